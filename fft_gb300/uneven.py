"""The mixed ("uneven") batch workload: many power-of-two transforms of
different sizes, dimensionalities and kinds run as one queue.

``uneven_batch(count, seed)`` draws the transform list: 75% 1D with
log2 n ~ U{6..18}, 20% 2D with each side's log2 ~ U{6..11}, 5% 3D with each
side's log2 ~ U{5..8} (sides drawn independently); 50/50 complex/real and
50/50 forward/inverse.  ``allocate(items, dev)`` carves every transform's
arrays out of one device allocation and fills the inputs with standard
normal values; ``descs(...)`` returns the tuples ``fft_gb300.Queue`` takes.
"""
import numpy as np


def uneven_batch(count=10000, seed=5, max_log1d=18, side2d=(6, 11), side3d=(5, 8)):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        u = rng.random()
        if u < 0.75:
            dims = [1 << int(rng.integers(6, max_log1d + 1))]
        elif u < 0.95:
            dims = [1 << int(rng.integers(side2d[0], side2d[1] + 1)) for _ in range(2)]
        else:
            dims = [1 << int(rng.integers(side3d[0], side3d[1] + 1)) for _ in range(3)]
        real = rng.random() < 0.5
        inverse = rng.random() < 0.5
        out.append((("r" if real else "c") + ("i" if inverse else ""), dims))
    return out


def elems(kind, dims):
    """(input elements, output elements) per array of one transform."""
    n = int(np.prod(dims))
    h = (dims[0] // 2 + 1) * (n // dims[0])
    return {"c": (n, n), "ci": (n, n), "r": (n, h), "ri": (h, n)}[kind]


def flops(kind, dims):
    n = int(np.prod(dims))
    return (5.0 if kind in ("c", "ci") else 2.5) * n * np.log2(n)


def bytes_moved(kind, dims):
    """Algorithmic bytes: one read of the input and one write of the output."""
    i, o = elems(kind, dims)
    ci = kind != "r"
    co = kind != "ri"
    return 4 * i * (2 if ci else 1) + 4 * o * (2 if co else 1)


def allocate(items, dev, seed=0, io_regions=False):
    """One device allocation holding every transform's input and output
    arrays (each 256-byte aligned), inputs standard normal.  With io_regions
    every input array comes first and every output array after them, so one
    copy moves all inputs and one all outputs; the boundary (in floats) is
    returned as a third value."""
    import torch
    align = 64
    offs = []
    total = 0
    pad = lambda m: (m + align - 1) // align * align
    if io_regions:
        for kind, dims in items:
            i, _ = elems(kind, dims)
            rec = []
            for m in (i, i if kind != "r" else 0):
                rec.append(total if m else None)
                total += pad(m)
            offs.append(rec)
        boundary = total
        for (kind, dims), rec in zip(items, offs):
            _, o = elems(kind, dims)
            for m in (o, o if kind != "ri" else 0):
                rec.append(total if m else None)
                total += pad(m)
    else:
        for kind, dims in items:
            i, o = elems(kind, dims)
            rec = []
            for m in (i, i if kind != "r" else 0, o, o if kind != "ri" else 0):
                rec.append(total if m else None)
                total += pad(m)
            offs.append(rec)
        boundary = None
    buf = torch.empty(total, dtype=torch.float32, device=dev)
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    buf.normal_(generator=g)
    return (buf, offs, boundary) if io_regions else (buf, offs)


def descs(items, buf, offs):
    base = buf.data_ptr()
    out = []
    for (kind, dims), rec in zip(items, offs):
        p = [None if r is None else base + 4 * r for r in rec]
        out.append((kind, dims, p[0], p[1], p[2], p[3]))
    return out
