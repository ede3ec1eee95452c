"""CPU emulation of a libafft_gb300 plan, for checking the host logic without a
GPU.

``describe(kind, dims, batch, fmt)`` returns the library's own JSON
description of the kernel launches a plan issues (afft_gb300_plan_describe,
no device calls).  ``run(desc, ...)`` executes those launches on float64
numpy buffers: every launch gathers and scatters through exactly the address
formulas the kernels use (off(q) = (q >> qshift) * hi + (q & qmask) * lo,
element stride es), applies the math each kernel type computes (a length-L
DFT per line with the four-step twiddle, the fused real post/pre pass, the
standalone real pass, the packing copy), and checks on the way that

* every address lies inside its buffer,
* no address is written twice within a launch,
* when a launch reads and writes the same buffer, no CTA writes an address
  that another CTA reads (the kernels rely on this to run in place).

The Stockham stages inside a kernel are not emulated (a line's DFT is taken
with numpy); those are checked on the GPU against the oracle.
"""
import ctypes
import json

import numpy as np

import fft_gb300 as G

SRC_RE, SRC_IM, DST_RE, DST_IM, SCR = range(5)


def describe(kind, dims, batch=1, fmt=0):
    """fmt may carry fft_gb300.FORM_TC."""
    L = G.lib()
    f = L.afft_gb300_plan_describe
    f.restype = ctypes.c_size_t
    f.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int,
                  ctypes.c_char_p, ctypes.c_size_t]
    k = G.KINDS[kind] if isinstance(kind, str) else kind
    arr = (ctypes.c_size_t * max(1, len(dims)))(*dims)
    n = f(k, len(dims), arr, batch, fmt, None, 0)
    if n == 0:
        raise ValueError(G.last_error())
    buf = ctypes.create_string_buffer(n)
    f(k, len(dims), arr, batch, fmt, buf, n)
    return json.loads(buf.value.decode())


def w(m, n):
    """exp(-2 pi i m / n) in float64."""
    return np.exp(-2j * np.pi * (np.asarray(m, np.float64) % n) / n)


class Buffers:
    def __init__(self, sizes):
        self.b = [None if s is None else np.full(s, np.nan) for s in sizes]

    def addr(self, ref, idx):
        buf, off = ref
        a = off + idx
        arr = self.b[buf]
        assert arr is not None, "launch touches an unbound buffer %d" % buf
        assert a.min() >= 0 and a.max() < arr.size, "out of bounds on buffer %d: [%d, %d] of %d" % (
            buf, a.min(), a.max(), arr.size)
        return buf, a


def line_offsets(spec, q):
    return (q >> spec["qshift"]) * spec["hi"] + (q & spec["qmask"]) * spec["lo"]


class Access:
    """Records reads/writes of one launch, per buffer, with the CTA id."""

    def __init__(self):
        self.reads = {}
        self.writes = {}

    def note(self, table, buf, addrs, cta):
        addrs = np.asarray(addrs)
        cta = np.broadcast_to(np.asarray(cta), addrs.shape)
        table.setdefault(buf, []).append((addrs.reshape(-1), cta.reshape(-1)))

    def check(self):
        for buf, lst in self.writes.items():
            a = np.concatenate([x for x, _ in lst])
            c = np.concatenate([y for _, y in lst])
            u, cnt = np.unique(a, return_counts=True)
            assert cnt.max() == 1, "address written twice in one launch (buffer %d)" % buf
            if buf in self.reads:
                ra = np.concatenate([x for x, _ in self.reads[buf]])
                rc = np.concatenate([y for _, y in self.reads[buf]])
                order = np.argsort(a)
                a_s, c_s = a[order], c[order]
                pos = np.searchsorted(a_s, ra)
                hit = (pos < a_s.size)
                hit[hit] &= a_s[pos[hit]] == ra[hit]
                bad = hit.copy()
                bad[hit] = c_s[pos[hit]] != rc[hit]
                assert not bad.any(), "CTA reads an address another CTA writes (buffer %d)" % buf


def _gather(B, acc, spec, q, idx, cta):
    ore = line_offsets(spec, q)[:, None] + idx[None, :] * spec["es"]
    bre, are = B.addr(spec["re"], ore)
    bim, aim = B.addr(spec["im"], ore)
    ctas = np.broadcast_to(cta[:, None], ore.shape)
    acc.note(acc.reads, bre, are, ctas)
    acc.note(acc.reads, bim, aim, ctas)
    return B.b[bre][are] + 1j * B.b[bim][aim]


def _scatter(B, acc, spec, q, idx, cta, val):
    """cta: per line, or per (line, element) when a line is split over CTAs."""
    ore = line_offsets(spec, q)[:, None] + idx[None, :] * spec["es"]
    bre, are = B.addr(spec["re"], ore)
    bim, aim = B.addr(spec["im"], ore)
    ctas = cta if cta.ndim == 2 else np.broadcast_to(cta[:, None], ore.shape)
    acc.note(acc.writes, bre, are, ctas)
    acc.note(acc.writes, bim, aim, ctas)
    return (bre, are, val.real), (bim, aim, val.imag)


def _scatter_re(B, acc, spec, q, idx, cta, val):
    ore = line_offsets(spec, q)[:, None] + idx[None, :] * spec["es"]
    bre, are = B.addr(spec["re"], ore)
    acc.note(acc.writes, bre, are, np.broadcast_to(cta[:, None], ore.shape))
    return (bre, are, val.real),


def run_op(B, op):
    acc = Access()
    pending = []
    t = op["type"]
    if t == "line" and op.get("plane"):
        # plane-fused pass: plane q (D1 rows x D2 points, dense from its
        # line offset), C / D1 planes per CTA, a 2D transform
        D1, D2 = 1 << op["plane"], 1 << op["logl"]
        n = op["nlines"] // D1
        q = np.arange(n, dtype=np.int64)
        cta = q // (op["C"] // D1)
        assert op["grid"] == -(-n // (op["C"] // D1))
        m = np.arange(D1 * D2)
        x = _gather(B, acc, op["in"], q, m, cta).reshape(n, D1, D2)
        y = np.fft.ifft2(x) * (D1 * D2) if op["inverse"] else np.fft.fft2(x)
        pending += _scatter(B, acc, op["out"], q, m, cta, y.reshape(n, D1 * D2))
    elif t == "line":
        L = 1 << op["logl"]
        q = np.arange(op["nlines"], dtype=np.int64)
        halves = op.get("halves", 1)
        cta = q // op["C"] * halves
        lk = op["lk"]
        if lk == 4:  # four-step pass B with the 1D real post-pass over mirrored column pairs
            L1, C = op["pcols"], op["C"]
            nt = op["nlines"] // L1
            k1 = q % L1
            H = C // 2
            tile = np.where(k1 < L1 // 2, k1 // H, np.where(k1 == L1 // 2, 0, (L1 - k1) // H))
            cta = (q // L1) * (L1 // C) + tile
            x = _gather(B, acc, op["in"], q, np.arange(L), cta)
            Xf = np.fft.fft(x, axis=1)
            N = L1 * L
            Z = Xf.reshape(nt, L1, L).transpose(0, 2, 1).reshape(nt, N)   # Z[o][k1 + L1 k2]
            k = np.arange(N + 1)
            s0 = Z[:, k % N]
            s1 = Z[:, (N - k) % N]
            X = (s0 + np.conj(s1)) / 2 - 0.5j * w(k, 2 * N) * (s0 - np.conj(s1))
            X[:, 0] = Z[:, 0].real + Z[:, 0].imag
            X[:, N] = Z[:, 0].real - Z[:, 0].imag
            out = X[:, :N].reshape(nt, L, L1).transpose(0, 2, 1).reshape(nt * L1, L)
            pending += _scatter(B, acc, op["out"], q, np.arange(L), cta, out)
            q0 = np.arange(nt, dtype=np.int64) * L1
            pending += _scatter(B, acc, op["out"], q0, np.array([L]), cta[q0], X[:, N:N + 1])
        elif lk == 5:  # inverse four-step pass A with the 1D real pre-pass over mirrored column pairs
            L2c, C = op["pcols"], op["C"]
            nt = op["nlines"] // L2c
            t2 = q % L2c
            H = C // 2
            tile = np.where(t2 < L2c // 2, t2 // H, np.where(t2 == L2c // 2, 0, (L2c - t2) // H))
            cta = (q // L2c) * (L2c // C) + tile
            N = L2c * L
            x = _gather(B, acc, op["in"], q, np.arange(L), cta)            # X[t2 + L2 t1]
            xl = _gather(B, acc, op["in"], np.arange(nt, dtype=np.int64) * L2c, np.array([L]),
                         cta[np.arange(nt) * L2c])                          # X[N]
            X = np.concatenate([x.reshape(nt, L2c, L).transpose(0, 2, 1).reshape(nt, N), xl], axis=1)
            k = np.arange(N)
            s0, s1 = X[:, k], X[:, N - k]
            Zp = (s0 + np.conj(s1)) - 1j * (np.conj(s1) - s0) * np.conj(w(k, 2 * N))
            Zp[:, 0] = (X[:, 0].real + X[:, N].real) + 1j * (X[:, 0].real - X[:, N].real)
            z = Zp.reshape(nt, L, L2c).transpose(0, 2, 1).reshape(nt * L2c, L)   # line (o, t2), element t1
            Xf = np.fft.ifft(z, axis=1) * L
            tw = w(t2[:, None] * np.arange(L)[None, :], op["tw_n"])
            Xf = Xf * np.conj(tw)
            pending += _scatter(B, acc, op["out"], q, np.arange(L), cta, Xf)
        elif lk == 2:  # C2R: reads L+1 bins
            X = _gather(B, acc, op["in"], q, np.arange(L + 1), cta)
            i = np.arange(L)
            s0, s1 = X[:, i], X[:, L - i]
            wv = w(i, 2 * L)
            a = s0 + np.conj(s1)
            b = (np.conj(s1) - s0) * np.conj(wv)
            Zp = a - 1j * b
            Zp[:, 0] = (X[:, 0].real + X[:, L].real) + 1j * (X[:, 0].real - X[:, L].real)
            z = np.fft.ifft(Zp, axis=1) * L
            pending += _scatter(B, acc, op["out"], q, np.arange(L), cta, z)
        else:
            x = _gather(B, acc, op["in"], q, np.arange(L), cta)
            Xf = np.fft.ifft(x, axis=1) * L if op["inverse"] else np.fft.fft(x, axis=1)
            if op["tw_n"]:
                col = (q >> op["tw_qshift"]) & op["tw_qmask"]
                tw = w(col[:, None] * np.arange(L)[None, :], op["tw_n"])
                Xf = Xf * (np.conj(tw) if op["inverse"] else tw)
            if lk == 0:
                pending += _scatter(B, acc, op["out"], q, np.arange(L), cta, Xf)
            else:  # R2C post pass: L+1 bins
                k = np.arange(L + 1)
                s0 = Xf[:, k % L]
                s1 = Xf[:, (L - k) % L]
                out = (s0 + np.conj(s1)) / 2 - 0.5j * w(k, 2 * L) * (s0 - np.conj(s1))
                out[:, 0] = Xf[:, 0].real + Xf[:, 0].imag
                out[:, L] = Xf[:, 0].real - Xf[:, 0].imag
                if halves == 2:
                    # both CTAs of a tile read the whole line; CTA h writes
                    # the bins of parity h
                    _gather(B, acc, op["in"], q, np.arange(L), cta + 1)
                    cta = cta[:, None] + (k[None, :] & 1)
                pending += _scatter(B, acc, op["out"], q, k, cta, out)
    elif t == "real":
        L = op["L"]
        q = np.arange(op["nlines"], dtype=np.int64)
        cta = q  # one thread per pair: reads and writes stay in a thread
        # the kernel's k = 0 thread also reads slot L in both directions
        X = _gather(B, acc, op["in"], q, np.arange(L + 1), cta)
        k = np.arange(L + 1) if not op["inverse"] else np.arange(L)
        if not op["inverse"]:
            Z = X[:, :L]
            s0, s1 = Z[:, k % L], Z[:, (L - k) % L]
            out = (s0 + np.conj(s1)) / 2 - 0.5j * w(k, 2 * L) * (s0 - np.conj(s1))
            out[:, 0] = Z[:, 0].real + Z[:, 0].imag
            out[:, L] = Z[:, 0].real - Z[:, 0].imag
        else:
            s0, s1 = X[:, k], X[:, L - k]
            out = (s0 + np.conj(s1)) - 1j * (np.conj(s1) - s0) * np.conj(w(k, 2 * L))
            out[:, 0] = (X[:, 0].real + X[:, L].real) + 1j * (X[:, 0].real - X[:, L].real)
        pending += _scatter(B, acc, op["out"], q, k, cta, out)
    elif t == "copy":
        q = np.arange(op["nlines"], dtype=np.int64)
        cta = np.zeros_like(q)  # copies never run in place
        x = _gather(B, acc, op["in"], q, np.arange(op["len"]), cta)
        pending += _scatter(B, acc, op["out"], q, np.arange(op["len"]), cta, x)
    elif t == "real1":
        q = np.arange(op["nlines"], dtype=np.int64)
        x = _gather(B, acc, op["in"], q, np.arange(1), q)
        if op["inverse"]:
            pending += _scatter_re(B, acc, op["out"], q, np.arange(1), q, x.real + 0j)
        else:
            pending += _scatter(B, acc, op["out"], q, np.arange(1), q, x.real + 0j)
    else:
        raise ValueError(t)
    acc.check()
    for buf, addr, val in pending:
        B.b[buf][addr] = val


def buffer_sizes(desc):
    kind, fmt, batch = desc["kind"], desc["format"], desc["batch"]
    ie, oe = desc["in_elems"] * batch, desc["out_elems"] * batch
    inter = fmt == 1
    cin = kind != 2      # complex input
    cout = kind != 3     # complex output
    src_re = ie * (2 if (inter and cin) else 1)
    src_im = ie if (cin and not inter) else None
    dst_re = oe * (2 if (inter and cout) else 1)
    dst_im = oe if (cout and not inter) else None
    return [src_re, src_im, dst_re, dst_im, desc["scratch_elems"] or None]


def run(desc, a, b=None):
    """Execute a described plan on inputs (split arrays); returns outputs as
    split arrays (re, im) or the real array."""
    B = Buffers(buffer_sizes(desc))
    kind, inter = desc["kind"], desc["format"] == 1
    if kind == 2:
        B.b[SRC_RE][:] = a
    elif inter:
        B.b[SRC_RE][0::2], B.b[SRC_RE][1::2] = a, b
    else:
        B.b[SRC_RE][:], B.b[SRC_IM][:] = a, b
    for op in desc["ops"]:
        run_op(B, op)
    if kind == 3:
        return B.b[DST_RE].copy()
    if inter:
        return B.b[DST_RE][0::2].copy(), B.b[DST_RE][1::2].copy()
    return B.b[DST_RE].copy(), B.b[DST_IM].copy()
