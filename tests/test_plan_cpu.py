"""Host logic without a GPU: the launch plans the library builds (described
by afft_gb300_plan_describe, no device calls) are executed by the numpy plan
emulator, which checks every address against its buffer and every in-place
launch for cross-CTA hazards, and must reproduce the FP64 oracle."""
import numpy as np
import pytest

import fft_gb300 as G
from oracle import oracle as O
from plan_emulator import describe, run

SHAPES = [[1], [2], [4], [16], [32], [256], [4096], [16384], [32768], [1 << 16], [1 << 19], [1 << 20], [1 << 21],
          [2, 2], [4, 8], [64, 4], [8, 4096], [4096, 8], [16, 2048, 2], [8192, 4], [2, 16384],
          [2, 4, 8], [16, 16, 16], [4, 4, 4, 4], [2, 2, 2, 2, 2], [1, 32, 1], [4, 1, 1, 8],
          # plane-fused last two axes (2^12 .. 2^14-point planes)
          [4, 64, 64], [32, 128], [2, 256, 32], [2, 2, 32, 512]]


def _inputs(kind, dims, batch, seed):
    n = int(np.prod(dims))
    h = O.half_elems(dims)
    m = (n if kind in ("c", "ci", "r") else h) * batch
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(m)
    b = None if kind == "r" else rng.standard_normal(m)
    return a, b


def _expected(kind, dims, batch, a, b):
    n = int(np.prod(dims))
    h = O.half_elems(dims)
    m_in = n if kind in ("c", "ci", "r") else h
    outs = []
    for j in range(batch):
        s = slice(j * m_in, (j + 1) * m_in)
        outs.append(O.oracle64(kind, dims, a[s], None if b is None else b[s]))
    if kind == "ri":
        return np.concatenate(outs)
    return np.concatenate([o[0] for o in outs]), np.concatenate([o[1] for o in outs])


@pytest.mark.parametrize("dims", SHAPES, ids=lambda d: "x".join(map(str, d)))
@pytest.mark.parametrize("kind", ["c", "ci", "r", "ri"])
def test_plan_emulation(kind, dims):
    n = int(np.prod(dims))
    if kind in ("r", "ri") and n == 1:
        dims = [1]
    for fmt in (G.afft_split, G.afft_interleaved):
        for batch in (1, 3):
            if n * batch > (1 << 20) and batch > 1:
                continue
            desc = describe(kind, dims, batch, fmt)
            a, b = _inputs(kind, dims, batch, n + batch)
            got = run(desc, a, b)
            ref = _expected(kind, dims, batch, a, b)
            assert O.rel_l2(got, ref) < 1e-12, (kind, dims, batch, fmt)


@pytest.mark.parametrize("kind,fmt", [("c", G.afft_split), ("ci", G.afft_interleaved), ("ri", G.afft_split)])
def test_plan_emulation_three_pass_2p22(kind, fmt):
    # the 2^22-point complex axis in three passes (256, then a strided
    # four-step through a second scratch region); one format per kind keeps
    # the CPU time to seconds
    dims = [1 << 22]
    desc = describe(kind, dims, 1, fmt)
    a, b = _inputs(kind, dims, 1, 22)
    got = run(desc, a, b)
    assert O.rel_l2(got, _expected(kind, dims, 1, a, b)) < 1e-12


def test_launch_counts():
    # one pass while a line fits one CTA, two (four-step) beyond
    assert len(describe("c", [4096], 16384)["ops"]) == 1
    assert len(describe("c", [1 << 16], 4)["ops"]) == 2
    assert len(describe("c", [256, 256, 256])["ops"]) == 3
    assert len(describe("r", [4096, 4096])["ops"]) == 2
    # long 1D real: the real post-pass rides in pass B, the pre-pass of the
    # inverse in pass A
    assert len(describe("r", [1 << 20], 2)["ops"]) == 2
    assert len(describe("ri", [1 << 19], 2)["ops"]) == 2
    assert len(describe("ri", [1 << 20], 2)["ops"]) == 3   # standalone pre-pass measured faster there
    # (the standalone pre-pass, then the complex 2^21 axis in three passes)
    assert len(describe("ri", [1 << 22], 1)["ops"]) == 4
    # complex axes of 2^21 and 2^22 points: three passes
    assert len(describe("c", [1 << 22], 1)["ops"]) == 3
    assert len(describe("ci", [1 << 21], 2)["ops"]) == 3


# FP64 plans (afft_64_*): rows up to 2^13 points, cols up to 2^11, standalone
# real passes beyond one CTA; the same emulation and oracle bar
SHAPES64 = [[1], [2], [8], [16], [512], [8192], [16384], [32768], [1 << 17], [1 << 22],
            [2, 2], [4096, 4], [8, 4096], [2048, 2], [16, 2048, 2], [2, 16384], [2, 4, 8], [4, 1, 1, 8]]


@pytest.mark.parametrize("dims", SHAPES64, ids=lambda d: "x".join(map(str, d)))
@pytest.mark.parametrize("kind", ["c", "ci", "r", "ri"])
def test_plan_emulation_f64(kind, dims):
    n = int(np.prod(dims))
    for fmt in (G.afft_split, G.afft_interleaved):
        for batch in (1, 3):
            if n * batch > (1 << 20) and batch > 1:
                continue
            desc = describe(kind, dims, batch, fmt | G.FORM_F64)
            assert desc["f64"] == 1
            for op in desc["ops"]:
                if op["type"] == "line":
                    assert op["lk"] in (0, 1, 2) and op["halves"] == 1 and op["tc"] == 0, op
            a, b = _inputs(kind, dims, batch, n + batch)
            got = run(desc, a, b)
            ref = _expected(kind, dims, batch, a, b)
            assert O.rel_l2(got, ref) < 1e-12, (kind, dims, batch, fmt)


def test_launch_counts_f64():
    F = G.FORM_F64
    assert len(describe("c", [8192], 4, F)["ops"]) == 1
    assert len(describe("c", [16384], 4, F)["ops"]) == 2
    assert len(describe("r", [16384], 4, F)["ops"]) == 1          # 8192 complex points, one CTA
    assert len(describe("r", [32768], 4, F)["ops"]) == 3          # four-step + standalone post-pass
    assert len(describe("ri", [32768], 4, F)["ops"]) == 3         # standalone pre-pass + four-step
    d = describe("r", [4096, 4096], 1, F)
    assert len(d["ops"]) == 2 and d["ops"][0]["logl"] == 11 and d["ops"][0]["C"] == 4
    assert describe("c", [256, 256, 256], 1, F)["scratch_elems"] == 0
    assert len(describe("c", [1 << 22], 1, F)["ops"]) == 2


def test_uneven_io_regions_layout():
    # the mixed batch's end-to-end leg copies all inputs and all outputs in
    # one piece each: inputs below the boundary, outputs above, disjoint,
    # every array 256-byte aligned
    import torch
    from fft_gb300 import uneven as U
    items = U.uneven_batch(300, seed=3, max_log1d=12, side2d=(4, 6), side3d=(3, 4))
    buf, offs, boundary = U.allocate(items, "cpu", io_regions=True)
    spans = []
    for (kind, dims), rec in zip(items, offs):
        i, o = U.elems(kind, dims)
        sizes = (i, i if kind != "r" else 0, o, o if kind != "ri" else 0)
        for slot, (off, m) in enumerate(zip(rec, sizes)):
            if not m:
                assert off is None
                continue
            assert off % 64 == 0
            assert (off + m <= boundary) if slot < 2 else (off >= boundary)
            spans.append((off, off + m))
    spans.sort()
    assert all(a[1] <= b[0] for a, b in zip(spans, spans[1:]))
    assert spans[-1][1] <= buf.numel()
    # the same transforms and descriptors as the interleaved layout
    assert len(U.descs(items, buf, offs)) == len(items)


def test_cols_pair_kernels_where_pairs_are():
    # cols passes over interleaved pairs (the real transforms' interleaved
    # views, the interleaved format) take the 8-byte-pair kernels; split
    # data keeps the plain ones
    units = lambda k, d, b, f=G.afft_split: [(o["cols"], o["tstore"], o["unit"]) for o in describe(k, d, b, f)["ops"]
                                            if o["type"] == "line"]
    assert units("r", [1 << 20], 4) == [(1, 1, 3), (1, 0, 1)]             # pairs: real input, scratch, scratch
    assert units("ri", [1 << 21], 4)[-1] == (1, 0, 2)                     # pass B writes them
    assert units("c", [65536], 4, G.afft_interleaved) == [(1, 1, 1), (1, 0, 2)]
    assert units("c", [256, 256, 256], 1, G.afft_interleaved)[1:] == [(1, 0, 3), (1, 0, 3)]
    assert all(u == 0 for c, _, u in units("c", [65536], 4) + units("c", [64, 64, 64], 1) if c)


def test_rows_real_pair_kernels():
    # rows C2R passes of 256 points and more write the real side as float2
    # pairs, rows R2C passes of 4096 points and more read it so; shorter
    # lines keep the strided or warp-staged accesses
    rows = lambda k, d, b: [(o["logl"], o["lk"], o["unit"]) for o in describe(k, d, b)["ops"]
                            if o["type"] == "line" and not o["cols"]]
    assert rows("r", [8192], 64) == [(12, 1, 2)]
    assert rows("ri", [1 << 15], 4) == [(14, 2, 2)]
    assert rows("r", [256], 64) == [(7, 1, 0)]
    assert rows("r", [4096], 64) == [(11, 1, 0)]
    assert rows("ri", [512], 8) == [(8, 2, 2)]
    assert rows("ri", [256], 8) == [(7, 2, 0)]
    assert all(u != 2 for _, _, u in rows("r", [4096, 4096], 1))        # N-D rows are complex


def test_long_real_scratch_is_pairs():
    # the long 1D real transforms keep their four-step scratch (and the long
    # inverse's standalone Z') as re,im pairs: every access on both sides of
    # it is an 8-byte pair, and the scratch size is unchanged
    def ops(k, d, b):
        return [(o["type"], o.get("cols"), o.get("tstore"), o.get("lk"), o.get("unit"))
                for o in describe(k, d, b)["ops"]]
    assert ops("r", [1 << 19], 8) == [("line", 1, 1, 0, 3), ("line", 1, 0, 4, 1)]
    assert ops("ri", [1 << 19], 8) == [("line", 1, 1, 5, 2), ("line", 1, 0, 0, 3)]
    assert ops("ri", [1 << 21], 2) == [("real", None, None, None, None), ("line", 1, 1, 0, 1),
                                      ("line", 1, 0, 0, 2)]
    for k, d, b in (("r", [1 << 19], 8), ("ri", [1 << 19], 8)):
        plan = describe(k, d, b)
        s = [o for o in plan["ops"] if o["type"] == "line"]
        scr = s[0]["out"]                                   # pass A's output, pass B's input
        assert scr["re"][0] == scr["im"][0] and scr["im"][1] == scr["re"][1] + 1 and scr["es"] == 2
        assert plan["scratch_elems"] >= 2 * b * (d[0] // 2)
    d = describe("ri", [1 << 21], 2)["ops"][0]["out"]       # Z' of the standalone pre-pass
    assert d["im"][1] == d["re"][1] + 1 and d["es"] == 2


@pytest.mark.parametrize("kind,dims,batch,expect", [
    ("c", [256, 256, 256], 1, [(0, 0), (1, 0), (1, 0)]),   # rows, then two 256-point cols passes by TMA
    ("c", [65536], 64, [(1, 0), (1, 0)]),                  # four-step: pass A (transposing store) and pass B by TMA
    ("c", [1024, 1024], 4, [(0, 0), (1, 1)]),              # 1024-point cols pass pipelined (taken at launch
                                                           # from two tiles per CTA slot)
    ("ri", [4096, 4096], 1, [(0, 0), (1, 1)]),             # the 2048-point C2R pass pipelined
    ("r", [4096, 4096], 1, [(0, 0), (0, 0)]),              # the split 2048-point R2C pass keeps LSU loads (measured)
    ("c", [2048, 2048], 2, [(0, 0), (1, 1)]),              # the 2048-point C2C cols pass pipelined
    ("c", [4096], 64, [(0, 0)]),                           # rows passes load through the LSU
], ids=str)
def test_tma_fed_passes(kind, dims, batch, expect):
    """Which passes take the TMA-fed cols kernels, as (tma, pipe): the plan's
    default choice.  pipe: the persistent pipelined form of the 1024- and
    2048-point cols passes.  At launch the LSU kernel of the same shape runs instead
    where the bound arrays miss the TMA alignment rules."""
    d = describe(kind, dims, batch)
    got = [(op.get("tma", 0), op.get("pipe", 0)) for op in d["ops"] if op["type"] == "line"]
    assert got == expect, (got, d["ops"])


@pytest.mark.parametrize("kind,dims,batch,expect", [
    ("c", [512, 512], 64, [0, 1]),             # 512-point complex cols pass: TMA stores
    ("ci", [8, 512, 64], 2, [0, 1, 0]),        # the 512-point middle axis; the 8-point one has no TMA form
    ("c", [1 << 18], 4, [0, 1]),               # 512 x 512 four-step: pass B (pass A: the transposing store,
                                               # TMA loads only)
    ("c", [256, 256, 256], 1, [0, 0, 0]),      # 256-point complex cols passes: per-thread stores (measured)
    ("ri", [512, 512], 64, [0, 1]),            # 256-point C2R cols pass: TMA stores
    ("ri", [1024, 1024], 16, [0, 0]),          # 512-point C2R cols pass: per-thread stores (measured)
    ("r", [512, 512], 64, [0, 0]),             # R2C cols passes: per-thread stores
    ("c", [2048, 2048], 2, [0, 0]),            # the pipelined passes store by TMA on their own
    ("c", [1024, 1024], 2, [0, 1]),            # 1024 points: the one-tile form below the pipelined
                                               # kernel's tile threshold stores by TMA too
    ("ri", [2048, 2048], 1, [0, 0]),           # 1024-point C2R one-tile form: per-thread stores (measured)
], ids=str)
def test_tma_store_passes(kind, dims, batch, expect):
    """Which passes have the one-tile TMA kernel that also stores its tile by
    TMA (line_fft_tma_bulk), taken at launch when both the input and the
    output maps encode (and, for 1024-point passes, when the tiles are too
    few for the pipelined kernel)."""
    d = describe(kind, dims, batch)
    got = [op.get("tma_store", 0) for op in d["ops"] if op["type"] == "line"]
    assert got == expect, (got, d["ops"])
