"""The exchange layouts of the pipelined cols kernels
(fft_gb300/csrc/line_fft_pipe.cuh), restated: element j of line c at float
row(j) * C + c, with row(j) = j + j/8 for 2048-point lines (tiles of C = 8 or
4 lines) and j + j/4 for 1024-point lines (C = 8).  Checked here for every
warp and element: the rows they give are the Stockham positions of the
stage scatter (stage() in line_fft.cuh) written as a per-thread base plus a
compile-time offset, every position is written once per stage, the map is
injective and fits pipe_rows rows, and every access of a warp (32/C
consecutive threads t x C lines) touches 32 distinct banks."""
import numpy as np
import pytest

E = 16
# LOGL: (L, T, radices (R, NS) of the two scattering stages, pad shift)
SCHED = {11: (2048, 128, [(8, 1), (16, 8)], 3), 10: (1024, 64, [(4, 1), (16, 4)], 2)}
CASES = [(11, 8), (11, 4), (10, 8)]


def row(logl, j):
    return j + (j >> SCHED[logl][3])


def rows_total(logl):
    L, _, _, sh = SCHED[logl]
    return L + (L >> sh)          # pipe_rows


def stockham_pos(logl, s, t, e):
    L, T, rad, _ = SCHED[logl]
    R, NS = rad[s]
    B = E // R
    u, r = e % B, e // B
    b = t + T * u
    return (b // NS) * NS * R + (b % NS) + r * NS


# the kernel's base/offset forms (pipe_wbase, pipe_woff, pipe_gbase, pipe_goff)
def wrow(logl, s, t, e):
    if logl == 11:
        return (9 * t + 1152 * (e % 2) + e // 2) if s == 0 else (144 * (t >> 3) + (t & 7) + 9 * e)
    return (5 * t + 320 * (e % 4) + e // 4) if s == 0 else (80 * (t >> 2) + (t & 3) + 5 * e)


def grow(logl, t, e):
    return (t + (t >> 3) + 144 * e) if logl == 11 else (t + (t >> 2) + 80 * e)


@pytest.mark.parametrize("logl", [11, 10])
def test_forms_match_the_stockham_positions(logl):
    L, T, _, _ = SCHED[logl]
    for t in range(T):
        for e in range(E):
            assert grow(logl, t, e) == row(logl, t + T * e)
            for s in range(2):
                assert wrow(logl, s, t, e) == row(logl, stockham_pos(logl, s, t, e))


@pytest.mark.parametrize("logl", [11, 10])
def test_every_position_is_written_once_per_stage(logl):
    L, T, _, _ = SCHED[logl]
    for s in range(2):
        pos = sorted(stockham_pos(logl, s, t, e) for t in range(T) for e in range(E))
        assert pos == list(range(L))


@pytest.mark.parametrize("logl,C", CASES)
def test_injective_and_in_bounds(logl, C):
    L = SCHED[logl][0]
    idx = np.array([row(logl, j) * C + c for j in range(L) for c in range(C)])
    assert len(set(idx.tolist())) == L * C and idx.max() < rows_total(logl) * C


@pytest.mark.parametrize("logl,C", CASES)
def test_one_wavefront_per_access(logl, C):
    # a warp covers 32 / C consecutive threads t (lanes C apart share a line)
    L, T, _, _ = SCHED[logl]
    W = 32 // C
    for w in range(T * C // 32):
        ts = [W * w + k for k in range(W)]
        for e in range(E):
            for f in (lambda t: grow(logl, t, e), lambda t: wrow(logl, 0, t, e), lambda t: wrow(logl, 1, t, e)):
                banks = {(f(t) * C + c) % 32 for t in ts for c in range(C)}
                assert len(banks) == 32, (w, e)


@pytest.mark.parametrize("logl,C", CASES)
def test_raw_tile_reads_one_wavefront(logl, C):
    # the raw tile is [rows][C] per plane (as is the bulk stores' staging);
    # the C2R pre-pass also reads the mirror rows L - i
    L, T, _, _ = SCHED[logl]
    W = 32 // C
    for w in range(T * C // 32):
        ts = [W * w + k for k in range(W)]
        for e in range(E):
            for f in (lambda t: t + T * e, lambda t: (L - (t + T * e)) % L):
                banks = {(f(t) * C + c) % 32 for t in ts for c in range(C)}
                assert len(banks) == 32
