"""The exchange layout of the pipelined 2048-point cols kernels
(fft_gb300/csrc/line_fft_pipe.cuh), restated: element j of line c at float
(j + j/8) * C + c, for tiles of C = 8 and of C = 4 lines.  Checked here for every warp and element: the rows it
gives are the Stockham positions of the stage scatter (stage() in
line_fft.cuh) written as a per-thread base plus a compile-time offset, the
map is injective and fits kPipeRows rows, and every access of a warp (32/C
consecutive threads t x C lines) touches 32 distinct banks."""
import numpy as np
import pytest

L, T, E = 2048, 128, 16
ROWS = L + L // 8                       # kPipeRows
RADIX = [(8, 1), (16, 8)]               # (R, NS) of the two stages that scatter


def row(j):
    return j + (j >> 3)


def stockham_pos(s, t, e):
    R, NS = RADIX[s]
    B = E // R
    u, r = e % B, e // B
    b = t + T * u
    return (b // NS) * NS * R + (b % NS) + r * NS


# the kernel's base/offset forms (pipe_wbase, pipe_woff, pipe_gbase, pipe_goff)
def wrow(s, t, e):
    return (9 * t + 1152 * (e % 2) + e // 2) if s == 0 else (144 * (t >> 3) + (t & 7) + 9 * e)


def grow(t, e):
    return t + (t >> 3) + 144 * e


def test_forms_match_the_stockham_positions():
    for t in range(T):
        for e in range(E):
            assert grow(t, e) == row(t + T * e)
            for s in range(2):
                assert wrow(s, t, e) == row(stockham_pos(s, t, e))


def test_every_position_is_written_once_per_stage():
    for s in range(2):
        pos = sorted(stockham_pos(s, t, e) for t in range(T) for e in range(E))
        assert pos == list(range(L))


@pytest.mark.parametrize("C", [8, 4])
def test_injective_and_in_bounds(C):
    idx = np.array([row(j) * C + c for j in range(L) for c in range(C)])
    assert len(set(idx.tolist())) == L * C and idx.max() < ROWS * C


@pytest.mark.parametrize("C", [8, 4])
def test_one_wavefront_per_access(C):
    # a warp covers 32 / C consecutive threads t (lanes C apart share a line)
    W = 32 // C
    for w in range(T * C // 32):
        ts = [W * w + k for k in range(W)]
        for e in range(E):
            for f in (lambda t: grow(t, e), lambda t: wrow(0, t, e), lambda t: wrow(1, t, e)):
                banks = {(f(t) * C + c) % 32 for t in ts for c in range(C)}
                assert len(banks) == 32, (w, e)


@pytest.mark.parametrize("C", [8, 4])
def test_raw_tile_reads_one_wavefront(C):
    # the raw tile is [rows][C] per plane (as is the bulk stores' staging);
    # the C2R pre-pass also reads the mirror rows L - i
    W = 32 // C
    for w in range(T * C // 32):
        ts = [W * w + k for k in range(W)]
        for e in range(E):
            for f in (lambda t: t + T * e, lambda t: (L - (t + T * e)) % L):
                banks = {(f(t) * C + c) % 32 for t in ts for c in range(C)}
                assert len(banks) == 32
