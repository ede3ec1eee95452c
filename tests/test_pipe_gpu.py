"""GPU parity of the persistent TMA-pipelined 1024- and 2048-point cols
passes (line_fft_pipe: C2C, and C2R; TMA output stores for C2C and the
1024-point C2R pass)
against the FP64 oracle:
tile counts below, at and above one per SM and not multiples of the grid,
in place and out of place, the four-step twiddle, and arrays off a 16-byte
boundary, where the one-tile-per-CTA kernels of the same shape run instead.
Also the one-tile 1024- and 512-point complex and 256-point C2R cols
passes that store their tile by TMA (line_fft_tma_bulk).
Tolerance: relative L2 <= 2e-6, as the other parity tests."""
import numpy as np
import pytest

import fft_gb300 as G
from oracle import oracle as O
from plan_emulator import describe

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
TOL = 2e-6


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def _pipe_ops(kind, dims, batch):
    return [op for op in describe(kind, dims, batch)["ops"] if op["type"] == "line" and op.get("pipe")]


def _c2c(kind, dims, batch, dev, pad=0, inplace=False, seed=0):
    from test_plane_gpu import _batch
    got, ref = _batch(kind, dims, batch, dev, inplace=inplace, pad=pad, seed=seed)
    return O.rel_l2(got, ref)


# tiles of 8 columns (one per transform of 8 columns): 1 tile, 151 / 152 /
# 153 tiles around one per SM, 2048 tiles (13.5 per SM)
@pytest.mark.parametrize("dims,batch", [([2048, 8], 1), ([2048, 8], 151), ([2048, 8], 152), ([2048, 8], 153),
                                        ([2048, 2048], 8), ([4, 2048, 64], 3)], ids=str)
@pytest.mark.parametrize("kind", ["c", "ci"])
def test_pipe_c2c_tile_counts(dev, kind, dims, batch):
    assert len(_pipe_ops(kind, dims, batch)) == 1
    for inplace in (False, True):
        err = _c2c(kind, dims, batch, dev, inplace=inplace, seed=dims[-1])
        assert err <= TOL, (kind, dims, batch, inplace, err)


@pytest.mark.parametrize("pad", [1, 2])
def test_pipe_c2c_unaligned_takes_the_one_tile_kernels(dev, pad):
    # the same plans on arrays off a 16-byte boundary: tma_tile refuses the
    # maps and the LSU kernel of the same shape runs
    for dims, batch in (([2048, 64], 2), ([2048, 2048], 1)):
        assert _c2c("c", dims, batch, dev, pad=pad, seed=pad) <= TOL, (dims, pad)


@pytest.mark.parametrize("kind,dims", [("c", [1 << 21, 8]), ("ci", [1 << 21, 4]), ("c", [1 << 22, 2])], ids=str)
def test_pipe_c2c_fourstep_twiddle(dev, kind, dims):
    # strided axes of 2^21 and 2^22 points: pass A of their four-step is a
    # 2048-point pipelined cols pass that applies the four-step twiddle
    ops = _pipe_ops(kind, dims, 1)
    assert ops and ops[0]["tw_n"] == dims[0], ops
    assert _c2c(kind, dims, 1, dev, seed=3) <= TOL, (kind, dims)


@pytest.mark.parametrize("dims,batch", [([4096, 8], 1), ([4096, 8], 153), ([4096, 4096], 2), ([4096, 64, 16], 3)],
                         ids=str)
def test_pipe_c2r_tile_counts(dev, dims, batch):
    # the real inverse's dim-0 pass (2048 complex points) pipelined
    from test_parity_gpu import check, inputs
    assert len(_pipe_ops("ri", dims, batch)) == 1
    n = int(np.prod(dims))
    h = O.half_elems(dims)
    rng = np.random.default_rng(batch)
    a = rng.standard_normal(h * batch).astype(np.float32)
    b = rng.standard_normal(h * batch).astype(np.float32)
    p = G.BatchPlan("ri", dims, batch)
    sr, si = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    d = torch.zeros(n * batch, dtype=torch.float32, device=dev)
    p.launch(sr, si, d, None)
    torch.cuda.synchronize()
    got = d.cpu().numpy()
    for j in range(batch):
        ref = O.oracle64("ri", dims, a[j * h:(j + 1) * h], b[j * h:(j + 1) * h])
        assert O.rel_l2(got[j * n:(j + 1) * n], ref) <= TOL, (dims, batch, j)


def test_pipe_c2r_unaligned(dev):
    from test_parity_gpu import check, inputs, run_plan
    for pad in (1, 3):
        a, b = inputs("ri", [4096, 64], pad)
        check("ri", [4096, 64], a, b, run_plan("ri", [4096, 64], a, b, dev, pad=pad))


# 1024-point tiles: the pipelined kernel from two tiles per CTA slot (608 on
# 152 SMs), the one-tile kernels below that; both sides of the threshold
@pytest.mark.parametrize("kind,dims,batch", [("c", [1024, 8], 1216), ("ci", [1024, 8], 700), ("c", [1024, 1024], 4),
                                             ("ci", [2, 1024, 512], 3)], ids=str)
def test_pipe_1024_c2c(dev, kind, dims, batch):
    assert len(_pipe_ops(kind, dims, batch)) == 1
    for inplace in (False, True):
        assert _c2c(kind, dims, batch, dev, inplace=inplace, seed=batch) <= TOL, (kind, dims, batch, inplace)


@pytest.mark.parametrize("dims,batch", [([2048, 8], 700), ([2048, 2048], 4), ([2048, 2048], 1)], ids=str)
def test_pipe_1024_c2r(dev, dims, batch):
    assert len(_pipe_ops("ri", dims, batch)) == 1
    n = int(np.prod(dims))
    h = O.half_elems(dims)
    rng = np.random.default_rng(batch + 1)
    a = rng.standard_normal(h * batch).astype(np.float32)
    b = rng.standard_normal(h * batch).astype(np.float32)
    p = G.BatchPlan("ri", dims, batch)
    d = torch.zeros(n * batch, dtype=torch.float32, device=dev)
    p.launch(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), d, None)
    torch.cuda.synchronize()
    got = d.cpu().numpy()
    for j in range(batch):
        ref = O.oracle64("ri", dims, a[j * h:(j + 1) * h], b[j * h:(j + 1) * h])
        assert O.rel_l2(got[j * n:(j + 1) * n], ref) <= TOL, (dims, batch, j)


# 512-point complex cols passes: TMA loads and TMA stores, one tile of 8
# columns per CTA (1 tile, 153 tiles, 64 tiles per transform, a 3D middle
# axis, the strided axis of a 2^18-point four-step with its twiddle)
@pytest.mark.parametrize("dims,batch", [([512, 8], 1), ([512, 8], 153), ([512, 512], 8), ([4, 512, 64], 3),
                                        ([64, 512, 256], 2), ([1 << 18], 4)], ids=str)
@pytest.mark.parametrize("kind", ["c", "ci"])
def test_tma_store_512(dev, kind, dims, batch):
    assert sum(op.get("tma_store", 0) for op in describe(kind, dims, batch)["ops"]) == 1
    for inplace in (False, True):
        err = _c2c(kind, dims, batch, dev, inplace=inplace, seed=batch)
        assert err <= TOL, (kind, dims, batch, inplace, err)


@pytest.mark.parametrize("pad", [1, 2])
def test_tma_store_512_unaligned(dev, pad):
    # off a 16-byte boundary neither map encodes and the LSU kernel runs
    for dims, batch in (([512, 64], 2), ([512, 512], 1)):
        assert _c2c("c", dims, batch, dev, pad=pad, seed=pad) <= TOL, (dims, pad)


def _c2r(dims, batch, dev, pad=0, seed=0):
    n = int(np.prod(dims))
    h = O.half_elems(dims)
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(h * batch).astype(np.float32)
    b = rng.standard_normal(h * batch).astype(np.float32)
    from test_plane_gpu import _dev
    d = _dev(np.zeros(n * batch, np.float32), dev, pad)
    G.BatchPlan("ri", dims, batch).launch(_dev(a, dev, pad), _dev(b, dev, pad), d, None)
    torch.cuda.synchronize()
    got = d.cpu().numpy()
    return max(O.rel_l2(got[j * n:(j + 1) * n], O.oracle64("ri", dims, a[j * h:(j + 1) * h], b[j * h:(j + 1) * h]))
               for j in range(batch))


# 256-point C2R cols passes (real inverse along a 512-point axis): TMA loads
# and stores, 16 columns per tile (one tile per transform, 153 tiles, 3D),
# and off a 16-byte boundary the load-only or LSU kernels
@pytest.mark.parametrize("dims,batch", [([512, 16], 3), ([512, 16], 153), ([512, 512], 4), ([512, 8, 64], 3),
                                        ([512, 64, 64], 2)], ids=str)
def test_tma_store_256_c2r(dev, dims, batch):
    assert sum(op.get("tma_store", 0) for op in describe("ri", dims, batch)["ops"]) == 1
    assert _c2r(dims, batch, dev, seed=batch) <= TOL, (dims, batch)


@pytest.mark.parametrize("pad", [1, 2])
def test_tma_store_256_c2r_unaligned(dev, pad):
    for dims, batch in (([512, 64], 2), ([512, 512], 1)):
        assert _c2r(dims, batch, dev, pad=pad, seed=pad) <= TOL, (dims, pad)


# 1024-point complex cols passes below the pipelined kernel's threshold
# (fewer than 608 tiles): the one-tile kernel with TMA loads and stores
# (1 tile, 128, 256 and 512 tiles, the four-step's pass B with its twiddle)
@pytest.mark.parametrize("dims,batch", [([1024, 8], 1), ([1024, 1024], 1), ([1024, 512], 4), ([1024, 1024], 4),
                                        ([1 << 20], 2)], ids=str)
@pytest.mark.parametrize("kind", ["c", "ci"])
def test_tma_store_1024_one_tile(dev, kind, dims, batch):
    assert sum(op.get("tma_store", 0) for op in describe(kind, dims, batch)["ops"]) == 1
    for inplace in (False, True):
        err = _c2c(kind, dims, batch, dev, inplace=inplace, seed=batch)
        assert err <= TOL, (kind, dims, batch, inplace, err)
