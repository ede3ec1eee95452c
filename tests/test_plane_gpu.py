"""GPU parity of the plane-fused passes (plane_fft: the last two axes of a
complex N-D transform in one CTA per plane) against the FP64 oracle, for
every plane shape built, in place and out of place, staged and unstaged
loads, as the first pass of 3D and 4D transforms and behind the real
transforms' dim-0 pass; plus the plans that must keep the per-axis passes.
Tolerance: relative L2 <= 2e-6, as the other parity tests."""
import numpy as np
import pytest

import fft_gb300 as G
from oracle import oracle as O
from plan_emulator import describe

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
TOL = 2e-6

# (log2 rows, log2 row length) of every plane_fft instantiation
PLANES = [(4, 4), (4, 5), (5, 4), (4, 6), (5, 5), (6, 4), (4, 7), (5, 6), (6, 5), (7, 4),
          (4, 8), (5, 7), (6, 6), (7, 5), (8, 4), (4, 9), (5, 8), (6, 7), (7, 6), (8, 5), (9, 4),
          (5, 9), (6, 8), (7, 7), (8, 6), (9, 5)]


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def _dev(a, dev, pad=0):
    t = torch.zeros(a.size + pad + 1, dtype=torch.float32, device=dev)
    t[pad:pad + a.size] = torch.from_numpy(np.ascontiguousarray(a, np.float32))
    return t[pad:pad + a.size]


def _batch(kind, dims, batch, dev, inplace=False, pad=0, seed=0):
    """A batched complex transform through BatchPlan; returns (got, ref)."""
    n = int(np.prod(dims))
    rng = np.random.default_rng(seed)
    a = rng.uniform(-1, 1, n * batch).astype(np.float32)
    b = rng.uniform(-1, 1, n * batch).astype(np.float32)
    p = G.BatchPlan(kind, dims, batch)
    sr, si = _dev(a, dev, pad), _dev(b, dev, pad)
    dr, di = (sr, si) if inplace else (_dev(np.zeros_like(a), dev, pad), _dev(np.zeros_like(b), dev, pad))
    p.launch(sr, si, dr, di)
    torch.cuda.synchronize()
    got = (dr.cpu().numpy(), di.cpu().numpy())
    outs = [O.oracle64(kind, dims, a[j * n:(j + 1) * n], b[j * n:(j + 1) * n]) for j in range(batch)]
    ref = (np.concatenate([o[0] for o in outs]), np.concatenate([o[1] for o in outs]))
    return got, ref


def _planes_of(kind, dims, batch=1):
    return [op["plane"] for op in describe(kind, dims, batch)["ops"] if op["type"] == "line" and op.get("plane")]


@pytest.mark.parametrize("lg", PLANES, ids=lambda v: "%dx%d" % (1 << v[0], 1 << v[1]))
@pytest.mark.parametrize("kind", ["c", "ci"])
def test_plane_2d(dev, kind, lg):
    dims = [1 << lg[0], 1 << lg[1]]
    # (2^14-point planes take the plane pass from 256 planes per launch)
    # (planes under 2^12 points share a CTA: a batch that leaves the last CTA part full)
    batch = 256 if lg[0] + lg[1] == 14 else 3 if lg[0] + lg[1] >= 12 else (1 << (12 - lg[0] - lg[1])) + 3
    assert _planes_of(kind, dims, batch) == [lg[0]]           # one plane pass is the whole transform
    for inplace in (False, True):
        got, ref = _batch(kind, dims, batch, dev, inplace=inplace, seed=lg[0] * 16 + lg[1])
        assert O.rel_l2(got, ref) <= TOL, (kind, dims, inplace)


@pytest.mark.parametrize("kind", ["c", "ci"])
@pytest.mark.parametrize("dims,batch", [([8, 64, 64], 2), ([4, 32, 128], 2), ([16, 128, 128], 16), ([2, 256, 32], 2),
                                        ([8, 32, 512], 32), ([2, 4, 64, 64], 2), ([16, 16, 16], 3),
                                        ([4, 32, 32], 5), ([2, 16, 64], 7), ([64, 128, 16], 1)], ids=str)
def test_plane_nd(dev, kind, dims, batch):
    # the plane pass first, then the leading axes in place
    assert len(_planes_of(kind, dims, batch)) == 1
    got, ref = _batch(kind, dims, batch, dev, seed=len(dims))
    assert O.rel_l2(got, ref) <= TOL, (kind, dims)


@pytest.mark.parametrize("dims,batch", [([64, 64], 3), ([32, 32], 7), ([8, 32, 128], 2), ([4, 16, 16], 5),
                                        ([128, 128], 256)], ids=str)
@pytest.mark.parametrize("kind", ["c", "ci"])
@pytest.mark.parametrize("inplace", [False, True], ids=["oop", "inplace"])
def test_plane_interleaved(dev, kind, dims, batch, inplace):
    # interleaved re,im pairs: the pair kernels (staged 16-byte loads of pair
    # lines, 8-byte stores)
    from test_parity_gpu import run_batch
    assert [op.get("plane") for op in describe(kind, dims, batch, G.afft_interleaved)["ops"]][0] == \
        {64: 6, 32: 5, 16: 4, 128: 7}[dims[-2]]
    n = int(np.prod(dims))
    rng = np.random.default_rng(len(dims) + batch)
    a = rng.uniform(-1, 1, n * batch).astype(np.float32)
    b = rng.uniform(-1, 1, n * batch).astype(np.float32)
    got = run_batch(kind, dims, batch, a, b, fmt=G.afft_interleaved, inplace=inplace)
    outs = [O.oracle64(kind, dims, a[j * n:(j + 1) * n], b[j * n:(j + 1) * n]) for j in range(batch)]
    ref = (np.concatenate([o[0] for o in outs]), np.concatenate([o[1] for o in outs]))
    assert O.rel_l2(got, ref) <= TOL, (kind, dims, inplace)


def test_plane_interleaved_unaligned(dev):
    # interleaved planes off an 8- and a 16-byte boundary (scalar and unstaged pair accesses)
    p = G.BatchPlan("c", [32, 64], 4, fmt=G.afft_interleaved)
    n = 32 * 64 * 4
    rng = np.random.default_rng(5)
    a = rng.uniform(-1, 1, n).astype(np.float32)
    b = rng.uniform(-1, 1, n).astype(np.float32)
    src = np.empty(2 * n, np.float32)
    src[0::2], src[1::2] = a, b
    outs = [O.oracle64("c", [32, 64], a[j * 2048:(j + 1) * 2048], b[j * 2048:(j + 1) * 2048]) for j in range(4)]
    ref = (np.concatenate([o[0] for o in outs]), np.concatenate([o[1] for o in outs]))
    for pad in (1, 2):
        s = _dev(src, dev, pad)
        d = _dev(np.zeros_like(src), dev, pad)
        p.launch(s, None, d, None)
        torch.cuda.synchronize()
        o = d.cpu().numpy()
        assert O.rel_l2((o[0::2], o[1::2]), ref) <= TOL, pad


@pytest.mark.parametrize("pad", [1, 2])
def test_plane_unaligned_loads(dev, pad):
    # planes that start off a 16-byte boundary load without the staging
    for dims in ([64, 64], [32, 128], [8, 32, 256], [32, 32], [16, 16, 64]):
        got, ref = _batch("c", dims, 2, dev, pad=pad, seed=pad)
        assert O.rel_l2(got, ref) <= TOL, (dims, pad)


@pytest.mark.parametrize("kind", ["r", "ri"])
@pytest.mark.parametrize("dims", [[16, 64, 64], [8, 32, 128], [64, 128, 64], [16, 16, 16], [32, 32, 32]], ids=str)
def test_plane_behind_real_pass(dev, kind, dims):
    from test_parity_gpu import check, inputs, run_plan
    assert len(_planes_of(kind, dims)) == 1
    a, b = inputs(kind, dims, 7)
    check(kind, dims, a, b, run_plan(kind, dims, a, b, dev))


def test_per_axis_where_no_plane_fits():
    # planes of other sizes, sides below 16 or above 512, and the FP64 form
    # keep one pass per axis (the tensor-core form takes the plain plane pass)
    assert _planes_of("c", [256, 256, 256]) == []                 # 2^16-point planes
    assert _planes_of("c", [64, 8, 256]) == []                    # a side of 8
    assert _planes_of("c", [1024, 16]) == []                      # a side of 1024
    assert _planes_of("c", [32, 32]) == [5]                       # 2^10 points: four planes per CTA
    assert _planes_of("c", [128, 128], 255) == [] and _planes_of("c", [128, 128], 256) == [7]   # 2^14: >= 256
    assert [op.get("plane", 0) for op in describe("c", [8, 64, 64], 1, G.FORM_F64)["ops"]] == [0, 0, 0]
    assert [op.get("plane", 0) for op in describe("c", [8, 64, 64], 1, G.FORM_TC)["ops"]] == [6, 0]


def test_queue_with_plane_segments(dev):
    # 3D and 2D transforms whose planes fuse, mixed with others, through the
    # queue's grouped plane kernels
    from fft_gb300 import uneven as U
    items = [("c", [8, 64, 64]), ("ci", [4, 32, 128]), ("r", [16, 64, 64]), ("ri", [8, 128, 64]),
             ("c", [64, 64]), ("ci", [128, 128]), ("c", [256]), ("r", [32, 32, 32]), ("c", [16, 256, 32])] * 3
    buf, offs = U.allocate(items, dev, seed=9)
    q = G.Queue(U.descs(items, buf, offs))
    q.run()
    torch.cuda.synchronize()
    host = buf.cpu().numpy()
    for j, (kind, dims) in enumerate(items):
        i_n, o_n = U.elems(kind, dims)
        r = offs[j]
        a = host[r[0]:r[0] + i_n]
        b = None if r[1] is None else host[r[1]:r[1] + i_n]
        got = host[r[2]:r[2] + o_n] if kind == "ri" else (host[r[2]:r[2] + o_n], host[r[3]:r[3] + o_n])
        assert O.rel_l2(got, O.oracle64(kind, dims, a, b)) <= TOL, (j, kind, dims)
