"""The split-precision tensor-core form (AFFT_GB300_FORM_TC): radix-16
butterflies of complex passes of length 256 and 4096 as tcgen05 DFT-matrix
products on FP16 hi + scaled lo operand pairs with FP32 accumulation in TMEM.
Bound: relative L2 error <= 5e-6 against the FP64 oracle, also on inputs with
a 1e-4 dynamic-range spread."""
import numpy as np
import pytest

import fft_gb300 as G
from fft_gb300 import uneven as U
from oracle import oracle as O
from plan_emulator import describe

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
TOL_TC = 5e-6


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def _inputs(n, batch, seed, spread=False):
    rng = np.random.default_rng(seed)
    if spread:
        mag = 10.0 ** rng.uniform(-4, 0, n * batch)
        ph = rng.uniform(0, 2 * np.pi, n * batch)
        return (mag * np.cos(ph)).astype(np.float32), (mag * np.sin(ph)).astype(np.float32)
    return rng.uniform(-1, 1, n * batch).astype(np.float32), rng.uniform(-1, 1, n * batch).astype(np.float32)


def _run(kind, dims, batch, a, b, dev):
    plan = G.BatchPlan(kind, dims, batch, form="tc")
    xa, xb = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
    ya, yb = torch.empty_like(xa), torch.empty_like(xb)
    plan(xa, xb, ya, yb)
    return ya.cpu().numpy(), yb.cpu().numpy()


def test_tc_kernels_selected():
    d = describe("c", [4096], 8, G.FORM_TC)
    assert [op["tc"] for op in d["ops"]] == [1]
    d = describe("c", [1 << 16], 2, G.FORM_TC)
    assert [op["tc"] for op in d["ops"]] == [1, 1]
    d = describe("c", [1024], 2, G.FORM_TC)       # radix schedule 4 x 16 x 16: plain
    assert [op["tc"] for op in d["ops"]] == [0]
    assert [op["tc"] for op in describe("c", [4096], 8)["ops"]] == [0]


@pytest.mark.parametrize("kind", ["c", "ci"])
@pytest.mark.parametrize("dims,batch", [([256], 300), ([4096], 40), ([1 << 16], 3), ([256, 256], 2),
                                        ([16, 256, 256], 1), ([1024], 5)], ids=str)
def test_tc_accuracy(kind, dims, batch, dev):
    n = int(np.prod(dims))
    a, b = _inputs(n, batch, n + batch)
    ya, yb = _run(kind, dims, batch, a, b, dev)
    worst = 0.0
    for j in range(batch):
        s = slice(j * n, (j + 1) * n)
        ref = O.oracle64(kind, dims, a[s], b[s])
        err = O.rel_l2((ya[s], yb[s]), ref)
        worst = max(worst, err)
        assert err <= TOL_TC, (j, err)
    print(kind, dims, "worst rel-L2 %.2e" % worst)


def test_tc_dynamic_range_spread(dev):
    # the 1e-4 magnitude spread input set of the split-precision comparison
    n, batch = 1 << 16, 4
    a, b = _inputs(n, batch, 77, spread=True)
    ya, yb = _run("c", [n], batch, a, b, dev)
    for j in range(batch):
        s = slice(j * n, (j + 1) * n)
        ref = O.oracle64("c", [n], a[s], b[s])
        assert O.rel_l2((ya[s], yb[s]), ref) <= TOL_TC


def test_tc_queue(dev):
    items = U.uneven_batch(120, seed=13, max_log1d=16, side2d=(6, 9), side3d=(4, 8))
    buf, offs = U.allocate(items, dev, seed=9)
    q = G.Queue(U.descs(items, buf, offs), form="tc")
    q.run()
    torch.cuda.synchronize()
    host = buf.cpu().numpy()
    for j, (kind, dims) in enumerate(items):
        i_n, o_n = U.elems(kind, dims)
        r = offs[j]
        a = host[r[0]:r[0] + i_n]
        b = None if r[1] is None else host[r[1]:r[1] + i_n]
        got = host[r[2]:r[2] + o_n] if kind == "ri" else (host[r[2]:r[2] + o_n], host[r[3]:r[3] + o_n])
        assert O.rel_l2(got, O.oracle64(kind, dims, a, b)) <= TOL_TC, (j, kind, dims)
