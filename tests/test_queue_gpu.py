"""The multi-transform queue (device-side descriptor tables, one grouped
launch per (pass level, kernel shape), graph-captured) against the FP64
oracle, transform by transform."""
import numpy as np
import pytest

import fft_gb300 as G
from fft_gb300 import uneven as U
from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
TOL = 2e-6


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def _check_all(items, buf, offs, sample=None):
    host = buf.cpu().numpy()
    idx = range(len(items)) if sample is None else sample
    worst = 0.0
    for j in idx:
        kind, dims = items[j]
        i_n, o_n = U.elems(kind, dims)
        r = offs[j]
        a = host[r[0]:r[0] + i_n]
        b = None if r[1] is None else host[r[1]:r[1] + i_n]
        got = host[r[2]:r[2] + o_n] if kind == "ri" else (host[r[2]:r[2] + o_n], host[r[3]:r[3] + o_n])
        ref = O.oracle64(kind, dims, a, b)
        err = O.rel_l2(got, ref)
        worst = max(worst, err)
        assert err <= TOL, (j, kind, dims, err)
    return worst


def test_uneven_small_sizes(dev):
    items = U.uneven_batch(400, seed=11, max_log1d=16, side2d=(2, 8), side3d=(1, 6))
    buf, offs = U.allocate(items, dev, seed=3)
    inputs = buf.clone()
    q = G.Queue(U.descs(items, buf, offs))
    for _ in range(3):   # replays of the captured graph give the same result
        q.run()
        torch.cuda.synchronize()
        # inputs untouched
        for j, (kind, dims) in enumerate(items[:50]):
            i_n, _ = U.elems(kind, dims)
            assert torch.equal(buf[offs[j][0]:offs[j][0] + i_n], inputs[offs[j][0]:offs[j][0] + i_n])
    worst = _check_all(items, buf, offs)
    # one launch per (pass level, kernel shape), far fewer than transforms
    assert q.launches < len(items) // 4
    print("400 mixed transforms, %d launches, worst rel-L2 %.2e" % (q.launches, worst))


def test_uneven_full_distribution_prefix(dev):
    # the mixed-batch distribution itself (1D up to 2^18, 2D up to 2048^2,
    # 3D up to 256^3), a prefix checked completely
    items = U.uneven_batch(10000, seed=5)[:160]
    buf, offs = U.allocate(items, dev, seed=4)
    q = G.Queue(U.descs(items, buf, offs))
    q.run()
    torch.cuda.synchronize()
    _check_all(items, buf, offs)


def test_queue_rejects_bad_descriptors(dev):
    x = torch.zeros(64, device=dev)
    with pytest.raises(G.AfftError):
        G.Queue([("c", [12], x, x, x, x)])
    with pytest.raises(G.AfftError):
        G.Queue([("c", [2, 2, 2, 2], x, x, x, x)])


def test_empty_queue_runs_nothing():
    q = G.Queue([])
    assert q.launches == 0
    q.run()
    assert G.last_error()[0] == 0


@pytest.mark.parametrize("form", [None, "tc"], ids=["plain", "tc"])
def test_full_uneven_batch_sampled(form, dev):
    # the whole 10,000-transform mixed batch (about 26 GB on the device) in
    # one queue run, plain and split-precision tensor-core forms, against the
    # FP64 oracle on a seeded sample of 256 transforms of every kind and
    # dimensionality (rel-L2 <= 2e-6 plain, 5e-6 tensor-core form)
    items = U.uneven_batch(10000, seed=5)
    buf, offs = U.allocate(items, dev, seed=8)
    q = G.Queue(U.descs(items, buf, offs), form=form)
    q.run()
    torch.cuda.synchronize()
    sample = sorted(int(j) for j in np.random.default_rng(99).choice(len(items), 256, replace=False))
    tol = TOL if form is None else 5e-6
    worst = 0.0
    for j in sample:
        kind, dims = items[j]
        i_n, o_n = U.elems(kind, dims)
        r = offs[j]
        a = buf[r[0]:r[0] + i_n].cpu().numpy()
        b = None if r[1] is None else buf[r[1]:r[1] + i_n].cpu().numpy()
        got = buf[r[2]:r[2] + o_n].cpu().numpy()
        if kind != "ri":
            got = (got, buf[r[3]:r[3] + o_n].cpu().numpy())
        err = O.rel_l2(got, O.oracle64(kind, dims, a, b))
        worst = max(worst, err)
        assert err <= tol, (j, kind, dims, err)
    print("10000 mixed transforms (%s), worst rel-L2 over 256 sampled: %.2e" % (form or "plain", worst))
    del q, buf
    torch.cuda.empty_cache()
