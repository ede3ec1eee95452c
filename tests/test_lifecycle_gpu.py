"""Plan lifecycle, concurrency and failure reporting on the GPU: distinct
plans used from several host threads at once (as run_all --threads does,
run_all.cpp:138-146), a plan re-created at the same caller memory, use after
release, and the bounded-wait failure path (a device wait that gives up and
reports AFFT_GB300_ETIMEOUT without faulting)."""
import ctypes
import threading

import numpy as np
import pytest

import fft_gb300 as G
from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def test_threads_with_distinct_plans(dev):
    errors = []

    def work(n, seed):
        try:
            rng = np.random.default_rng(seed)
            p = G.complex_transform([n])
            for _ in range(20):
                a = rng.standard_normal(n).astype(np.float32)
                b = rng.standard_normal(n).astype(np.float32)
                yr, yi = np.zeros(n, np.float32), np.zeros(n, np.float32)
                p(a, b, yr, yi)
                if O.rel_l2((yr, yi), O.c2c64([n], a, b)) > 2e-6:
                    errors.append((n, seed))
        except Exception as e:   # surfaced below
            errors.append(repr(e))

    ts = [threading.Thread(target=work, args=(n, s)) for s, n in enumerate([256, 1024, 4096, 1 << 16, 64, 512])]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors, errors


def test_recreate_at_same_mem_and_use_after_release(dev):
    L = G.lib()
    mem = ctypes.create_string_buffer(256)
    d1 = (ctypes.c_size_t * 1)(1024)
    p1 = L.afft_32_c_create(1, d1, 0, ctypes.addressof(mem), 0)
    assert p1 == ctypes.addressof(mem)
    assert L.afft_gb300_plan_launches(p1) == 1
    # a new plan at the same memory replaces the old one
    d2 = (ctypes.c_size_t * 1)(1 << 16)
    p2 = L.afft_32_c_create(1, d2, 0, ctypes.addressof(mem), 0)
    assert p2 == p1 and L.afft_gb300_plan_launches(p2) == 2
    x = np.ones(1 << 16, np.float32)
    y = np.zeros(1 << 16, np.float32)
    L.afft_32_c_transform(p2, x.ctypes.data, x.ctypes.data, y.ctypes.data, y.ctypes.data)
    assert G.last_error()[0] == 0
    assert L.afft_gb300_release(p2) == 0
    # after release the plan is reported, not used
    L.afft_32_c_transform(p2, x.ctypes.data, x.ctypes.data, y.ctypes.data, y.ctypes.data)
    assert G.last_error()[0] == 5
    assert L.afft_gb300_release(p2) == 5


def test_bounded_wait_reports_timeout(dev):
    f = G.lib().afft_gb300_selftest_bounded_wait
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int]
    assert f(1000) == 6            # AFFT_GB300_ETIMEOUT
    # the context is still usable afterwards
    p = G.complex_transform([256])
    x = np.ones(256, np.float32)
    yr, yi = np.zeros(256, np.float32), np.zeros(256, np.float32)
    p(x, x, yr, yi)
    assert yr[0] == 256.0 and yi[0] == 256.0


def test_tma_tile_wait_reports_timeout(dev):
    # the cols passes' TMA tile wait, made to run out on purpose (a copy of
    # half the announced bytes): 20 ms limit, reported as ETIMEOUT
    f = G.lib().afft_gb300_selftest_tma_wait
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int]
    assert f(20000) == 6, G.last_error()
    # the context is still usable: a TMA-fed cols pass runs and is right
    p = G.BatchPlan("c", [256, 256], 4)
    x = torch.ones(256 * 256 * 4, device=dev)
    yr, yi = torch.zeros_like(x), torch.zeros_like(x)
    p(x, x, yr, yi)
    torch.cuda.synchronize()
    assert float(yr[0]) == 65536.0 and float(yr[1:65536].abs().max()) == 0.0


def test_missing_data_pointers_are_rejected(dev):
    # a NULL array the transform reads or writes is reported (EINVAL) before
    # anything is launched, through the synchronous, async and queue entry
    # points; the context stays usable
    L = G.lib()
    n = 1024
    x = torch.ones(n, device=dev)
    y = torch.zeros(n + 2, device=dev)
    z = torch.zeros(n + 2, device=dev)
    cases = [
        (G.complex_transform([n]), (x, None, y, z)),
        (G.complex_transform([n]), (x, x, None, z)),
        (G.inverse_complex_transform([n]), (x, x, y, None)),
        (G.real_transform([n]), (x, None, z)),
        (G.real_transform([n]), (None, y, z)),
        (G.inverse_real_transform([n]), (x, None, y)),
    ]
    for plan, args in cases:
        with pytest.raises(G.AfftError):
            plan(*args)
        assert G.last_error()[0] == 1
    p = G.BatchPlan("r", [n], 1)
    rc = L.afft_gb300_transform_async(p.state, G.ptr(x), None, None, G.ptr(z), None)
    assert rc == 1
    with pytest.raises(G.AfftError):
        G.Queue([("c", [n], x, None, y, z)])
    # still usable
    plan = G.complex_transform([n])
    yr, yi = torch.zeros(n, device=dev), torch.zeros(n, device=dev)
    plan(x, torch.zeros(n, device=dev), yr, yi)
    torch.cuda.synchronize()
    assert abs(float(yr[0]) - n) < 1e-3 and float(yr[1:].abs().max()) < 1e-3
