"""The no-allocation entry point afft_gb300_c2c_noalloc, for callers that
cannot allocate device memory at call time (fixed memory budgets, custom
allocators that own the free memory, loops that cannot afford cudaMalloc's
synchronisation).  Its output, over two calls in a row through the C ABI,
must match the ordinary batched entry point's within the parity tolerance.
This file sorts last so a run that stops at the first failure has already
run every other test; it also passes on its own in a fresh process."""
import ctypes
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

import fft_gb300 as G
from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
TOL = 2e-6


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def noalloc():
    f = G.lib().afft_gb300_c2c_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p]
    return f


@pytest.mark.parametrize("n,batch", [(1 << 15, 4), (1 << 16, 8), (1 << 18, 2), (1 << 21, 1)])
@pytest.mark.parametrize("inverse", [0, 1])
def test_noalloc_matches_batched_entry_point(n, batch, inverse, dev):
    f = noalloc()
    plan = G.BatchPlan("ci" if inverse else "c", [n], batch)
    rng = np.random.default_rng(n + batch + inverse)
    for call in range(2):   # two calls in a row; the second reuses the scratch
        xr = torch.from_numpy(rng.standard_normal(n * batch).astype(np.float32)).to(dev)
        xi = torch.from_numpy(rng.standard_normal(n * batch).astype(np.float32)).to(dev)
        ref_r, ref_i = torch.empty_like(xr), torch.empty_like(xi)
        plan(xr, xi, ref_r, ref_i)
        yr = torch.full_like(xr, float("nan"))
        yi = torch.full_like(xi, float("nan"))
        rc = f(xr.data_ptr(), xi.data_ptr(), yr.data_ptr(), yi.data_ptr(), n, batch, inverse, None)
        assert rc == 0, G.last_error()
        torch.cuda.synchronize()
        err = O.rel_l2((yr.cpu().numpy(), yi.cpu().numpy()), (ref_r.cpu().numpy(), ref_i.cpu().numpy()))
        assert err <= TOL, (call, err)


def test_noalloc_rejects_sizes_beyond_its_scratch(dev):
    f = noalloc()
    x = torch.zeros(16, device=dev)
    p = x.data_ptr()
    assert f(p, p, p, p, 1 << 22, 1, 0, None) == 1
    assert "2^21" in G.last_error()[1]
    assert f(p, p, p, p, 1 << 16, 64, 0, None) == 1     # n * batch > 2^21
    assert f(p, p, p, p, 1 << 14, 1, 0, None) == 1      # one-pass sizes need no scratch
    assert f(p, p, p, p, 3 << 15, 1, 0, None) == 1
    # n * batch wraps to 2^15 in 64 bits; it must still be refused
    assert f(p, p, p, p, 1 << 15, (1 << 49) + 1, 0, None) == 1
    assert f(p, p, p, p, 1 << 15, 0, 0, None) == 1


def test_noalloc_call_takes_no_device_memory(dev):
    """The point of the entry point: once a device is set up (first call,
    which also loads its kernels), a call leaves free device memory as it
    found it."""
    f = noalloc()
    n, batch = 1 << 16, 8
    rng = np.random.default_rng(7)
    xr = torch.from_numpy(rng.standard_normal(n * batch).astype(np.float32)).to(dev)
    xi = torch.from_numpy(rng.standard_normal(n * batch).astype(np.float32)).to(dev)
    yr, yi = torch.empty_like(xr), torch.empty_like(xi)
    assert f(xr.data_ptr(), xi.data_ptr(), yr.data_ptr(), yi.data_ptr(), n, batch, 0, None) == 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(dev)[0]
    assert f(xr.data_ptr(), xi.data_ptr(), yr.data_ptr(), yi.data_ptr(), n, batch, 0, None) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(dev)[0] == free0


_FRESH = textwrap.dedent("""
    import ctypes
    import sys
    import numpy as np
    import torch
    sys.path.insert(0, sys.argv[1])
    import fft_gb300 as G
    from oracle import oracle as O
    f = G.lib().afft_gb300_c2c_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p]
    dev = torch.device("cuda:0")
    n, batch = 1 << 17, 4
    rng = np.random.default_rng(11)
    xr = torch.from_numpy(rng.standard_normal(n * batch).astype(np.float32)).to(dev)
    xi = torch.from_numpy(rng.standard_normal(n * batch).astype(np.float32)).to(dev)
    yr, yi = torch.empty_like(xr), torch.empty_like(xi)
    torch.cuda.synchronize()
    side = torch.cuda.Stream()          # torch side streams do not order after the default stream
    rc = f(xr.data_ptr(), xi.data_ptr(), yr.data_ptr(), yi.data_ptr(), n, batch, 0, side.cuda_stream)
    assert rc == 0, G.last_error()
    side.synchronize()
    rr, ri = torch.empty_like(xr), torch.empty_like(xi)
    G.BatchPlan("c", [n], batch)(xr, xi, rr, ri)
    torch.cuda.synchronize()
    err = O.rel_l2((yr.cpu().numpy(), yi.cpu().numpy()), (rr.cpu().numpy(), ri.cpu().numpy()))
    assert err <= 2e-6, err
    print("fresh-process first call on a side stream: rel-L2 %.2e" % err)
""")


def test_noalloc_first_call_on_a_side_stream_in_a_fresh_process(dev):
    """The device set-up happens inside the first call; that call here runs
    on a non-blocking stream in a new process, so its kernels must not
    overtake the set-up's table uploads."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _FRESH, root], capture_output=True, text=True, timeout=300,
                       cwd=root)
    assert r.returncode == 0, r.stdout + r.stderr
