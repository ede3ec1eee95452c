"""GPU parity of the FP64 transforms (afft_64_*, fft.h:52-80) through the C
ABI: against the reference library's own double outputs (tests/golden,
afft_golden64) and the FP64 oracle, on device and host arrays, for every
kind, split and interleaved, batched and N-D.

Tolerance: relative L2 error <= 1e-13 against the oracle and against afft's
double output (FP64 roundoff is ~1e-16 per operation; an FP32 step anywhere
in the path would show as ~1e-7).
"""
import ctypes

import numpy as np
import pytest

import fft_gb300 as G
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL64 = 1e-13

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def _arrays(kind, n, h, batch=1):
    m_in = {"c": n, "ci": n, "r": n, "ri": h}[kind] * batch
    m_out = {"c": n, "ci": n, "r": h, "ri": n}[kind] * batch
    return m_in, m_out


def run64(kind, dims, a, b, dev, fmt=G.afft_split, host=False, batch=1):
    """One FP64 call (fft.hpp-style classes with bits=64, or a batched plan
    of form 'f64'); returns numpy float64 output (tuple for complex)."""
    n = int(np.prod(dims))
    h = O.half_elems(dims)
    m_in, m_out = _arrays(kind, n, h, batch)
    inter = fmt == G.afft_interleaved
    if batch == 1:
        cls = {"c": G.complex_transform, "ci": G.inverse_complex_transform,
               "r": G.real_transform, "ri": G.inverse_real_transform}[kind]
        plan = cls(dims, fmt=fmt, bits=64)
    else:
        plan = G.BatchPlan(kind, dims, batch, fmt=fmt, form="f64")
    if host:
        conv = lambda x: np.ascontiguousarray(x, np.float64)
        zeros = lambda m: np.zeros(m, np.float64)
        back = lambda x: x
    else:
        conv = lambda x: torch.from_numpy(np.ascontiguousarray(x, np.float64)).to(dev)
        zeros = lambda m: torch.zeros(m, dtype=torch.float64, device=dev)
        back = lambda x: x.cpu().numpy()
    cin = kind != "r"
    cout = kind != "ri"
    if cin and inter:
        src = np.empty(2 * m_in)
        src[0::2], src[1::2] = a, b
        s0, s1 = conv(src), None
    else:
        s0, s1 = conv(a), (conv(b) if cin else None)
    if cout and inter:
        d0, d1 = zeros(2 * m_out), None
    else:
        d0, d1 = zeros(m_out), (zeros(m_out) if cout else None)
    if kind in ("c", "ci"):
        plan(s0, s1, d0, d1)
    elif kind == "r":
        plan(s0, d0, d1)
    else:
        plan(s0, s1, d0)
    torch.cuda.synchronize()
    if not cout:
        return back(d0)
    if inter:
        o = back(d0)
        return o[0::2].copy(), o[1::2].copy()
    return back(d0), back(d1)


def oracle_batch(kind, dims, a, b, batch):
    n = int(np.prod(dims))
    h = O.half_elems(dims)
    m = {"c": n, "ci": n, "r": n, "ri": h}[kind]
    outs = [O.oracle64(kind, dims, a[j * m:(j + 1) * m], None if b is None else b[j * m:(j + 1) * m])
            for j in range(batch)]
    if kind == "ri":
        return np.concatenate(outs)
    return np.concatenate([o[0] for o in outs]), np.concatenate([o[1] for o in outs])


def inputs(kind, dims, batch, seed):
    n = int(np.prod(dims))
    m, _ = _arrays(kind, n, O.half_elems(dims), batch)
    rng = np.random.default_rng(seed)
    return rng.standard_normal(m), (None if kind == "r" else rng.standard_normal(m))


# --- the reference's own double outputs ---------------------------------------

def test_golden64_device(golden64, dev):
    z, cases = golden64
    worst = 0.0
    for case in cases:
        nm, kind, dims = case["name"], case["kind"], case["dims"]
        a = z[nm + "/in0"].astype(np.float64)
        b = z[nm + "/in1"].astype(np.float64) if nm + "/in1" in z else None
        got = run64(kind, dims, a, b, dev)
        ref = z[nm + "/scalar0"] if kind == "ri" else (z[nm + "/scalar0"], z[nm + "/scalar1"])
        err = O.rel_l2(got, ref)
        worst = max(worst, err)
        assert err <= TOL64, (nm, err)
        assert O.rel_l2(got, O.oracle64(kind, dims, a, b)) <= TOL64, nm
    print("worst FP64 rel-L2 vs afft_64 over golden cases: %.2e" % worst)


def test_golden64_host_and_interleaved(golden64, dev):
    # host arrays (staged through device buffers) and the interleaved format
    z, cases = golden64
    for i, case in enumerate(cases[::3]):
        nm, kind, dims = case["name"], case["kind"], case["dims"]
        a = z[nm + "/in0"].astype(np.float64)
        b = z[nm + "/in1"].astype(np.float64) if nm + "/in1" in z else None
        ref = z[nm + "/scalar0"] if kind == "ri" else (z[nm + "/scalar0"], z[nm + "/scalar1"])
        fmt = G.afft_interleaved if i % 2 else G.afft_split
        got = run64(kind, dims, a, b, dev, fmt=fmt, host=(i % 3 == 0))
        assert O.rel_l2(got, ref) <= TOL64, (nm, fmt)


# --- larger and batched shapes against the oracle -----------------------------

BATCHED = [("c", [4096], 64), ("ci", [8192], 16), ("c", [16384], 8), ("ci", [1 << 16], 4), ("c", [1 << 22], 1),
           ("r", [16384], 8), ("ri", [16384], 8), ("r", [1 << 20], 2), ("ri", [1 << 17], 3),
           ("c", [2048, 2048], 1), ("r", [4096, 4096], 1), ("ri", [4096, 512], 2), ("r", [8192, 64], 1),
           ("c", [256, 256, 256], 1), ("ci", [32, 64, 128], 3), ("ri", [64, 32, 16], 2), ("r", [1 << 15, 4], 1)]


@pytest.mark.parametrize("kind,dims,batch", BATCHED, ids=str)
def test_batched_f64(kind, dims, batch, dev):
    a, b = inputs(kind, dims, batch, len(dims) * 31 + batch)
    got = run64(kind, dims, a, b, dev, batch=batch)
    err = O.rel_l2(got, oracle_batch(kind, dims, a, b, batch))
    assert err <= TOL64, (kind, dims, batch, err)


@pytest.mark.parametrize("kind,dims", [("c", [1 << 15]), ("r", [4096, 8]), ("ri", [1 << 16]), ("ci", [16, 16, 16])],
                         ids=str)
def test_batched_f64_interleaved(kind, dims, dev):
    a, b = inputs(kind, dims, 3, 7)
    got = run64(kind, dims, a, b, dev, fmt=G.afft_interleaved, batch=3)
    assert O.rel_l2(got, oracle_batch(kind, dims, a, b, 3)) <= TOL64


@pytest.mark.parametrize("dims", [[1024], [1 << 18], [512, 256], [64, 64, 64]], ids=str)
def test_round_trip_f64(dims, dev):
    n = int(np.prod(dims))
    a, b = inputs("c", dims, 1, n)
    fr, fi = run64("c", dims, a, b, dev)
    br, bi = run64("ci", dims, fr, fi, dev)
    assert O.rel_l2((br / n, bi / n), (a, b)) <= TOL64
    x = np.random.default_rng(n).standard_normal(n)
    hr, hi = run64("r", dims, x, None, dev)
    y = run64("ri", dims, hr, hi, dev)
    assert O.rel_l2(y / n, x) <= TOL64


def test_precision_mismatch_is_refused(dev):
    # an FP32 plan through an afft_64 transform (and the reverse) is reported,
    # never launched
    L = G.lib()
    p32 = G.complex_transform([64])
    p64 = G.complex_transform([64], bits=64)
    x = torch.zeros(128, dtype=torch.float64, device=dev)
    P = ctypes.c_void_p
    L.afft_64_c_transform(P(p32.state), P(x.data_ptr()), P(x.data_ptr() + 512), P(x.data_ptr()),
                          P(x.data_ptr() + 512))
    code, msg = G.last_error()
    assert code == 1 and "FP32 plan" in msg
    L.afft_32_c_transform(P(p64.state), P(x.data_ptr()), P(x.data_ptr() + 256), P(x.data_ptr()),
                          P(x.data_ptr() + 256))
    code, msg = G.last_error()
    assert code == 1 and "FP64 plan" in msg
    torch.cuda.synchronize()


def test_f64_plans_describe_and_count(dev):
    p = G.BatchPlan("r", [1 << 15], 2, form="f64")
    assert p.launches == 3
    d = G.describe("c", [8192], 1, G.FORM_F64)
    assert d["f64"] == 1 and len(d["ops"]) == 1


def test_misaligned_f64_pointers_are_refused(dev):
    # double arrays off an 8-byte boundary are reported before any launch
    L = G.lib()
    p64 = G.complex_transform([64], bits=64)
    x = torch.zeros(1024, dtype=torch.float64, device=dev)   # 8 KB: every array below fits inside
    P = ctypes.c_void_p
    base = x.data_ptr()
    L.afft_64_c_transform(P(p64.state), P(base + 4), P(base + 1028), P(base + 2052), P(base + 3076))
    code, msg = G.last_error()
    assert code == 1 and "8-byte aligned" in msg
    L.afft_64_c_transform(P(p64.state), P(base), P(base + 1024), P(base + 2048), P(base + 3072))
    assert G.last_error()[0] == 0
    torch.cuda.synchronize()


@pytest.mark.parametrize("n", [1, 2, 4])
@pytest.mark.parametrize("batch", [1, 5])
def test_tiny_real_f64(n, batch, dev):
    # real transforms of total size 1 (the length-1 DFT), 2 and 4: the
    # smallest FP64 line kernels and the size-1 elementwise kernel
    a, _ = inputs("r", [n], batch, 11 * n + batch)
    hr, hi = run64("r", [n], a, None, dev, batch=batch)
    assert O.rel_l2((hr, hi), oracle_batch("r", [n], a, None, batch)) <= TOL64
    br, bi = inputs("ri", [n], batch, 13 * n + batch)
    y = run64("ri", [n], br, bi, dev, batch=batch)
    assert O.rel_l2(y, oracle_batch("ri", [n], br, bi, batch)) <= TOL64
