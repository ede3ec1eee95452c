"""The benchmark configurations at their full sizes, checked through
properties that do not depend on the size plus a sample of transforms against
the FP64 oracle:

* C1  1 x c2c n=1024 (the reference harness's own input), forward + inverse/n
* C2  16384 x c2c n=4096, forward and inverse
* C3a c2c 256^3; C3b r2c 4096^2 and its inverse; C3c 64 x r2c n=2^20
* C4  4096 x c2c n=65536 (plain and split-precision tensor-core forms; the
      second input set has magnitudes spread over 1e-4)

Properties: inverse(forward(x))/N recovers x (rel-L2 <= 2e-6 plain, 5e-6
tensor-core form); Parseval, sum |X|^2 = N sum |x|^2 (rel. 1e-5); linearity
F(a x + y) = a F(x) + F(y) on the full batch (rel-L2 <= 4e-6)."""
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


def rel(a, b):
    return (torch.linalg.vector_norm((a - b).double()) / torch.linalg.vector_norm(b.double())).item()


def _c2c_config(dims, batch, dev, form=None, spread=False, tol=2e-6, samples=(0,)):
    n = int(np.prod(dims))
    g = torch.Generator(device=dev)
    g.manual_seed(n + batch)
    if spread:
        mag = 10.0 ** (-4 * torch.rand(n * batch, generator=g, device=dev))
        ph = 2 * np.pi * torch.rand(n * batch, generator=g, device=dev)
        xr, xi = mag * torch.cos(ph), mag * torch.sin(ph)
    else:
        xr = torch.randn(n * batch, generator=g, device=dev)
        xi = torch.randn(n * batch, generator=g, device=dev)
    fwd = G.BatchPlan("c", dims, batch, form=form)
    inv = G.BatchPlan("ci", dims, batch, form=form)
    yr, yi = torch.empty_like(xr), torch.empty_like(xi)
    zr, zi = torch.empty_like(xr), torch.empty_like(xi)
    fwd(xr, xi, yr, yi)
    inv(yr, yi, zr, zi)
    # round trip
    assert rel(torch.cat([zr, zi]) / n, torch.cat([xr, xi])) <= tol
    # Parseval
    ex = (xr.double() ** 2 + xi.double() ** 2).sum().item()
    ey = (yr.double() ** 2 + yi.double() ** 2).sum().item()
    assert abs(ey / (n * ex) - 1) <= 1e-5
    # linearity on the whole batch
    a = 0.75
    sr, si = torch.roll(xr, 12345), torch.roll(xi, 12345)
    ur, ui = torch.empty_like(xr), torch.empty_like(xi)
    fwd(a * xr + sr, a * xi + si, ur, ui)
    vr, vi = torch.empty_like(xr), torch.empty_like(xi)
    fwd(sr, si, vr, vi)
    assert rel(torch.cat([ur, ui]), torch.cat([a * yr + vr, a * yi + vi])) <= 2 * tol
    # sampled transforms against the FP64 oracle
    for j in samples:
        s = slice(j * n, (j + 1) * n)
        ref = O.c2c64(dims, xr[s].cpu().numpy(), xi[s].cpu().numpy())
        assert O.rel_l2((yr[s].cpu().numpy(), yi[s].cpu().numpy()), ref) <= tol


def test_c1_harness_input(golden, dev):
    z, _ = golden
    a, b = torch.from_numpy(z["c1/in0"]).to(dev), torch.from_numpy(z["c1/in1"]).to(dev)
    yr, yi = torch.empty_like(a), torch.empty_like(b)
    zr, zi = torch.empty_like(a), torch.empty_like(b)
    G.BatchPlan("c", [1024], 1)(a, b, yr, yi)
    G.BatchPlan("ci", [1024], 1)(yr, yi, zr, zi)
    ref = O.c2c64([1024], z["c1/in0"], z["c1/in1"])
    assert O.rel_l2((yr.cpu().numpy(), yi.cpu().numpy()), ref) <= 2e-6
    assert O.rel_l2((zr.cpu().numpy() / 1024, zi.cpu().numpy() / 1024), (z["c1/in0"], z["c1/in1"])) <= 2e-6


def test_c2_full(dev):
    _c2c_config([4096], 16384, dev, samples=(0, 8191, 16383))


def test_c3a_full(dev):
    _c2c_config([256, 256, 256], 1, dev)


def test_c4_full_plain(dev):
    _c2c_config([65536], 4096, dev, samples=(0, 4095))


def test_c4_full_tensor_core_form(dev):
    _c2c_config([65536], 4096, dev, form="tc", tol=5e-6, samples=(0, 2048))
    _c2c_config([65536], 4096, dev, form="tc", spread=True, tol=5e-6, samples=(7,))


@pytest.mark.parametrize("dims,batch", [([4096, 4096], 1), ([1 << 20], 64)], ids=["c3b", "c3c"])
def test_c3_real_full(dims, batch, dev):
    n = int(np.prod(dims))
    h = O.half_elems(dims)
    g = torch.Generator(device=dev)
    g.manual_seed(n)
    x = torch.randn(n * batch, generator=g, device=dev)
    hr, hi = torch.empty(h * batch, device=dev), torch.empty(h * batch, device=dev)
    y = torch.empty_like(x)
    G.BatchPlan("r", dims, batch)(x, hr, hi)
    G.BatchPlan("ri", dims, batch)(hr, hi, y)
    assert rel(y / n, x) <= 2e-6
    # sampled transform against the FP64 oracle (batch entry 0)
    ref = O.r2c64(dims, x[:n].cpu().numpy())
    assert O.rel_l2((hr[:h].cpu().numpy(), hi[:h].cpu().numpy()), ref) <= 2e-6
    # the DC bin is the sum of the input
    assert abs(hr[0].item() - x[:n].double().sum().item()) <= 1e-4 * max(1.0, float(np.sqrt(n)))
