"""Randomised shape sweep in the manner of the reference's run_all
(run_all.cpp:149-219): every 1D size, cubic 2D/3D sizes, and random shapes of
up to 5 dims and 2^22 elements drawn with a fixed seed, all four kinds, split
and interleaved, each through the C ABI against the FP64 oracle (rel-L2 <= 2e-6)."""
import numpy as np
import pytest

import fft_gb300 as G
from oracle import oracle as O
from test_parity_gpu import TOL, dev, inputs, run_plan  # noqa: F401

pytestmark = pytest.mark.gpu


def sweep_shapes(seed=2024, count=40, max_log=22, max_dims=5):
    rng = np.random.default_rng(seed)
    shapes = [[2 ** k, 2 ** k] for k in range(1, 12)] + [[2 ** k] * 3 for k in range(1, 8)]
    while len(shapes) < 18 + count:
        nd = int(rng.integers(1, max_dims + 1))
        total = int(rng.integers(nd, max_log + 1))
        # split `total` bits over nd dims (zero bits allowed: size-1 dims)
        cuts = np.sort(rng.integers(0, total + 1, nd - 1))
        bits = np.diff(np.concatenate([[0], cuts, [total]]))
        shapes.append([int(2 ** b) for b in bits])
    return shapes


SHAPES = sweep_shapes()


@pytest.mark.parametrize("dims", SHAPES, ids=lambda d: "x".join(map(str, d)))
def test_sweep(dims, dev):
    n = int(np.prod(dims))
    for i, kind in enumerate(("c", "ci", "r", "ri")):
        if kind in ("r", "ri") and n == 1:
            continue
        fmt = G.afft_interleaved if (n + i) % 3 == 0 else G.afft_split
        a, b = inputs(kind, dims, n + i)
        got = run_plan(kind, dims, a, b, dev, fmt=fmt)
        err = O.rel_l2(got, O.oracle64(kind, dims, a, b))
        assert err <= TOL, (kind, dims, fmt, err)


@pytest.mark.parametrize("dims", SHAPES[::2], ids=lambda d: "x".join(map(str, d)))
def test_sweep_f64(dims, dev):
    # the same shapes through the FP64 transforms (afft_64_*), FP64 bound
    from test_f64_gpu import TOL64, run64
    n = int(np.prod(dims))
    for i, kind in enumerate(("c", "ci", "r", "ri")):
        fmt = G.afft_interleaved if (n + i) % 3 == 1 else G.afft_split
        a, b = inputs(kind, dims, n + i)
        a = np.asarray(a, np.float64)
        b = None if b is None else np.asarray(b, np.float64)
        got = run64(kind, dims, a, b, dev, fmt=fmt)
        err = O.rel_l2(got, O.oracle64(kind, dims, a, b))
        assert err <= TOL64, (kind, dims, fmt, err)
