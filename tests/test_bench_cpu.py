"""The benchmark's reference arm runs on the host alone (afft itself through
its C API on all host threads where its library is built, else the oracle's
port of afft) and prints the one JSON line the bench contract asks for, with
the same config record as the GPU arm; checked here without a GPU.  Also the
bench's FP64 accuracy reference against the FP64 oracle."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

REQUIRED = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling", "vs_baseline",
            "dtype", "data", "config", "impl", "cpu_baseline", "e2e")


@pytest.mark.parametrize("args", [[], ["--form", "f64"], ["--config", "c3b"], ["--config", "c5"]],
                         ids=["c2", "c2-f64", "c3b", "c5"])
def test_reference_arm_line(args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"] + args, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    for k in REQUIRED:
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "GFLOP/s"
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] in ("reference", "port") and d["cpu_baseline"]["cores"] >= 1
    assert d["dtype"] == ("f64" if "f64" in args else "f32")
    sys.path.insert(0, ROOT)
    import bench
    cfg = args[args.index("--config") + 1] if "--config" in args else "c2"
    ns = bench.argparse.Namespace(batch=0, form="f64" if "f64" in args else "plain")
    assert d["config"] == json.loads(json.dumps(bench.config_record(cfg, ns)))


def test_reference_arm_times_afft_itself_when_built():
    from oracle import oracle as O
    if O.ref_bench_lib() is None:
        pytest.skip("reference afft library not built on this host")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--config", "c3b"], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads(r.stdout.strip().splitlines()[-1])
    assert d["cpu_baseline"]["kind"] == "reference" and "afft" in d["cpu_baseline"]["impl"]


@pytest.mark.parametrize("kind", ["c", "ci", "r", "ri"])
@pytest.mark.parametrize("dims", [[64], [16, 8], [8, 4, 16], [1, 32, 1, 4]])
def test_bench_fp64_reference_matches_oracle(kind, dims):
    """The bench checks GPU outputs against numpy's float64 FFT under afft's
    conventions (unnormalised inverses, dim 0 halved for real transforms,
    the real inverse's map); that must agree with the FP64 oracle."""
    sys.path.insert(0, ROOT)
    import bench
    from oracle import oracle as O
    rng = np.random.default_rng(len(dims) * 10 + len(kind))
    n = int(np.prod(dims))
    ni = O.half_elems(dims) if kind == "ri" else n
    a = rng.standard_normal(ni)
    b = None if kind == "r" else rng.standard_normal(ni)
    got = bench.fp64_reference(kind, dims, a, b)
    o = O.oracle64(kind, dims, a, b)
    ref = o if kind == "ri" else o[0] + 1j * o[1]
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
