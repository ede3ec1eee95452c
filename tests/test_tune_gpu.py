"""GPU tests of the autotuner (afft_gb300_tune): it times the plan variants a
shape allows, keeps the fastest for later plans of that shape, and persists
choices in the file named by AFFT_GB300_TUNE_CACHE; plans built from a tuned
choice must still agree with the FP64 oracle."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import fft_gb300 as G
from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def batched_parity(kind, dims, batch):
    n = int(np.prod(dims))
    h = O.half_elems(dims)
    nin = (h if kind == "ri" else n)
    nout = (h if kind == "r" else n)
    rng = np.random.default_rng(n + batch)
    a = rng.standard_normal(nin * batch).astype(np.float32)
    b = rng.standard_normal(nin * batch).astype(np.float32)
    p = G.BatchPlan(kind, dims, batch)
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    oa = torch.zeros(nout * batch, device="cuda")
    ob = torch.zeros_like(oa)
    p.launch(da, None if kind == "r" else db, oa, None if kind == "ri" else ob)
    torch.cuda.synchronize()
    ga, gb = oa.cpu().numpy(), ob.cpu().numpy()
    for t in (0, batch - 1):
        si, so = slice(t * nin, (t + 1) * nin), slice(t * nout, (t + 1) * nout)
        ref = O.oracle64(kind, dims, a[si], None if kind == "r" else b[si])
        got = ga[so] if kind == "ri" else (ga[so], gb[so])
        assert O.rel_l2(got, ref) <= 2e-6, (kind, dims, t)


@pytest.mark.parametrize("kind,dims,batch", [("c", [1 << 17], 16), ("ci", [1 << 15], 64), ("r", [1 << 18], 8),
                                             ("ri", [1 << 16], 32), ("c", [4, 1 << 17], 2)], ids=str)
def test_tune_picks_the_fastest_and_plans_stay_correct(kind, dims, batch, dev):
    rep = G.tune(kind, dims, batch)
    cands = rep["candidates"]
    assert len(cands) >= 2, rep            # odd-length four-step axes: two splits at least
    timed = [c for c in cands if c["ms"] > 0]
    assert timed, rep
    best = min(timed, key=lambda c: c["ms"])
    assert rep["chosen"]["ms"] == best["ms"]
    assert G.tuned(kind, dims, batch) == {"split": rep["chosen"]["split"], "real_inv": rep["chosen"]["real_inv"]}
    batched_parity(kind, dims, batch)


def test_tune_shape_without_choices(dev):
    rep = G.tune("c", [4096], 64)
    assert len(rep["candidates"]) == 1 and rep["chosen"]["ms"] < 0


def test_every_variant_is_correct(tmp_path, dev):
    # force each choice through the cache file, one fresh process per variant
    for split in (0, 1):
        for real_inv in (0, 1):
            code = ("import sys; sys.path.insert(0, %r); sys.path.insert(0, %r)\n"
                    "import test_tune_gpu as T\nT.batched_parity('ri', [1 << 16], 8)\n"
                    "T.batched_parity('c', [1 << 17], 4)\n" % (ROOT, os.path.join(ROOT, "tests")))
            path = str(tmp_path / ("tune_variant_%d_%d.json" % (split, real_inv)))
            name = torch.cuda.get_device_name(0).replace(" ", "_")
            with open(path, "w") as f:
                f.write("{\n\"%s|3|65536|8|0\": {\"split\": %d, \"real_inv\": %d, \"ms\": 1.0},\n"
                        "\"%s|0|131072|4|0\": {\"split\": %d, \"real_inv\": %d, \"ms\": 1.0}\n}\n"
                        % (name, split, real_inv, name, split, real_inv))
            env = dict(os.environ, AFFT_GB300_TUNE_CACHE=path)
            r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
            assert r.returncode == 0, r.stderr[-2000:]


def test_cache_file_round_trip_and_autotune(tmp_path, dev):
    path = str(tmp_path / "tune.json")
    env = dict(os.environ, AFFT_GB300_TUNE_CACHE=path)
    code1 = ("import sys; sys.path.insert(0, %r)\nimport fft_gb300 as G\n"
             "r = G.tune('c', [1 << 17], 8)\nprint(r['chosen']['split'])\n" % ROOT)
    r1 = subprocess.run([sys.executable, "-c", code1], env=env, capture_output=True, text=True, timeout=600)
    assert r1.returncode == 0, r1.stderr[-2000:]
    text = open(path).read()
    assert "|0|131072|8|0" in text
    json.loads(text)                      # the file is valid JSON
    code2 = ("import sys; sys.path.insert(0, %r)\nimport fft_gb300 as G\n"
             "print(G.tuned('c', [1 << 17], 8)['split'])\n" % ROOT)
    r2 = subprocess.run([sys.executable, "-c", code2], env=env, capture_output=True, text=True, timeout=600)
    assert r2.returncode == 0 and r2.stdout.strip() == r1.stdout.strip(), (r1.stdout, r2.stdout, r2.stderr[-2000:])
    # AFFT_GB300_AUTOTUNE=1: a new shape is tuned when its first plan is built
    env2 = dict(env, AFFT_GB300_AUTOTUNE="1")
    code3 = ("import sys; sys.path.insert(0, %r)\nimport fft_gb300 as G\n"
             "assert G.tuned('c', [1 << 15], 32) is None\np = G.BatchPlan('c', [1 << 15], 32)\n"
             "print(G.tuned('c', [1 << 15], 32) is not None)\n" % ROOT)
    r3 = subprocess.run([sys.executable, "-c", code3], env=env2, capture_output=True, text=True, timeout=600)
    assert r3.returncode == 0 and r3.stdout.strip() == "True", (r3.stdout, r3.stderr[-2000:])
