"""GPU tests of the autotuner (afft_gb300_tune): it times the plan variants a
shape allows (four-step split, fused or standalone real pre-pass, TMA or LSU
tile loads, cols tile width, plain or tensor-core form), keeps the fastest
for later plans of that shape, and persists choices in the file named by
AFFT_GB300_TUNE_CACHE; plans built from any variant must still agree with
the FP64 oracle, and so must a queue built from tuned per-shape choices."""
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


def test_tune_weighs_plane_fusion(tmp_path, dev):
    # the last two axes of a 3D transform: one plane-fused pass or one pass
    # each; both timed, the faster kept
    rep = G.tune("c", [16, 64, 64], 4)
    cands = rep["candidates"]
    assert {c["no_plane"] for c in cands} == {0, 1}, rep    # (2, fused at any count, is the rule here)
    assert {c["launches"] for c in cands if c["no_plane"]} == {3} and {c["launches"] for c in cands
                                                                      if not c["no_plane"]} == {2}, rep
    timed = [c for c in cands if c["ms"] > 0]
    assert rep["chosen"]["ms"] == min(c["ms"] for c in timed)
    batched_parity("c", [16, 64, 64], 4)
    # the per-axis form forced through the cache file, in a fresh process
    name = torch.cuda.get_device_name(0).replace(" ", "_")
    path = str(tmp_path / "tune_no_plane.json")
    with open(path, "w") as f:
        f.write("{\n\"%s|1|8x64x128|3|0\": {\"split\": 0, \"real_inv\": 0, \"cols_lsu\": 0, \"tc\": 0, "
                "\"cols_c\": 0, \"passes\": 0, \"no_plane\": 1, \"ms\": 1.0}\n}\n" % name)
    code = ("import sys; sys.path.insert(0, %r); sys.path.insert(0, %r)\n"
            "import test_tune_gpu as T\nT.batched_parity('ci', [8, 64, 128], 3)\n" % (ROOT, os.path.join(ROOT, "tests")))
    r = subprocess.run([sys.executable, "-c", code], env=dict(os.environ, AFFT_GB300_TUNE_CACHE=path),
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]


def test_tune_weighs_large_planes_at_small_counts(dev):
    # 2^14-point planes below 256 per launch: the rule takes a pass per
    # axis, and the tuner also times the plane pass (no_plane = 2)
    rep = G.tune("c", [8, 128, 128], 2)
    assert {c["no_plane"] for c in rep["candidates"]} == {0, 2}, rep
    batched_parity("c", [8, 128, 128], 2)


def test_tune_weighs_pipelined_form(dev):
    # 2048-point cols passes: the persistent pipelined kernel or one tile
    # per CTA (at 2048 points the one-tile complex pass loads through the
    # LSU, so that variant and cols_lsu build the same launches); both timed,
    # the faster kept
    rep = G.tune("c", [2048, 2048], 4)
    cands = rep["candidates"]
    assert {c["no_pipe"] for c in cands} == {0, 1}, rep
    timed = [c for c in cands if c["ms"] > 0]
    assert rep["chosen"]["ms"] == min(c["ms"] for c in timed)
    batched_parity("c", [2048, 2048], 4)


def test_tune_shape_without_choices(dev):
    rep = G.tune("c", [1024], 64)
    assert len(rep["candidates"]) == 1 and rep["chosen"]["ms"] < 0


def test_tune_weighs_tile_loads_widths_and_form(dev):
    # 256-point cols passes: TMA or LSU loads, 8/16/32-line tiles, and the
    # tensor-core form; every distinct variant is timed
    rep = G.tune("c", [256, 256, 16], 2)
    cands = rep["candidates"]
    seen = {(c["cols_lsu"], c["cols_c"], c["tc"]) for c in cands}
    assert {(0, 0, 0), (1, 0, 0), (0, 8, 0), (0, 32, 0)} <= seen, rep
    assert any(c["tc"] for c in cands), rep
    timed = [c for c in cands if c["ms"] > 0]
    assert rep["chosen"]["ms"] == min(c["ms"] for c in timed)
    batched_parity("c", [256, 256, 16], 2)


# variants forced through the cache file: the key holds the batch, so each
# batch of one shape can take another variant in one process
VARIANTS = [dict(split=0, real_inv=0, cols_lsu=l, tc=t, cols_c=w)
            for l in (0, 1) for t in (0, 1) for w in (0, 8, 32)]


def test_every_tile_and_form_variant_is_correct(tmp_path, dev):
    name = torch.cuda.get_device_name(0).replace(" ", "_")
    path = str(tmp_path / "tune_variants.json")
    lines = []
    for i, v in enumerate(VARIANTS):
        for kind, code in (("c", 0), ("ci", 1)):
            lines.append("\"%s|%d|256x256x8|%d|0\": {\"split\": 0, \"real_inv\": 0, \"cols_lsu\": %d, \"tc\": %d, "
                         "\"cols_c\": %d, \"ms\": 1.0}" % (name, code, i + 1, v["cols_lsu"], v["tc"], v["cols_c"]))
        lines.append("\"%s|0|512x512|%d|0\": {\"split\": 0, \"real_inv\": 0, \"cols_lsu\": %d, \"tc\": %d, "
                     "\"cols_c\": %d, \"ms\": 1.0}" % (name, i + 1, v["cols_lsu"], v["tc"], 16 if v["cols_c"] else 0))
    with open(path, "w") as f:
        f.write("{\n" + ",\n".join(lines) + "\n}\n")
    code = ("import sys; sys.path.insert(0, %r); sys.path.insert(0, %r)\n"
            "import test_tune_gpu as T\n"
            "for b in range(1, %d):\n"
            "    T.batched_parity('c', [256, 256, 8], b)\n"
            "    T.batched_parity('ci', [256, 256, 8], b)\n"
            "    T.batched_parity('c', [512, 512], b)\n" % (ROOT, os.path.join(ROOT, "tests"), len(VARIANTS) + 1))
    env = dict(os.environ, AFFT_GB300_TUNE_CACHE=path)
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]


def test_tuned_queue_matches_fp64(tmp_path, dev):
    # a queue whose plans take the per-shape queue choices (tuned on first
    # use) against the FP64 oracle, transform by transform
    from fft_gb300 import uneven as U
    code = ("import sys; sys.path.insert(0, %r); sys.path.insert(0, %r)\n"
            "import torch, fft_gb300 as G\nfrom fft_gb300 import uneven as U\n"
            "import test_queue_gpu as Q\n"
            "items = U.uneven_batch(10000, seed=5)[:120]\n"
            "buf, offs = U.allocate(items, torch.device('cuda:0'), seed=6)\n"
            "q = G.Queue(U.descs(items, buf, offs), tuned=True)\n"
            "q.run(); torch.cuda.synchronize()\n"
            "print('worst %%.2e' %% Q._check_all(items, buf, offs))\n" % (ROOT, os.path.join(ROOT, "tests")))
    env = dict(os.environ, AFFT_GB300_TUNE_CACHE=str(tmp_path / "queue_tune.json"))
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    text = open(str(tmp_path / "queue_tune.json")).read()
    assert "|0|0\"" in text          # entries kept under batch 0 (the queue's)
    json.loads(text)


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
