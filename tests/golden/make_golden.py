"""Generate the golden fixtures that pin the oracle and the GPU library to the
reference afft library's own float outputs.

Runs HERE only (x86-64 with the reference sources): it builds
oracle/_ref/libafft_ref.so from the reference's source files (oracle/Makefile
target ``ref``), then for every case calls the reference's C API (fft.h) with
afft_scalar and with afft_auto (its best SIMD backend on this host) and saves
inputs and both outputs to ``afft_golden.npz``.  The committed .npz travels to
the GPU machine; the reference does not.

Inputs follow the reference harness (testing.cpp:1064-1067): std::mt19937
seeded per case, uniform_real_distribution<float>(-1, 1).  Real-inverse inputs
are a random (non-Hermitian) half spectrum, so the fixture pins the exact map
afft computes, including how it ignores the imaginary parts of planes 0 and
d0/2.  Case 'c1' is the reference harness's own n=1024 input (default seed,
re block then im block).

With ``--f64`` it writes ``afft_golden64.npz`` / ``.json`` instead: the same
cases plus the lengths where FP64 plans change shape, through the
reference's double entry points (afft_64_*, fft.h:52-80).  Inputs are the
same mt19937 floats (stored as float32, exact) widened to double; the output
stored is afft_scalar's, and the json records how far afft_auto's differs.

With ``--configs`` it writes ``afft_golden_configs.npz`` / ``.json``: afft's
float outputs (scalar backend and afft_auto) at the benchmark configurations'
full sizes -- n=4096, n=65536, 256^3 complex, a 2^20-point real transform, and
4096^2 real forward and inverse.  The inputs are not stored: they are the
mt19937 uniform[-1,1) values of the case's seed, which the oracle's
generator reproduces on any host.  Only the outputs at a seeded sample of
4096 indices per array are stored, to keep the fixture small.

    python tests/golden/make_golden.py            # FP32 fixtures
    python tests/golden/make_golden.py --f64      # FP64 fixtures
    python tests/golden/make_golden.py --configs  # config-size samples
"""
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

AFFT_SCALAR = 1
AFFT_AUTO = 0

SHAPES = [
    [1], [2], [4], [8], [16], [32], [64], [128], [256], [512], [1024], [2048],
    [4096], [8192],
    [2, 2], [4, 8], [8, 4], [16, 16], [2, 64], [64, 2], [32, 128], [128, 32],
    [2, 4, 8], [8, 8, 8], [4, 16, 2], [16, 16, 16],
    [4, 4, 4, 4], [2, 8, 2, 8], [2, 2, 4, 2, 8],
    [1, 64], [16, 1, 8], [32, 1], [1, 1, 1], [1, 1, 4, 1],
]
KINDS = ["c", "ci", "r", "ri"]
# FP64 fixtures also cover the lengths where the FP64 plans change shape
# (one CTA up to 2^13 points in rows, 2^11 in cols)
SHAPES64 = SHAPES + [[16384], [32768], [4096, 4]]


def cases(shapes=SHAPES):
    seed = 1
    for dims in shapes:
        n = int(np.prod(dims))
        for kind in KINDS:
            # the reference crashes on real transforms of total size 1
            if kind in ("r", "ri") and n == 1:
                continue
            seed += 1
            yield "%s_%s" % (kind, "x".join(map(str, dims))), kind, dims, seed


def main_f64():
    arrays = {}
    index = []
    for name, kind, dims, seed in cases(SHAPES64):
        # the longer real shapes only for the real kinds (their complex
        # cases repeat the four-step of [16384]), keeping the fixture small
        if dims in ([32768], [4096, 4]) and kind in ("c", "ci"):
            continue
        n = int(np.prod(dims))
        h = O.half_elems(dims)
        m = 2 * n if kind in ("c", "ci") else (n if kind == "r" else 2 * h)
        v32 = O.mt19937_uniform(m, seed)
        v = v32.astype(np.float64)
        if kind in ("c", "ci"):
            a, b = v[:n], v[n:]
            arrays[name + "/in0"], arrays[name + "/in1"] = v32[:n], v32[n:]
        elif kind == "r":
            a, b = v, None
            arrays[name + "/in0"] = v32
        else:
            a, b = v[:h], v[h:]
            arrays[name + "/in0"], arrays[name + "/in1"] = v32[:h], v32[h:]
        out = O.ref_run(kind, dims, a, b, AFFT_SCALAR, bits=64)
        alt = O.ref_run(kind, dims, a, b, AFFT_AUTO, bits=64)
        if kind == "ri":
            arrays[name + "/scalar0"] = out
        else:
            arrays[name + "/scalar0"], arrays[name + "/scalar1"] = out
        index.append({"name": name, "kind": kind, "dims": dims, "seed": seed,
                      "auto_vs_scalar_rel_l2": O.rel_l2(alt, out)})
    np.savez_compressed(os.path.join(HERE, "afft_golden64.npz"), **arrays)
    with open(os.path.join(HERE, "afft_golden64.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py --f64",
                   "reference_impls": {"scalar": AFFT_SCALAR},
                   "inputs": "float32 values, widened to double for the transform",
                   "cases": index}, f, indent=1)
    print("wrote %d FP64 cases" % len(index))


# (name, kind, dims, seed) of the config-size cases
CONFIG_CASES = [("c_4096", "c", [4096], 101), ("c_65536", "c", [65536], 102), ("c_256x256x256", "c", [256, 256, 256], 103),
                ("r_1048576", "r", [1 << 20], 104), ("r_4096x4096", "r", [4096, 4096], 105),
                ("ri_4096x4096", "ri", [4096, 4096], 106)]
CONFIG_SAMPLE = 4096


def config_inputs(kind, dims, seed):
    """The inputs of a config-size case: mt19937(seed) uniform[-1,1)
    floats, re block then im block (the harness's layout)."""
    n = int(np.prod(dims))
    h = O.half_elems(dims)
    if kind in ("c", "ci"):
        v = O.mt19937_uniform(2 * n, seed)
        return v[:n], v[n:]
    if kind == "r":
        return O.mt19937_uniform(n, seed), None
    v = O.mt19937_uniform(2 * h, seed)
    return v[:h], v[h:]


def config_sample_index(kind, dims, seed):
    n = int(np.prod(dims))
    m = O.half_elems(dims) if kind == "r" else n
    return np.sort(np.random.default_rng(seed).choice(m, CONFIG_SAMPLE, replace=False)).astype(np.int64)


def main_configs():
    arrays = {}
    index = []
    for name, kind, dims, seed in CONFIG_CASES:
        a, b = config_inputs(kind, dims, seed)
        idx = config_sample_index(kind, dims, seed)
        arrays[name + "/index"] = idx
        for tag, impl in (("scalar", AFFT_SCALAR), ("auto", AFFT_AUTO)):
            out = O.ref_run(kind, dims, a, b, impl)
            if kind == "ri":
                arrays[name + "/%s0" % tag] = out[idx]
            else:
                arrays[name + "/%s0" % tag] = out[0][idx]
                arrays[name + "/%s1" % tag] = out[1][idx]
        index.append({"name": name, "kind": kind, "dims": dims, "seed": seed, "sample": CONFIG_SAMPLE})
        print(name, flush=True)
    np.savez_compressed(os.path.join(HERE, "afft_golden_configs.npz"), **arrays)
    with open(os.path.join(HERE, "afft_golden_configs.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py --configs",
                   "reference_impls": {"scalar": AFFT_SCALAR, "auto": AFFT_AUTO},
                   "inputs": "mt19937(seed) uniform[-1,1) floats (oracle.mt19937_uniform), re block then im block",
                   "outputs": "sampled at the stored indices (np.random.default_rng(seed).choice, sorted)",
                   "cases": index}, f, indent=1)
    print("wrote %d config-size cases" % len(index))


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all", "ref"], check=True)
    if "--f64" in sys.argv[1:]:
        return main_f64()
    if "--configs" in sys.argv[1:]:
        return main_configs()
    arrays = {}
    index = []
    for name, kind, dims, seed in cases():
        n = int(np.prod(dims))
        h = O.half_elems(dims)
        if kind in ("c", "ci"):
            v = O.mt19937_uniform(2 * n, seed)
            a, b = v[:n], v[n:]
        elif kind == "r":
            a, b = O.mt19937_uniform(n, seed), None
        else:
            v = O.mt19937_uniform(2 * h, seed)
            a, b = v[:h], v[h:]
        arrays[name + "/in0"] = a
        if b is not None:
            arrays[name + "/in1"] = b
        for tag, impl in (("scalar", AFFT_SCALAR), ("auto", AFFT_AUTO)):
            out = O.ref_run(kind, dims, a, b, impl)
            if kind == "ri":
                arrays[name + "/%s0" % tag] = out
            else:
                arrays[name + "/%s0" % tag] = out[0]
                arrays[name + "/%s1" % tag] = out[1]
        index.append({"name": name, "kind": kind, "dims": dims, "seed": seed})

    # C1: the reference harness's own n=1024 complex input, then its inverse
    n = 1024
    v = O.mt19937_uniform(2 * n, 5489)
    arrays["c1/in0"], arrays["c1/in1"] = v[:n], v[n:]
    for tag, impl in (("scalar", AFFT_SCALAR), ("auto", AFFT_AUTO)):
        fr, fi = O.ref_run("c", [n], v[:n], v[n:], impl)
        arrays["c1/%s0" % tag], arrays["c1/%s1" % tag] = fr, fi
        br, bi = O.ref_run("ci", [n], fr, fi, impl)
        arrays["c1/%s_inv0" % tag], arrays["c1/%s_inv1" % tag] = br / n, bi / n
    index.append({"name": "c1", "kind": "c", "dims": [n], "seed": 5489})

    np.savez_compressed(os.path.join(HERE, "afft_golden.npz"), **arrays)
    with open(os.path.join(HERE, "afft_golden.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py",
                   "reference_impls": {"scalar": AFFT_SCALAR, "auto": AFFT_AUTO},
                   "cases": index}, f, indent=1)
    print("wrote %d cases" % len(index))


if __name__ == "__main__":
    main()
