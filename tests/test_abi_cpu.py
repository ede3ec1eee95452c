"""The C-ABI library without a GPU: it loads, exports every symbol the public
header declares, and rejects what afft rejects before touching the device."""
import ctypes
import os
import re

import pytest

import fft_gb300 as G
from conftest import ROOT, cuda_available

HEADER = os.path.join(ROOT, "include", "afft_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"#define[^\n]*\n", "", text)
    funcs = set(re.findall(r"AFFT_GB300_API\s+[\w\s\*]*?\b(\w+)\s*\(", text))
    data = set(re.findall(r"extern\s+AFFT_GB300_API\s+const\s+\w+\s+(\w+)\s*;", text))
    return funcs, data


def exported_symbols():
    import subprocess
    out = subprocess.run(["nm", "-D", "--defined-only", G.LIB_PATH], capture_output=True, text=True, check=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def test_library_builds_and_loads():
    assert os.path.exists(G.LIB_PATH)
    G.lib()


def test_every_declared_symbol_is_exported():
    funcs, data = declared_symbols()
    assert len(funcs) >= 38 and data == {"afft_alignment"}
    exported = exported_symbols()
    missing = (funcs | data) - exported
    assert not missing, missing
    for name in funcs | data:
        getattr(G.lib(), name)


def test_fft_h_symbols_present():
    # every entry point of afft's fft.h (fft.h:22-84)
    exported = exported_symbols()
    for bits in ("32", "64"):
        for k in ("c", "ci", "r", "ri"):
            for f in ("memsize", "create", "transform"):
                assert "afft_%s_%s_%s" % (bits, k, f) in exported
        assert "afft_%s_align_size" % bits in exported
    assert {"afft_supported", "afft_alignment"} <= exported


def test_constants():
    assert G.alignment() == 64
    assert G.align_size(0) == 0
    assert G.align_size(1) == 16
    assert G.align_size(16) == 16
    assert G.align_size(17) == 32
    assert G.lib().afft_64_align_size(3) == 8


def _memsize(kind, dims, fmt=0, impl=0):
    arr = (ctypes.c_size_t * len(dims))(*dims)
    return getattr(G.lib(), "afft_32_%s_memsize" % kind)(len(dims), arr, fmt, impl)


@pytest.mark.parametrize("kind", ["c", "ci", "r", "ri"])
def test_rejections_before_device(kind):
    # non power of two: afft hangs here; this library returns 0 with EINVAL
    assert _memsize(kind, [12]) == 0
    assert G.last_error()[0] == 1
    assert _memsize(kind, [4, 0]) == 0
    # a CPU backend of afft: not available here
    assert _memsize(kind, [16], impl=G.afft_avx2) == 0
    # unknown format: (size_t)-1 as afft's impl.hpp:38-39
    assert _memsize(kind, [16], fmt=7) == ctypes.c_size_t(-1).value
    # FP64 entry points: the same validation
    ms64 = getattr(G.lib(), "afft_64_%s_memsize" % kind)
    assert ms64(1, (ctypes.c_size_t * 1)(12), 0, 0) == 0
    assert G.last_error()[0] == 1
    assert ms64(1, (ctypes.c_size_t * 1)(16), 0, G.afft_avx2) == 0
    assert ms64(1, (ctypes.c_size_t * 1)(16), 7, 0) == ctypes.c_size_t(-1).value


@pytest.mark.skipif(cuda_available(), reason="checks the no-device path")
def test_no_device():
    assert not G.supported(G.afft_auto)
    assert not G.supported(G.afft_gb300)
    assert _memsize("c", [16]) == 0
    assert G.last_error()[0] == 2
    with pytest.raises(G.AfftError):
        G.complex_transform([16])


def test_release_unknown_plan():
    buf = ctypes.create_string_buffer(128)
    assert G.lib().afft_gb300_release(ctypes.addressof(buf)) == 5
    assert G.lib().afft_gb300_plan_launches(ctypes.addressof(buf)) == -1


def test_python_front_end_checks_arrays():
    # a wrong element type, a short array or a strided view is refused before
    # any pointer reaches the library
    import numpy as np
    V = G._validate
    f32, f64 = np.zeros(64, np.float32), np.zeros(64, np.float64)
    V("c", [64], 1, G.afft_split, 32, f32, f32, f32, f32)
    V("c", [64], 1, G.afft_split, 64, f64, f64, f64, f64)
    V("r", [64], 1, G.afft_split, 32, f32, None, np.zeros(33, np.float32), np.zeros(33, np.float32))
    V("ri", [64], 1, G.afft_interleaved, 32, np.zeros(66, np.float32), None, f32, None)
    V("c", [64], 1, G.afft_split, 32, 12345, 12345, 12345, 12345)            # raw pointers: unchecked
    with pytest.raises(G.AfftError, match="float64"):
        V("c", [64], 1, G.afft_split, 64, f32, f32, f32, f32)
    with pytest.raises(G.AfftError, match="elements"):
        V("c", [64], 2, G.afft_split, 32, f32, f32, f32, f32)
    with pytest.raises(G.AfftError, match="elements"):
        V("c", [64], 1, G.afft_interleaved, 32, f32, None, f32, None)        # needs 128 per array
    with pytest.raises(G.AfftError, match="contiguous"):
        V("c", [32], 1, G.afft_split, 32, f32[::2], f32, f32, f32)
