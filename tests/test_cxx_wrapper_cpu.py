"""Drop-in check for C++ callers: afft's own C++ wrapper header fft.hpp,
unchanged, compiles against include/afft_gb300.h (through a two-line fft.h
stand-in) and links against libafft_gb300.so.  The wrapper header is read
from the reference sources, so this runs only where they are present."""
import os
import subprocess

import pytest

import fft_gb300 as G
from conftest import ROOT

REF = os.environ.get("AFFT_REF_SRC", "/root/reference")
HERE = os.path.join(ROOT, "tests", "cxx")


def _build(tmp_path):
    exe = str(tmp_path / "wrapper")
    libdir = os.path.dirname(G.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O1", "-I", HERE, "-I", REF, os.path.join(HERE, "wrapper_main.cpp"),
           "-L", libdir, "-lafft_gb300", "-Wl,-rpath," + libdir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.skipif(not os.path.exists(os.path.join(REF, "fft.hpp")), reason="reference sources absent")
def test_reference_cxx_wrapper_links_and_runs(tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
