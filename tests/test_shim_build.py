"""The C++ header shims (include/tira_gb300/) compile against tiralib-style
caller code and link to libtvgb.so (CPU-side: build only)."""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_shim_check(out_dir):
    from tiralib_gb300 import _lib, build as kb
    if not os.path.exists(_lib.LIB_PATH):
        kb.build()
    nvcc = kb.nvcc_path()
    exe = os.path.join(out_dir, "shim_check")
    libdir = os.path.dirname(_lib.LIB_PATH)
    cmd = [nvcc, "-x", "c++", "-std=c++17", os.path.join(REPO, "tests", "cpp", "shim_check.cpp"),
           "-I", os.path.join(REPO, "include"), "-L", libdir, "-ltvgb", "-Xlinker", f"-rpath,{libdir}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_shim_header_compiles_and_links(tmp_path):
    if shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("nvcc not available")
    exe = build_shim_check(str(tmp_path))
    assert os.path.exists(exe)
