"""The atmosphere::Model C++ facade (include/atmosphere/model.h): a program
written against the reference's atmosphere/model.h compiles unchanged and
links libatmo_gb300.so.  The C++ test program builds with g++ here and on the
GPU host; its host checks run everywhere, Init only on a GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def facade_binary(atmo, tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    out = str(tmp_path_factory.mktemp("cxx") / "model_facade_test")
    libdir = os.path.dirname(atmo.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror",
           "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cxx", "model_facade_test.cc"),
           "-o", out, "-L", libdir, "-l:" + os.path.basename(atmo.LIB_PATH),
           "-Wl,-rpath," + libdir]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def run(binary, mode):
    p = subprocess.run([binary, mode], capture_output=True, text=True, timeout=600)
    assert p.returncode == 0 and p.stdout.strip().endswith("ok"), p.stdout + p.stderr


def test_facade_host_behaviour(facade_binary):
    run(facade_binary, "host")


@pytest.mark.gpu
def test_facade_init_matches_c_abi(facade_binary, torch_cuda):
    run(facade_binary, "gpu")
