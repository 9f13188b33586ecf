"""Native (C++) unit tests of host code in the renderer library, compiled
here with g++ against the built libgbr.so; no GPU."""
import os
import shutil
import subprocess

import pytest

import __graft_entry__ as graft

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "habitat-sim_gb300", "csrc")


def _cuda_include():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.isdir(os.path.join(c, "include")):
            return os.path.join(c, "include")
    pytest.skip("CUDA headers not found")


@pytest.mark.parametrize("name", ["worker_pool_test", "json_test", "c_abi_test", "work_items_test"])
def test_native(name, tmp_path):
    if shutil.which("g++") is None or shutil.which("gcc") is None:
        pytest.skip("g++/gcc not available")
    graft.load_package()
    from habitat_sim_gb300 import _lib
    lib = _lib._build.build()
    exe = str(tmp_path / name)
    src = os.path.join(ROOT, "tests", "native", name + ".cpp")
    if os.path.exists(src):
        cmd = ["g++", "-O1", "-std=c++17", "-pthread", "-I" + CSRC, "-I" + _cuda_include()]
    else:  # the public headers as plain C, without the CUDA headers
        src = os.path.join(ROOT, "tests", "native", name + ".c")
        cmd = ["gcc", "-O1", "-std=c99", "-Wall", "-Werror", "-pedantic"]
    subprocess.check_call(cmd + ["-I" + os.path.join(ROOT, "include"), src, "-o", exe,
                                 "-L" + os.path.dirname(lib), "-lgbr", "-Wl,-rpath," + os.path.dirname(lib)])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert "ok" in out.stdout
