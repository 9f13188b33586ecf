"""The public C++ API (include/gbr.hpp) compiled by a caller and run on the GPU.

tests/native/cpp_api_gpu_test.cpp is the reference's singleMesh test
(src/tests/GfxBatchRendererTest.cpp:1524-1600) written against
gbr::gfx_batch::RendererStandalone; it checks the known-answer pixels and
depths itself, and its colour image must equal the reference's golden
screenshot pixel for pixel (the test's thresholds for uncompressed textures
are 0/0)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import __graft_entry__ as graft
import scenarios

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile(tmp_path, name, src):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    graft.load_package()
    from habitat_sim_gb300 import _lib
    lib = _lib._build.build()
    exe = str(tmp_path / name)
    subprocess.check_call(["g++", "-O1", "-std=c++17", "-Wall", "-Werror", "-ffp-contract=off",
                           "-I" + os.path.join(ROOT, "include"), src, "-o", exe,
                           "-L" + os.path.dirname(lib), "-lgbr",
                           "-Wl,-rpath," + os.path.dirname(lib)])
    return exe


def test_cpp_header_compiles_without_cuda_headers(tmp_path):
    """gbr.hpp needs only gbr.h and the C++ standard library."""
    src = tmp_path / "use.cpp"
    src.write_text('#include "gbr.hpp"\n'
                   "int main() {\n"
                   "  gbr::gfx_batch::RendererConfiguration c;\n"
                   "  c.setTileSizeCount({64, 32}, {2, 3}).setMaxLightCount(0).setAmbientFactor(0.1f);\n"
                   "  gbr::gfx_batch::Matrix4 m = gbr::gfx_batch::Matrix4::scaling(2, 2, 2);\n"
                   "  return (c.raw().tile_size[0] == 64 && m[0][0] == 2.0f) ? 0 : 1;\n"
                   "}\n")
    exe = _compile(tmp_path, "use", str(src))
    assert subprocess.run([exe], timeout=60).returncode == 0


@pytest.mark.gpu
def test_cpp_single_mesh_matches_reference_golden(tmp_path):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    exe = _compile(tmp_path, "cpp_api_gpu_test",
                   os.path.join(ROOT, "tests", "native", "cpp_api_gpu_test.cpp"))
    out_img = tmp_path / "color.rgba"
    res = subprocess.run([exe, scenarios.SCENES, str(out_img)], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "ok" in res.stdout
    img = np.frombuffer(out_img.read_bytes(), np.uint8).reshape(96, 128, 4)
    gold = scenarios.load_png("GfxBatchRendererTestSingleMesh.png")
    assert img.shape == gold.shape
    assert np.array_equal(img, gold)
