"""Collect the batch renderer's golden fixtures from a habitat-sim checkout.

Run once in a container that has the habitat-sim source tree:

    python tests/golden/make_golden.py /path/to/habitat-sim

It copies, byte for byte, the batch-friendly glTF test scenes and the
expected-output screenshots that habitat-sim's own batch renderer test
(``src/tests/GfxBatchRendererTest.cpp``) renders and compares against, and
writes ``manifest.json`` with their sizes and SHA-256 sums.  The files are
test data (meshes, textures, PNG screenshots), not source code:

* ``data/test_assets/scenes/batch*.gltf|.bin|.ktx2`` -- the scenes the test
  feeds to ``Renderer::addFile`` (``GfxBatchRendererTest.cpp:100-220``);
* ``data/test_assets/screenshots/GfxBatchRendererTest*.png`` -- the golden
  colour images (``GfxBatchRendererTest.cpp:1514-1906``);
* ``data/test_assets/objects/*.glb`` -- the untextured binary glTF objects
  that habitat-sim's replay tests instance through keyframes
  (``BatchReplayRendererTest.cpp:400-487`` uses ``sphere.glb``).

The tests read only the copies in this folder, so they run where the
habitat-sim tree is absent.
"""
import hashlib
import json
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))

SCENES = [
    "batch.gltf", "batch.bin",
    "batch-multiple-meshes.gltf", "batch-multiple-meshes.bin",
    "batch-multiple-textures.gltf", "batch-multiple-textures.bin",
    "batch-square-circle-triangle.gltf", "batch-square-circle-triangle.bin",
    "batch-square-circle-triangle-compressed.gltf",
    "batch-square-circle-triangle.0.2x.dxt.ktx2",
    "batch-four-squares.gltf", "batch-four-squares.bin",
    "batch-four-squares-compressed.gltf", "batch-four-squares.4x.dxt.ktx2",
    "batch-four-squares-no-materials.gltf", "batch-four-squares-no-materials.bin",
    "batch-four-squares-deep-hierarchy-whole-file.gltf",
    "batch-four-squares-deep-hierarchy-whole-file.bin",
    "batch-four-squares-no-scene.gltf", "batch-four-squares-no-scene.bin",
]

OBJECTS = ["sphere.glb", "transform_box.glb", "nested_box.glb", "5boxes.glb"]

SCREENSHOTS = [
    "GfxBatchRendererTestDefaults.png",
    "GfxBatchRendererTestSingleMesh.png",
    "GfxBatchRendererTestMeshHierarchy.png",
    "GfxBatchRendererTestMeshHierarchyNoTextures.png",
    "GfxBatchRendererTestMultipleMeshes.png",
    "GfxBatchRendererTestMultipleScenes.png",
    "GfxBatchRendererTestMultipleScenesClearScene1.png",
    "GfxBatchRendererTestLights.png",
    "GfxBatchRendererTestLightsDisabled.png",
    "GfxBatchRendererTestLightsNone.png",
]


def main(root):
    manifest = {}
    for sub, names in (("scenes", SCENES), ("screenshots", SCREENSHOTS), ("objects", OBJECTS)):
        os.makedirs(os.path.join(HERE, sub), exist_ok=True)
        for name in names:
            src = os.path.join(root, "data", "test_assets", sub, name)
            dst = os.path.join(HERE, sub, name)
            shutil.copyfile(src, dst)
            data = open(dst, "rb").read()
            manifest[f"{sub}/{name}"] = {
                "bytes": len(data),
                "sha256": hashlib.sha256(data).hexdigest(),
                "source": f"data/test_assets/{sub}/{name}",
            }
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
    print(f"wrote {len(manifest)} fixtures")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py /path/to/habitat-sim")
    main(sys.argv[1])
