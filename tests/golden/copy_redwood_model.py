"""Copy the Redwood depth distortion model from a habitat-sim checkout.

    python tests/golden/copy_redwood_model.py /path/to/habitat-sim

The model (80 x 400 float32: an 80 x 80 grid over a 640 x 480 sensor, 5
depth bins per cell) is the published Redwood / CLAMS PrimeSense distortion
table that habitat-sim ships as
``src_python/habitat_sim/sensors/noise_models/data/redwood-depth-dist-model.npy``;
it is data, copied byte for byte, with its SHA-256 written beside it.
"""
import hashlib
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
DATA = os.path.join(os.path.dirname(os.path.dirname(HERE)), "habitat-sim_gb300", "data")
NAME = "redwood-depth-dist-model.npy"


def main(root):
    src = os.path.join(root, "src_python", "habitat_sim", "sensors", "noise_models", "data", NAME)
    dst = os.path.join(DATA, NAME)
    shutil.copyfile(src, dst)
    digest = hashlib.sha256(open(dst, "rb").read()).hexdigest()
    with open(dst + ".sha256", "w") as f:
        f.write(f"{digest}  {NAME}\n")
    print(dst, digest)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: copy_redwood_model.py /path/to/habitat-sim")
    main(sys.argv[1])
