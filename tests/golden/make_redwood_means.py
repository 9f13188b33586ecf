"""Fixtures of the Redwood depth-noise model computed by habitat-sim's own code.

    python tests/golden/make_redwood_means.py /path/to/habitat-sim

Reads ``src_python/habitat_sim/sensors/noise_models/redwood_depth_noise_model.py``
from the checkout, takes its two model functions ``_undistort`` and
``_simulate`` out of the source with ``ast`` (without importing
``habitat_sim``, which needs the compiled simulator), and runs them with numba's
``jit`` replaced by an identity decorator and ``prange`` by ``range`` (numba is
not installed here; the functions are plain numpy/Python).  The workload is the
reference's own GPU-versus-CPU test (``tests/test_noise_models.py:24-51``): a
256 x 256 ramp of depths 0-20 m, noise multipliers 0 and 1, the mean of 100
simulations (one for multiplier 0, where the model draws no noise: every
simulation is the same).  Writes ``redwood/reference_means.npz`` beside this
script with those means, the sha256 of the source file and the seed of numpy's
global generator, which ``_simulate`` draws its normals from.
"""
import ast
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCE = os.path.join("src_python", "habitat_sim", "sensors", "noise_models",
                      "redwood_depth_noise_model.py")
MODEL = os.path.join("src_python", "habitat_sim", "sensors", "noise_models", "data",
                     "redwood-depth-dist-model.npy")
SEED = 20240517
SIMS = 100


class _NumbaStub:
    """jit(...) returns the function unchanged; prange is range."""

    @staticmethod
    def jit(*args, **kwargs):
        if args and callable(args[0]) and not kwargs:
            return args[0]
        return lambda f: f

    prange = range


def reference_functions(path):
    """(_undistort, _simulate) compiled from the reference file's source."""
    text = open(path).read()
    tree = ast.parse(text)
    wanted = [n for n in tree.body if isinstance(n, ast.FunctionDef)
              and n.name in ("_undistort", "_simulate")]
    assert [n.name for n in wanted] == ["_undistort", "_simulate"], "functions not found"
    module = ast.Module(body=wanted, type_ignores=[])
    ns = {"np": np, "numba": _NumbaStub()}
    exec(compile(module, path, "exec"), ns)
    return ns["_undistort"], ns["_simulate"], hashlib.sha256(text.encode()).hexdigest()


def main(root):
    _, simulate, digest = reference_functions(os.path.join(root, SOURCE))
    model = np.load(os.path.join(root, MODEL)).reshape(80, 80, 5)
    depth = np.linspace(0, 20, num=256 * 256, dtype=np.float32).reshape(256, 256)
    np.random.seed(SEED)
    t0 = time.time()
    mean0 = simulate(depth, model, 0.0).astype(np.float32)
    runs = [simulate(depth, model, 1.0) for _ in range(SIMS)]
    mean1 = np.mean(np.stack(runs, 0), 0).astype(np.float32)
    os.makedirs(os.path.join(HERE, "redwood"), exist_ok=True)
    out = os.path.join(HERE, "redwood", "reference_means.npz")
    np.savez_compressed(out, mult0=mean0, mult1=mean1, sims1=np.int64(SIMS), seed=np.int64(SEED),
                        source_sha256=np.array(digest), source=np.array(SOURCE))
    print(f"{out}: {time.time() - t0:.1f} s, source sha256 {digest}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_redwood_means.py /path/to/habitat-sim")
    main(sys.argv[1])
