"""Build recipe for libgbr.so, the renderer's C-ABI library.

nvcc compiles the kernels for sm_103a only (``--fmad=false`` so no
multiply-add fuses unless the source asks for it); g++ compiles the host
runtime with ``-ffp-contract=off`` for the same reason; the result links
against the static CUDA runtime.  Objects build in parallel and are reused
while their sources are unchanged."""
import hashlib
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libgbr.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
CU_SOURCES = ["kernels.cu", "noise.cu", "hbao.cu"]
CPP_SOURCES = ["renderer.cpp", "importer.cpp", "capi.cpp", "replay.cpp", "pool.cpp"]
HEADERS = ["kernels.h", "records.h", "renderer.h", "importer.h", "json.h", "replay.h", "hbao.h", "mips.h",
           "trace.h", "pool.h", "work_items.h"]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _digest(paths, extra):
    h = hashlib.sha256((extra + platform.machine()).encode())
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def build(verbose=False):
    """Compile (if needed) and return the path of libgbr.so."""
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [
        os.path.join(INCLUDE, h) for h in ("gbr.h", "gbr_replay.h", "gbr_noise.h", "gbr_hbao.h")]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        path = os.path.join(CSRC, src)
        cmd = [nvcc, ARCH, "-O3", "-lineinfo", "--fmad=false", "-std=c++17",
               "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + INCLUDE, "-c", path]
        key = _digest([path] + headers, " ".join(cmd[1:]))
        obj = os.path.join(BUILD, f"{src}.{key}.o")
        objs.append(obj)
        if not os.path.exists(obj):
            jobs.append(cmd + ["-o", obj])
    for src in CPP_SOURCES:
        path = os.path.join(CSRC, src)
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
               "-Wall", "-Wno-unused-function", "-I" + os.path.join(cuda, "include"),
               "-I" + INCLUDE, "-c", path]
        key = _digest([path] + headers, " ".join(cmd[1:]))
        obj = os.path.join(BUILD, f"{src}.{key}.o")
        objs.append(obj)
        if not os.path.exists(obj):
            jobs.append(cmd + ["-o", obj])
    procs = [(j, subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT))
             for j in jobs]
    failed = []
    for j, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0 or verbose:
            sys.stderr.write(out.decode(errors="replace"))
        if p.returncode != 0:
            failed.append(" ".join(j))
    if failed:
        raise RuntimeError("compilation failed:\n" + "\n".join(failed))
    link_key = _digest(objs, "link")
    stamp = LIB + ".key"
    if jobs or not os.path.exists(LIB) or not os.path.exists(stamp) or open(stamp).read() != link_key:
        tmp = LIB + f".tmp{os.getpid()}"
        subprocess.check_call([nvcc, ARCH, "-shared", "-cudart", "static", "-o", tmp] + objs +
                              ["-Xlinker", "--no-undefined", "-lpthread", "-ldl", "-lrt"])
        os.replace(tmp, LIB)
        with open(stamp, "w") as f:
            f.write(link_key)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
