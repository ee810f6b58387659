"""Builds the native parts of mantiis_gb300 in-tree.

Outputs (git-ignored, rebuilt on each machine):
  mantiis_gb300/lib/libmantiis_gpu.so  C ABI of include/mantiis_gpu.h: host grid
                                       builder (C++) + sm_103a kernels (CUDA)
  mantiis_gb300/bin/mantiis            drop-in for the reference executable
  mantiis_gb300/lib/libmantiis_cnn.so  C ABI of include/mantiis_cnn.h: the warm-start
                                       network's kernels (CUDA)
Object files go to _build/.  Everything is compiled for sm_103a only.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "mantiis_gb300"
CSRC = PKG / "csrc"
OBJ = ROOT / "_build"
LIB = PKG / "lib" / "libmantiis_gpu.so"
BIN = PKG / "bin" / "mantiis"
CNN_LIB = PKG / "lib" / "libmantiis_cnn.so"
CNN_SOURCES = ["cnn/cnn.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

HOST_SOURCES = [
    "host/units.cpp",
    "host/geometry.cpp",
    "host/grid.cpp",
    "host/capi_host.cpp",
    "solver/layout.cpp",
]
CUDA_SOURCES = ["solver/solver.cu", "geometry/pore_props.cu"]
APP_SOURCES = ["app/mantiis_main.cpp"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build mantiis_gb300")


def _headers():
    return [p for p in CSRC.rglob("*") if p.suffix in (".h", ".hpp", ".cuh")] + [ROOT / "include" / "mantiis_gpu.h",
                                                                               ROOT / "include" / "mantiis_cnn.h"]


def _stale(target: Path, deps):
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(str(c) for c in cmd), flush=True)
    r = subprocess.run([str(c) for c in cmd], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(str(c) for c in cmd) + "\n" + r.stdout)
    return r.stdout


def build(verbose=False, jobs=None):
    nvcc = _nvcc()
    OBJ.mkdir(exist_ok=True)
    LIB.parent.mkdir(exist_ok=True)
    BIN.parent.mkdir(exist_ok=True)
    hdrs = _headers()
    steps = []
    objs = []
    for src in HOST_SOURCES:
        s = CSRC / src
        o = OBJ / (src.replace("/", "_") + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            steps.append(["g++", "-std=c++17", "-O2", "-fPIC", "-Wall", "-c", s, "-o", o])
    for src in CUDA_SOURCES:
        s = CSRC / src
        o = OBJ / (src.replace("/", "_") + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            steps.append([nvcc, "-std=c++17", *ARCH, "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-c", s, "-o", o])
    cnn_objs = []
    for src in CNN_SOURCES:
        s = CSRC / src
        o = OBJ / (src.replace("/", "_") + ".o")
        cnn_objs.append(o)
        if _stale(o, [s] + hdrs):
            steps.append([nvcc, "-std=c++17", *ARCH, "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        for out in ex.map(lambda c: _run(c, verbose), steps):
            pass
    if steps or not LIB.exists() or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lpthread"], verbose)
    if not CNN_LIB.exists() or _stale(CNN_LIB, cnn_objs):
        _run([nvcc, *ARCH, "-shared", "-o", CNN_LIB, *cnn_objs], verbose)
    app = [CSRC / a for a in APP_SOURCES]
    if _stale(BIN, app + hdrs + [LIB]):
        _run(["g++", "-std=c++17", "-O2", "-Wall", *app, "-o", BIN, "-L", LIB.parent, "-lmantiis_gpu",
              "-Wl,-rpath,$ORIGIN/../lib"], verbose)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
