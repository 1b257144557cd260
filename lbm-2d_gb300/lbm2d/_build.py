"""In-tree build of liblbm2d.so (CUDA kernels for sm_103a + C++ host runtime).

Translation units are compiled in parallel; the library links the CUDA
runtime statically so it does not depend on which libcudart a host process
(e.g. PyTorch) has loaded.  Rebuilds only when a source is newer than the
library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))  # lbm-2d_gb300/
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "liblbm2d.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _nvcc() -> str:
    p = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblbm2d")
    return p


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]


def _compile(src: str) -> str:
    nvcc = _nvcc()
    base = os.path.splitext(os.path.basename(src))[0]
    out = os.path.join(OBJ, base + ".o")
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", f"-I{INCLUDE}", f"-I{CSRC}"]
    if src.endswith(".cu"):
        cmd = [nvcc, *ARCH, "-lineinfo", *common, "-Xptxas", "-v", "-c", src, "-o", out]
    else:
        # host code: -ffp-contract=off keeps the reference's double rounding
        cmd = [nvcc, *common, "-Xcompiler", "-ffp-contract=off", "-c", src, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if src.endswith(".cu"):
        with open(os.path.join(OBJ, base + ".ptxas.txt"), "w") as fh:
            fh.write(r.stderr)
    return out


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in sources() + _headers())


def build(force: bool = False, quiet: bool = False) -> str:
    if not force and not needs_build():
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        objs = list(ex.map(_compile, sources()))
    tmp = LIB + ".tmp"
    cmd = [_nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if not quiet:
        print(f"built {LIB}")
    return LIB
