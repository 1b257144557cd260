"""Compile C++ programs against the drop-in headers and liblbm2d."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DROPIN = os.path.join(ROOT, "lbm-2d_gb300", "dropin")
INCLUDE = os.path.join(ROOT, "include")
SHIM = os.path.join(ROOT, "tests", "dropin")
LIBDIR = os.path.join(ROOT, "lbm-2d_gb300", "lib")


def compile_dropin(src: str, out: str, extra_after: str | None = None,
                   flags: tuple = ()) -> subprocess.CompletedProcess:
    cmd = ["g++", "-std=c++20", "-O2", "-fopenmp", *flags, f"-I{SHIM}", f"-I{DROPIN}", f"-I{INCLUDE}"]
    if extra_after:
        cmd += ["-idirafter", extra_after]
    cmd += [src, f"-L{LIBDIR}", "-llbm2d", f"-Wl,-rpath,{LIBDIR}", "-o", out]
    return subprocess.run(cmd, capture_output=True, text=True)
