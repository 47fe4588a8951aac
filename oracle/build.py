"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/orc.c`` twice with gcc and OpenMP into ``oracle/_build/``:
``liborc_f64.so`` (REAL=double, the float64 oracle) and ``liborc_f32.so``
(REAL=float, the reference's working precision, used for the timed CPU
baseline).  Portable flags only (the same source builds on x86_64 and aarch64).
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")


def lib_path(precision: str) -> str:
    return os.path.join(BUILD, f"liborc_{precision}.so")


def build(force: bool = False) -> None:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "orc.c")
    jobs = []
    for prec, real in (("f64", "double"), ("f32", "float")):
        out = lib_path(prec)
        if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
            continue
        cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", f"-DREAL={real}",
               "-D_DEFAULT_SOURCE", src, "-o", out + ".tmp", "-lm"]
        jobs.append((subprocess.Popen(cmd), out))
    for p, out in jobs:
        if p.wait() != 0:
            raise RuntimeError(f"oracle build failed for {out}")
        os.replace(out + ".tmp", out)


if __name__ == "__main__":
    build(force=True)
    print("built", lib_path("f64"), lib_path("f32"))
