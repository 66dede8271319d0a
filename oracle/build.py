"""Build the CPU oracle (test infrastructure only).

Two artefacts:

* ``oracle/liboracle.so`` -- the plain-C restatement in ``oracle/oracle.c``.  Builds
  anywhere gcc exists (x86-64 and aarch64 alike).
* ``oracle/_ref/librbref.so`` -- the reference's own RandBLAS headers, compiled directly
  with g++ (no CMake) against the project-written Random123 / BLAS++ stand-ins in
  ``oracle/shim/`` plus ``oracle/ref_driver.cc``.  Built only where the reference source
  tree is present (``RANDBLAS_REF_DIR``, else ``reference/`` beside the repository); used to pin the
  restatement and to generate ``tests/golden/``.

Nothing in the product imports this module.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference source tree: RANDBLAS_REF_DIR, else a "reference" directory beside this
# repository's root (where the build container mounts it).
REF_DIR = os.environ.get("RANDBLAS_REF_DIR") or os.path.join(
    os.path.dirname(os.path.dirname(HERE)), "reference")
# the float-float sin / cos / log shared by the GPU and the oracle's shared-math mode
FFMATH = os.path.join(os.path.dirname(HERE), "randblas_gb300", "csrc", "rbg_ffmath.cuh")
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "librbref.so")


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources if os.path.exists(s))


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "oracle.c")
    shared = os.path.join(HERE, "shared_math.cc")
    if force or not _newer(ORACLE_SO, [src, shared, FFMATH]):
        with tempfile.TemporaryDirectory() as tmp:
            o1, o2 = os.path.join(tmp, "oracle.o"), os.path.join(tmp, "shared_math.o")
            subprocess.run(["gcc", "-O2", "-std=gnu11", "-fPIC", "-ffp-contract=off", "-fopenmp",
                            "-c", src, "-o", o1], check=True)
            subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I",
                            os.path.dirname(FFMATH), "-c", shared, "-o", o2], check=True)
            subprocess.run(["g++", "-shared", "-fopenmp", o1, o2, "-o", ORACLE_SO, "-lm"],
                           check=True)
    return ORACLE_SO


def ref_available() -> bool:
    return os.path.isfile(os.path.join(REF_DIR, "RandBLAS.hh"))


def build_ref(force: bool = False) -> str | None:
    """Compile the reference headers + shims; returns the .so path or None if no reference."""
    if not ref_available():
        return None
    src = os.path.join(HERE, "ref_driver.cc")
    shim = os.path.join(HERE, "shim")
    deps = [src, FFMATH] + [os.path.join(dp, f) for dp, _, fs in os.walk(shim) for f in fs]
    if force or not _newer(REF_SO, deps):
        os.makedirs(os.path.dirname(REF_SO), exist_ok=True)
        # -I order: the reference tree first (RandBLAS/*.hh), then the shims (Random123/*,
        # blas.hh and the RandBLAS/config.h that CMake would otherwise generate).
        cmd = ["g++", "-O2", "-std=c++20", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
               "-w", "-I", REF_DIR, "-I", shim, "-I", os.path.dirname(FFMATH), src, "-o",
               REF_SO]
        subprocess.run(cmd, check=True)
    return REF_SO


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_oracle(force))
    print(build_ref(force) or "reference tree not present: oracle/_ref not built")
