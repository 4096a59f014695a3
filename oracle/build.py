"""Build recipe for the CPU oracle (test infrastructure, never the product).

Compiles ``oracle/meshode_oracle.c`` into ``oracle/_build/libmeshode_oracle.so``
with gcc.  ``-ffp-contract=off`` is required: the oracle reproduces the
reference's float arithmetic operation by operation, and aarch64 gcc would
otherwise fuse multiply-adds.

The reference itself (hjwdzh/MeshODE) is not compiled into ``oracle/_ref``: its
hot-path sources include Eigen, ceres/jet.h, libigl and torch/extension.h, and
none of those un-vendored dependencies is available, so it is unbuildable here.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "meshode_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
OUT = os.path.join(OUT_DIR, "libmeshode_oracle.so")


def build(force: bool = False) -> str:
    """Compile the oracle shared library if it is missing or stale."""
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(OUT)
            and os.path.getmtime(OUT) >= os.path.getmtime(SRC)):
        return OUT
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math",
           "-fopenmp", "-fPIC", "-shared", "-Wall", "-Wno-unknown-pragmas",
           "-o", OUT + ".tmp", SRC, "-lm"]
    subprocess.check_call(cmd)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
