"""Build recipe for oracle/_ref: the reference's own pyDeform loops, compiled
unchanged from the reference tree (test infrastructure, never the product).

The reference's hot-path sources are compiled where they lie, with g++ -O2
like the reference's CMakeLists.txt:14, against the stand-in headers in
``oracle/ref_shim`` for its un-vendored dependencies:

* ``Eigen/Core``: fixed and dynamic matrices, coefficient-wise arithmetic;
* ``ceres/jet.h``: Ceres' forward-mode Jet rules;
* ``torch/extension.h``: a contiguous tensor with ``size()``,
  ``storage().data()`` and ``torch::full``;
* ``igl/point_mesh_squared_distance.h``: the oracle's FP64 AABB-tree query.

``-ffp-contract=off`` keeps every float operation separately rounded, as the
reference's x86-64 build without FMA instructions does.  The output goes to
``oracle/_ref/libpydeform_ref.so`` (git-ignored), with the C entry points of
``oracle/ref_abi.cc``.  The reference tree exists only where the reference
is mounted; elsewhere ``build()`` returns None and the tests that need the
library skip.
"""
import concurrent.futures as cf
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("MESHODE_REFERENCE", "/root/reference")
OUT_DIR = os.path.join(HERE, "_ref")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
OUT = os.path.join(OUT_DIR, "libpydeform_ref.so")

# The reference files compiled unchanged (paths inside the reference tree).
REF_SOURCES = [
    "src/lib/uniformgrid.cc",
    "src/lib/mesh.cc",
    "src/interface/deform_params.cc",
    "src/interface/mesh_tensor.cc",
    "src/interface/distance_layer.cc",
    "src/interface/rigid_layer.cc",
    "src/interface/graph_layer.cc",
    "src/interface/cad_layer.cc",
    "src/interface/normalize.cc",
]
SHIM = os.path.join(HERE, "ref_shim")
OWN_SOURCES = [os.path.join(HERE, "ref_abi.cc"), os.path.join(HERE, "meshode_oracle.c")]
CXXFLAGS = ["-std=c++14", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-fopenmp", "-w"]
CFLAGS = ["-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-fopenmp", "-w"]


def available() -> bool:
    return all(os.path.exists(os.path.join(REF_ROOT, s)) for s in REF_SOURCES)


def _deps():
    out = [os.path.join(REF_ROOT, s) for s in REF_SOURCES] + OWN_SOURCES + [os.path.abspath(__file__)]
    for d, _, files in os.walk(SHIM):
        out += [os.path.join(d, f) for f in files]
    return out


def build(force: bool = False):
    """Compile oracle/_ref/libpydeform_ref.so; None when the reference is absent."""
    if not available():
        return None
    deps = _deps()
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= max(os.path.getmtime(d) for d in deps):
        return OUT
    os.makedirs(OBJ_DIR, exist_ok=True)
    inc = ["-I", SHIM, "-I", os.path.join(REF_ROOT, "src", "lib"), "-I", os.path.join(REF_ROOT, "src", "interface")]
    jobs = []
    objs = []
    for s in [os.path.join(REF_ROOT, s) for s in REF_SOURCES] + OWN_SOURCES:
        stem = os.path.relpath(s, REF_ROOT if s.startswith(REF_ROOT) else HERE).replace(os.sep, "_")
        obj = os.path.join(OBJ_DIR, stem + ".o")
        objs.append(obj)
        if s.endswith(".c"):
            jobs.append(["gcc"] + CFLAGS + ["-c", s, "-o", obj])
        else:
            jobs.append(["g++"] + CXXFLAGS + inc + ["-c", s, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle/_ref build failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))

    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        list(ex.map(run, jobs))
    run(["g++", "-shared", "-fopenmp", "-o", OUT + ".tmp"] + objs)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
