"""Recipe for oracle/_ref: the parts of the reference that compile here.

TEST INFRASTRUCTURE ONLY (a checker, never part of the product).  Compiles,
unchanged and where they lie in the reference checkout, the reference's
source files whose arithmetic sits on a path this repository restates, with
a small C driver of this repository's own, into oracle/_ref/:

  libref_hitscan.so  sutil/hitscanprocessing.cpp (isPointWithinMesh, float
                     point-in-mesh parity ray cast) + oracle/ref_hitscan.cpp.
                     Needs only headers from the checkout (sutil/vec_math.h,
                     sutil/Matrix.h, sutil/Aabb.h, support/tinygltf) and CUDA's
                     vector_types.h.

Not buildable here, and therefore not built: the pose math of
libEyeRenderer3/cameras/DataRecordCamera.h:42-87 (its base class header
GenericCamera.h includes optix.h, an external library absent from this
machine), and every device program of libEyeRenderer3/shaders.cu (OptiX).

The checkout's location: argument 1, else $CR_REFERENCE_ROOT, else
/root/reference.  When the checkout is absent (as on a GPU machine) nothing is
built and the tests that need the library skip; the golden fixtures made from
it (tests/golden/make_hitscan_golden.py) stand in there.  The checkout's path
is recorded in oracle/_ref/reference_root.txt for the CPU tests.

Flags: -O2 without floating-point contraction (-ffp-contract=off), so the
float operations are the ones the source writes, on x86-64 and aarch64 alike.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def reference_root(arg=None):
    return arg or os.environ.get("CR_REFERENCE_ROOT") or "/root/reference"


def build(root=None, force=False):
    """Builds oracle/_ref/libref_hitscan.so; returns its path, or None when the
    reference checkout is not present."""
    root = reference_root(root)
    src = os.path.join(root, "sutil", "hitscanprocessing.cpp")
    if not os.path.isfile(src):
        return None
    os.makedirs(OUT, exist_ok=True)
    lib = os.path.join(OUT, "libref_hitscan.so")
    driver = os.path.join(HERE, "ref_hitscan.cpp")
    if force or not os.path.exists(lib) or os.path.getmtime(lib) < max(os.path.getmtime(src), os.path.getmtime(driver)):
        tmp = lib + ".tmp"
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-w",
               "-I" + root, "-I" + os.path.join(root, "support"), "-I" + os.path.join(CUDA_HOME, "include"),
               src, driver, "-o", tmp]
        proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if proc.returncode != 0:
            raise RuntimeError("reference build failed:\n" + " ".join(cmd) + "\n" + proc.stdout)
        os.replace(tmp, lib)
    with open(os.path.join(OUT, "reference_root.txt"), "w") as f:
        f.write(os.path.abspath(root) + "\n")
    return lib


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None, force="-f" in sys.argv))
