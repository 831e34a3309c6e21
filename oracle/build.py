"""Build recipes for the oracle (test infrastructure only).

build_oracle(): gcc -> oracle/liboracle.so   (the C restatement, cm_oracle.c)
build_ref():    nvcc -> oracle/_ref/libref.so (include-harness around the
                unmodified reference sources; only where the reference tree
                is present, i.e. never on a machine that only runs tests)
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference tree: $CM_REFERENCE_TREE, else a directory named "reference"
# beside this repository.
REF_TREE = os.environ.get("CM_REFERENCE_TREE") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_oracle(force=False):
    src = os.path.join(HERE, "cm_oracle.c")
    out = os.path.join(HERE, "liboracle.so")
    if force or not _newer(out, [src]):
        subprocess.check_call(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", src, "-o", out])
    return out


def build_ref(force=False):
    """Returns the path of libref.so, or None when the reference tree is absent."""
    if not os.path.isfile(os.path.join(REF_TREE, "cuMetis.cu")):
        return None
    src = os.path.join(HERE, "ref_harness.cu")
    outdir = os.path.join(HERE, "_ref")
    out = os.path.join(outdir, "libref.so")
    if not force and _newer(out, [src]):
        return out
    os.makedirs(outdir, exist_ok=True)
    # The reference's own Makefile line (-std=c++11, sm_80 only) does not
    # build with CUDA 13; its sources compile unchanged with -std=c++17.
    cmd = ["nvcc", "-std=c++17", "-O2", "-shared", "-Xcompiler", "-fPIC",
           "-gencode", "arch=compute_103a,code=sm_103a", "--expt-relaxed-constexpr", "-w",
           "-I" + REF_TREE, "-I" + os.path.join(REF_TREE, "include"), src, "-o", out]
    subprocess.check_call(cmd)
    return out


if __name__ == "__main__":
    print(build_oracle(force="-f" in sys.argv))
    print(build_ref(force="-f" in sys.argv))
