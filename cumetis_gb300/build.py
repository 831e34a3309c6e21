"""Build recipe for libcm.so (CUDA kernels for sm_103a + C++ host code) and
the `cuMetis` command-line tool, in-tree under cumetis_gb300/.

    python -m cumetis_gb300.build [-f] [-v]

Translation units compile in parallel; objects go to cumetis_gb300/_build/.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcm.so")
CLI = os.path.join(HERE, "cuMetis")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["cm_ctx.cu", "cm_match.cu", "cm_cmap.cu", "cm_contract.cu", "cm_refine.cu"]
CPP_SOURCES = ["cm_graph.cpp", "cm_initpart.cpp", "cm_engine.cpp"]
CLI_SOURCES = ["cm_cli.cpp"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _deps():
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return headers + [os.path.join(INCLUDE, "cm.h"), os.path.abspath(__file__)]


def _stale(obj, src, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src] + deps)


def _compile(args):
    cmd, src = args
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (src, " ".join(cmd), r.stdout))
    return r.stdout


def build(force=False, verbose=False):
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    deps = _deps()
    extra = []
    extra += os.environ.get("CM_EXTRA_DEFINES", "").split()  # e.g. "-DCM_MID_THREADS0=512" for tuning runs
    jobs, objs = [], []
    for f in CU_SOURCES:
        src = os.path.join(CSRC, f)
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if force or _stale(obj, src, deps):
            jobs.append(([nvcc, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", "-I" + INCLUDE,
                          "-Xptxas", "-v" if verbose else "-O3", *extra, "-c", src, "-o", obj], src))
    for f in CPP_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if force or _stale(obj, src, deps):
            jobs.append((["g++", "-std=c++17", "-O2", "-fPIC", "-fopenmp", "-I" + INCLUDE, *extra, "-c", src, "-o",
                          obj], src))
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            logs = list(ex.map(_compile, jobs))
    if jobs or not os.path.exists(LIB):
        subprocess.check_call([nvcc, "-shared", *ARCH, "-o", LIB, *objs, "-Xcompiler", "-fopenmp", "-lgomp",
                               "-lpthread"])
    cli_srcs = [os.path.join(CSRC, f) for f in CLI_SOURCES if os.path.exists(os.path.join(CSRC, f))]
    if cli_srcs and (force or jobs or not os.path.exists(CLI) or _stale(CLI, cli_srcs[0], deps + [LIB])):
        subprocess.check_call(["g++", "-std=c++17", "-O2", "-I" + INCLUDE, *cli_srcs, "-o", CLI, "-L" + HERE, "-lcm",
                               "-Wl,-rpath,$ORIGIN"])
    if verbose:
        for l in logs:
            sys.stdout.write(l)
    return LIB


if __name__ == "__main__":
    print(build(force="-f" in sys.argv, verbose="-v" in sys.argv))
