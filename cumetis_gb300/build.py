"""Build recipe for libcm.so (CUDA kernels for sm_103a + C++ host code) and
the `cuMetis` command-line tool, in-tree under cumetis_gb300/.

    python -m cumetis_gb300.build [-f] [-v]

Translation units compile in parallel; objects go to cumetis_gb300/_build/.
The kernels' tuning macros (thresholds, block shapes) come from
cumetis_gb300/tuned.json when it exists (written by cumetis_gb300.autotune),
then from the CM_EXTRA_DEFINES environment variable.
"""
import concurrent.futures as cf
import hashlib
import json
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
TUNED = os.path.join(HERE, "tuned.json")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["cm_ctx.cu", "cm_match.cu", "cm_cmap.cu", "cm_contract.cu", "cm_refine.cu", "cm_batch.cu", "cm_engine.cu"]
CPP_SOURCES = ["cm_graph.cpp", "cm_initpart.cpp"]
CLI_SOURCES = ["cm_cli.cpp"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _deps():
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    extra = [TUNED] if os.path.exists(TUNED) else []
    return headers + [os.path.join(INCLUDE, "cm.h"), os.path.abspath(__file__)] + extra


def tuned_defines(path=TUNED):
    """-D flags of a tuning file ({"defines": {"CM_X": value, ...}, ...}); none
    when the file does not exist."""
    if not os.path.exists(path):
        return []
    with open(path) as f:
        d = json.load(f).get("defines", {})
    for k, v in d.items():
        if not (k.startswith("CM_") and k.replace("_", "").isalnum() and isinstance(v, int)):
            raise ValueError("%s: bad tuning entry %r=%r" % (path, k, v))
    return ["-D%s=%d" % (k, v) for k, v in sorted(d.items())]


def _cu_cmd(nvcc, src, obj, defines, verbose=False):
    return [nvcc, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", "-I" + INCLUDE,
            "-Xptxas", "-v" if verbose else "-O3", *defines, "-c", src, "-o", obj]


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
    extra = tuned_defines()
    extra += os.environ.get("CM_EXTRA_DEFINES", "").split()  # e.g. "-DCM_MID_THREADS0=512" for tuning runs
    jobs, objs = [], []
    for f in CU_SOURCES:
        src = os.path.join(CSRC, f)
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if force or _stale(obj, src, deps):
            jobs.append((_cu_cmd(nvcc, src, obj, extra, verbose), src))
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


def build_variant(defines_by_source, out_dir):
    """Builds a libcm.so variant into out_dir: each CUDA source compiled with
    its own -D flags (defines_by_source: {"cm_match.cu": ["-DCM_X=1"], ...};
    sources not named get none), linked with the main build's C++ objects.
    Objects are cached under _build/variants by source and flags, so a
    variant that changes one source recompiles only that one.  Returns the
    library path."""
    build()  # the C++ objects (and an up-to-date default library)
    nvcc = _nvcc()
    cache = os.path.join(BUILD, "variants")
    os.makedirs(cache, exist_ok=True)
    os.makedirs(out_dir, exist_ok=True)
    deps = _deps()
    jobs, objs = [], []
    for f in CU_SOURCES:
        src = os.path.join(CSRC, f)
        defs = list(defines_by_source.get(f, []))
        key = hashlib.sha1((f + "|" + " ".join(defs)).encode()).hexdigest()[:16]
        obj = os.path.join(cache, "%s.%s.o" % (f, key))
        objs.append(obj)
        if _stale(obj, src, deps):
            jobs.append((_cu_cmd(nvcc, src, obj, defs), src))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            list(ex.map(_compile, jobs))
    objs += [os.path.join(BUILD, f + ".o") for f in CPP_SOURCES]
    lib = os.path.join(out_dir, "libcm.so")
    subprocess.check_call([nvcc, "-shared", *ARCH, "-o", lib, *objs, "-Xcompiler", "-fopenmp", "-lgomp", "-lpthread"])
    return lib


if __name__ == "__main__":
    print(build(force="-f" in sys.argv, verbose="-v" in sys.argv))
