"""Autotuner for the kernels' thresholds and block shapes.

    python -m cumetis_gb300.autotune [--workload rmat22] [--steps 40] [--out cumetis_gb300/tuned.json]

Each tuning parameter is a macro of one CUDA source (the warp-per-vertex
threshold and the warp work-item size of the matching, the longest row the
contraction sorts in one-warp batches and its chunk size, the block shapes of
their kernels, the resident blocks per SM each size-class shape is compiled
for).  The search is coordinate descent from the current tuning file (or
the compiled-in defaults): for each parameter in turn every other candidate
value is built as a library variant (only the source it belongs to is
recompiled), timed with bench.py in a fresh process on the same workload,
and kept when it is at least --min-gain faster than the incumbent.  The
winner must then pass a parity subset of the GPU tests before the tuning
file is written; `build()` compiles it in from then on.  Needs a GPU.
"""
import argparse
import json
import os
import subprocess
import sys
import time

from . import build as B

ROOT = os.path.dirname(B.HERE)

# (macro, compiled-in default, candidates, source it belongs to)
PARAMS = [
    ("CM_SERIAL_DEG", 16, [8, 16], "cm_match.cu"),          # rows scanned by one lane (warp-per-vertex threshold)
    ("CM_MATCH_CHUNK", 256, [128, 256, 512], "cm_match.cu"),  # entries per warp work item
    ("CM_FIRST_MINBLOCKS", 8, [4, 6, 8], "cm_match.cu"),     # first-round kernel: blocks per SM (register cap)
    ("CM_FIRST_KEEP_SHORT", 2, [1, 2, 4], "cm_match.cu"),    # candidates the first round keeps (lane rows)
    ("CM_FIRST_KEEP_CHUNK", 2, [1, 2, 4], "cm_match.cu"),    # ... and per chunked row
    ("CM_TAIL_ITEMS", 4096, [1024, 4096, 16384], "cm_match.cu"),  # rounds this small run in one block
    ("CM_TINY_MAX", 64, [16, 32, 64], "cm_contract.cu"),    # rows sorted in one-warp batches; larger rows by size class
    ("CM_CHUNK", 16384, [8192, 16384], "cm_contract.cu"),    # huge-row segment (chunk) size
    ("CM_CHUNK_THREADS", 1024, [512, 1024], "cm_contract.cu"),  # threads sorting one chunk
    ("CM_CLASS_ITEMS", 16, [8, 16], "cm_contract.cu"),        # entries per thread of the size-class blocks
    ("CM_MERGE_THREADS", 256, [256, 512], "cm_contract.cu"),
    # resident blocks per SM asked of the compiler for a size-class shape (0: no launch bound)
    ("CM_MB_32_12", 32, [0, 32], "cm_contract.cu"),
    ("CM_MB_32_16", 22, [0, 22, 28], "cm_contract.cu"),
    ("CM_MB_64_16", 13, [0, 13, 16], "cm_contract.cu"),
    ("CM_MB_128_12", 9, [0, 9, 12], "cm_contract.cu"),
    ("CM_MB_128_16", 6, [0, 6, 8], "cm_contract.cu"),
    ("CM_MB_256_16", 3, [0, 3, 4], "cm_contract.cu"),
    ("CM_MB_512_16", 2, [0, 2], "cm_contract.cu"),
]
DEFAULTS = {name: d for name, d, _, _ in PARAMS}
SOURCE = {name: src for name, _, _, src in PARAMS}
CHECK_TESTS = "test_long_rows or test_contract_bitexact or test_coarsen_hierarchy or test_match_bitexact_synthetic"


def valid(cfg):
    """The sources' static constraints on combinations."""
    return (cfg["CM_CHUNK"] // cfg["CM_TINY_MAX"] <= 256  # at most sixteen size classes
            and cfg["CM_CHUNK"] // cfg["CM_CHUNK_THREADS"] <= 16  # at most 16 pairs per thread of a chunk sort
            and cfg["CM_CHUNK"] // cfg["CM_CLASS_ITEMS"] <= 1024)  # the largest class's block fits 1024 threads


def defines_by_source(cfg):
    """Non-default values as -D flags, per source."""
    out = {}
    for name, v in cfg.items():
        if v != DEFAULTS[name]:
            out.setdefault(SOURCE[name], []).append("-D%s=%d" % (name, v))
    return {k: sorted(v) for k, v in out.items()}


def variant_dir(cfg):
    tag = "_".join("%s%d" % (n.replace("CM_", "").lower(), cfg[n]) for n in sorted(cfg) if cfg[n] != DEFAULTS[n])
    return os.path.join(B.BUILD, "variants", "lib_" + (tag or "default"))


def bench_ms(lib, workload, steps, warmup, timeout=900):
    """ms per step of bench.py on `workload`, run against the library `lib`."""
    env = dict(os.environ, CUMETIS_LIB=lib)
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--workload", workload, "--steps", str(steps),
           "--warmup", str(warmup), "--no-cpu-baseline", "--no-e2e"]
    r = subprocess.run(cmd, env=env, cwd=ROOT, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError("bench failed (%s):\n%s" % (lib, r.stdout[-2000:]))
    for line in r.stdout.splitlines():
        if line.startswith("{"):
            return float(json.loads(line)["ms_per_step"])
    raise RuntimeError("no JSON line from bench:\n" + r.stdout[-2000:])


def search(start, measure, min_gain=0.01, log=print):
    """Coordinate descent over PARAMS from `start` with measure(cfg) -> ms.
    Returns (best cfg, its ms, trials [(cfg, ms or None)])."""
    cfg = dict(start)
    best = measure(cfg)
    trials = [(dict(cfg), best)]
    log("start %.3f ms %s" % (best, defines_by_source(cfg)))
    for name, _, cands, _ in PARAMS:
        for v in cands:
            if v == cfg[name]:
                continue
            c2 = dict(cfg, **{name: v})
            if not valid(c2):
                continue
            try:
                t = measure(c2)
            except Exception as e:  # a variant that fails to build or run is skipped, not fatal
                log("  %s=%d failed: %s" % (name, v, str(e).splitlines()[0] if str(e) else e))
                trials.append((c2, None))
                continue
            trials.append((c2, t))
            log("  %s=%d: %.3f ms (best %.3f)" % (name, v, t, best))
            if t < best * (1.0 - min_gain):
                cfg, best = c2, t
        log("%s -> %d" % (name, cfg[name]))
    return cfg, best, trials


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--workload", default="rmat22")
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--min-gain", type=float, default=0.01, help="relative gain a change must bring")
    ap.add_argument("--out", default=B.TUNED)
    ap.add_argument("--no-check", action="store_true", help="skip the parity subset on the winner")
    args = ap.parse_args(argv)
    start = dict(DEFAULTS)
    if os.path.exists(B.TUNED):
        with open(B.TUNED) as f:
            start.update({k: v for k, v in json.load(f).get("defines", {}).items() if k in DEFAULTS})
    t0 = time.time()

    def measure(cfg):
        lib = B.build_variant(defines_by_source(cfg), variant_dir(cfg))
        return bench_ms(lib, args.workload, args.steps, args.warmup)

    base = measure(dict(DEFAULTS))
    cfg, best, trials = search(start, measure, args.min_gain)
    lib = os.path.join(variant_dir(cfg), "libcm.so")
    if not args.no_check:
        r = subprocess.run([sys.executable, "-m", "pytest", "tests/test_parity_gpu.py", "-x", "-q", "-k", CHECK_TESTS],
                           env=dict(os.environ, CUMETIS_LIB=lib), cwd=ROOT, stdout=subprocess.PIPE,
                           stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            print(r.stdout[-3000:])
            raise SystemExit("the tuned variant failed the parity subset; tuning file not written")
    out = {"defines": {k: v for k, v in sorted(cfg.items()) if v != DEFAULTS[k]},
           "workload": args.workload, "steps": args.steps, "ms_per_step": best, "default_ms_per_step": base,
           "search_s": round(time.time() - t0, 1),
           "trials": [{"defines": {k: v for k, v in sorted(c.items()) if v != DEFAULTS[k]}, "ms_per_step": t}
                      for c, t in trials]}
    with open(args.out, "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print(json.dumps({k: out[k] for k in ("defines", "ms_per_step", "default_ms_per_step", "search_s")}))


if __name__ == "__main__":
    main()
