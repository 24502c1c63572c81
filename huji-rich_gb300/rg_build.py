"""Builds librich_gb300.so in-tree with nvcc for sm_103a.

FP64-exact translation units are compiled with --fmad=false (no multiply-add
contraction, so every result rounds as the reference's FP64 does); the host
code has no floating point on the hot path.  Objects are compiled in
parallel and linked into one shared library with the CUDA runtime linked
statically.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librich_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# source -> extra flags
UNITS = {
    "rg_fp64.cu": ["--fmad=false"],
    "rg_capi.cu": [],
    "rg_mixed.cu": [],
    "rg_noalloc.cu": ["--fmad=false"],
    "rg_adjoint.cu": ["--fmad=false"],
    "rg_adjoint_rev.cu": [],
    "rg_adjoint_api.cu": [],
    "rg_tune.cu": [],
    "rg_3d.cu": ["--fmad=false"],
    "rg_3d_api.cu": [],
    "rg_3d_mixed.cu": [],
    "rg_tracers.cu": ["--fmad=false"],
    "rg_tracer_api.cu": [],
    "rg_rules_api.cu": [],
    "rg_motion.cu": ["--fmad=false"],
    "rg_motion_api.cu": [],
    "rg_adjoint_rev32.cu": [],
}
# units that include another unit's source
EXTRA_DEPS = {"rg_adjoint_rev32.cu": ["rg_adjoint_rev.cu"]}


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _newer(out, deps):
    return os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps)


def _deps():
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hdrs + [os.path.join(ROOT, "include", "rich_gb300.h"), __file__]


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    deps = _deps()
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                     "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    if verbose:
        common += ["-Xptxas", "-v"]
    jobs = []
    objs = []
    for src, flags in UNITS.items():
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT_DIR, src + ".o")
        objs.append(o)
        extra = [os.path.join(CSRC, d) for d in EXTRA_DEPS.get(src, [])]
        if force or not _newer(o, deps + [s] + extra):
            jobs.append([cc] + common + flags + ["-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        res = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
    for c, r in zip(jobs, res):
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(c) + "\n" + r.stdout + r.stderr)
    if force or jobs or not _newer(LIB, objs):
        tmp = LIB + ".tmp"
        r = subprocess.run([cc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs,
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
