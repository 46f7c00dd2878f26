"""Build libgfx.so (the sm_103a CUDA library behind include/gfx.h) in-tree.

Each translation unit is compiled in parallel with nvcc (CUDA sources) or g++
(host sources); objects go to cudagfx_gb300/_build/ and the shared library to
cudagfx_gb300/libgfx.so.  A unit is recompiled when it or any header is newer
than its object.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build", __import__("platform").machine())
LIB = os.path.join(HERE, "libgfx.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                      "-I" + INCLUDE, "-I" + CSRC]
# translation unit -> extra flags.  The twister bank uses the reference build's
# floating-point flags (-prec-div=false -prec-sqrt=false -ftz=false).
UNITS = {
    "gfx_kernels.cu": [],
    "gfx_heatbath.cu": [],
    "gfx_mt.cu": ["-prec-sqrt=false", "-prec-div=false", "-ftz=false"],
    "gfx_api.cu": [],
    "gfx_tune.cu": [],
    "gfx_ctx_files.cu": [],
    "gfx_noalloc.cu": [],
    "gfx_batch.cu": [],
    "gfx_rebased.cu": [],
    "gfx_host.cpp": [],
    "gfx_legacy.cpp": [],
    "gfx_lime.cpp": [],
    "gfx_io.cpp": [],
}


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(obj, src, headers):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + headers + [__file__])


def _compile(unit, extra, verbose):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, unit + ".o")
    if unit.endswith(".cu"):
        cmd = [_nvcc(), "-c", src, "-o", obj] + NVCC_COMMON + extra
    else:
        cmd = ["g++", "-c", src, "-o", obj, "-O2", "-fPIC", "-std=c++17",
               "-ffp-contract=off", "-I" + INCLUDE, "-I" + CSRC,
               "-I/usr/local/cuda/include"] + extra
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj, r.stderr


def build(verbose=False, force=False, ptxas_info=False):
    """Compile every unit that is out of date and link libgfx.so; returns its path.
    Concurrent callers (several ranks on one machine) serialize on a lock file."""
    import fcntl
    os.makedirs(BUILD, exist_ok=True)
    with open(os.path.join(BUILD, ".lock"), "w") as lk:
        fcntl.flock(lk, fcntl.LOCK_EX)
        try:
            return _build_locked(verbose, force, ptxas_info)
        finally:
            fcntl.flock(lk, fcntl.LOCK_UN)


def _build_locked(verbose, force, ptxas_info):
    headers = _headers()
    jobs = []
    for unit, extra in UNITS.items():
        obj = os.path.join(BUILD, unit + ".o")
        if force or _stale(obj, os.path.join(CSRC, unit), headers):
            flags = list(extra)
            if ptxas_info and unit.endswith(".cu"):
                flags += ["-Xptxas", "-v"]
            jobs.append((unit, flags))
    logs = {}
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for unit, (obj, err) in zip([j[0] for j in jobs],
                                        ex.map(lambda j: _compile(j[0], j[1], verbose), jobs)):
                logs[unit] = err
    objs = [os.path.join(BUILD, u + ".o") for u in UNITS]
    if jobs or not os.path.exists(LIB):
        cmd = [_nvcc(), "-shared", "-o", LIB] + ARCH + objs + ["-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (r.stdout, r.stderr))
    _build_program(verbose, force or bool(jobs))
    if ptxas_info:
        for u, e in logs.items():
            if e:
                print("== %s\n%s" % (u, e))
    return LIB


PROGRAM = os.path.join(HERE, "gfx_gaugefix")


def _build_program(verbose, force):
    """host/gfx_gaugefix.c -> gfx_gaugefix, linked against libgfx.so next to it"""
    src = os.path.join(HERE, "host", "gfx_gaugefix.c")
    if not force and os.path.exists(PROGRAM) and not _stale(PROGRAM, src, _headers()):
        return PROGRAM
    cmd = ["gcc", "-O2", "-std=gnu99", "-Wall", "-I" + INCLUDE, src, "-o", PROGRAM,
           "-L" + HERE, "-lgfx", "-Wl,-rpath,$ORIGIN"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("program link failed: %s\n%s" % (r.stdout, r.stderr))
    return PROGRAM


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
