"""Build recipe for the oracle (test infrastructure only).

  oracle/liboracle.so        the CPU restatement in gfx_oracle.c (gcc, -ffp-contract=off)
  oracle/liboracle_fast.so   the same restatement built for speed (-O3, FMA contraction
                             allowed): the timed CPU baseline, not a checker
  oracle/_ref/host_src/      unchanged copies of the reference's host C files and
                             headers, made by copy_reference() from a reference
                             checkout (its path is an argument or GFX_REFERENCE_DIR).
                             The copies travel with the repository's working tree, so
                             the builds below also run where no checkout exists.
  oracle/_ref/libref_host.so the reference's su3manip.c, observables.c, rngs.c and
                             complex.c, plus ref_globals.c which defines the globals
                             the reference's main would define.
  oracle/_ref/libref_io.so   gauge_io.c, spinor_io.c, cksum.c with libgfx's LIME records.
  oracle/_ref/ref_gaugefix   the reference's host program flow (ref_link_main.c) over
                             its host C files, linked against libgfx.so.
  oracle/_ref/MersenneTwister.dat   the reference's twister-parameter file.

Nothing here is part of the product; only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg use it.
"""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(REF_DIR, "libref_host.so")
REF_DAT = os.path.join(REF_DIR, "MersenneTwister.dat")
FAST_LIB = os.path.join(HERE, "liboracle_fast.so")
# unchanged copies of the reference's host files (git-ignored; made by copy_reference)
REFERENCE = os.path.join(REF_DIR, "host_src")
REF_SOURCES = ["su3manip.c", "observables.c", "rngs.c", "complex.c"]
REF_HOST_FILES = ["read_input.c", "gauge_io.c", "spinor_io.c", "cksum.c", "su3manip.c",
                  "observables.c", "rngs.c", "complex.c", "complex.h", "cudaglobal.h",
                  "gauge_io.h", "global.h", "observables.h", "read_input.h", "rngs.h",
                  "spinor_io.h", "su3.h", "su3manip.h", "MersenneTwister.dat"]


def reference_checkout(path=None):
    """The reference checkout to copy from: `path`, else $GFX_REFERENCE_DIR, else None."""
    path = path or os.environ.get("GFX_REFERENCE_DIR")
    if path and os.path.exists(os.path.join(path, "global.h")):
        return path
    return None


def copy_reference(path=None):
    """Copy the reference's host files, unchanged, into oracle/_ref/host_src."""
    src = reference_checkout(path)
    if not src:
        return os.path.isdir(REFERENCE)
    os.makedirs(REFERENCE, exist_ok=True)
    for f in REF_HOST_FILES:
        a, b = os.path.join(src, f), os.path.join(REFERENCE, f)
        if os.path.exists(a) and _newer(b, [a]):
            shutil.copyfile(a, b)
            os.chmod(b, 0o644)
    return True


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("%s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_oracle():
    src = os.path.join(HERE, "gfx_oracle.c")
    if _newer(ORACLE_LIB, [src, os.path.join(HERE, "gfx_oracle.h"), __file__]):
        _run(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-shared", "-fPIC", "-std=c99",
              src, "-o", ORACLE_LIB, "-lm"])
    return ORACLE_LIB


def build_fast():
    """The CPU baseline build of the restatement: -O3 with FMA contraction allowed
    (portable flags: the same command on x86-64 and aarch64).  Its results differ from
    the oracle's in the last bits, so it is only timed, never used as the checker."""
    src = os.path.join(HERE, "gfx_oracle.c")
    if _newer(FAST_LIB, [src, os.path.join(HERE, "gfx_oracle.h"), __file__]):
        _run(["gcc", "-O3", "-ffp-contract=fast", "-fopenmp", "-shared", "-fPIC", "-std=c99",
              src, "-o", FAST_LIB, "-lm"])
    return FAST_LIB


def reference_present():
    return all(os.path.exists(os.path.join(REFERENCE, f)) for f in REF_SOURCES + ["global.h"])


def build_reference_host():
    """Compile the reference's host observables/initializers; None if the reference
    checkout is not present (as on a machine that only has this repository)."""
    if not reference_present():
        return REF_LIB if os.path.exists(REF_LIB) else None
    os.makedirs(REF_DIR, exist_ok=True)
    srcs = [os.path.join(REFERENCE, f) for f in REF_SOURCES]
    glob = os.path.join(HERE, "ref_globals.c")
    if _newer(REF_LIB, srcs + [glob, __file__]):
        cuda_inc = "/usr/local/cuda/include"
        _run(["gcc", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-w",
              "-I" + REFERENCE, "-I" + cuda_inc] + srcs + [glob, "-o", REF_LIB, "-lm"])
    dat = os.path.join(REFERENCE, "MersenneTwister.dat")
    if os.path.exists(dat) and _newer(REF_DAT, [dat]):
        shutil.copyfile(dat, REF_DAT)
    return REF_LIB


REF_IO_LIB = os.path.join(REF_DIR, "libref_io.so")
REF_IO_SOURCES = ["gauge_io.c", "spinor_io.c", "cksum.c", "complex.c"]


def build_reference_io():
    """The reference's file code (gauge_io.c, spinor_io.c, cksum.c) with libgfx's
    LIME implementation standing in for c-lime, plus ref_io_driver.c."""
    if not all(os.path.exists(os.path.join(REFERENCE, f)) for f in REF_IO_SOURCES):
        return REF_IO_LIB if os.path.exists(REF_IO_LIB) else None
    os.makedirs(REF_DIR, exist_ok=True)
    repo = os.path.dirname(HERE)
    lime = os.path.join(repo, "cudagfx_gb300", "csrc", "gfx_lime.cpp")
    srcs = [os.path.join(REFERENCE, f) for f in REF_IO_SOURCES]
    drv = [os.path.join(HERE, "ref_io_driver.c"), os.path.join(HERE, "ref_globals.c")]
    if _newer(REF_IO_LIB, srcs + drv + [lime, os.path.join(repo, "include", "lime.h"), __file__]):
        cuda_inc = "/usr/local/cuda/include"
        inc = ["-I" + REFERENCE, "-I" + os.path.join(repo, "include"), "-I" + cuda_inc]
        lime_obj = os.path.join(REF_DIR, "gfx_lime.o")
        _run(["g++", "-O2", "-fPIC", "-std=c++17", "-c", lime, "-o", lime_obj] + inc)
        _run(["gcc", "-O2", "-shared", "-fPIC", "-w", "-std=gnu99"] + inc + srcs + drv +
             [lime_obj, "-o", REF_IO_LIB, "-lstdc++", "-lm"])
    return REF_IO_LIB


REF_PROGRAM = os.path.join(REF_DIR, "ref_gaugefix")
REF_LINK_SOURCES = ["read_input.c", "gauge_io.c", "spinor_io.c", "cksum.c", "su3manip.c",
                    "observables.c", "rngs.c", "complex.c"]


def build_reference_link():
    """The reference's host C files, unchanged, with ref_link_main.c, linked against
    libgfx.so: the program the reference's main is, with libgfx as its CUDA side."""
    if not all(os.path.exists(os.path.join(REFERENCE, f)) for f in REF_LINK_SOURCES):
        return REF_PROGRAM if os.path.exists(REF_PROGRAM) else None
    os.makedirs(REF_DIR, exist_ok=True)
    repo = os.path.dirname(HERE)
    pkg = os.path.join(repo, "cudagfx_gb300")
    libgfx = os.path.join(pkg, "libgfx.so")
    srcs = [os.path.join(REFERENCE, f) for f in REF_LINK_SOURCES]
    main = os.path.join(HERE, "ref_link_main.c")
    if _newer(REF_PROGRAM, srcs + [main, libgfx, __file__]):
        inc = ["-I" + REFERENCE, "-I" + os.path.join(repo, "include"), "-I/usr/local/cuda/include"]
        # -ffp-contract=off: aarch64 gcc fuses a*b+c into FMA by default, x86-64 without
        # -march does not; with it off both give the reference's random start bit for bit
        _run(["gcc", "-O2", "-w", "-std=gnu99", "-ffp-contract=off"] + inc + srcs +
             [main, "-o", REF_PROGRAM, "-L" + pkg, "-lgfx", "-Wl,-rpath," + pkg, "-lm"])
    return REF_PROGRAM


def build(reference=None):
    """Build the oracle and its baseline copy; with a reference checkout (argument or
    $GFX_REFERENCE_DIR) refresh the copies of its host files first; build the
    reference's host libraries from the copies when they exist."""
    build_oracle()
    build_fast()
    copy_reference(reference)
    build_reference_host()
    build_reference_io()


if __name__ == "__main__":
    build()
    print(ORACLE_LIB, REF_LIB if os.path.exists(REF_LIB) else "(reference not built)")
