"""Recipe: the reference's own CUDA code, built for sm_103a, as a second checker.

Test infrastructure only.  Two steps:

prepare(path)  (needs the reference checkout: `path` or $GFX_REFERENCE_DIR) copies the
           reference's CUDA translation unit (cudagaugefix.cu and the .cu/.h files it
           includes) and the host C files it links into oracle/_ref/gpu_src/
           (git-ignored) and applies the compatibility shim the current toolkit needs:
             - the texture-reference declarations, fetch helpers and bind functions
               (dev_su3.cu:4-12, 208-218, 1644-1693) are blanked: CUDA 12+ removed
               texture references, and the reference's texture path is compiled out
               (USETEXTURE is undefined in cudaglobal.h:13);
             - cudaMemcpyToSymbol("sa_beta"/"therm_beta", ...) uses the symbol instead
               of its name (simulated_annealing.cu:298, heatbath_thermalization.cu:561);
             - cudaThreadSynchronize -> cudaDeviceSynchronize (a -D flag);
             - empty cublas.h (included, never used) and a lime.h with the reader/writer
               types only (the ILDG I/O is not linked);
             - the overrelaxation parameter, a literal 1.68 at overrelax.cu:416, reads
               the __constant__ ref_omega that ref_gpu_driver.cu defines with the same
               default 1.68 (ref_set_omega changes it), so workloads quoted at another
               omega run through the reference's own kernel.
build()    (needs nvcc; runs where the copied sources are, e.g. the GPU machine)
           compiles oracle/ref_gpu_driver.cu -- which includes the shimmed
           cudagaugefix.cu -- with the reference's floating-point flags into
           oracle/_ref/libref_gpu.so.
"""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
SRC = os.path.join(REF_DIR, "gpu_src")
LIB = os.path.join(REF_DIR, "libref_gpu.so")

CUDA_FILES = ["cudagaugefix.cu", "dev_su3.cu", "dev_su3.h", "overrelax.cu", "MersenneTwister.cu",
              "MersenneTwister.h", "simulated_annealing.cu", "heatbath_thermalization.cu",
              "cudaglobal.h", "global.h", "complex.h", "rngs.h", "su3manip.h", "observables.h",
              "read_input.h", "gauge_io.h"]
HOST_C = ["complex.c", "rngs.c", "su3manip.c", "observables.c"]
# (file, first line, last line, text that must appear in the range): blanked ranges
BLANK = [("dev_su3.cu", 4, 12, "texture<int4,1> gf_tex"),
         ("dev_su3.cu", 208, 218, "tex1Dfetch_gf"),
         ("dev_su3.cu", 1644, 1693, "bind_texture_gf")]
REPLACE = [("simulated_annealing.cu", 'cudaMemcpyToSymbol("sa_beta"', "cudaMemcpyToSymbol(sa_beta"),
           ("heatbath_thermalization.cu", 'cudaMemcpyToSymbol("therm_beta"',
            "cudaMemcpyToSymbol(therm_beta"),
           ("overrelax.cu", "overrelax(&(trafosmem[ix]), &(help), 1.68, 3);",
            "overrelax(&(trafosmem[ix]), &(help), ref_omega, 3);")]


def prepare(path=None):
    REFERENCE = path or os.environ.get("GFX_REFERENCE_DIR")
    if not REFERENCE or not os.path.exists(os.path.join(REFERENCE, "cudagaugefix.cu")):
        return os.path.isdir(SRC)
    os.makedirs(SRC, exist_ok=True)
    for f in CUDA_FILES + HOST_C:
        dst = os.path.join(SRC, f)
        shutil.copyfile(os.path.join(REFERENCE, f), dst)
        os.chmod(dst, 0o644)
    for f, a, b, marker in BLANK:
        p = os.path.join(SRC, f)
        lines = open(p, encoding="latin-1").read().split("\n")
        chunk = "\n".join(lines[a - 1:b])
        if marker not in chunk:
            raise RuntimeError("%s:%d-%d does not contain %r" % (f, a, b, marker))
        for k in range(a - 1, b):
            lines[k] = ""
        open(p, "w", encoding="latin-1").write("\n".join(lines))
    for f, old, new in REPLACE:
        p = os.path.join(SRC, f)
        s = open(p, encoding="latin-1").read()
        if old not in s:
            raise RuntimeError("%s: %r not found" % (f, old))
        open(p, "w", encoding="latin-1").write(s.replace(old, new))
    open(os.path.join(SRC, "cublas.h"), "w").write("/* unused by the reference */\n")
    open(os.path.join(SRC, "lime.h"), "w").write(
        "typedef unsigned long long n_uint64_t;\n"
        "typedef struct LimeReader LimeReader;\n"
        "typedef struct LimeWriter LimeWriter;\n"
        "typedef struct LimeRecordHeader LimeRecordHeader;\n")
    return True


def build(force=False):
    if not os.path.isdir(SRC):
        return None
    driver = os.path.join(HERE, "ref_gpu_driver.cu")
    deps = [driver, __file__] + [os.path.join(SRC, f) for f in os.listdir(SRC)]
    if not force and os.path.exists(LIB) and \
            all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    nvcc = "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc"
    cmd = [nvcc, "-shared", "-Xcompiler", "-fPIC", "-gencode", "arch=compute_103a,code=sm_103a",
           "-O3", "-ftz=false", "-prec-div=false", "-prec-sqrt=false", "-w",
           "-DcudaThreadSynchronize=cudaDeviceSynchronize", "-I" + SRC, driver] + \
          [os.path.join(SRC, f) for f in HOST_C] + ["-o", LIB]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("%s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    import sys
    prepare(sys.argv[1] if len(sys.argv) > 1 else None)
    print(build(force=True))
