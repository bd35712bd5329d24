"""In-tree build of libimexlb.so and the imexlb_run driver for sm_103a.

nvcc compiles the CUDA kernels for sm_103a only (-gencode arch=compute_103a,
code=sm_103a); g++ compiles the host code. Everything is built with
contraction off (-fmad=false / -ffp-contract=off) so that every floating-point
operation rounds as in the reference's serial build. Outputs go to
imexlb-1.0_gb300/_build/. Translation units compile in parallel and are
rebuilt only when a source or header changed.
"""
import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libimexlb.so")
EXE = os.path.join(OUT, "imexlb_run")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, extra nvcc flags): the FP64 reference-order kernels never contract
# a*b+c; the FP32-arithmetic kernels may.
LIB_CU = [("kernels.cu", ["-fmad=false"]), ("step_split2.cu", ["-fmad=false"]),
          ("step_split3.cu", ["-fmad=false"]), ("step_fused.cu", ["-fmad=false"]),
          ("noalloc.cu", ["-fmad=false"]), ("setup_device.cu", ["-fmad=false"]),
          ("kernels_lp.cu", []), ("kernels_fx.cu", []), ("batch.cu", []), ("batch_persist.cu", []),
          ("nn.cu", [])]
LIB_CPP = ["imexlb.cpp", "bcmap.cpp", "fused_plan.cpp", "host_setup.cpp", "testing.cpp", "plt_writer.cpp"]
EXE_CPP = ["imexlb_run.cpp"]


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INC, "*.h"))


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _obj(src):
    return os.path.join(OUT, os.path.basename(src) + ".o")


def build(force=False, verbose=False):
    """Compile what is stale; return the path of libimexlb.so."""
    os.makedirs(OUT, exist_ok=True)
    hdrs = _headers() + [__file__]
    jobs = []
    for s, flags in LIB_CU:
        src = os.path.join(CSRC, s)
        if force or _newer(_obj(src), [src] + hdrs):
            jobs.append([os.path.join(CUDA, "bin", "nvcc"), "-std=c++17", "-O3"] + ARCH + flags +
                        ["-lineinfo", "-Xptxas", "-warn-spills",
                         "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", INC, "-I", CSRC,
                         "-c", src, "-o", _obj(src)])
    for s in LIB_CPP + EXE_CPP:
        src = os.path.join(CSRC, s)
        if force or _newer(_obj(src), [src] + hdrs):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall",
                         "-I", INC, "-I", CSRC, "-I", os.path.join(CUDA, "include"),
                         "-c", src, "-o", _obj(src)])
    procs = [(j, subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for j in jobs]
    failed = []
    for j, p in procs:
        out = p.communicate()[0].decode(errors="replace")
        if p.returncode != 0:
            failed.append((j, out))
        elif verbose and out.strip():
            print(out)
    if failed:
        msg = "\n\n".join(" ".join(j) + "\n" + o for j, o in failed)
        raise RuntimeError("libimexlb build failed:\n" + msg)
    lib_objs = [_obj(os.path.join(CSRC, s)) for s, _ in LIB_CU] + \
        [_obj(os.path.join(CSRC, s)) for s in LIB_CPP]
    cudart = ["-L" + os.path.join(CUDA, "lib64"), "-lcudart_static", "-ldl", "-lrt", "-lpthread"]
    if force or _newer(LIB, lib_objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        subprocess.run(["g++", "-shared", "-o", tmp] + lib_objs + cudart, check=True)
        os.replace(tmp, LIB)
    exe_objs = lib_objs + [_obj(os.path.join(CSRC, s)) for s in EXE_CPP]
    if force or _newer(EXE, exe_objs):
        subprocess.run(["g++", "-o", EXE] + exe_objs + cudart, check=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
