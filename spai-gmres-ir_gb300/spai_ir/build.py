"""Build libspai_ir.so and the drop-in CLIs in-tree (spai-gmres-ir_gb300/_build/).

nvcc -gencode arch=compute_103a,code=sm_103a for every CUDA translation unit, compiled in
parallel; the SPAI construction unit is compiled with --fmad=false so its arithmetic follows the
reference's unfused operation order. The CLIs are plain C++ linked against the library.
"""
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC]

UNITS = {
    "spai_build.o": ("spai_build.cu", ["--fmad=false"]),
    "api.o": ("api.cu", []),
    "noalloc.o": ("noalloc.cu", []),
    "batched.o": ("batched.cu", []),
    "mm_device.o": ("mm_device.cu", []),
}
HEADERS = ["common.cuh", "exact_math.cuh", "spai_internal.hpp", "krylov.cuh", "krylov_kernels.cuh",
           "cgs_tiles.cuh", "adjoint.cuh", "sell.cuh", "dia.cuh", "mm_text.hpp", "cli_read.hpp"]
CLIS = {"gpu_fp64_ir": ("cli_main.cpp", "-DSOLVER_F64"), "gpu_fp32_ir": ("cli_main.cpp", "-DSOLVER_F32"),
        "gpu_mixed_ir": ("cli_main.cpp", "-DSOLVER_MIXED"), "gpu_diag_ir": ("diag_main.cpp", "")}

LIB = os.path.join(OUT, "libspai_ir.so")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(OUT, exist_ok=True)
    hdr = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "spai_ir.h")]
    procs = []
    for obj, (src, extra) in UNITS.items():
        target = os.path.join(OUT, obj)
        deps = [os.path.join(CSRC, src)] + hdr
        if force or _stale(target, deps):
            cmd = [NVCC] + COMMON + extra + ["-c", os.path.join(CSRC, src), "-o", target]
            if verbose:
                print(" ".join(cmd))
            procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("nvcc failed: %s\n%s" % (" ".join(cmd), out.decode(errors="replace")))
    objs = [os.path.join(OUT, o) for o in UNITS]
    if force or procs or _stale(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static"]
        subprocess.run(cmd, check=True)
    cli_procs = []
    for name, (src, flag) in CLIS.items():
        target = os.path.join(OUT, name)
        deps = [os.path.join(CSRC, src), LIB] + hdr
        if force or _stale(target, deps):
            cmd = ["g++", "-O2", "-std=c++17"] + ([flag] if flag else []) + ["-I" + INCLUDE, "-I" + CSRC,
                   os.path.join(CSRC, src), "-o", target, "-L" + OUT, "-lspai_ir",
                   "-Wl,-rpath,$ORIGIN"]
            cli_procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in cli_procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("g++ failed: %s\n%s" % (" ".join(cmd), out.decode(errors="replace")))
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
