"""Builds libbmf_gb300.so (the C-ABI library of include/bmf.h) in-tree.

nvcc compiles each translation unit under csrc/ for sm_103a in parallel, then
links one shared library into binarymeshfitting_gb300/_build/.  Every TU is
built with --fmad=false and IEEE division / square root: the kernels reproduce
the reference's single-precision arithmetic operation by operation.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libbmf_gb300.so")
# A compiled C++ caller of the library (include/bmf.h + include/bmf_adapter.hpp).
DROPIN_SRC = os.path.join(HERE, "dropin", "bmf_dropin.cpp")
DROPIN = os.path.join(BUILD, "bmf_dropin")
SOURCES = ["bmf_sample.cu", "bmf_extract.cu", "bmf_process.cu", "bmf_capi.cu", "bmf_noalloc.cu", "bmf_lod.cu",
           "bmf_adjoint64.cu", "bmf_fit_loss.cu"]
# Sources whose arithmetic does not mirror the reference's float rounding may
# contract multiplies and adds (every other TU is built with --fmad=false).
FMA_SOURCES = {"bmf_adjoint64.cu"}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
                     "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden", "-I" + os.path.join(HERE, "..")]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libbmf_gb300.so")
    return path


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h"))]
    files.append(os.path.join(HERE, "..", "include", "bmf.h"))
    files.append(os.path.join(HERE, "..", "include", "bmf_fields.h"))
    files.append(os.path.join(HERE, "..", "include", "bmf_adapter.hpp"))
    files.append(DROPIN_SRC)
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files)


def build(force=False, verbose=False, extra_flags=()):
    """Compiles (if stale) and returns the library path."""
    if (not force and os.path.exists(LIB) and os.path.exists(DROPIN)
            and min(os.path.getmtime(LIB), os.path.getmtime(DROPIN)) >= _deps()):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        flags = [("--fmad=true" if f == "--fmad=false" and src in FMA_SOURCES else f) for f in NVCC_FLAGS]
        cmd = [cc, "-c", os.path.join(CSRC, src), "-o", obj] + flags + list(extra_flags)
        if verbose:
            cmd += ["-Xptxas", "-v"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
        return obj, r.stderr

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    if verbose:
        for _, err in results:
            sys.stderr.write(err)
    tmp = LIB + ".tmp"
    cmd = [cc, "-shared"] + ARCH + ["-o", tmp] + [o for o, _ in results] + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    build_dropin(cc)
    return LIB


def build_dropin(cc):
    """The drop-in caller: host C++ only, linked against the library (rpath
    $ORIGIN, both live in _build/)."""
    tmp = DROPIN + ".tmp"
    cmd = [cc, "-std=c++17", "-O2", "-Xcompiler", "-ffp-contract=off", "-I" + os.path.join(HERE, ".."), DROPIN_SRC,
           "-o", tmp, "-L" + BUILD, "-lbmf_gb300", "-lcudart", "-Xlinker", "-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("drop-in caller build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, DROPIN)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
