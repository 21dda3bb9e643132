"""Build libgbrelion (the sm_103a CUDA E-step) in-tree with nvcc.

The translation units are compiled in parallel and linked into
relion_gb300/_build/libgbrelion.so.  Host code is compiled with
-ffp-contract=off so that the pose enumeration is bit-identical to the
reference's double-precision arithmetic.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libgbrelion.so")
ACC = os.path.join(HERE, "acc")
ACC_LIB = os.path.join(BUILD, "libgbrelion_acc.so")
INCLUDE = os.path.join(HERE, "..", "include")
SOURCES = ["k_project.cu", "k_gemm.cu", "k_estep.cu", "estep.cu", "k_noalloc.cu", "k_tc.cu", "k_prepimg.cu", "k_recon.cu",
           "k_posenet.cu", "io.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _run(cmd):
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, errors="replace")
    if proc.returncode != 0:
        raise RuntimeError("command failed: %s\n%s" % (" ".join(cmd), proc.stdout))
    return proc.stdout


def build_acc(force=False):
    """Compile the C++ façade (relion_gb300/acc: AccProjector, AccBackprojector,
    MlDeviceBundle, MlOptimiserCuda over the C ABI) into libgbrelion_acc.so,
    linked against libgbrelion.so; return its path."""
    srcs = [os.path.join(ACC, f) for f in sorted(os.listdir(ACC)) if f.endswith(".cpp")]
    deps = [os.path.join(ACC, f) for f in os.listdir(ACC)] + [os.path.join(INCLUDE, "gbrelion.h"), LIB]
    if (not force and os.path.exists(ACC_LIB)
            and os.path.getmtime(ACC_LIB) >= max(os.path.getmtime(d) for d in deps)):
        return ACC_LIB
    tmp = ACC_LIB + ".tmp"
    _run(["g++", "-std=c++17", "-O2", "-Wall", "-fPIC", "-shared", "-I", INCLUDE, "-I", ACC] + srcs +
         ["-o", tmp, "-L", BUILD, "-lgbrelion", "-Wl,-rpath,$ORIGIN"])
    os.replace(tmp, ACC_LIB)
    return ACC_LIB


def build(verbose=False, force=False):
    """Compile libgbrelion.so if any source is newer than it, then the C++
    façade library; return the path of libgbrelion.so."""
    os.makedirs(BUILD, exist_ok=True)
    _build_lib(verbose, force)
    build_acc(force)
    if verbose:
        print("built", ACC_LIB)
    return LIB


def _build_lib(verbose, force):
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "gbrelion.h"))
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps)):
        return LIB
    nvcc = _nvcc()
    flags = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                    "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fopenmp", "-Xptxas", "-v"]

    def one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        out = _run([nvcc] + flags + ["-c", os.path.join(CSRC, src), "-o", obj])
        with open(obj + ".ptxas.txt", "w") as fh:
            fh.write(out)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(one, SOURCES))
    tmp = LIB + ".tmp"
    _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lcufft", "-lgomp"])
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
