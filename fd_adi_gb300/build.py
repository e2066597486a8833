"""Build libfdadi.so in-tree with nvcc for sm_103a (GB300).

The library exports the C ABI declared in include/fdadi.h. Translation units
are compiled in parallel and linked into fd_adi_gb300/_build/libfdadi.so.
"""
import concurrent.futures
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libfdadi.so")
SOURCES = ["fdadi_ops.cu", "fdadi_engine.cu", "fdadi_bs.cu", "fdadi_mlp.cu", "fdadi_mesh.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              "-I" + os.path.join(ROOT, "include")]
# Host-only sources restate the reference's Python float arithmetic: no
# floating-point contraction (a fused multiply-add would change the bits).
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread",
             "-I" + os.path.join(ROOT, "include")]


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if d and os.path.isdir(os.path.join(d, "include")):
            return os.path.join(d, "include")
    return None


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _deps():
    out = [os.path.join(CSRC, s) for s in SOURCES]
    out += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    out.append(os.path.join(ROOT, "include", "fdadi.h"))
    out.append(os.path.abspath(__file__))
    return out


def stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(d) > t for d in _deps())


def build(force=False, verbose=False):
    """Compile every translation unit and link libfdadi.so; returns its path."""
    if not force and not stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        if src.endswith(".cpp"):
            inc = _cuda_include()
            cmd = [os.environ.get("CXX", "g++")] + CXX_FLAGS + \
                (["-I" + inc] if inc else []) + ["-c", os.path.join(CSRC, src), "-o", obj]
        else:
            cmd = [nvcc] + ARCH + NVCC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".%d.tmp" % os.getpid()
    subprocess.check_call([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
