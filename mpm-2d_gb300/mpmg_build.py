"""Build recipe of the mpm_gb300 shared library (the product).

Compiles every CUDA translation unit of ``csrc/`` for sm_103a (GB300) with
nvcc, in parallel, and links ``_build/libmpm_gb300.so``.  Runs the same on the
x86 build container (cross-compile) and on the Arm GPU host.
"""
import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(OUT, "libmpm_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code is compiled without contraction of multiply-adds, so host-side
# arithmetic (file writers, the libmpm layer) rounds the same on x86 and Arm
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I", INCLUDE]
CU_SOURCES = ["mpmg_api.cu", "mpmg_step.cu", "mpmg_sort.cu", "mpmg_nonlocal.cu", "mpmg_sort_noalloc.cu",
              "mpmg_libmpm.cu", "mpmg_mixed.cu", "mpmg_bin.cu", "mpmg_adjoint.cu",
              "mpmg_io.cu", "mpmg_split.cu"]
CPP_SOURCES = []


def nvcc():
    path = shutil.which("nvcc")
    if path is None and os.path.exists("/usr/local/cuda/bin/nvcc"):
        path = "/usr/local/cuda/bin/nvcc"
    if path is None:
        raise RuntimeError("nvcc not found")
    return path


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    files.append(os.path.abspath(__file__))   # the flags
    return max(os.path.getmtime(f) for f in files)


def _compile(src, verbose=False, extra=()):
    obj = os.path.join(OUT, os.path.splitext(os.path.basename(src))[0] + ".o")
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + list(extra) + ["-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        print(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def build(verbose=False, force=False, extra=()):
    """Compile (when sources changed) and return the path of the library."""
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps():
        return LIB
    srcs = CU_SOURCES + CPP_SOURCES
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose, extra), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, err in results:
            if err:
                print(err)
    cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-ldl", "-lpthread"]
    if verbose:
        print(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose=True, force=True, extra=sys.argv[1:]))
