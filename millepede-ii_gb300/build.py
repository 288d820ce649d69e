"""Build libmpgpu.so (sm_103a CUDA + C++ host side) and, for the tests, the
CPU oracle library.  Plain nvcc/g++ invocations, run in parallel; no cmake.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(HERE, "_build")
ORACLE = os.path.join(ROOT, "oracle")
ORACLE_BUILD = os.path.join(ORACLE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off"]
# the local-fit and preconditioner units keep the reference's separate
# multiply and add so that record decisions and the band factor are
# bit-identical; fused products are requested explicitly
PER_FILE = {"mpgpu_fit.cu": ["-fmad=false"], "mpgpu_precond.cu": ["-fmad=false"]}
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-pthread"]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build_lib(verbose=False):
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    for f in sorted(os.listdir(CSRC)):
        src = os.path.join(CSRC, f)
        obj = os.path.join(OBJDIR, f + ".o")
        if f.endswith(".cu"):
            jobs.append([nvcc] + NVCC_FLAGS + PER_FILE.get(f, []) + ["-c", src, "-o", obj])
        elif f.endswith(".cpp"):
            jobs.append(["g++"] + CXX_FLAGS + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        list(ex.map(_run, jobs))
    objs = [j[-1] for j in jobs]
    out = os.path.join(LIBDIR, "libmpgpu.so")
    _run([nvcc] + ARCH + ["-shared", "-o", out] + objs + ["-lpthread", "-ldl"])
    if verbose:
        print("built", out)
    return out


def build_oracle(verbose=False):
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    srcs = [os.path.join(ORACLE, f) for f in sorted(os.listdir(ORACLE)) if f.endswith(".c")]
    out = os.path.join(ORACLE_BUILD, "libmpref.so")
    _run(["gcc", "-O3", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp", "-o", out] + srcs + ["-lm"])
    if verbose:
        print("built", out)
    return out


def build_all(verbose=False):
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        a = ex.submit(build_lib, verbose)
        b = ex.submit(build_oracle, verbose)
        return a.result(), b.result()


if __name__ == "__main__":
    build_all(verbose=True)
