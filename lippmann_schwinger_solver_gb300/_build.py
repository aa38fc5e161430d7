"""Builds liblsdafmm.so in-tree: host C++ with g++ (OpenMP, no FMA
contraction so that assembly decisions are identical on x86 and aarch64)
and the CUDA sources with nvcc for sm_103a only."""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "liblsdafmm.so")
DRIVER = os.path.join(PKG, "gmres_driver")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CXX_SOURCES = ["assemble.cpp", "capi.cpp"]
CU_SOURCES = ["matvec.cu", "matvec_df.cu", "gmres.cu", "batched.cu", "fno.cu", "nn_precond.cu", "peaks.cu", "batched_tc.cu",
              "quadrature.cu", "far_gpu.cu"]
# The far-field assembly on the GPU rounds every product and sum on its own,
# as the host assembler (-ffp-contract=off) does.
CU_EXTRA = {"far_gpu.cu": ["--fmad=false"]}


def _nvcc():
    p = os.path.join(CUDA_HOME, "bin", "nvcc")
    return p if os.path.exists(p) else (shutil.which("nvcc") or "nvcc")


def _cmds():
    inc = ["-I" + os.path.join(CUDA_HOME, "include"), "-I" + os.path.join(ROOT, "include")]
    cmds = []
    for s in CXX_SOURCES:
        o = os.path.join(OBJ, s + ".o")
        cmds.append((o, ["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off",
                         "-Wall", "-Wno-sign-compare", "-Wno-unused-function"] + inc +
                     ["-c", os.path.join(CSRC, s), "-o", o], [os.path.join(CSRC, s)]))
    for s in CU_SOURCES:
        o = os.path.join(OBJ, s + ".o")
        cmds.append((o, [_nvcc(), "-O3", "-std=c++17", ARCH, "-lineinfo", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-v" if os.environ.get("LS_PTXAS_VERBOSE") else "-O3"] + CU_EXTRA.get(s, []) + inc +
                     ["-c", os.path.join(CSRC, s), "-o", o], [os.path.join(CSRC, s)]))
    return cmds


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    headers += [os.path.join(ROOT, "include", "ls_dafmm.h"), os.path.join(ROOT, "include", "ls_fno.h")]
    return any(os.path.getmtime(d) > t for d in list(deps) + headers)


def build(verbose=False, force=False):
    os.makedirs(OBJ, exist_ok=True)
    jobs = [(o, c) for o, c, deps in _cmds() if force or _stale(o, deps)]

    def run(job):
        o, c = job
        if verbose:
            print(" ".join(c), flush=True)
        r = subprocess.run(c, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed:\n" + " ".join(c) + "\n" + r.stdout + r.stderr)
        return r.stdout + r.stderr

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for out in ex.map(run, jobs):
            if verbose and out.strip():
                print(out)
    objs = [o for o, _, _ in _cmds()]
    if force or jobs or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        link = ["g++", "-shared", "-fopenmp", "-o", LIB] + objs + [
            "-L" + os.path.join(CUDA_HOME, "lib64"), "-Wl,-rpath," + os.path.join(CUDA_HOME, "lib64"), "-lcudart"]
        r = subprocess.run(link, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + " ".join(link) + "\n" + r.stdout + r.stderr)
    # Reference-style C++ driver over the facade (include/ls_dafmm.hpp).
    src = os.path.join(PKG, "examples", "gmres_driver.cpp")
    hpp = os.path.join(ROOT, "include", "ls_dafmm.hpp")
    if force or not os.path.exists(DRIVER) or max(os.path.getmtime(src), os.path.getmtime(hpp),
                                                   os.path.getmtime(LIB)) > os.path.getmtime(DRIVER):
        cmd = ["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), src, "-o", DRIVER, "-L" + PKG,
               "-llsdafmm", "-Wl,-rpath," + PKG]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("driver build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
