"""In-tree build of the shared objects (nvcc for sm_103a, g++ for host code).

* ``lib/libcudaLduSolvers.so``  CUDA kernels + host C++ solvers + C ABI
* ``lib/libcfxcase.so``         synthetic case generator (host only)

Translation units are compiled in parallel and only when a source or header
is newer than the object.  There is no CPU fallback: if nvcc is missing the
build fails.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

from . import CSRC_DIR, INCLUDE_DIR, LIB_DIR

NVCC_ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--fmad=false", "-Xptxas", "-O3"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall"]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required (no CPU fallback)")


def _cuda_home(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose=False, jobs=None):
    os.makedirs(LIB_DIR, exist_ok=True)
    objdir = os.path.join(LIB_DIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC_DIR, "*.h")) + glob.glob(os.path.join(CSRC_DIR, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE_DIR, "*.h"))

    # host-only case generator
    case_so = os.path.join(LIB_DIR, "libcfxcase.so")
    case_src = os.path.join(CSRC_DIR, "cases.cpp")
    if _stale(case_so, [case_src] + headers):
        _run(["g++", *CXX_FLAGS, "-shared", "-o", case_so, case_src])

    nvcc = _nvcc()
    cuda = _cuda_home(nvcc)
    cu_srcs = sorted(glob.glob(os.path.join(CSRC_DIR, "*.cu")))
    cpp_srcs = sorted(s for s in glob.glob(os.path.join(CSRC_DIR, "*.cpp")) if not s.endswith("cases.cpp"))
    jobs_ = []
    objs = []
    for s in cu_srcs:
        o = os.path.join(objdir, os.path.basename(s) + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs_.append([nvcc, *NVCC_ARCH, *NVCC_FLAGS, "-I", INCLUDE_DIR, "-I", CSRC_DIR, "-c", s, "-o", o])
    for s in cpp_srcs:
        o = os.path.join(objdir, os.path.basename(s) + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs_.append(["g++", *CXX_FLAGS, "-I", INCLUDE_DIR, "-I", CSRC_DIR, "-I",
                          os.path.join(cuda, "include"), "-c", s, "-o", o])
    logs = []
    if jobs_:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(jobs_), os.cpu_count() or 4)) as ex:
            for out in ex.map(_run, jobs_):
                logs.append(out)
    so = os.path.join(LIB_DIR, "libcudaLduSolvers.so")
    if objs and _stale(so, objs):
        _run([nvcc, *NVCC_ARCH, "-shared", "-o", so, *objs, "-lcudart", "-lpthread"])
    if verbose:
        print("\n".join(x for x in logs if x.strip()))
    return so
