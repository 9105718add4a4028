"""Build liblbm_gb300.so (sm_103a) in-tree with nvcc.

Five translation units are compiled in parallel and linked with the static
CUDA runtime:

* ``lbm_fused.cu``   fused pull-scheme engine (all storage forms)
* ``lbm_unfused.cu`` one kernel per reference function, ``-fmad=false``
* ``lbm_api.cu``     C-ABI front, CUDA-graph cache, storage conversion
* ``lbm_batch.cu``   batched lattices (work-queue and per-tile kernels)
* ``lbm_adjoint.cu`` discrete adjoint of the FP64 fused step

Processes that build at the same time (one per rank under torchrun) take
turns on a lock file; each rebuilds only if the library is still stale.
"""
import concurrent.futures
import fcntl
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "liblbm_gb300.so")
OBJ_DIR = os.path.join(HERE, "_lib", "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "--expt-relaxed-constexpr"]
UNITS = {
    "lbm_fused.cu": [],
    "lbm_unfused.cu": ["-fmad=false"],
    "lbm_api.cu": [],
    "lbm_batch.cu": [],
    "lbm_adjoint.cu": [],
}


def nvcc():
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found (set NVCC)")
    return cand


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(HERE, "..", "include", "lbm_gb300.h"), __file__]


def up_to_date():
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force=False, verbose=False, extra=()):
    """Compile and link; returns the library path.  verbose: print every
    nvcc command line (and anything nvcc prints) to stdout."""
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(OBJ_DIR, exist_ok=True)
    with open(os.path.join(OBJ_DIR, "build.lock"), "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        try:
            if not force and up_to_date():  # built by another process meanwhile
                return LIB_PATH
            return _compile_and_link(verbose, extra)
        finally:
            fcntl.flock(lock, fcntl.LOCK_UN)


def _compile_and_link(verbose, extra):
    nv = nvcc()

    def compile_unit(item):
        src, flags = item
        obj = os.path.join(OBJ_DIR, src.replace(".cu", ".o"))
        cmd = [nv, *ARCH, *COMMON, *flags, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS.items()))
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = [nv, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs]
    if verbose:
        print(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose=True, extra=tuple(sys.argv[1:])))
