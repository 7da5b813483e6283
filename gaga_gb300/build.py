"""Build libgb_cs.so for sm_103a with nvcc (in-tree, no torch needed).

Translation units are compiled in parallel, then linked into
gaga_gb300/lib/libgb_cs.so.  Object files go to gaga_gb300/_build/.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libgb_cs.so")
ROOT = os.path.dirname(HERE)
SOURCES = ["gb_ops.cu", "gb_solver.cu", "gb_api.cu", "gb_batch.cu", "gb_noalloc.cu", "gb_gemm.cu", "gb_gemm_tc.cu",
           "gb_shared.cu", "gb_learned.cu", "gb_resident.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
         "-I", os.path.join(ROOT, "include")]


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(ROOT, "include", "gb_cs.h"))
    files.append(os.path.abspath(__file__))  # the source list and flags
    return files


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [NVCC] + ARCH + FLAGS + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def build(force=False, verbose=False, extra=None):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    if not force and not _stale(LIB, _deps()):
        return LIB
    extra = list(extra or [])
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    if verbose:
        for obj, err in results:
            if err:
                print(err)
    objs = [o for o, _ in results]
    cmd = [NVCC] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs
    subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    v = "-v" in sys.argv
    print(build(force="-f" in sys.argv, verbose=v, extra=["-Xptxas", "-v"] if v else None))
