"""Build recipe for the oracle (test infrastructure only).

* ``build_oracle()`` compiles oracle/gbo.c into oracle/_build/libgbo.so.
* ``build_ref()`` compiles a few of the reference's own source files, unmodified,
  from the reference tree (GAGA/gaga/kernels.cu, expander/kernels.cu,
  expander/serial_l0.cu) with the CUDA host-emulation shim into
  oracle/_ref/libgaga_ref.so.  It runs only where the reference tree exists; the
  golden fixtures it produces are committed under tests/golden.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
REFERENCE_ROOT = os.environ.get("GAGA_REFERENCE_ROOT", "/root/reference")
LIBGBO = os.path.join(BUILD, "libgbo.so")
LIBREF = os.path.join(REF_OUT, "libgaga_ref.so")


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_oracle(force=False):
    os.makedirs(BUILD, exist_ok=True)
    src = [os.path.join(HERE, "gbo.c"), os.path.join(HERE, "gbo.h")]
    if not force and _newer(LIBGBO, src):
        return LIBGBO
    cmd = ["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-D_DEFAULT_SOURCE", src[0], "-o", LIBGBO, "-lm"]
    subprocess.check_call(cmd)
    return LIBGBO


def build_ref(force=False):
    gaga = os.path.join(REFERENCE_ROOT, "GAGA", "gaga")
    if not os.path.isdir(gaga):
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    drv = os.path.join(HERE, "ref_shim", "ref_driver.cpp")
    shim = os.path.join(HERE, "ref_shim", "cuda_host_shim.h")
    if not force and _newer(LIBREF, [drv, shim]):
        return LIBREF
    cmd = ["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-ffp-contract=off", "-w",
           "-include", shim, "-I", gaga, drv, "-o", LIBREF]
    subprocess.check_call(cmd)
    return LIBREF


if __name__ == "__main__":
    print(build_oracle(force="-f" in sys.argv))
    print(build_ref(force="-f" in sys.argv))
