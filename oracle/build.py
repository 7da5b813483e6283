"""Build recipe for the oracle (test infrastructure only).

* ``build_oracle()`` compiles oracle/gbo.c into oracle/_build/libgbo.so.
* ``build_ref()`` compiles a few of the reference's own source files, unmodified,
  from the reference tree (GAGA/gaga/kernels.cu, expander/kernels.cu,
  expander/serial_l0.cu) with the CUDA host-emulation shim into
  oracle/_ref/libgaga_ref.so.
* ``build_ref_gateways()`` compiles the reference's three MEX gateways
  (GAGA/gaga/gaga_gen.cu, gaga_dct.cu, gaga_smv.cu, with everything they include)
  for the CPU into oracle/_ref/libgaga_{gen,dct,smv}_ref.so, over the host emulation
  of the CUDA runtime and of the closed libraries in ref_shim/host/.  The sources are
  read where they lie; the one textual step is on the preprocessed translation unit
  (oracle/_ref/*.ii, a build intermediate): the kernel-launch syntax
  ``k<<<grid, block>>>(args)``, which g++ cannot parse, becomes
  ``::gbh::launch(k, grid, block)(args)``, and ``extern __shared__ T a[]`` becomes a
  pointer to the emulated dynamic shared memory.  No other line changes.

Both run only where the reference tree exists (GAGA_REFERENCE_ROOT, default the
read-only reference checkout this recipe was written against); the golden fixtures
they produce are committed under tests/golden, so nothing else needs them.
"""
import concurrent.futures as cf
import os
import re
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


_LAUNCH = re.compile(r"\b([A-Za-z_][A-Za-z_0-9]*)\s*<<<(.*?)>>>", re.S)
_EXTERN_SHARED = re.compile(r"\bextern\s+static\s+([A-Za-z_][A-Za-z_0-9 ]*?)\s+([A-Za-z_][A-Za-z_0-9]*)\s*\[\s*\]\s*;")
GATEWAYS = ("gen", "dct", "smv")
HOST = os.path.join(HERE, "ref_shim", "host")
_HOST_FLAGS = ["-std=c++17", "-fPIC", "-ffp-contract=off", "-U_FORTIFY_SOURCE", "-w", "-I", HOST]


def lib_gateway(name):
    return os.path.join(REF_OUT, "libgaga_%s_ref.so" % name)


def rewrite_launches(text):
    """The two mechanical rewrites of a preprocessed reference translation unit."""
    text = _LAUNCH.sub(lambda mo: "::gbh::launch(%s, %s)" % (mo.group(1), mo.group(2).strip()), text)
    return _EXTERN_SHARED.sub(lambda mo: "%s *%s = (%s *)::gbh::dynamic_shared();" % (mo.group(1), mo.group(2),
                                                                                    mo.group(1)), text)


def _build_gateway(name, runtime_obj):
    src = os.path.join(REFERENCE_ROOT, "GAGA", "gaga", "gaga_%s.cu" % name)
    drv = os.path.join(HERE, "ref_shim", "ref_gateway.cpp")
    ii = os.path.join(REF_OUT, "gaga_%s.ii" % name)
    ii_host = os.path.join(REF_OUT, "gaga_%s_host.ii" % name)
    obj = os.path.join(REF_OUT, "gaga_%s.o" % name)
    subprocess.check_call(["g++", "-E"] + _HOST_FLAGS + ['-DGB_GATEWAY_SRC="%s"' % src, drv, "-o", ii])
    with open(ii) as f:
        text = f.read()
    with open(ii_host, "w") as f:
        f.write(rewrite_launches(text))
    subprocess.check_call(["g++", "-c", "-O2", "-x", "c++"] + _HOST_FLAGS + [ii_host, "-o", obj])
    subprocess.check_call(["g++", "-shared", obj, runtime_obj, "-o", lib_gateway(name)])
    return lib_gateway(name)


def build_ref_gateways(force=False):
    gaga = os.path.join(REFERENCE_ROOT, "GAGA", "gaga")
    if not os.path.isdir(gaga):
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    shim = [os.path.join(HERE, "ref_shim", "ref_gateway.cpp"), os.path.abspath(__file__)]
    shim += [os.path.join(d, f) for d, _, fs in os.walk(HOST) for f in fs]
    if not force and all(_newer(lib_gateway(g), shim) for g in GATEWAYS):
        return [lib_gateway(g) for g in GATEWAYS]
    runtime_obj = os.path.join(REF_OUT, "gb_host_runtime.o")
    subprocess.check_call(["g++", "-c", "-O2"] + _HOST_FLAGS +
                          [os.path.join(HOST, "gb_host_runtime.cpp"), "-o", runtime_obj])
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        return list(ex.map(lambda g: _build_gateway(g, runtime_obj), GATEWAYS))


if __name__ == "__main__":
    print(build_oracle(force="-f" in sys.argv))
    print(build_ref(force="-f" in sys.argv))
    print(build_ref_gateways(force="-f" in sys.argv))
