"""Builds this library's MEX gateways (gaga_gb300/mex/gb_gaga_mex.cpp) against the stand-in
MATLAB API of oracle/ref_shim/host/mex.h, so the tests can call them as MATLAB would
(test infrastructure; MATLAB itself is not needed).  One shared object per gateway in
gaga_gb300/_build/mex_stub/, linked to gaga_gb300/lib/libgb_cs.so."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "gaga_gb300", "mex", "gb_gaga_mex.cpp")
HOST = os.path.join(ROOT, "oracle", "ref_shim", "host")
LIBDIR = os.path.join(ROOT, "gaga_gb300", "lib")
OUT = os.path.join(ROOT, "gaga_gb300", "_build", "mex_stub")
GATEWAYS = {"gen": 1, "dct": 2, "smv": 3}


def build(gateway):
    os.makedirs(OUT, exist_ok=True)
    so = os.path.join(OUT, "gaga_%s_mex.so" % gateway)
    deps = [SRC, os.path.join(HOST, "mex.h"), os.path.join(HOST, "gb_host_runtime.cpp"),
            os.path.join(ROOT, "include", "gb_cs.h"), os.path.join(LIBDIR, "libgb_cs.so")]
    if os.path.exists(so) and all(os.path.getmtime(d) <= os.path.getmtime(so) for d in deps):
        return so
    cmd = ["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-U_FORTIFY_SOURCE", "-Wall", "-Wextra", "-Werror",
           "-Wno-unused-parameter", "-DGB_MEX_GATEWAY=%d" % GATEWAYS[gateway], "-I", os.path.join(ROOT, "include"),
           "-I", HOST, SRC, os.path.join(HOST, "gb_host_runtime.cpp"), "-L", LIBDIR, "-lgb_cs",
           "-Wl,-rpath," + LIBDIR, "-o", so]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("MEX shim build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    return so


def load(gateway):
    from oracle import ref_gateway

    return ref_gateway.bind(build(gateway))
