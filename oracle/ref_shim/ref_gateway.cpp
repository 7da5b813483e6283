/*
 * ref_gateway.cpp -- wraps one of the reference's MEX gateways (GAGA/gaga/gaga_gen.cu,
 * gaga_dct.cu or gaga_smv.cu, named by GB_GATEWAY_SRC and included unmodified from the
 * reference tree) so that a test can call its mexFunction (C linkage, as mex.h declares it) on the CPU through the host
 * emulation (host/gb_host_cuda.h, host/gb_host_libs.h, host/mex.h).  oracle/build.py
 * preprocesses this file, rewrites the kernel-launch syntax g++ cannot parse, and builds
 * oracle/_ref/libgaga_<gateway>_ref.so.  TEST INFRASTRUCTURE ONLY: it produces the
 * reference's own outputs as golden fixtures.
 */
#include "gb_host_libs.h"
#include "mex.h"

#include GB_GATEWAY_SRC
