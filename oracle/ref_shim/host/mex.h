/*
 * mex.h -- a minimal stand-in for MATLAB's MEX API: enough for the reference's gateways
 * (GAGA/gaga/gaga_{gen,dct,smv}.cu) and for a MEX shim over libgb_cs.so to compile and
 * run without MATLAB.  Arrays are column-major M x N of one class; cells hold element
 * pointers.  The gbmx_* calls (C linkage) let a test build arguments and call the
 * gateway's mexFunction.  TEST INFRASTRUCTURE ONLY.
 */
#pragma once
#include <stddef.h>

typedef enum {
  mxUNKNOWN_CLASS = 0,
  mxCELL_CLASS = 1,
  mxSTRUCT_CLASS = 2,
  mxLOGICAL_CLASS = 3,
  mxCHAR_CLASS = 4,
  mxVOID_CLASS = 5,
  mxDOUBLE_CLASS = 6,
  mxSINGLE_CLASS = 7,
  mxINT8_CLASS = 8,
  mxUINT8_CLASS = 9,
  mxINT16_CLASS = 10,
  mxUINT16_CLASS = 11,
  mxINT32_CLASS = 12,
  mxUINT32_CLASS = 13,
  mxINT64_CLASS = 14,
  mxUINT64_CLASS = 15
} mxClassID;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;
typedef struct gbmx_array mxArray;

#ifdef __cplusplus
extern "C" {
#endif
mxArray *mxCreateNumericMatrix(size_t m, size_t n, mxClassID cls, mxComplexity cplx);
void *mxGetData(const mxArray *a);
size_t mxGetM(const mxArray *a);
size_t mxGetN(const mxArray *a);
double mxGetScalar(const mxArray *a);
int mxGetString(const mxArray *a, char *buf, size_t buflen);
int mxIsCell(const mxArray *a);
mxArray *mxGetCell(const mxArray *a, size_t index);
size_t mxCalcSingleSubscript(const mxArray *a, size_t nsubs, const int *subs);
int mexPrintf(const char *fmt, ...);
/* the gateway's entry point, with C linkage as MATLAB declares it */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);
/* MATLAB raises an error and leaves the MEX function; the stand-in records the message
 * (gbmx_last_error) and returns, so a gateway returns right after calling it */
void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...);

/* test-side construction of arguments (not part of MATLAB's API) */
mxArray *gbmx_numeric(int cls, int m, int n, const void *data);
mxArray *gbmx_string(const char *s);
mxArray *gbmx_cell(int m, int n);
void gbmx_cell_set(mxArray *cell, int index, mxArray *elem);
int gbmx_class(const mxArray *a);
const char *gbmx_last_error(void);
void gbmx_clear_error(void);
void gbmx_free(mxArray *a);
#ifdef __cplusplus
}
#endif
