/* Minimal MATLAB MEX API for running MEX gateways outside MATLAB.
 *
 * TEST INFRASTRUCTURE ONLY (oracle/ref_mex/): declares the mx and mex functions that the
 * reference's +scattering/combined_quick_gpu.cu and this library's gateways
 * (comp_ui_toolbox_gb300/mex/) call, implemented by mex_stub.cpp over an in-memory property
 * tree that the runners fill from Python.
 * Interleaved complex storage (R2018a API, combined_quick_gpu.m:32). */
#ifndef CUI_REF_MEX_H
#define CUI_REF_MEX_H

#include <stddef.h>
#include <stdbool.h>
#include <float.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mxArray_tag mxArray;
typedef size_t mwSize;
typedef size_t mwIndex;
typedef double mxDouble;
typedef struct { mxDouble real, imag; } mxComplexDouble;
typedef enum { mxUNKNOWN_CLASS = 0, mxDOUBLE_CLASS = 6 } mxClassID;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;

mxArray* mxGetProperty(const mxArray* pa, mwIndex index, const char* name);
mxArray* mxGetCell(const mxArray* pa, mwIndex index);
mxDouble* mxGetDoubles(const mxArray* pa);
mxComplexDouble* mxGetComplexDoubles(const mxArray* pa);
double mxGetScalar(const mxArray* pa);
size_t mxGetNumberOfElements(const mxArray* pa);
size_t mxGetM(const mxArray* pa);
size_t mxGetN(const mxArray* pa);
mwSize mxGetNumberOfDimensions(const mxArray* pa);
bool mxIsClass(const mxArray* pa, const char* name);
bool mxIsScalar(const mxArray* pa);
bool mxIsDouble(const mxArray* pa);
bool mxIsComplex(const mxArray* pa);
bool mxIsNumeric(const mxArray* pa);
bool mxIsEmpty(const mxArray* pa);
mxArray* mxDuplicateArray(const mxArray* pa);
int mxMakeArrayComplex(mxArray* pa);
mxArray* mxCreateNumericArray(mwSize ndim, const mwSize* dims, mxClassID classid, mxComplexity flag);
void* mxMalloc(size_t n);
void* mxCalloc(size_t n, size_t size);
void* mxRealloc(void* ptr, size_t size);
void mxFree(void* ptr);
void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...);
int mexPrintf(const char* fmt, ...);
int mexAtExit(void (*fn)(void));
/* the gateway every MEX file defines (C linkage, as MATLAB's header declares it) */
void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]);

#ifdef __cplusplus
}
#endif

#endif
