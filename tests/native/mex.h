/* Declarations of the documented MATLAB C MEX API (R2018a interleaved-complex
 * names and signatures, as published in MathWorks' External Interfaces
 * reference) used by voxscatter_gb300/matlab/voxscatter_mex.c -- a stand-in
 * so that the gateway can be compile-checked where MATLAB is not installed.
 * Test infrastructure only: nothing is implemented here. */
#ifndef VS_TEST_MEX_DECLS_H
#define VS_TEST_MEX_DECLS_H
#include <stdbool.h>
#include <stddef.h>

typedef struct mxArray_tag mxArray;
typedef size_t mwSize;
typedef size_t mwIndex;
typedef double mxDouble;
typedef struct { mxDouble real, imag; } mxComplexDouble;
typedef enum { mxUNKNOWN_CLASS = 0, mxDOUBLE_CLASS = 6, mxUINT64_CLASS = 15 } mxClassID;
typedef enum { mxREAL, mxCOMPLEX } mxComplexity;

int mxGetString(const mxArray* pm, char* str, mwSize strlen);
size_t mxGetNumberOfElements(const mxArray* pm);
mwSize mxGetNumberOfDimensions(const mxArray* pm);
const mwSize* mxGetDimensions(const mxArray* pm);
size_t mxGetM(const mxArray* pm);
size_t mxGetN(const mxArray* pm);
mxDouble* mxGetDoubles(const mxArray* pa);
mxComplexDouble* mxGetComplexDoubles(const mxArray* pa);
void* mxGetData(const mxArray* pm);
bool mxIsDouble(const mxArray* pm);
bool mxIsComplex(const mxArray* pm);
bool mxIsUint64(const mxArray* pm);
bool mxIsStruct(const mxArray* pm);
mxArray* mxGetField(const mxArray* pm, mwIndex index, const char* fieldname);
double mxGetScalar(const mxArray* pm);
mxArray* mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID classid, mxComplexity flag);
mxArray* mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity flag);
mxArray* mxCreateDoubleScalar(double value);
void* mxMalloc(mwSize n);
void mxFree(void* ptr);
void mexErrMsgIdAndTxt(const char* errorid, const char* errormsg, ...);
int mexAtExit(void (*ExitFcn)(void));
void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]);
#endif
