/*
 * Minimal stand-in for MATLAB's MEX API: just the declarations the
 * reference's omc_matrad front end uses, so that its source compiles
 * unmodified outside MATLAB.  TEST INFRASTRUCTURE ONLY: the implementation
 * lives in oracle/matrad_harness.c, which feeds mexFunction its five
 * input arrays from files and writes the sparse dose-influence matrix it
 * returns.
 */
#ifndef OMC_MEXSHIM_MEX_H
#define OMC_MEXSHIM_MEX_H

/* Like MATLAB's header, this brings in stdio.h and stdlib.h, so that a
 * later include of them does not see a user macro named exit. */
#include <stdbool.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>

typedef struct mxArray_tag mxArray;
typedef size_t mwSize;
typedef size_t mwIndex;
typedef bool mxLogical;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;

mxArray *mxGetField(const mxArray *a, mwIndex i, const char *name);
int mxGetNumberOfFields(const mxArray *a);
double *mxGetPr(const mxArray *a);
double mxGetScalar(const mxArray *a);
mxLogical *mxGetLogicals(const mxArray *a);
const mwSize *mxGetDimensions(const mxArray *a);
mwSize mxGetNumberOfDimensions(const mxArray *a);
bool mxIsDouble(const mxArray *a);
bool mxIsInt32(const mxArray *a);
bool mxIsStruct(const mxArray *a);
mxArray *mxGetCell(const mxArray *a, mwIndex i);
mwIndex mxCalcSingleSubscript(const mxArray *a, mwSize nsubs, const mwIndex *subs);
char *mxArrayToString(const mxArray *a);
mxArray *mxCreateDoubleScalar(double v);
mxArray *mxCreateString(const char *s);
mxArray *mxCreateSparse(mwSize m, mwSize n, mwSize nzmax, mxComplexity c);
mwIndex *mxGetIr(const mxArray *a);
mwIndex *mxGetJc(const mxArray *a);
void mxSetNzmax(mxArray *a, mwSize nzmax);
void mxSetPr(mxArray *a, double *pr);
void mxSetIr(mxArray *a, mwIndex *ir);
void *mxRealloc(void *p, mwSize n);
void mxDestroyArray(mxArray *a);
int mexCallMATLAB(int nlhs, mxArray *plhs[], int nrhs, mxArray *prhs[], const char *name);
int mexPrintf(const char *fmt, ...);
void mexErrMsgIdAndTxt(const char *id, const char *fmt, ...);

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);

#endif
