/*
 * Minimal mxArray runtime: the subset of MATLAB's matrix API that the QSM.m
 * MEX sources call, written for this project so that those sources compile
 * and run outside MATLAB as a test oracle.  Only numeric, real, dense arrays
 * exist; data is zero-filled on creation, as mxCreateNumericArray does.
 *
 * Test infrastructure only: nothing in the product links this.
 */
#pragma once

#include <stddef.h>
#include <stdint.h>
#include <stdbool.h>

typedef size_t mwSize;
typedef size_t mwIndex;

typedef enum {
    mxUNKNOWN_CLASS = 0,
    mxCELL_CLASS,
    mxSTRUCT_CLASS,
    mxLOGICAL_CLASS,
    mxCHAR_CLASS,
    mxVOID_CLASS,
    mxDOUBLE_CLASS,
    mxSINGLE_CLASS,
    mxINT8_CLASS,
    mxUINT8_CLASS,
    mxINT16_CLASS,
    mxUINT16_CLASS,
    mxINT32_CLASS,
    mxUINT32_CLASS,
    mxINT64_CLASS,
    mxUINT64_CLASS
} mxClassID;

typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;

typedef struct mxArray_tag mxArray;

/* creation / destruction */
mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims,
                              mxClassID classid, mxComplexity flag);
mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity flag);
mxArray *mxCreateLogicalArray(mwSize ndim, const mwSize *dims);
mxArray *mxCreateDoubleScalar(double value);
mxArray *mxDuplicateArray(const mxArray *in);
void mxDestroyArray(mxArray *pa);

/* queries */
void *mxGetData(const mxArray *pa);
const mwSize *mxGetDimensions(const mxArray *pa);
mwSize mxGetNumberOfDimensions(const mxArray *pa);
size_t mxGetNumberOfElements(const mxArray *pa);
size_t mxGetElementSize(const mxArray *pa);
mxClassID mxGetClassID(const mxArray *pa);
double mxGetScalar(const mxArray *pa);
bool mxIsSingle(const mxArray *pa);
bool mxIsDouble(const mxArray *pa);
bool mxIsLogical(const mxArray *pa);
