/*
 * The mxArray runtime behind matrix.h / mex.h, plus shim_call(), the entry
 * point a Python harness uses to run one MEX gateway (mexFunction) with
 * arrays it built through the same runtime.
 *
 * Test infrastructure only: nothing in the product links this.
 */
#include <setjmp.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "mex.h"

struct mxArray_tag {
    mxClassID cls;
    mwSize ndim;
    mwSize dims[8];
    size_t numel;
    size_t elsize;
    void *data;
};

static size_t class_size(mxClassID c)
{
    switch (c) {
    case mxDOUBLE_CLASS: case mxINT64_CLASS: case mxUINT64_CLASS: return 8;
    case mxSINGLE_CLASS: case mxINT32_CLASS: case mxUINT32_CLASS: return 4;
    case mxINT16_CLASS: case mxUINT16_CLASS: case mxCHAR_CLASS: return 2;
    case mxLOGICAL_CLASS: case mxINT8_CLASS: case mxUINT8_CLASS: return 1;
    default: return 0;
    }
}

mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims,
                              mxClassID classid, mxComplexity flag)
{
    (void)flag;
    if (ndim > 8) return NULL;
    mxArray *a = (mxArray *)calloc(1, sizeof(mxArray));
    a->cls = classid;
    a->ndim = ndim < 2 ? 2 : ndim;
    a->dims[0] = 1;
    a->dims[1] = 1;
    a->numel = 1;
    for (mwSize d = 0; d < ndim; ++d) {
        a->dims[d] = dims[d];
        a->numel *= dims[d];
    }
    a->elsize = class_size(classid);
    /* +64 bytes so that an empty array still has a valid pointer */
    a->data = calloc(a->numel * a->elsize + 64, 1);
    return a;
}

mxArray *mxCreateLogicalArray(mwSize ndim, const mwSize *dims)
{
    return mxCreateNumericArray(ndim, dims, mxLOGICAL_CLASS, mxREAL);
}

mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity flag)
{
    mwSize d[2] = {m, n};
    return mxCreateNumericArray(2, d, mxDOUBLE_CLASS, flag);
}

mxArray *mxCreateDoubleScalar(double value)
{
    mxArray *a = mxCreateDoubleMatrix(1, 1, mxREAL);
    *(double *)a->data = value;
    return a;
}

mxArray *mxDuplicateArray(const mxArray *in)
{
    mxArray *a = mxCreateNumericArray(in->ndim, in->dims, in->cls, mxREAL);
    memcpy(a->data, in->data, in->numel * in->elsize);
    return a;
}

void mxDestroyArray(mxArray *pa)
{
    if (!pa) return;
    free(pa->data);
    free(pa);
}

void *mxGetData(const mxArray *pa) { return pa->data; }
const mwSize *mxGetDimensions(const mxArray *pa) { return pa->dims; }
mwSize mxGetNumberOfDimensions(const mxArray *pa) { return pa->ndim; }
size_t mxGetNumberOfElements(const mxArray *pa) { return pa->numel; }
size_t mxGetElementSize(const mxArray *pa) { return pa->elsize; }
mxClassID mxGetClassID(const mxArray *pa) { return pa->cls; }
bool mxIsSingle(const mxArray *pa) { return pa->cls == mxSINGLE_CLASS; }
bool mxIsDouble(const mxArray *pa) { return pa->cls == mxDOUBLE_CLASS; }
bool mxIsLogical(const mxArray *pa) { return pa->cls == mxLOGICAL_CLASS; }

double mxGetScalar(const mxArray *pa)
{
    if (pa->numel == 0) return 0.0;
    switch (pa->cls) {
    case mxDOUBLE_CLASS: return *(const double *)pa->data;
    case mxSINGLE_CLASS: return *(const float *)pa->data;
    case mxLOGICAL_CLASS: case mxUINT8_CLASS: return *(const uint8_t *)pa->data;
    case mxINT8_CLASS: return *(const int8_t *)pa->data;
    case mxINT32_CLASS: return *(const int32_t *)pa->data;
    case mxUINT32_CLASS: return *(const uint32_t *)pa->data;
    case mxINT64_CLASS: return (double)*(const int64_t *)pa->data;
    case mxUINT64_CLASS: return (double)*(const uint64_t *)pa->data;
    default: return 0.0;
    }
}

/* ---- error / print ---- */

static jmp_buf *g_jmp = NULL;
static char g_err[512];
static int g_verbose = 0;

void mexErrMsgTxt(const char *msg)
{
    snprintf(g_err, sizeof g_err, "%s", msg);
    if (g_jmp) longjmp(*g_jmp, 1);
    fprintf(stderr, "mexErrMsgTxt outside shim_call: %s\n", msg);
    abort();
}

int mexPrintf(const char *fmt, ...)
{
    if (!g_verbose) return 0;
    va_list ap;
    va_start(ap, fmt);
    int r = vprintf(fmt, ap);
    va_end(ap);
    fflush(stdout);
    return r;
}

/* mexAtExit: the function runs at shim_clear(), as MATLAB runs it at `clear mex` */
static void (*g_atexit)(void) = NULL;

int mexAtExit(void (*fn)(void))
{
    g_atexit = fn;
    return 0;
}

void shim_clear(void)
{
    if (g_atexit) g_atexit();
    g_atexit = NULL;
}

/* Run the gateway; returns 0 on success, 1 if it raised mexErrMsgTxt
 * (the message is then available from shim_last_error()). */
int shim_call(int nlhs, mxArray **plhs, int nrhs, const mxArray **prhs, int verbose)
{
    jmp_buf jb;
    g_verbose = verbose;
    g_err[0] = 0;
    g_jmp = &jb;
    if (setjmp(jb)) {
        g_jmp = NULL;
        return 1;
    }
    mexFunction(nlhs, plhs, nrhs, prhs);
    g_jmp = NULL;
    return 0;
}

const char *shim_last_error(void) { return g_err; }
