/*
 * Minimal MEX gateway API for running QSM.m's C-MEX sources as a test
 * oracle outside MATLAB.  mexErrMsgTxt does not return: it long-jumps back
 * to shim_call(), which reports the message to the caller as an error.
 *
 * Test infrastructure only: nothing in the product links this.
 */
#pragma once

#include "matrix.h"

#ifndef MEXFUNCTION_DECLARED
#define MEXFUNCTION_DECLARED
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);
#endif

void mexErrMsgTxt(const char *msg);
int mexPrintf(const char *fmt, ...);
int mexAtExit(void (*fn)(void));
