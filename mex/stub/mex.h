/*
 * mex.h - a stand-in for MATLAB's MEX / C Matrix API, just the calls the
 * gateways in mex/ use, with MATLAB's names and signatures.  It lets the
 * gateways compile and run without MATLAB: against this header and
 * mx_stub.cpp (plain C++ structs behind mxArray) for the CPU tests and the
 * standalone driver's gateway mode.  Inside MATLAB, `mex` compiles the same
 * gateway sources against MATLAB's own mex.h instead.
 *
 * Differences from MATLAB, where the stub cannot do what MATLAB does:
 *   - mexErrMsgIdAndTxt throws mx_stub_error (MATLAB unwinds to its prompt);
 *   - every mxArray owns its memory until mxDestroyArray (no garbage
 *     collection of temporaries).
 */
#ifndef BAMF_MX_STUB_MEX_H
#define BAMF_MX_STUB_MEX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
#include <stdexcept>
#include <string>
extern "C" {
#endif

typedef size_t mwSize;
typedef size_t mwIndex;
typedef struct mxArray_tag mxArray;

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

typedef enum { mxREAL = 0, mxCOMPLEX } mxComplexity;

/* creation and destruction */
mxArray *mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID classid, mxComplexity flag);
mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID classid, mxComplexity flag);
mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity flag);
mxArray *mxCreateDoubleScalar(double value);
mxArray *mxCreateStructMatrix(mwSize m, mwSize n, int nfields, const char **fieldnames);
mxArray *mxCreateString(const char *str);
void mxDestroyArray(mxArray *pa);

/* queries */
mxClassID mxGetClassID(const mxArray *pa);
int mxIsSingle(const mxArray *pa);
int mxIsDouble(const mxArray *pa);
int mxIsStruct(const mxArray *pa);
int mxIsChar(const mxArray *pa);
int mxIsNumeric(const mxArray *pa);
mwSize mxGetM(const mxArray *pa);
mwSize mxGetN(const mxArray *pa);
mwSize mxGetNumberOfElements(const mxArray *pa);
mwSize mxGetNumberOfDimensions(const mxArray *pa);
const mwSize *mxGetDimensions(const mxArray *pa);
int mxGetNumberOfFields(const mxArray *pa);
const char *mxGetFieldNameByNumber(const mxArray *pa, int n);

/* data */
void *mxGetData(const mxArray *pa);
double *mxGetPr(const mxArray *pa);
double mxGetScalar(const mxArray *pa);
int mxGetString(const mxArray *pa, char *buf, mwSize buflen);
mxArray *mxGetField(const mxArray *pa, mwIndex i, const char *fieldname);
mxArray *mxGetFieldByNumber(const mxArray *pa, mwIndex i, int fieldnumber);
int mxGetFieldNumber(const mxArray *pa, const char *name);
void mxSetField(mxArray *pa, mwIndex i, const char *fieldname, mxArray *value);
void mxSetFieldByNumber(mxArray *pa, mwIndex i, int fieldnumber, mxArray *value);

/* MEX services */
void mexErrMsgIdAndTxt(const char *errorid, const char *errormsg, ...);
int mexPrintf(const char *fmt, ...);

/* the gateway every MEX file defines */
void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]);

#ifdef __cplusplus
}

/* what mexErrMsgIdAndTxt throws under the stub */
struct mx_stub_error : std::runtime_error {
    std::string id;
    mx_stub_error(const std::string &i, const std::string &m) : std::runtime_error(m), id(i) {}
};
#endif

#endif /* BAMF_MX_STUB_MEX_H */
