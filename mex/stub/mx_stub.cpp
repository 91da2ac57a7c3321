/*
 * mx_stub.cpp - plain C++ implementation of the mxArray subset declared in
 * mex/stub/mex.h: numeric arrays (column-major, any class), char strings
 * and struct arrays (one mxArray* per element and field, owned by the
 * struct).  Enough for the gateways of mex/ to run outside MATLAB.
 */
#include "mex.h"

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

struct mxArray_tag {
    mxClassID cls = mxUNKNOWN_CLASS;
    std::vector<mwSize> dims;
    std::vector<unsigned char> data;      /* numeric / char payload       */
    std::vector<std::string> fields;      /* struct field names           */
    std::vector<mxArray *> values;        /* struct: [element][field]     */
};

static size_t elem_size(mxClassID c)
{
    switch (c) {
    case mxDOUBLE_CLASS: case mxINT64_CLASS: case mxUINT64_CLASS: return 8;
    case mxSINGLE_CLASS: case mxINT32_CLASS: case mxUINT32_CLASS: return 4;
    case mxINT16_CLASS: case mxUINT16_CLASS: case mxCHAR_CLASS: return 2;
    case mxINT8_CLASS: case mxUINT8_CLASS: case mxLOGICAL_CLASS: return 1;
    default: return 0;
    }
}

static mwSize count(const std::vector<mwSize> &d)
{
    mwSize n = 1;
    for (mwSize v : d) n *= v;
    return n;
}

extern "C" {

mxArray *mxCreateNumericArray(mwSize ndim, const mwSize *dims, mxClassID classid, mxComplexity flag)
{
    if (flag != mxREAL || elem_size(classid) == 0) return nullptr;
    mxArray *a = new mxArray_tag();
    a->cls = classid;
    a->dims.assign(dims, dims + ndim);
    while (a->dims.size() < 2) a->dims.push_back(1);
    a->data.assign(count(a->dims) * elem_size(classid), 0);
    return a;
}

mxArray *mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID classid, mxComplexity flag)
{
    const mwSize d[2] = {m, n};
    return mxCreateNumericArray(2, d, classid, flag);
}

mxArray *mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity flag)
{
    return mxCreateNumericMatrix(m, n, mxDOUBLE_CLASS, flag);
}

mxArray *mxCreateDoubleScalar(double value)
{
    mxArray *a = mxCreateNumericMatrix(1, 1, mxDOUBLE_CLASS, mxREAL);
    std::memcpy(a->data.data(), &value, sizeof value);
    return a;
}

mxArray *mxCreateStructMatrix(mwSize m, mwSize n, int nfields, const char **fieldnames)
{
    mxArray *a = new mxArray_tag();
    a->cls = mxSTRUCT_CLASS;
    a->dims = {m, n};
    for (int f = 0; f < nfields; ++f) a->fields.emplace_back(fieldnames[f]);
    a->values.assign((size_t)(m * n) * (size_t)nfields, nullptr);
    return a;
}

mxArray *mxCreateString(const char *str)
{
    const size_t L = std::strlen(str);
    mxArray *a = new mxArray_tag();
    a->cls = mxCHAR_CLASS;
    a->dims = {1, L};
    a->data.assign(2 * L, 0);
    for (size_t i = 0; i < L; ++i) a->data[2 * i] = (unsigned char)str[i];
    return a;
}

void mxDestroyArray(mxArray *pa)
{
    if (!pa) return;
    for (mxArray *v : pa->values) mxDestroyArray(v);
    delete pa;
}

mxClassID mxGetClassID(const mxArray *pa) { return pa ? pa->cls : mxUNKNOWN_CLASS; }
int mxIsSingle(const mxArray *pa) { return pa && pa->cls == mxSINGLE_CLASS; }
int mxIsDouble(const mxArray *pa) { return pa && pa->cls == mxDOUBLE_CLASS; }
int mxIsStruct(const mxArray *pa) { return pa && pa->cls == mxSTRUCT_CLASS; }
int mxIsChar(const mxArray *pa) { return pa && pa->cls == mxCHAR_CLASS; }
int mxIsNumeric(const mxArray *pa)
{
    return pa && pa->cls >= mxDOUBLE_CLASS && pa->cls <= mxUINT64_CLASS;
}
mwSize mxGetM(const mxArray *pa) { return pa ? pa->dims[0] : 0; }
mwSize mxGetN(const mxArray *pa)
{
    if (!pa) return 0;
    mwSize n = 1;
    for (size_t k = 1; k < pa->dims.size(); ++k) n *= pa->dims[k];
    return n;
}
mwSize mxGetNumberOfElements(const mxArray *pa) { return pa ? count(pa->dims) : 0; }
mwSize mxGetNumberOfDimensions(const mxArray *pa) { return pa ? pa->dims.size() : 0; }
const mwSize *mxGetDimensions(const mxArray *pa) { return pa ? pa->dims.data() : nullptr; }
int mxGetNumberOfFields(const mxArray *pa) { return pa ? (int)pa->fields.size() : 0; }
const char *mxGetFieldNameByNumber(const mxArray *pa, int n)
{
    return pa && n >= 0 && n < (int)pa->fields.size() ? pa->fields[n].c_str() : nullptr;
}

void *mxGetData(const mxArray *pa)
{
    if (!pa || pa->data.empty()) return nullptr;
    return (void *)pa->data.data();
}
double *mxGetPr(const mxArray *pa) { return pa && pa->cls == mxDOUBLE_CLASS ? (double *)mxGetData(pa) : nullptr; }

double mxGetScalar(const mxArray *pa)
{
    if (!pa || pa->data.empty()) return 0.0;
    const void *p = pa->data.data();
    switch (pa->cls) {
    case mxDOUBLE_CLASS: return *(const double *)p;
    case mxSINGLE_CLASS: return *(const float *)p;
    case mxINT64_CLASS: return (double)*(const int64_t *)p;
    case mxUINT64_CLASS: return (double)*(const uint64_t *)p;
    case mxINT32_CLASS: return *(const int32_t *)p;
    case mxUINT32_CLASS: return *(const uint32_t *)p;
    case mxINT16_CLASS: return *(const int16_t *)p;
    case mxUINT16_CLASS: case mxCHAR_CLASS: return *(const uint16_t *)p;
    case mxINT8_CLASS: return *(const int8_t *)p;
    case mxUINT8_CLASS: case mxLOGICAL_CLASS: return *(const uint8_t *)p;
    default: return 0.0;
    }
}

int mxGetString(const mxArray *pa, char *buf, mwSize buflen)
{
    if (!pa || pa->cls != mxCHAR_CLASS || buflen < 1) return 1;
    const mwSize n = count(pa->dims);
    mwSize k = 0;
    for (; k < n && k + 1 < buflen; ++k) buf[k] = (char)pa->data[2 * k];
    buf[k] = 0;
    return k < n ? 1 : 0;
}

int mxGetFieldNumber(const mxArray *pa, const char *name)
{
    if (!pa || pa->cls != mxSTRUCT_CLASS) return -1;
    for (size_t f = 0; f < pa->fields.size(); ++f)
        if (pa->fields[f] == name) return (int)f;
    return -1;
}

mxArray *mxGetFieldByNumber(const mxArray *pa, mwIndex i, int fieldnumber)
{
    if (!pa || pa->cls != mxSTRUCT_CLASS || fieldnumber < 0 || fieldnumber >= (int)pa->fields.size() ||
        i >= count(pa->dims))
        return nullptr;
    return pa->values[i * pa->fields.size() + (size_t)fieldnumber];
}

mxArray *mxGetField(const mxArray *pa, mwIndex i, const char *fieldname)
{
    return mxGetFieldByNumber(pa, i, mxGetFieldNumber(pa, fieldname));
}

void mxSetFieldByNumber(mxArray *pa, mwIndex i, int fieldnumber, mxArray *value)
{
    if (!pa || pa->cls != mxSTRUCT_CLASS || fieldnumber < 0 || fieldnumber >= (int)pa->fields.size() ||
        i >= count(pa->dims))
        return;
    mxArray *&slot = pa->values[i * pa->fields.size() + (size_t)fieldnumber];
    if (slot && slot != value) mxDestroyArray(slot);
    slot = value;
}

void mxSetField(mxArray *pa, mwIndex i, const char *fieldname, mxArray *value)
{
    mxSetFieldByNumber(pa, i, mxGetFieldNumber(pa, fieldname), value);
}

void mexErrMsgIdAndTxt(const char *errorid, const char *errormsg, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, errormsg);
    std::vsnprintf(buf, sizeof buf, errormsg, ap);
    va_end(ap);
    throw mx_stub_error(errorid ? errorid : "", buf);
}

int mexPrintf(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    int r = std::vprintf(fmt, ap);
    va_end(ap);
    return r;
}

}  // extern "C"

/* For hosts that cannot catch C++ exceptions (a C program, Python's
 * ctypes): calls the linked gateway's mexFunction and turns an error raised
 * by mexErrMsgIdAndTxt into a return value of 1 with its identifier and
 * message copied out (0: the gateway returned normally). */
extern "C" int mx_stub_call_gateway(int nlhs, mxArray **plhs, int nrhs, const mxArray **prhs, char *errid,
                                    size_t idlen, char *errmsg, size_t msglen)
{
    try {
        mexFunction(nlhs, plhs, nrhs, prhs);
        return 0;
    } catch (const mx_stub_error &e) {
        if (errid && idlen) std::snprintf(errid, idlen, "%s", e.id.c_str());
        if (errmsg && msglen) std::snprintf(errmsg, msglen, "%s", e.what());
        return 1;
    }
}
