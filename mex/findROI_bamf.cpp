/*
 * findROI_bamf.cpp - MEX gateway that does the work of @RJ/findROI.m
 * (its kernel calls, findROI.m:98-122, driving
 * source/cuda/cuda_FindROI/cuda_FindROI.cu, and the find / box / crop steps
 * of findROI.m:124-163) in one call through the C ABI (bamf_find_roi_host,
 * include/bamf.h):
 *
 *   [SMD, ROIStack, Res] = findROI_bamf(Image, Sigma1, Sigma2, Boxsize, Minval)
 *
 * Inputs and defaults are findROI.m's: Image single Y x X x Z; Sigma1 1.3;
 * Sigma2 2*1.3; Boxsize 7; Minval (1/4)*2000*(1/(2*pi*2*1.3^2)).  Outputs
 * as findROI.m returns them: SMD.XBoxCorner, SMD.YBoxCorner, SMD.FrameNum
 * (double column vectors, 1-based, MATLAB find order), ROIStack (double
 * Boxsize x Boxsize x N crops of Image), Res (double, the size of Image, 1 at
 * every maximum).  findROI.m's own body can call this in place of its
 * CUDAKernel feval calls.  Errors raise bamf:findROI:<what>.
 */
#include <mex.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "bamf.h"

namespace {

[[noreturn]] void fail(const char *what, const std::string &msg)
{
    const std::string id = std::string("bamf:findROI:") + what;
    mexErrMsgIdAndTxt(id.c_str(), "%s", msg.c_str());
    throw 0;
}

double arg_or(int nrhs, const mxArray *prhs[], int k, double dflt)
{
    if (k >= nrhs || mxGetNumberOfElements(prhs[k]) == 0) return dflt;
    if (!mxIsNumeric(prhs[k])) fail("type", "Sigma1, Sigma2, Boxsize and Minval must be numeric");
    return mxGetScalar(prhs[k]);
}

mxArray *column(const std::vector<double> &v)
{
    mxArray *a = mxCreateDoubleMatrix((mwSize)v.size(), 1, mxREAL);
    if (!v.empty()) std::memcpy(mxGetPr(a), v.data(), v.size() * sizeof(double));
    return a;
}

}  // namespace

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    if (nrhs < 1 || nrhs > 5) fail("nrhs", "findROI_bamf(Image, Sigma1, Sigma2, Boxsize, Minval)");
    if (nlhs > 3) fail("nlhs", "findROI_bamf has 3 outputs");
    const mxArray *im = prhs[0];
    if (!mxIsSingle(im)) fail("type", "Image must be single");
    const mwSize nd = mxGetNumberOfDimensions(im);
    if (nd > 3) fail("size", "Image must be Y x X x Z");
    const mwSize *d = mxGetDimensions(im);
    const int Y = (int)d[0], X = (int)d[1], Z = nd > 2 ? (int)d[2] : 1;
    const double pi = 3.14159265358979323846;
    const double s1 = arg_or(nrhs, prhs, 1, 1.3);
    const double s2 = arg_or(nrhs, prhs, 2, 2 * 1.3);
    const int box = (int)arg_or(nrhs, prhs, 3, 7);
    const float minval = (float)arg_or(nrhs, prhs, 4, (1.0 / 4) * 2000 * (1 / (2 * pi * 2 * 1.3 * 1.3)));
    if (box < 1 || box > Y || box > X) fail("size", "Boxsize must be between 1 and the frame size");
    const float *frames = (const float *)mxGetData(im);

    /* maxima are at least Boxsize apart in some direction, so this rarely
     * needs the second call */
    int64_t cap = (int64_t)(Y / (box + 1) + 1) * (X / (box + 1) + 1) * Z + 16;
    std::vector<int32_t> coords, corners;
    std::vector<float> stack;
    int64_t count = 0;
    for (int pass = 0; pass < 2; ++pass) {
        coords.assign((size_t)cap * 3, 0);
        corners.assign((size_t)cap * 2, 0);
        stack.assign((size_t)cap * box * box, 0.0f);
        const bamf_status st = bamf_find_roi_host(frames, Y, X, Z, s1, s2, box, minval, cap, coords.data(),
                                                  corners.data(), stack.data(), &count);
        if (st != BAMF_OK)
            fail("status", std::string("bamf_find_roi_host returned ") + std::to_string(st) + " " + bamf_last_error());
        if (count <= cap) break;
        cap = count;
    }
    const size_t n = (size_t)count;
    std::vector<double> xc(n), yc(n), fr(n);
    for (size_t k = 0; k < n; ++k) {
        yc[k] = corners[2 * k];
        xc[k] = corners[2 * k + 1];
        fr[k] = coords[3 * k + 2];
    }
    const char *fields[3] = {"XBoxCorner", "YBoxCorner", "FrameNum"};
    mxArray *smd = mxCreateStructMatrix(1, 1, 3, fields);
    mxSetFieldByNumber(smd, 0, 0, column(xc));
    mxSetFieldByNumber(smd, 0, 1, column(yc));
    mxSetFieldByNumber(smd, 0, 2, column(fr));
    plhs[0] = smd;
    if (nlhs > 1) {
        const mwSize sd[3] = {(mwSize)box, (mwSize)box, (mwSize)n};
        mxArray *rs = mxCreateNumericArray(3, sd, mxDOUBLE_CLASS, mxREAL);
        double *r = mxGetPr(rs);
        for (size_t k = 0; k < n * box * box; ++k) r[k] = stack[k];
        plhs[1] = rs;
    }
    if (nlhs > 2) {
        mxArray *res = mxCreateNumericArray(nd, d, mxDOUBLE_CLASS, mxREAL);
        double *r = mxGetPr(res);
        for (size_t k = 0; k < n; ++k) {
            const size_t row = (size_t)coords[3 * k] - 1, col = (size_t)coords[3 * k + 1] - 1,
                         f = (size_t)coords[3 * k + 2] - 1;
            r[row + (size_t)Y * (col + (size_t)X * f)] = 1.0;
        }
        plhs[2] = res;
    }
}
