/*
 * gaussMLE_bamf.cpp - MEX gateway with the inputs and outputs of
 * @RJ/gaussMLE.m (:64-211), whose kernel calls (cuda_gaussMLEv2.cu, all
 * eight kernel_MLEFit_* variants) run through the C ABI
 * (bamf_gauss_mle_fit_host, include/bamf.h):
 *
 *   [Results, Statistics] = gaussMLE_bamf(Data, FitType, CameraType, Sigma)
 *   ... gaussMLE_bamf(Data, 'Z', 'CCD', Sigma, ZStruct)
 *   ... gaussMLE_bamf(Data, FitType, 'SCMOS', Sigma, VarianceImage, BoxCorners [, ZStruct])
 *   ... and optionally 'Iterations', n as the last two inputs (gaussMLE.m
 *       fixes 20 Newton iterations, :98; that stays the default)
 *
 * FitType 'Basic' | 'Sigma' | 'Z' | 'SigmaYX', CameraType 'CCD' | 'SCMOS'.
 * Results has gaussMLE.m's fields (single columns): Y, X, Photons, BG, their
 * _SE (square roots of the CRLB diagonal), the fit type's extra parameter
 * (Sigma | Z | SigmaY, SigmaX) with its _SE, LogLikelihood; Statistics has
 * FitTime, FitPerSecond, NKernelsCalls (1), NFitsPerCall.  Errors raise
 * bamf:gaussMLE:<what>.
 */
#include <mex.h>

#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "bamf.h"

namespace {

[[noreturn]] void fail(const char *what, const std::string &msg)
{
    const std::string id = std::string("bamf:gaussMLE:") + what;
    mexErrMsgIdAndTxt(id.c_str(), "%s", msg.c_str());
    throw 0;
}

std::string str(const mxArray *a, const char *name)
{
    char buf[32] = {0};
    if (!mxIsChar(a) || mxGetString(a, buf, sizeof buf)) fail("type", std::string(name) + " must be a string");
    return buf;
}

float zfield(const mxArray *z, const char *name)
{
    const mxArray *f = mxIsStruct(z) ? mxGetField(z, 0, name) : nullptr;
    if (!f || !mxIsNumeric(f)) fail("field", std::string("ZStruct.") + name + " is missing");
    return (float)mxGetScalar(f);
}

mxArray *column(const float *v, size_t n, bool root)
{
    mxArray *a = mxCreateNumericMatrix((mwSize)n, 1, mxSINGLE_CLASS, mxREAL);
    float *d = (float *)mxGetData(a);
    for (size_t k = 0; k < n; ++k) d[k] = root ? std::sqrt(v[k]) : v[k];
    return a;
}

}  // namespace

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
    int iterations = 20;
    if (nrhs >= 6 && mxIsChar(prhs[nrhs - 2])) { /* after Data, FitType, CameraType, Sigma */
        if (str(prhs[nrhs - 2], "option") != "Iterations") fail("option", "the only option is 'Iterations', n");
        iterations = (int)mxGetScalar(prhs[nrhs - 1]);
        if (iterations < 1) fail("option", "Iterations must be positive");
        nrhs -= 2;
    }
    if (nrhs < 4 || nrhs > 7) fail("nrhs", "gaussMLE must have 4 to 7 inputs. See doc gaussMLE");
    if (nlhs > 2) fail("nlhs", "gaussMLE_bamf has 2 outputs");
    const mxArray *D = prhs[0];
    if (!mxIsSingle(D)) fail("type", "Data must be single");
    const mwSize nd = mxGetNumberOfDimensions(D);
    const mwSize *dims = mxGetDimensions(D);
    const int sz = (int)dims[0];
    const int n = nd > 2 ? (int)dims[2] : 1;
    if (nd > 3 || (int)dims[1] != sz) fail("size", "Data must be sz x sz x N");
    const std::string fit = str(prhs[1], "FitType"), cam = str(prhs[2], "CameraType");
    int fit_type;
    if (fit == "Basic") fit_type = BAMF_FIT_BASIC;
    else if (fit == "Sigma") fit_type = BAMF_FIT_SIGMA;
    else if (fit == "Z") fit_type = BAMF_FIT_Z;
    else if (fit == "SigmaYX") fit_type = BAMF_FIT_SIGMAYX;
    else fail("FitType", "gaussMLE: Unknown fit type: " + fit);
    if (cam != "CCD" && cam != "SCMOS") fail("CameraType", "CameraType must be 'CCD' or 'SCMOS'");
    const mxArray *S = prhs[3];
    if (!mxIsNumeric(S) || mxGetNumberOfElements(S) < 1) fail("type", "Sigma must be numeric");
    const mwSize ns = mxGetNumberOfElements(S);
    std::vector<double> sig(ns);
    for (mwSize k = 0; k < ns; ++k) {
        if (mxIsDouble(S)) sig[k] = mxGetPr(S)[k];
        else if (mxIsSingle(S)) sig[k] = ((const float *)mxGetData(S))[k];
        else fail("type", "Sigma must be single or double");
    }
    double mean = 0;
    for (double v : sig) mean += v;
    mean /= (double)ns;

    int next = 4;
    const float *var = nullptr, *corners = nullptr;
    int map_size = 0;
    std::vector<float> corner_buf;
    if (cam == "SCMOS") {
        if (nrhs < 6) fail("nrhs", "SCMOS needs VarianceImage and BoxCorners");
        const mxArray *V = prhs[4], *B = prhs[5];
        if (!mxIsSingle(V)) fail("type", "VarianceImage must be single");
        if (mxGetM(V) != mxGetN(V)) fail("size", "gaussMLE: SCMOS fitting is only implemented for square Camera ROI");
        var = (const float *)mxGetData(V);
        map_size = (int)mxGetM(V);
        if (mxGetNumberOfElements(B) < (mwSize)(2 * n)) fail("size", "BoxCorners needs 2 values per fit");
        corner_buf.resize((size_t)2 * n);
        for (size_t k = 0; k < corner_buf.size(); ++k)
            corner_buf[k] = mxIsSingle(B) ? ((const float *)mxGetData(B))[k] : (float)mxGetPr(B)[k];
        corners = corner_buf.data();
        next = 6;
    }
    bamf_zfit z;
    const bamf_zfit *zp = nullptr;
    if (fit_type == BAMF_FIT_Z) {
        if (nrhs <= next) fail("nrhs", "the 'Z' fit needs ZStruct");
        const mxArray *Zs = prhs[next];
        z.sigma_x = (float)sig[0];
        z.sigma_y = (float)(ns > 1 ? sig[1] : sig[0]);
        z.Ax = zfield(Zs, "Ax"); z.Ay = zfield(Zs, "Ay"); z.Bx = zfield(Zs, "Bx"); z.By = zfield(Zs, "By");
        z.gamma = zfield(Zs, "Gamma"); z.d = zfield(Zs, "D");
        zp = &z;
    }
    const int np = bamf_gauss_mle_nparams(fit_type);
    std::vector<float> P((size_t)np * n), CR((size_t)np * n), LL((size_t)n);
    const auto t0 = std::chrono::steady_clock::now();
    const bamf_status st = bamf_gauss_mle_fit_host((const float *)mxGetData(D), sz, n, fit_type, (float)mean, zp,
                                                   corners, var, map_size, iterations, P.data(), CR.data(),
                                                   LL.data());
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (st != BAMF_OK)
        fail("status", std::string("bamf_gauss_mle_fit_host returned ") + std::to_string(st) + " " + bamf_last_error());

    /* param-major outputs: parameter k of fit i at k*n + i, as Params_out(:, k) */
    std::vector<const char *> names = {"Y", "X", "Photons", "BG", "Y_SE", "X_SE", "Photons_SE", "BG_SE"};
    std::vector<std::pair<const char *, const char *>> extra;
    if (fit_type == BAMF_FIT_SIGMA) extra = {{"Sigma", "Sigma_SE"}};
    else if (fit_type == BAMF_FIT_Z) extra = {{"Z", "Z_SE"}};
    else if (fit_type == BAMF_FIT_SIGMAYX) extra = {{"SigmaY", "SigmaY_SE"}, {"SigmaX", "SigmaX_SE"}};
    for (auto &e : extra) names.push_back(e.first);
    for (auto &e : extra) names.push_back(e.second);
    names.push_back("LogLikelihood");
    mxArray *R = mxCreateStructMatrix(1, 1, (int)names.size(), names.data());
    for (int k = 0; k < 4; ++k) {
        mxSetField(R, 0, names[k], column(&P[(size_t)k * n], (size_t)n, false));
        mxSetField(R, 0, names[4 + k], column(&CR[(size_t)k * n], (size_t)n, true));
    }
    for (size_t e = 0; e < extra.size(); ++e) {
        mxSetField(R, 0, extra[e].first, column(&P[(4 + e) * (size_t)n], (size_t)n, false));
        mxSetField(R, 0, extra[e].second, column(&CR[(4 + e) * (size_t)n], (size_t)n, true));
    }
    mxSetField(R, 0, "LogLikelihood", column(LL.data(), (size_t)n, false));
    plhs[0] = R;
    if (nlhs > 1) {
        const char *sf[4] = {"FitTime", "FitPerSecond", "NKernelsCalls", "NFitsPerCall"};
        mxArray *St = mxCreateStructMatrix(1, 1, 4, sf);
        mxSetField(St, 0, "FitTime", mxCreateDoubleScalar(secs));
        mxSetField(St, 0, "FitPerSecond", mxCreateDoubleScalar(secs > 0 ? n / secs : 0.0));
        mxSetField(St, 0, "NKernelsCalls", mxCreateDoubleScalar(1.0));
        mxSetField(St, 0, "NFitsPerCall", mxCreateDoubleScalar((double)n));
        plhs[1] = St;
    }
}
