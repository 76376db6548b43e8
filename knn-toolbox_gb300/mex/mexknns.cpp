// mexknns.cpp -- the MATLAB MEX gateways mexknnsBitonic, mexknnsHeap (single)
// and mexknnsDBitonic, mexknnsDHeap (double) over the GB300 engine.
//
// Interface of src/mexknnsGen.cu:55-98 and src/mexknnsHeap.cu:185-274:
//   [dist, idx, time, dTime, sTime] = mexknns...(query, data, k, numStreams)
//   query  d x Q (columns are vectors), data d x N, same class (single for the
//          plain gateways, double for the D ones); k, numStreams scalars;
//   dist, idx  k x Q of the inputs' class, idx 0-based (toolbox/gpuknnBitonic.m
//          adds 1 and sorts); time, dTime, sTime  1 x 1 doubles: seconds of the
//          whole call, of the distance stage and of the selection stage.
// Differences: results arrive sorted by (distance, index); numStreams is a hint
// only; errors raise mexErrMsgIdAndTxt with the engine's message instead of
// returning garbage; the device is not reset (src/mexknnsGen.cu:266 resets it).
//
// Build (MATLAB present): mex -R2018a mexknns.cpp [-DKNN_GATEWAY_DOUBLE]
//   [-DKNN_GATEWAY_HEAP] -I<repo>/include -L<repo>/knn-toolbox_gb300/_build
//   -lknngb300 (or -lknngb300_double) -output mexknns[D]{Bitonic,Heap}
#include <chrono>
#include <cfloat>
#include <cstdint>
#include <cstring>
#include <vector>

#include "mex.h"

#ifdef KNN_GATEWAY_DOUBLE
#define __DOUBLE__ 1
#endif
#include "cuknns.h"
#ifdef KNN_GATEWAY_DOUBLE
#include "knn_gb300_f64.h"
#else
#include "knn_gb300.h"
#endif

#ifdef KNN_GATEWAY_DOUBLE
static const mxClassID kClass = mxDOUBLE_CLASS;
static const char* kClassName = "double";
#else
static const mxClassID kClass = mxSINGLE_CLASS;
static const char* kClassName = "single";
#endif

extern "C" void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[])
{
    if (nrhs != 4) mexErrMsgIdAndTxt("knns:nrhs", "four inputs: query (d x Q), data (d x N), k, numStreams");
    if (nlhs > 5) mexErrMsgIdAndTxt("knns:nlhs", "at most five outputs: dist, idx, time, dTime, sTime");
    if (mxGetClassID(prhs[0]) != kClass || mxGetClassID(prhs[1]) != kClass)
        mexErrMsgIdAndTxt("knns:class", "query and data must be %s matrices", kClassName);
    const size_t D = mxGetM(prhs[0]), Q = mxGetN(prhs[0]), N = mxGetN(prhs[1]);
    if (mxGetM(prhs[1]) != D) mexErrMsgIdAndTxt("knns:dims", "query and data need the same number of rows");
    const double kd = mxGetScalar(prhs[2]);
    const int numStreams = (int)mxGetScalar(prhs[3]);
    if (D == 0 || N == 0 || !(kd >= 1.0) || kd != (double)(int)kd || (size_t)kd > N)
        mexErrMsgIdAndTxt("knns:k", "k must be an integer in 1..N (N = %d)", (int)N);
    const int k = (int)kd;
    if (N > 0x7fffffff || Q > 0x7fffffff) mexErrMsgIdAndTxt("knns:size", "more than 2^31-1 vectors");
    knntype* query = (knntype*)mxGetData(prhs[0]);
    knntype* data = (knntype*)mxGetData(prhs[1]);

    plhs[0] = mxCreateNumericMatrix(k, Q, kClass, mxREAL);
    plhs[1] = mxCreateNumericMatrix(k, Q, kClass, mxREAL);
    for (int i = 2; i < 5; ++i) plhs[i] = mxCreateDoubleMatrix(1, 1, mxREAL);
    knntype* values = (knntype*)mxGetData(plhs[0]);
    knntype* indices = (knntype*)mxGetData(plhs[1]);
    double* t_all = mxGetPr(plhs[2]);
    double* t_dst = mxGetPr(plhs[3]);
    double* t_srch = mxGetPr(plhs[4]);
    *t_all = *t_dst = *t_srch = 0.0;
    if (Q == 0) return;

#ifdef KNN_GATEWAY_DOUBLE
    // the double library's drop-in entry points (same engine for both names)
#ifdef KNN_GATEWAY_HEAP
    const double t = gpuknnsHeap(query, data, values, indices, (int)N, (int)Q, (int)D, k, numStreams);
#else
    const double t = gpuknnsBitonic(query, data, values, indices, (int)N, (int)Q, (int)D, k, numStreams);
#endif
    if (t >= DBL_MAX) mexErrMsgIdAndTxt("knns:engine", "%s", knns_f64_last_error());
    *t_all = t;
    *t_dst = t;  // one fused stage: no separate selection time
#else
    (void)numStreams;
    knns_options o;
    knns_default_options(&o);
    o.timing = 1;
    double ms5[5];
    int cnt = 0;
    knns_timing_collect5(ms5, &cnt);  // drop stage times recorded earlier in this process
    std::vector<int32_t> idx((size_t)Q * k);
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = knns_search_host(data, (int64_t)N, query, (int64_t)Q, (int)D, k, values, idx.data(), &o);
    const auto t1 = std::chrono::steady_clock::now();
    if (rc != KNNS_OK) mexErrMsgIdAndTxt("knns:engine", "%s", knns_last_error());
    for (size_t i = 0; i < idx.size(); ++i) indices[i] = (knntype)idx[i];
    *t_all = std::chrono::duration<double>(t1 - t0).count();
    if (knns_timing_collect5(ms5, &cnt) == KNNS_OK && cnt > 0) {
        *t_dst = (ms5[0] + ms5[1] + ms5[2]) / 1000.0;
        *t_srch = (ms5[3] + ms5[4]) / 1000.0;
    }
#endif
}
