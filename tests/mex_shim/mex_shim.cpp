// mex_shim.cpp -- implementation of the mex.h stand-in (TEST INFRASTRUCTURE ONLY).
// Matrices are column-major buffers owned by the shim; mexErrMsgIdAndTxt throws,
// and shim_call() turns that into an error code and a message, as MATLAB turns
// it into an error at the prompt.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "mex.h"

struct mxArray_tag {
    size_t m = 0, n = 0;
    mxClassID cls = mxUNKNOWN_CLASS;
    std::vector<unsigned char> bytes;
};

namespace {
size_t elem(mxClassID c) { return c == mxDOUBLE_CLASS ? 8 : c == mxSINGLE_CLASS ? 4 : 0; }

struct MexError : std::runtime_error {
    std::string id;
    MexError(const char* i, const std::string& msg) : std::runtime_error(msg), id(i) {}
};
}  // namespace

extern "C" {

size_t mxGetM(const mxArray* a) { return a->m; }
size_t mxGetN(const mxArray* a) { return a->n; }
void* mxGetData(const mxArray* a) { return const_cast<unsigned char*>(a->bytes.data()); }
double* mxGetPr(const mxArray* a) { return reinterpret_cast<double*>(const_cast<unsigned char*>(a->bytes.data())); }
mxClassID mxGetClassID(const mxArray* a) { return a->cls; }

double mxGetScalar(const mxArray* a)
{
    if (a->bytes.empty()) return 0.0;
    if (a->cls == mxDOUBLE_CLASS) return *reinterpret_cast<const double*>(a->bytes.data());
    if (a->cls == mxSINGLE_CLASS) return *reinterpret_cast<const float*>(a->bytes.data());
    return 0.0;
}

mxArray* mxCreateNumericMatrix(size_t m, size_t n, mxClassID c, mxComplexity)
{
    mxArray* a = new mxArray_tag();
    a->m = m;
    a->n = n;
    a->cls = c;
    a->bytes.assign(m * n * elem(c), 0);
    return a;
}

mxArray* mxCreateDoubleMatrix(size_t m, size_t n, mxComplexity f) { return mxCreateNumericMatrix(m, n, mxDOUBLE_CLASS, f); }

void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    throw MexError(id, buf);
}

// ---- test harness helpers
mxArray* shim_matrix(size_t m, size_t n, int cls, const void* data)
{
    mxArray* a = mxCreateNumericMatrix(m, n, (mxClassID)cls, mxREAL);
    if (data && !a->bytes.empty()) memcpy(a->bytes.data(), data, a->bytes.size());
    return a;
}

void shim_destroy(mxArray* a) { delete a; }

typedef void (*mex_fn)(int, mxArray**, int, const mxArray**);

// Calls a gateway; returns 0, or 1 with the error id and message in err.
int shim_call(mex_fn fn, int nlhs, mxArray** plhs, int nrhs, const mxArray** prhs, char* err, size_t errlen)
{
    try {
        fn(nlhs, plhs, nrhs, prhs);
        return 0;
    } catch (const MexError& e) {
        snprintf(err, errlen, "%s: %s", e.id.c_str(), e.what());
        return 1;
    }
}

}  // extern "C"
