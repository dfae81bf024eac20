// cublas_v2.h -- TEST INFRASTRUCTURE: the cuBLAS calls of the reference's
// scalarslice::toImage (scalarslice.cu:93-138), with the semantics the cuBLAS
// documentation gives them: cublasI?amax returns the smallest 1-based index of
// the entry of largest magnitude (|x| for real data) over n entries at
// stride incx.  Host memory stands in for device memory (cuda_runtime.h).
#ifndef BS_REF_CUBLAS_H
#define BS_REF_CUBLAS_H
#include <cmath>

typedef int cublasStatus_t;
typedef struct bs_ref_cublas* cublasHandle_t;
enum { CUBLAS_STATUS_SUCCESS = 0, CUBLAS_STATUS_INVALID_VALUE = 7 };
inline cublasStatus_t cublasCreate(cublasHandle_t* h) {
    *h = nullptr;
    return CUBLAS_STATUS_SUCCESS;
}
inline cublasStatus_t cublasDestroy(cublasHandle_t) { return CUBLAS_STATUS_SUCCESS; }

template <class T>
inline cublasStatus_t bs_ref_iamax(int n, const T* x, int incx, int* r) {
    *r = 0;
    if (n <= 0 || incx <= 0) return CUBLAS_STATUS_SUCCESS;
    int best = 0;
    for (int i = 1; i < n; i++)
        if (std::fabs(x[(long)i * incx]) > std::fabs(x[(long)best * incx])) best = i;
    *r = best + 1;
    return CUBLAS_STATUS_SUCCESS;
}
inline cublasStatus_t cublasIsamax(cublasHandle_t, int n, const float* x, int incx, int* r) {
    return bs_ref_iamax(n, x, incx, r);
}
inline cublasStatus_t cublasIdamax(cublasHandle_t, int n, const double* x, int incx, int* r) {
    return bs_ref_iamax(n, x, incx, r);
}
#endif
