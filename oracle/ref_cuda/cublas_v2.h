// cublas_v2.h -- TEST INFRASTRUCTURE: declarations for the cuBLAS calls of the
// reference's scalarslice::toImage (image output, which the oracle checks
// never call); every call reports failure.
#ifndef BS_REF_CUBLAS_H
#define BS_REF_CUBLAS_H
typedef int cublasStatus_t;
typedef struct bs_ref_cublas* cublasHandle_t;
enum { CUBLAS_STATUS_SUCCESS = 0, CUBLAS_STATUS_NOT_SUPPORTED = 15 };
inline cublasStatus_t cublasCreate(cublasHandle_t* h) { *h = nullptr; return CUBLAS_STATUS_NOT_SUPPORTED; }
inline cublasStatus_t cublasDestroy(cublasHandle_t) { return CUBLAS_STATUS_SUCCESS; }
inline cublasStatus_t cublasIsamax(cublasHandle_t, int, const float*, int, int* r) { *r = 1; return CUBLAS_STATUS_NOT_SUPPORTED; }
inline cublasStatus_t cublasIdamax(cublasHandle_t, int, const double*, int, int* r) { *r = 1; return CUBLAS_STATUS_NOT_SUPPORTED; }
#endif
