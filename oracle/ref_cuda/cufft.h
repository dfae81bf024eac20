// cufft.h -- TEST INFRASTRUCTURE: host stand-in for the cuFFT calls of the
// reference's fieldslice.cpp (cufftPlan2d, cufftExecC2C/Z2Z, cufftDestroy).
// The transforms are this project's own row-column DFT in double precision
// with exact twiddles (ref_runtime.cpp); C2C results are rounded to float as
// cuFFT's single-precision output is.  Unnormalised, sign -1 forward, +1
// inverse, row-major nx x ny with ny contiguous, as cuFFT documents.
#ifndef BS_REF_CUFFT_H
#define BS_REF_CUFFT_H
#include "cuda_runtime.h"

typedef int cufftHandle;
typedef float2 cufftComplex;
typedef double2 cufftDoubleComplex;
typedef enum cufftResult_t {
    CUFFT_SUCCESS = 0,
    CUFFT_INVALID_PLAN = 1,
    CUFFT_ALLOC_FAILED = 2,
    CUFFT_INVALID_TYPE = 3,
    CUFFT_INVALID_VALUE = 4,
    CUFFT_INTERNAL_ERROR = 5,
    CUFFT_EXEC_FAILED = 6,
    CUFFT_SETUP_FAILED = 7,
    CUFFT_INVALID_SIZE = 8
} cufftResult;
typedef enum cufftType_t { CUFFT_C2C = 0x29, CUFFT_Z2Z = 0x69 } cufftType;
#define CUFFT_FORWARD -1
#define CUFFT_INVERSE 1

cufftResult cufftPlan2d(cufftHandle* plan, int nx, int ny, cufftType type);
cufftResult cufftExecC2C(cufftHandle plan, cufftComplex* in, cufftComplex* out, int direction);
cufftResult cufftExecZ2Z(cufftHandle plan, cufftDoubleComplex* in, cufftDoubleComplex* out, int direction);
cufftResult cufftDestroy(cufftHandle plan);
#endif
