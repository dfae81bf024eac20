// prelude.h -- TEST INFRASTRUCTURE, force-included (g++ -include) ahead of every
// reference source that oracle/Makefile compiles for the host-run build of the
// reference (target ref-sim).  It defines the CUDA keywords away and turns a
// kernel launch into a loop over the grid: the recipe rewrites
// `kernel<<<grid, block[, shmem]>>>(args)` into
// `BS_REF_LAUNCH(kernel, grid, block[, shmem])(args)` while piping the source to
// the compiler (no copy of the source is written).  The arguments are
// evaluated once; then blocks (z, y, x) and their threads (z, y, x) run one
// after another on the calling host thread, each a plain call of the kernel
// body with threadIdx/blockIdx set, so an early `return` ends that thread only.
// A launch with dynamic shared memory (the reference's only kernels that
// synchronise threads: the ring reductions of microscope.cu) runs each block's
// threads as coroutines instead (ref_runtime.cpp): __syncthreads() suspends the
// calling thread until every thread of the block that has not returned reaches
// it.  Elsewhere __syncthreads() does nothing.
#ifndef BS_REF_PRELUDE_H
#define BS_REF_PRELUDE_H

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <functional>
#include <utility>

#include "cuda_runtime.h"

#define __global__
#define __device__
#define __host__
#define __shared__
#define __constant__
#define __forceinline__ inline
#define __launch_bounds__(...)
#define HANDLE_ERROR(e) (e)

void bs_ref_syncthreads();
inline void __syncthreads() { bs_ref_syncthreads(); }

// CUDA's max/min overloads of the device math library, as plain functions so
// that mixed argument types promote as they do in device code.
inline int max(int a, int b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline unsigned max(unsigned a, unsigned b) { return a > b ? a : b; }
inline unsigned min(unsigned a, unsigned b) { return a < b ? a : b; }
inline float max(float a, float b) { return std::fmax(a, b); }
inline float min(float a, float b) { return std::fmin(a, b); }
inline double max(double a, double b) { return std::fmax(a, b); }
inline double min(double a, double b) { return std::fmin(a, b); }
inline double max(float a, double b) { return std::fmax((double)a, b); }
inline double max(double a, float b) { return std::fmax(a, (double)b); }
inline double min(float a, double b) { return std::fmin((double)a, b); }
inline double min(double a, float b) { return std::fmin(a, (double)b); }

namespace bs_ref {
// runs body() once per thread of a block of `block` threads, as coroutines that
// __syncthreads() switches between (ref_runtime.cpp)
void coop_block(const dim3& block, const std::function<void()>& body);

template <class F>
struct Launch {
    F f;
    dim3 grid, block;
    size_t shmem;
    template <class... A>
    void operator()(A&&... a) {
        ::gridDim = grid;
        ::blockDim = block;
        if (shmem > 0) {
            const std::function<void()> body = [&]() { f(a...); };
            for (unsigned bz = 0; bz < grid.z; bz++)
                for (unsigned by = 0; by < grid.y; by++)
                    for (unsigned bx = 0; bx < grid.x; bx++) {
                        ::blockIdx = uint3{bx, by, bz};
                        coop_block(block, body);
                    }
            return;
        }
        for (unsigned bz = 0; bz < grid.z; bz++)
            for (unsigned by = 0; by < grid.y; by++)
                for (unsigned bx = 0; bx < grid.x; bx++)
                    for (unsigned tz = 0; tz < block.z; tz++)
                        for (unsigned ty = 0; ty < block.y; ty++)
                            for (unsigned tx = 0; tx < block.x; tx++) {
                                ::blockIdx = uint3{bx, by, bz};
                                ::threadIdx = uint3{tx, ty, tz};
                                f(a...);
                            }
    }
};
template <class F>
Launch<F> launch_of(F f, dim3 g, dim3 b, size_t shmem = 0, void* = nullptr) {
    return Launch<F>{f, g, b, shmem};
}
}  // namespace bs_ref

#define BS_REF_LAUNCH(k, ...) ::bs_ref::launch_of([&](auto&... bs_a) { k(bs_a...); }, __VA_ARGS__)

#endif
