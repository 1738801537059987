/*
 * ref_shim.hpp -- lets a reference CUDA kernel file compile as host C++ (TEST
 * INFRASTRUCTURE ONLY).  The reference's own .cu sources are included unchanged from the
 * reference checkout by the wrapper translation units beside this file; nothing of them
 * is copied here.  Each wrapper includes one reference file inside its own namespace
 * (the files define the same helper names) and runs the kernel body once per node with
 * blockDim = 1 and blockIdx = (row, column, page), which is the reference launch with
 * one node per thread.
 */
#ifndef VSL_REF_SHIM_HPP
#define VSL_REF_SHIM_HPP

#include <cmath>
#include <cstdlib>

struct vsl_ref_dim3 {
    int x, y, z;
};
extern thread_local vsl_ref_dim3 blockIdx, threadIdx, blockDim;

#define __global__
#define __device__
#define __host__

/* Run `body` for every node of a rows x cols x pges grid, pages spread over OpenMP. */
#define VSL_REF_LAUNCH(rows, cols, pges, body)                                  \
    do {                                                                        \
        _Pragma("omp parallel for schedule(static)")                            \
        for (int pg_ = 0; pg_ < (pges); ++pg_) {                                \
            blockDim = vsl_ref_dim3{1, 1, 1};                                   \
            threadIdx = vsl_ref_dim3{0, 0, 0};                                  \
            for (int cl_ = 0; cl_ < (cols); ++cl_)                              \
                for (int rw_ = 0; rw_ < (rows); ++rw_) {                        \
                    blockIdx = vsl_ref_dim3{rw_, cl_, pg_};                     \
                    body;                                                       \
                }                                                               \
        }                                                                       \
    } while (0)

#define VSL_REF_MATH using std::pow; using std::fabs; using std::sqrt; using std::abs;

#endif
