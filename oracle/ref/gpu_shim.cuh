/*
 * gpu_shim.cuh -- device build of the reference's own CUDA kernel files, the "plain FP64
 * reference GPU form" (TEST AND MEASUREMENT INFRASTRUCTURE ONLY).  The reference's .cu
 * sources are included unchanged from the reference checkout by the wrapper translation
 * units beside this file; nothing of them is copied here.  Around each include the
 * reference's kernels are made device functions of a namespace of their own (the files
 * define the same helper names); the wrapper's extern "C" kernels call them one to one, so
 * the compiled code is the reference kernel's and a launch with the reference's geometry
 * (GPUInitialize.m:7-10) runs exactly the reference's work.  Each wrapper is compiled like
 * the reference's own Makefiles do (plain `nvcc -ptx`, default flags), for sm_103a, into
 * PTX that oracle/refgpu.py loads through the CUDA driver.
 */
#ifndef VSL_REF_GPU_SHIM_CUH
#define VSL_REF_GPU_SHIM_CUH

#include <cmath>
#include <cuda_runtime.h>

#define VSL_REF_KERNEL extern "C" __global__

#endif
