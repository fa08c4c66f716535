// Host-only stand-in for <cuda_runtime.h>, used only by oracle/ref_kat.cpp: it lets g++ compile
// the reference's __device__ inline helpers (SmoothingKernelsCUDA.h, MathUtilsCUDA.h) unchanged
// as plain host functions.  Not used by any product or oracle build.
#pragma once
#define __device__
#define __host__
#define __forceinline__ inline
