// Directed-rounding FP32 operations for watertight bounding-volume math.
//
// Same names and guarantees as the reference's approx:: namespace
// (include/neighbor/ApproximateMath.h:55-345 in mphowardlab/neighbor): each function returns an
// FP32 value on the requested side of the exact result.  On sm_103a every one of them is a single
// IEEE-754 instruction with a static rounding mode, so they are the CUDA __f*_rd/_ru intrinsics.
// There is no emulated (nextafter) branch: this library targets NVIDIA Blackwell only.
#ifndef NEIGHBOR_APPROXIMATE_MATH_H_
#define NEIGHBOR_APPROXIMATE_MATH_H_

#include <cuda_runtime.h>

namespace neighbor
{
namespace approx
{
__device__ __forceinline__ float double2float_rd(double x) { return __double2float_rd(x); }
__device__ __forceinline__ float double2float_ru(double x) { return __double2float_ru(x); }
__device__ __forceinline__ float fadd_rd(float x, float y) { return __fadd_rd(x, y); }
__device__ __forceinline__ float fadd_ru(float x, float y) { return __fadd_ru(x, y); }
__device__ __forceinline__ float fsub_rd(float x, float y) { return __fsub_rd(x, y); }
__device__ __forceinline__ float fsub_ru(float x, float y) { return __fsub_ru(x, y); }
__device__ __forceinline__ float fmul_rd(float x, float y) { return __fmul_rd(x, y); }
__device__ __forceinline__ float fmul_ru(float x, float y) { return __fmul_ru(x, y); }
__device__ __forceinline__ float fdiv_rd(float x, float y) { return __fdiv_rd(x, y); }
__device__ __forceinline__ float fdiv_ru(float x, float y) { return __fdiv_ru(x, y); }
__device__ __forceinline__ float frcp_rd(float x) { return __frcp_rd(x); }
__device__ __forceinline__ float frcp_ru(float x) { return __frcp_ru(x); }
__device__ __forceinline__ float fmaf_rd(float x, float y, float z) { return __fmaf_rd(x, y, z); }
__device__ __forceinline__ float fmaf_ru(float x, float y, float z) { return __fmaf_ru(x, y, z); }
} // namespace approx
} // namespace neighbor

#endif // NEIGHBOR_APPROXIMATE_MATH_H_
