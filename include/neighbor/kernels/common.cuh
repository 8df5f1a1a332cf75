// Device helpers shared by the build and traversal kernels (sm_103a).
#ifndef NEIGHBOR_KERNELS_COMMON_CUH_
#define NEIGHBOR_KERNELS_COMMON_CUH_

#include <cstdint>

#include <cuda_runtime.h>

#include "../BoundingVolumes.h"
#include "../LBVHData.h"

namespace neighbor
{
namespace gpu
{

// Bits of the device status word an LBVH keeps.  A bounded spin that gives up sets its bit and
// the kernel finishes without waiting further; LBVH::checkStatus() turns it into an exception.
enum StatusBits : unsigned int
    {
    kStatusOk = 0u,
    kStatusSortLookback = 1u,
    kStatusScanLookback = 2u,
    kStatusTensorWait = 4u,   // a wait for a tensor-core MMA gave up
    };

// Upper bound on polls of one look-back word (each poll sleeps ~64 ns after the first few), so a
// wait that can never end gives up after well under a second instead of hanging the GPU.  A
// legitimate wait (a predecessor tile finishing its local work) takes a few thousand polls.
constexpr unsigned int kSpinLimit = 1u << 22;

// Decoupled look-back status words: tag (30 bits, distinguishes builds and passes so the buffer
// never needs clearing) | flag (2 bits) | value (32 bits).
constexpr unsigned long long kFlagAggregate = 1ull;
constexpr unsigned long long kFlagInclusive = 2ull;

__device__ __forceinline__ unsigned long long make_status(unsigned int tag, unsigned long long flag,
                                                          unsigned int value)
    {
    return ((unsigned long long)tag << 34) | (flag << 32) | (unsigned long long)value;
    }

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p)
    {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
    }

__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v)
    {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
    }

__device__ __forceinline__ unsigned int lanemask_lt()
    {
    unsigned int m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
    }

// Look back over the status words of tiles tile-1, tile-2, ... (stride words apart) until an
// inclusive prefix is found; returns the sum of everything before `tile`.  Bounded.
__device__ __forceinline__ unsigned int lookback(const unsigned long long* status, int tile,
                                                 size_t stride, unsigned int tag,
                                                 unsigned int* error, unsigned int error_bit,
                                                 bool& timed_out)
    {
    unsigned int excl = 0;
    int k = tile - 1;
    unsigned int spins = 0;
    timed_out = false;
    while (k >= 0)
        {
        const unsigned long long s = ld_relaxed_u64(status + (size_t)k * stride);
        const unsigned int stag = (unsigned int)(s >> 34);
        const unsigned long long flag = (s >> 32) & 3ull;
        if (stag != tag || flag == 0ull)
            {
            if (++spins > kSpinLimit)
                {
                atomicOr(error, error_bit);
                timed_out = true;
                return excl;
                }
            if (spins > 8) __nanosleep(64);
            continue;
            }
        excl += (unsigned int)s;
        if (flag == kFlagInclusive) break;
        --k;
        }
    return excl;
    }

// Status word read that bypasses L1 (it may be set by another block of the same grid).
__device__ __forceinline__ unsigned int ld_status(const unsigned int* p)
    {
    return *reinterpret_cast<const volatile unsigned int*>(p);
    }

// Order-preserving map FP32 -> uint32 (for atomic min/max of bounds).
__device__ __forceinline__ unsigned int float_to_ordered(float f)
    {
    const unsigned int u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    }
__device__ __forceinline__ float ordered_to_float(unsigned int u)
    {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
    }

// ---------------------------------------------------------------------------------------------
// 30-bit Morton codes.  Same arithmetic as the reference's gen_codes (include/neighbor/kernels/
// LBVH.cuh:140-152): box centre, fractional coordinate by IEEE division, bin = truncation of
// clamp(f*1023, 0, 1023), bits interleaved x above y above z.
// ---------------------------------------------------------------------------------------------

// Insert two zero bits above each of the low 10 bits ("part 1 by 2").
__device__ __forceinline__ unsigned int part1by2(unsigned int v)
    {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
    }

__device__ __forceinline__ unsigned int morton_bin(float f)
    {
    return (unsigned int)fminf(fmaxf(__fmul_rn(f, 1023.f), 0.f), 1023.f);
    }

__device__ __forceinline__ unsigned int morton_code(const BoundingBox& b, const float3& lo,
                                                    const float3& ext)
    {
    const float3 c = b.getCenter();
    const unsigned int x = morton_bin(__fdiv_rn(__fsub_rn(c.x, lo.x), ext.x));
    const unsigned int y = morton_bin(__fdiv_rn(__fsub_rn(c.y, lo.y), ext.y));
    const unsigned int z = morton_bin(__fdiv_rn(__fsub_rn(c.z, lo.z), ext.z));
    return (part1by2(x) << 2) | (part1by2(y) << 1) | part1by2(z);
    }

// ---------------------------------------------------------------------------------------------
// Record boxes: 15-bit bins (0..32767) of the root box held in 16-bit fields.  Bins are measured
// from the root's lower corner with scale = 32767/extent rounded down; lower bounds round down,
// upper bounds round up, both clamped to [0, 32767].  Upper bins are stored complemented
// (32767-h), so "box overlaps query" is "every field of the box <= the matching field of the
// query".  The query's fields carry the guard bit 0x8000: (query|guard) - box is then computed
// in each 16-bit half without borrowing from its neighbour, and the guard bit survives exactly
// when box <= query.
// ---------------------------------------------------------------------------------------------
constexpr unsigned int kBinMax = 32767u;
constexpr unsigned int kGuard = 0x80008000u;

__device__ __forceinline__ unsigned int bin_down(float x, float o, float s)
    {
    const int v = __float2int_rd(approx::fmul_rd(approx::fsub_rd(x, o), s));
    return (unsigned int)min(max(v, 0), (int)kBinMax);
    }
__device__ __forceinline__ unsigned int bin_up(float x, float o, float s)
    {
    const int v = __float2int_ru(approx::fmul_ru(approx::fsub_ru(x, o), s));
    return (unsigned int)min(max(v, 0), (int)kBinMax);
    }

__device__ __forceinline__ uint3 pack_node_box(const QuantFrame& f, const float3& lo, const float3& hi)
    {
    const unsigned int lx = bin_down(lo.x, f.lo.x, f.scale.x);
    const unsigned int ly = bin_down(lo.y, f.lo.y, f.scale.y);
    const unsigned int lz = bin_down(lo.z, f.lo.z, f.scale.z);
    const unsigned int hx = bin_up(hi.x, f.lo.x, f.scale.x);
    const unsigned int hy = bin_up(hi.y, f.lo.y, f.scale.y);
    const unsigned int hz = bin_up(hi.z, f.lo.z, f.scale.z);
    return make_uint3(lx | (ly << 16), lz | ((kBinMax - hx) << 16),
                      (kBinMax - hy) | ((kBinMax - hz) << 16));
    }

// Query box packed as {hi.x|hi.y<<16, hi.z|~lo.x<<16, ~lo.y|~lo.z<<16} with the guard bits set.
__device__ __forceinline__ uint3 pack_query_box(const QuantFrame& f, const float3& lo, const float3& hi)
    {
    const unsigned int lx = bin_down(lo.x, f.lo.x, f.scale.x);
    const unsigned int ly = bin_down(lo.y, f.lo.y, f.scale.y);
    const unsigned int lz = bin_down(lo.z, f.lo.z, f.scale.z);
    const unsigned int hx = bin_up(hi.x, f.lo.x, f.scale.x);
    const unsigned int hy = bin_up(hi.y, f.lo.y, f.scale.y);
    const unsigned int hz = bin_up(hi.z, f.lo.z, f.scale.z);
    return make_uint3((hx | (hy << 16)) | kGuard, (hz | ((kBinMax - lx) << 16)) | kGuard,
                      ((kBinMax - ly) | ((kBinMax - lz) << 16)) | kGuard);
    }

__device__ __forceinline__ bool node_overlaps(const uint4& n, const uint3& q)
    {
    return ((q.x - n.x) & (q.y - n.y) & (q.z - n.z) & kGuard) == kGuard;
    }

constexpr unsigned int kLeafFlag = 0x80000000u;

} // namespace gpu
} // namespace neighbor

#endif // NEIGHBOR_KERNELS_COMMON_CUH_
