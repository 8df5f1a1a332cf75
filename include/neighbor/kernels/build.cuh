// LBVH build kernels for sm_103a.
//
// Stages of a build (one stream, no host synchronisation):
//   k_codes_histogram  Morton codes of every primitive -> digit histograms of all radix passes
//                      and the scene bounds (root box) in one read of the inputs.
//   k_digit_offsets    exclusive scan of each pass histogram.
//   k_onesweep         one stable LSD radix pass with decoupled look-back (Adinets & Merrill,
//                      "Onesweep", 2022); the first pass computes keys from the insert op.
//   k_climb            agglomerative bottom-up construction of the radix tree (the Karras tree of
//                      the reference, include/neighbor/kernels/LBVH.cuh:169-243) with packed
//                      15-bit boxes, block-local in shared memory, global across block edges;
//                      counts the box records of the traversal tree per first primitive.
//   k_scan_exclusive   chained exclusive scan of those counts (pre-order positions).
//   k_emit             writes every box and point record at its pre-order slot.
// Reference-layout arrays (parents, children, float boxes), on demand or for non-point trees:
//   k_gen_hierarchy    the Karras kernel, k_ref_bubble the reference's bubbling of float boxes
//                      (include/neighbor/kernels/LBVH.cuh:270-327).
#ifndef NEIGHBOR_KERNELS_BUILD_CUH_
#define NEIGHBOR_KERNELS_BUILD_CUH_

#include <cfloat>
#include <cstdint>
#include <type_traits>

#include "../InsertOps.h"
#include "common.cuh"

namespace neighbor
{
namespace gpu
{

template<int RB>
struct RadixConfig
    {
    static constexpr int kRadix = 1 << RB;
    static constexpr int kPasses = (30 + RB - 1) / RB;
    };

// ---------------------------------------------------------------------------------------------
// Block-wide exclusive scan of n values in shared memory (in place); s_tmp holds >= 32 words.
// ---------------------------------------------------------------------------------------------
template<int BLOCK, int NVALS>
__device__ __forceinline__ unsigned int block_exclusive_scan_smem(unsigned int* data, unsigned int* s_tmp)
    {
    constexpr int PER = (NVALS + BLOCK - 1) / BLOCK;
    constexpr int NW = BLOCK / 32;
    const int t = threadIdx.x;
    const int lane = t & 31;
    const int warp = t >> 5;
    unsigned int v[PER];
    unsigned int sum = 0;
#pragma unroll
    for (int k = 0; k < PER; ++k)
        {
        const int idx = t * PER + k;
        v[k] = idx < NVALS ? data[idx] : 0u;
        sum += v[k];
        }
    unsigned int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
        {
        const unsigned int n = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += n;
        }
    if (lane == 31) s_tmp[warp] = incl;
    __syncthreads();
    if (warp == 0)
        {
        const unsigned int w = lane < NW ? s_tmp[lane] : 0u;
        unsigned int wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
            {
            const unsigned int n = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += n;
            }
        if (lane < NW) s_tmp[lane] = wi - w;
        if (lane == 31) s_tmp[NW] = wi;
        }
    __syncthreads();
    unsigned int run = s_tmp[warp] + incl - sum;
#pragma unroll
    for (int k = 0; k < PER; ++k)
        {
        const int idx = t * PER + k;
        if (idx < NVALS) data[idx] = run;
        run += v[k];
        }
    const unsigned int total = s_tmp[NW];
    __syncthreads();
    return total;
    }

// ---------------------------------------------------------------------------------------------
// Morton codes -> histograms of every pass, and the bounds of all leaf boxes; the codes go to
// codes_out too when it is given (the first sort pass then reads them instead of recomputing).
// bounds[0..2] = max of ~ordered(lo), bounds[3..5] = max of ordered(hi); all start at zero.
// ---------------------------------------------------------------------------------------------
template<class InsertOpT, int RB>
__global__ void __launch_bounds__(256) k_codes_histogram(const InsertOpT insert, unsigned int N,
                                                         float3 scene_lo, float3 scene_ext,
                                                         unsigned int* __restrict__ hist,
                                                         unsigned int* __restrict__ bounds,
                                                         unsigned int* __restrict__ codes_out = nullptr)
    {
    constexpr int R = RadixConfig<RB>::kRadix;
    constexpr int P = RadixConfig<RB>::kPasses;
    __shared__ unsigned int s_hist[P * R];
    __shared__ float s_red[6][8];
    for (int i = threadIdx.x; i < P * R; i += blockDim.x) s_hist[i] = 0u;
    __syncthreads();

    float3 bmin = make_float3(FLT_MAX, FLT_MAX, FLT_MAX);
    float3 bmax = make_float3(-FLT_MAX, -FLT_MAX, -FLT_MAX);
    const unsigned int stride = gridDim.x * blockDim.x;
    // one primitive's box: bounds, code, histograms
    const auto one = [&](const BoundingBox& b) -> unsigned int {
        bmin.x = fminf(bmin.x, b.lo.x);
        bmin.y = fminf(bmin.y, b.lo.y);
        bmin.z = fminf(bmin.z, b.lo.z);
        bmax.x = fmaxf(bmax.x, b.hi.x);
        bmax.y = fmaxf(bmax.y, b.hi.y);
        bmax.z = fmaxf(bmax.z, b.hi.z);
        const unsigned int code = morton_code(b, scene_lo, scene_ext);
#pragma unroll
        for (int p = 0; p < P; ++p) atomicAdd(&s_hist[p * R + ((code >> (p * RB)) & (R - 1))], 1u);
        return code;
    };
    unsigned int first_scalar = 0u;
    if constexpr (std::is_same<InsertOpT, PointInsertOp>::value)
        {
        // Points: each thread reads four consecutive float3 as three aligned float4 (48 bytes)
        // and writes their four codes as one uint4, when the arrays are 16-byte aligned; the
        // last N % 4 points take the loop below.
        const bool aligned = ((reinterpret_cast<uintptr_t>(insert.points) | reinterpret_cast<uintptr_t>(codes_out)) & 15u) == 0u;
        if (aligned)
            {
            const unsigned int groups = N / 4u;
            const float4* p4 = reinterpret_cast<const float4*>(insert.points);
            for (unsigned int g = blockIdx.x * blockDim.x + threadIdx.x; g < groups; g += stride)
                {
                const float4 a = __ldg(p4 + 3u * g);
                const float4 b = __ldg(p4 + 3u * g + 1u);
                const float4 c = __ldg(p4 + 3u * g + 2u);
                const float3 q[4] = {make_float3(a.x, a.y, a.z), make_float3(a.w, b.x, b.y),
                                     make_float3(b.z, b.w, c.x), make_float3(c.y, c.z, c.w)};
                unsigned int code[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) code[k] = one(BoundingBox(q[k], q[k]));
                if (codes_out)
                    reinterpret_cast<uint4*>(codes_out)[g] = make_uint4(code[0], code[1], code[2], code[3]);
                }
            first_scalar = groups * 4u;
            }
        }
    for (unsigned int i = first_scalar + blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride)
        {
        const unsigned int code = one(insert.get(i));
        if (codes_out) codes_out[i] = code;
        }
    float vals[6] = {bmin.x, bmin.y, bmin.z, bmax.x, bmax.y, bmax.z};
#pragma unroll
    for (int k = 0; k < 6; ++k)
        {
        float v = vals[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            {
            const float n = __shfl_xor_sync(0xffffffffu, v, o);
            v = (k < 3) ? fminf(v, n) : fmaxf(v, n);
            }
        if ((threadIdx.x & 31) == 0) s_red[k][threadIdx.x >> 5] = v;
        }
    __syncthreads();
    if (threadIdx.x < 6)
        {
        const int k = threadIdx.x;
        float v = s_red[k][0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) v = (k < 3) ? fminf(v, s_red[k][w]) : fmaxf(v, s_red[k][w]);
        if (k < 3)
            atomicMax(&bounds[k], ~float_to_ordered(v));
        else
            atomicMax(&bounds[k], float_to_ordered(v));
        }
    for (int i = threadIdx.x; i < P * R; i += blockDim.x)
        {
        const unsigned int c = s_hist[i];
        if (c) atomicAdd(&hist[i], c);
        }
    }

// Exclusive scan of each pass histogram: one block per pass.
template<int RB>
__global__ void __launch_bounds__(1024) k_digit_offsets(const unsigned int* __restrict__ hist,
                                                        unsigned int* __restrict__ offsets)
    {
    constexpr int R = RadixConfig<RB>::kRadix;
    __shared__ unsigned int s_data[R];
    __shared__ unsigned int s_tmp[40];
    const int p = blockIdx.x;
    for (int i = threadIdx.x; i < R; i += blockDim.x) s_data[i] = hist[p * R + i];
    __syncthreads();
    block_exclusive_scan_smem<1024, R>(s_data, s_tmp);
    for (int i = threadIdx.x; i < R; i += blockDim.x) offsets[p * R + i] = s_data[i];
    }

// ---------------------------------------------------------------------------------------------
// One stable radix pass.  A block takes the next tile in launch order (atomic ticket), ranks its
// keys per warp with match.any (stable: items are visited in key order), publishes the tile's
// digit counts, stages the tile in shared memory in digit order, and scatters it after the
// decoupled look-back has produced each digit's global base.  Dynamic shared memory layout:
// warp histograms [NW*R], counts [R], local offsets [R], global bases [R], keys [TILE],
// values [TILE], scratch [40].
// ---------------------------------------------------------------------------------------------
template<int RB, int BLOCK, int ITEMS>
struct OnesweepConfig
    {
    static constexpr int kRadix = 1 << RB;
    static constexpr int kWarps = BLOCK / 32;
    static constexpr int kTile = BLOCK * ITEMS;
    static constexpr size_t kSmemBytes =
        sizeof(unsigned int) * ((size_t)kWarps * kRadix + 3 * kRadix + 2 * (size_t)kTile + 40);
    };

template<class InsertOpT, int RB, int BLOCK, int ITEMS, bool FIRST>
__global__ void __launch_bounds__(BLOCK, ITEMS <= 8 ? 6 : 4) k_onesweep(const InsertOpT insert, float3 scene_lo,
                                                    float3 scene_ext,
                                                    const unsigned int* __restrict__ keys_in,
                                                    const unsigned int* __restrict__ vals_in,
                                                    unsigned int* __restrict__ keys_out,
                                                    unsigned int* __restrict__ vals_out,
                                                    unsigned int N, int shift,
                                                    const unsigned int* __restrict__ offsets,
                                                    unsigned long long* __restrict__ status,
                                                    unsigned int tag,
                                                    unsigned int* __restrict__ tile_counter,
                                                    unsigned int* __restrict__ error)
    {
    typedef OnesweepConfig<RB, BLOCK, ITEMS> Cfg;
    constexpr int R = Cfg::kRadix;
    constexpr int NW = Cfg::kWarps;
    constexpr int TILE = Cfg::kTile;
    constexpr int WT = 32 * ITEMS;
    extern __shared__ __align__(16) unsigned int smem_sort[];
    unsigned int* s_whist = smem_sort;
    unsigned int* s_count = s_whist + NW * R;
    unsigned int* s_local = s_count + R;
    unsigned int* s_gbase = s_local + R;
    unsigned int* s_keys = s_gbase + R;
    unsigned int* s_vals = s_keys + TILE;
    unsigned int* s_tmp = s_vals + TILE;

    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    if (tid == 0)
        {
        s_tmp[39] = atomicAdd(tile_counter, 1u);
        s_tmp[38] = ld_status(error);
        s_tmp[37] = 0u;
        }
    for (int i = tid; i < NW * R; i += BLOCK) s_whist[i] = 0u;
    __syncthreads();
    const unsigned int tile = s_tmp[39];
    if (s_tmp[38] != 0u)
        {
        // An earlier wait of this build gave up: release successors at once and write nothing.
        for (int d = tid; d < R; d += BLOCK)
            st_relaxed_u64(status + (size_t)tile * R + d, make_status(tag, kFlagInclusive, 0u));
        return;
        }
    const unsigned int base = tile * TILE;
    const unsigned int wbase = base + warp * WT;

    unsigned int keys[ITEMS];
    unsigned int vals[ITEMS];
    unsigned int ranks[ITEMS];
#pragma unroll
    for (int j = 0; j < ITEMS; ++j)
        {
        const unsigned int idx = wbase + j * 32 + lane;
        keys[j] = 0u;
        vals[j] = 0u;
        if (idx < N)
            {
            if (FIRST)
                {
                // the codes of the histogram pass when given, else computed here
                keys[j] = keys_in ? keys_in[idx] : morton_code(insert.get(idx), scene_lo, scene_ext);
                vals[j] = idx;
                }
            else
                {
                keys[j] = keys_in[idx];
                vals[j] = vals_in[idx];
                }
            }
        }

    unsigned int* my_hist = s_whist + warp * R;
#pragma unroll
    for (int j = 0; j < ITEMS; ++j)
        {
        const bool valid = (wbase + j * 32 + lane) < N;
        const unsigned int d = (keys[j] >> shift) & (R - 1);
        const unsigned int peers = __match_any_sync(0xffffffffu, valid ? d : (unsigned int)(R + lane));
        const unsigned int prior = my_hist[d];
        __syncwarp();
        if (valid && lane == 31 - __clz(peers)) my_hist[d] = prior + __popc(peers);
        __syncwarp();
        ranks[j] = prior + __popc(peers & lanemask_lt());
        }
    __syncthreads();

    for (int d = tid; d < R; d += BLOCK)
        {
        unsigned int run = 0;
#pragma unroll
        for (int w = 0; w < NW; ++w)
            {
            const unsigned int c = s_whist[w * R + d];
            s_whist[w * R + d] = run;
            run += c;
            }
        s_count[d] = run;
        s_local[d] = run;
        st_relaxed_u64(status + (size_t)tile * R + d,
                       make_status(tag, tile == 0 ? kFlagInclusive : kFlagAggregate, run));
        }
    __syncthreads();
    block_exclusive_scan_smem<BLOCK, R>(s_local, s_tmp);

#pragma unroll
    for (int j = 0; j < ITEMS; ++j)
        {
        if ((wbase + j * 32 + lane) < N)
            {
            const unsigned int d = (keys[j] >> shift) & (R - 1);
            const unsigned int lp = s_local[d] + my_hist[d] + ranks[j];
            s_keys[lp] = keys[j];
            s_vals[lp] = vals[j];
            }
        }

    for (int d = tid; d < R; d += BLOCK)
        {
        unsigned int excl = 0;
        if (tile > 0)
            {
            bool timed_out;
            excl = lookback(status + d, (int)tile, R, tag, error, kStatusSortLookback, timed_out);
            if (timed_out) s_tmp[37] = 1u;
            st_relaxed_u64(status + (size_t)tile * R + d, make_status(tag, kFlagInclusive, excl + s_count[d]));
            }
        s_gbase[d] = offsets[d] + excl - s_local[d];
        }
    __syncthreads();
    if (s_tmp[37] != 0u) return;

    // Offsets are only wrong after a wait gave up elsewhere; the bound keeps stores in range.
    const unsigned int n_valid = min((unsigned int)TILE, N - base);
    for (unsigned int i = tid; i < n_valid; i += BLOCK)
        {
        const unsigned int k = s_keys[i];
        const unsigned int g = s_gbase[(k >> shift) & (R - 1)] + i;
        if (g < N)
            {
            keys_out[g] = k;
            vals_out[g] = s_vals[i];
            }
        }
    }

// ---------------------------------------------------------------------------------------------
// Karras hierarchy (reference layout).  One thread per internal node i: direction, range end j by
// exponential and binary search, split by binary search over the longest common prefix with the
// index tie-break; left/right children (leaves at N-1+s) and parents.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ int karras_delta(const unsigned int* __restrict__ codes, unsigned int ci,
                                            long long i, long long j, long long N)
    {
    if (j < 0 || j >= N) return -1;
    const unsigned int cj = __ldg(codes + j);
    if (ci == cj) return 32 + __clz((unsigned int)i ^ (unsigned int)j);
    return __clz(ci ^ cj);
    }

static __global__ void k_gen_hierarchy(const unsigned int* __restrict__ codes, unsigned int N,
                                       int* __restrict__ left, int* __restrict__ right,
                                       int* __restrict__ parent, const unsigned int* __restrict__ error)
    {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = N;
    if (i >= n - 1 || ld_status(error) != 0u) return;
    const unsigned int ci = __ldg(codes + i);
    const int fwd = karras_delta(codes, ci, i, i + 1, n);
    const int bwd = karras_delta(codes, ci, i, i - 1, n);
    const long long d = (fwd >= bwd) ? 1 : -1;
    const int min_prefix = karras_delta(codes, ci, i, i - d, n);
    long long lmax = 2;
    while (karras_delta(codes, ci, i, i + d * lmax, n) > min_prefix) lmax <<= 1;
    long long l = 0;
    for (long long t = lmax >> 1; t >= 1; t >>= 1)
        if (karras_delta(codes, ci, i, i + (l + t) * d, n) > min_prefix) l += t;
    const long long j = i + l * d;
    const int node_prefix = karras_delta(codes, ci, i, j, n);
    long long s = 0;
    long long t = l;
    do
        {
        t = (t + 1) >> 1;
        if (s + t < l && karras_delta(codes, ci, i, i + (s + t) * d, n) > node_prefix) s += t;
        } while (t > 1);
    const long long split = i + s * d + (d < 0 ? -1 : 0);
    const long long first = i < j ? i : j;
    const long long last = i < j ? j : i;
    const int lc = (int)((first == split) ? split + n - 1 : split);
    const int rc = (int)((last == split + 1) ? split + n : split + 1);
    left[i] = lc;
    right[i] = rc;
    parent[lc] = (int)i;
    parent[rc] = (int)i;
    if (i == 0) parent[0] = LBVHSentinel;
    }

// ---------------------------------------------------------------------------------------------
// Chained exclusive scan: out[i] = sum(in[0..i)), out[n] = total, *total_out = total.
// 512 threads x 16 items per tile (16M counts: 2.054 -> 2.043 ms whole build against 256 x 16);
// tiles taken in launch order; look-back on one status word.
// ---------------------------------------------------------------------------------------------
constexpr int kScanBlock = 512;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanBlock * kScanItems;

static __global__ void __launch_bounds__(kScanBlock) k_scan_exclusive(const unsigned int* __restrict__ in,
                                                               unsigned int* __restrict__ out,
                                                               unsigned int n,
                                                               unsigned long long* __restrict__ status,
                                                               unsigned int tag,
                                                               unsigned int* __restrict__ tile_counter,
                                                               unsigned int* __restrict__ total_out,
                                                               unsigned int* __restrict__ error)
    {
    __shared__ unsigned int s_tile;
    __shared__ unsigned int s_warp[kScanBlock / 32 + 1];
    __shared__ unsigned int s_excl;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    __shared__ unsigned int s_err;
    if (tid == 0)
        {
        s_tile = atomicAdd(tile_counter, 1u);
        s_err = ld_status(error);
        }
    __syncthreads();
    const unsigned int tile = s_tile;
    if (s_err != 0u)
        {
        if (tid == 0) st_relaxed_u64(status + tile, make_status(tag, kFlagInclusive, 0u));
        return;
        }
    const unsigned int base = tile * kScanTile + tid * kScanItems;
    unsigned int v[kScanItems];
    unsigned int sum = 0;
    static_assert(kScanItems % 4 == 0, "16-byte loads");
    if (base + kScanItems <= n)
        {
        // a whole thread's items in range: 16-byte loads (base is a multiple of 16 words)
        const uint4* in4 = reinterpret_cast<const uint4*>(in + base);
#pragma unroll
        for (int k = 0; k < kScanItems / 4; ++k)
            {
            const uint4 w = in4[k];
            v[4 * k] = w.x;
            v[4 * k + 1] = w.y;
            v[4 * k + 2] = w.z;
            v[4 * k + 3] = w.w;
            }
        }
    else
        {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) v[k] = (base + k < n) ? in[base + k] : 0u;
        }
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) sum += v[k];
    unsigned int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
        {
        const unsigned int x = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += x;
        }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0)
        {
        constexpr int NW = kScanBlock / 32;
        const unsigned int w = lane < NW ? s_warp[lane] : 0u;
        unsigned int wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
            {
            const unsigned int x = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += x;
            }
        if (lane < NW) s_warp[lane] = wi - w;
        if (lane == 31)
            {
            s_warp[NW] = wi;
            st_relaxed_u64(status + tile, make_status(tag, tile == 0 ? kFlagInclusive : kFlagAggregate, wi));
            unsigned int excl = 0;
            if (tile > 0)
                {
                bool timed_out;
                excl = lookback(status, (int)tile, 1, tag, error, kStatusScanLookback, timed_out);
                st_relaxed_u64(status + tile, make_status(tag, kFlagInclusive, excl + wi));
                }
            s_excl = excl;
            }
        }
    __syncthreads();
    unsigned int run = s_excl + s_warp[warp] + incl - sum;
    if (base + kScanItems <= n)
        {
        // every output of the thread lies before out[n] (the total, written by the thread whose
        // items start at n): 16-byte stores
        uint4* out4 = reinterpret_cast<uint4*>(out + base);
#pragma unroll
        for (int k = 0; k < kScanItems / 4; ++k)
            {
            uint4 w;
            w.x = run;
            run += v[4 * k];
            w.y = run;
            run += v[4 * k + 1];
            w.z = run;
            run += v[4 * k + 2];
            w.w = run;
            run += v[4 * k + 3];
            out4[k] = w;
            }
        }
    else
        {
#pragma unroll
        for (int k = 0; k < kScanItems; ++k)
            {
            if (base + k <= n) out[base + k] = run;
            if (base + k == n && total_out) *total_out = run;
            run += v[k];
            }
        }
    }

// ---------------------------------------------------------------------------------------------
// Root-box frame of the record bins from the root box (or from the bounds words).
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ QuantFrame frame_from_box(const float3& lo, const float3& hi)
    {
    QuantFrame f;
    f.lo = lo;
    f.hi = hi;
    float ex = approx::fsub_ru(f.hi.x, f.lo.x);
    float ey = approx::fsub_ru(f.hi.y, f.lo.y);
    float ez = approx::fsub_ru(f.hi.z, f.lo.z);
    if (!(ex > 0.f)) ex = 1.0f;
    if (!(ey > 0.f)) ey = 1.0f;
    if (!(ez > 0.f)) ez = 1.0f;
    f.scale = make_float3(approx::fdiv_rd((float)kBinMax, ex), approx::fdiv_rd((float)kBinMax, ey),
                          approx::fdiv_rd((float)kBinMax, ez));
    return f;
    }

__device__ __forceinline__ QuantFrame frame_from_bounds(const unsigned int* bounds)
    {
    return frame_from_box(
        make_float3(ordered_to_float(~bounds[0]), ordered_to_float(~bounds[1]), ordered_to_float(~bounds[2])),
        make_float3(ordered_to_float(bounds[3]), ordered_to_float(bounds[4]), ordered_to_float(bounds[5])));
    }

// ---------------------------------------------------------------------------------------------
// Agglomerative construction of the traversal tree (Apetrei, "Fast and Simple Agglomerative LBVH
// Construction", 2014).  The binary radix tree over the sorted (code, index) keys is unique, so
// this is the Karras tree above: node [l, r] is the left child of split r or the right child of
// split l-1, whichever boundary has the longer common prefix (the Karras delta with its index
// tie-break, include/neighbor/kernels/LBVH.cuh:73-94); the two can never be equal.
//
// One thread per sorted leaf climbs while it is the second child to arrive at a split.  Splits
// whose two subtrees lie inside the block's range of leaves meet in shared memory; a node whose
// parent split lies on the block boundary, and a split that only one child reached inside the
// block, continue after the block's local phase with one global arrival word per split.  Boxes
// are the packed 15-bit records' words: every field is a "min" field, so the union of two boxes
// is three 16x2 minima and equals the packing of the union of the float boxes (packing is
// monotone).  Each internal node p (split index) gets {box, first} and {last, db | live}; a node
// becomes a box record (live) when its parent has more than leaf_size primitives, or when it is
// the root, and is then counted at its first primitive for the pre-order scan.
// ---------------------------------------------------------------------------------------------
constexpr unsigned int kNodeLeaf = 0x80000000u;  // node id of sorted leaf s: s | kNodeLeaf
constexpr unsigned int kMetaLive = 0x80000000u;  // set in nmeta.y when the node is a box record

// Common-prefix length of the (code, index) keys at sorted positions i and i + 1.
__device__ __forceinline__ int adjacent_delta(unsigned int ci, unsigned int cj, unsigned int i)
    {
    return (ci != cj) ? __clz(ci ^ cj) : 32 + __clz(i ^ (i + 1u));
    }

// Split index of the parent of node [l, r] (not the root).
template<class DeltaF>
__device__ __forceinline__ unsigned int parent_split(unsigned int l, unsigned int r, unsigned int N,
                                                     const DeltaF& delta)
    {
    if (l == 0u) return r;
    if (r == N - 1u) return l - 1u;
    return delta(r) > delta(l - 1u) ? r : l - 1u;
    }

struct ClimbArgs
    {
    unsigned int N;
    const unsigned int* codes;      // sorted Morton codes
    const unsigned int* primitive;  // sorted primitive ids
    float4* payload;                // per sorted leaf: lower corner of its box, primitive id bits
    uint4* nbox;                    // internal node p: {packed box (3 words), first}
    uint2* nmeta;                   // internal node p: {last, db | kMetaLive}
    unsigned int* kids;             // 2 words per split: child ids met through the arrival words
    unsigned int* locks;            // arrival word per split, tagged per build
    unsigned int tag;
    unsigned int* counts;           // box records per first primitive (written for every position)
    uint2* items;                   // nodes whose climb continues across blocks: {id, parent split}
    unsigned int* n_items;          // zero on entry
    unsigned int item_capacity;
    const unsigned int* bounds;
    QuantFrame* frame_out;
    unsigned int leaf_size;
    const unsigned int* error;
    // double point trees (PointInsertOpF64): per sorted leaf, bit c set when the leaf box's upper
    // bound in axis c lies above its lower bound (the double point is not a float); NULL otherwise
    unsigned char* hi_bits = nullptr;
    };

struct ClimbNode
    {
    uint3 box;          // packed bins
    unsigned int l, r;  // sorted primitive range
    unsigned int id;    // internal: split index; leaf: s | kNodeLeaf
    unsigned int db;    // box records below it on its left spine
    };

__device__ __forceinline__ uint3 merge_boxes(const uint3& a, const uint3& b)
    {
    return make_uint3(__vminu2(a.x, b.x), __vminu2(a.y, b.y), __vminu2(a.z, b.z));
    }

template<class InsertOpT>
__device__ __forceinline__ ClimbNode climb_leaf(const InsertOpT& insert, const ClimbArgs& A,
                                                const QuantFrame& f, unsigned int s, bool store)
    {
    const unsigned int prim = A.primitive[s];
    const BoundingBox b = insert.get(prim);
    if (store) A.payload[s] = make_float4(b.lo.x, b.lo.y, b.lo.z, __uint_as_float(prim));
    if constexpr (std::is_same<InsertOpT, PointInsertOpF64>::value)
        {
        // the payload keeps the lower corner; these bits give back the upper one
        if (store && A.hi_bits)
            A.hi_bits[s] = (unsigned char)((b.hi.x != b.lo.x ? 1u : 0u) | (b.hi.y != b.lo.y ? 2u : 0u)
                                           | (b.hi.z != b.lo.z ? 4u : 0u));
        }
    const uint3 w = pack_node_box(f, b.lo, b.hi);
    ClimbNode n;
    n.box = w;
    n.l = s;
    n.r = s;
    n.id = s | kNodeLeaf;
    n.db = 0u;
    return n;
    }

// Form internal node p from its left child L and right child R.  LOCAL: counts go to the block's
// shared counters (index - base), else to the global ones.
template<bool LOCAL>
__device__ __forceinline__ ClimbNode form_parent(const ClimbArgs& A, unsigned int p, const ClimbNode& L,
                                                 const ClimbNode& R, unsigned int* s_count,
                                                 unsigned int base)
    {
    ClimbNode P;
    P.box = merge_boxes(L.box, R.box);
    P.l = L.l;
    P.r = R.r;
    P.id = p;
    const bool big = (P.r - P.l + 1u) > A.leaf_size;
    const bool root = (P.l == 0u && P.r == A.N - 1u);
    const bool l_internal = !(L.id & kNodeLeaf);
    const bool r_internal = !(R.id & kNodeLeaf);
    P.db = (big && l_internal) ? L.db + 1u : 0u;
    A.nbox[p] = make_uint4(P.box.x, P.box.y, P.box.z, P.l);
    A.nmeta[p] = make_uint2(P.r, P.db | (root ? kMetaLive : 0u));
    unsigned int c0 = root ? 1u : 0u;  // records counted at P.l (root, left child)
    if (big && l_internal)
        {
        A.nmeta[L.id] = make_uint2(L.r, L.db | kMetaLive);
        ++c0;
        }
    if (c0)
        {
        if (LOCAL) atomicAdd(s_count + (P.l - base), c0);
        else atomicAdd(A.counts + P.l, c0);
        }
    if (big && r_internal)
        {
        A.nmeta[R.id] = make_uint2(R.r, R.db | kMetaLive);
        if (LOCAL) atomicAdd(s_count + (R.l - base), 1u);
        else atomicAdd(A.counts + R.l, 1u);
        }
    return P;
    }

// Continue a climb from node X at split p.  Arrivals are counted in the global arrival words
// (any number of blocks, GPU-scope fences), or with BLOCK in a shared bitmap of all splits when a
// single block runs the whole stage (block-scope fences: the children's records are still in
// global memory, but every reader is in the same block).
template<bool BLOCK, class InsertOpT>
__device__ void climb_global(const InsertOpT& insert, const ClimbArgs& A, const QuantFrame& f,
                             ClimbNode X, unsigned int p, unsigned int* s_arrived)
    {
    const unsigned int N = A.N;
    const unsigned int* codes = A.codes;
    const auto delta = [codes](unsigned int i) { return adjacent_delta(__ldg(codes + i), __ldg(codes + i + 1u), i); };
    while (true)
        {
        const unsigned int side = (p == X.r) ? 0u : 1u;
        A.kids[2 * (size_t)p + side] = X.id;
        // the first child to arrive leaves; the second finds the first's node complete
        if (BLOCK)
            {
            __threadfence_block();
            const unsigned int bit = 1u << (p & 31u);
            if (!(atomicOr(s_arrived + (p >> 5), bit) & bit)) return;
            __threadfence_block();
            }
        else
            {
            __threadfence();
            if (atomicMax(A.locks + p, A.tag) != A.tag) return;
            __threadfence();
            }
        const unsigned int oid = __ldcg(A.kids + 2 * (size_t)p + (side ^ 1u));
        ClimbNode S;
        if (oid & kNodeLeaf)
            {
            S = climb_leaf(insert, A, f, oid & ~kNodeLeaf, false);
            }
        else
            {
            const uint4 nb = __ldcg(A.nbox + oid);
            const uint2 nm = __ldcg(A.nmeta + oid);
            S.box = make_uint3(nb.x, nb.y, nb.z);
            S.l = nb.w;
            S.r = nm.x;
            S.id = oid;
            S.db = nm.y & ~kMetaLive;
            }
        X = side == 0u ? form_parent<false>(A, p, X, S, nullptr, 0u) : form_parent<false>(A, p, S, X, nullptr, 0u);
        if (X.l == 0u && X.r == N - 1u) return;
        p = parent_split(X.l, X.r, N, delta);
        }
    }

template<class InsertOpT, int T>
__global__ void __launch_bounds__(T) k_climb(const InsertOpT insert, const ClimbArgs A)
    {
    __shared__ unsigned int s_codes[T + 2];  // codes[base - 1 .. base + T]
    __shared__ unsigned int s_arrive[T];     // arrivals per split of the block
    __shared__ unsigned int s_count[T];      // box records per first primitive of the block
    __shared__ uint4 s_box[2 * T];           // per split and side: child box, far end of its range
    __shared__ uint2 s_idb[2 * T];           // per split and side: child id, child db
    __shared__ unsigned char s_side[T];
    __shared__ QuantFrame s_frame;
    __shared__ unsigned int s_err;

    const unsigned int N = A.N;
    const unsigned int base = blockIdx.x * T;
    const unsigned int end = min(base + (unsigned int)T, N);
    const unsigned int t = threadIdx.x;
    if (t == 0)
        {
        const QuantFrame fr = frame_from_bounds(A.bounds);
        s_frame = fr;
        s_err = ld_status(A.error);
        if (blockIdx.x == 0) *A.frame_out = fr;
        }
    for (unsigned int k = t; k < (unsigned int)T + 2u; k += T)
        {
        const long long i = (long long)base - 1 + k;
        s_codes[k] = (i >= 0 && i < (long long)N) ? A.codes[i] : 0u;
        }
    s_arrive[t] = 0u;
    s_count[t] = 0u;
    __syncthreads();
    if (s_err != 0u) return;
    const QuantFrame f = s_frame;
    const auto delta = [&](unsigned int i) { return adjacent_delta(s_codes[i - base + 1u], s_codes[i - base + 2u], i); };

    // local phase
    const unsigned int s = base + t;
    bool boundary = false;
    unsigned int gp = 0u;
    ClimbNode X;
    if (s < end)
        {
        X = climb_leaf(insert, A, f, s, true);
        while (!(X.l == 0u && X.r == N - 1u))
            {
            const unsigned int p = parent_split(X.l, X.r, N, delta);
            if (p < base || p + 1u >= end)
                {
                boundary = true;
                gp = p;
                break;
                }
            const unsigned int side = (p == X.r) ? 0u : 1u;
            const unsigned int j = p - base;
            s_box[2 * j + side] = make_uint4(X.box.x, X.box.y, X.box.z, side == 0u ? X.l : X.r);
            s_idb[2 * j + side] = make_uint2(X.id, X.db);
            s_side[j] = (unsigned char)side;
            __threadfence_block();
            if (atomicAdd(s_arrive + j, 1u) == 0u) break;
            __threadfence_block();
            const uint4 ob = s_box[2 * j + (side ^ 1u)];
            const uint2 oi = s_idb[2 * j + (side ^ 1u)];
            ClimbNode S;
            S.box = make_uint3(ob.x, ob.y, ob.z);
            S.id = oi.x;
            S.db = oi.y;
            if (side == 0u)
                {
                S.l = p + 1u;
                S.r = ob.w;
                X = form_parent<true>(A, p, X, S, s_count, base);
                }
            else
                {
                S.l = ob.w;
                S.r = p;
                X = form_parent<true>(A, p, S, X, s_count, base);
                }
            }
        }
    __syncthreads();
    // every position of the block is written here (k_climb_global adds to them afterwards)
    if (s < end) A.counts[s] = s_count[t];

    // the climb continues across blocks (k_climb_global) from the splits of this block that only
    // one child reached and from the nodes whose parent split is on the block's edge; the block's
    // items take one range of the list (one global atomic per block; their order does not matter)
    const bool half = t + 1u < end - base && s_arrive[t] == 1u;
    const unsigned int mine = (half ? 1u : 0u) + (boundary ? 1u : 0u);
    __shared__ unsigned int s_items, s_items_base;
    if (t == 0) s_items = 0u;
    __syncthreads();
    const unsigned int local = mine ? atomicAdd(&s_items, mine) : 0u;
    __syncthreads();
    if (t == 0) s_items_base = s_items ? atomicAdd(A.n_items, s_items) : 0u;
    __syncthreads();
    unsigned int k = s_items_base + local;
    if (half)
        {
        if (k < A.item_capacity) A.items[k] = make_uint2(s_idb[2 * t + s_side[t]].x, base + t);
        ++k;
        }
    if (boundary && k < A.item_capacity) A.items[k] = make_uint2(X.id, gp);
    }

// Second stage of the climb: one thread per pending node, arrival words in global memory.
template<class InsertOpT>
__device__ __forceinline__ ClimbNode climb_item(const InsertOpT& insert, const ClimbArgs& A, const QuantFrame& f,
                                                const uint2& it)
    {
    ClimbNode X;
    if (it.x & kNodeLeaf)
        {
        X = climb_leaf(insert, A, f, it.x & ~kNodeLeaf, false);
        }
    else
        {
        const uint4 nb = A.nbox[it.x];
        const uint2 nm = A.nmeta[it.x];
        X.box = make_uint3(nb.x, nb.y, nb.z);
        X.l = nb.w;
        X.r = nm.x;
        X.id = it.x;
        X.db = nm.y & ~kMetaLive;
        }
    return X;
    }

template<class InsertOpT>
__global__ void __launch_bounds__(256) k_climb_global(const InsertOpT insert, const ClimbArgs A)
    {
    __shared__ QuantFrame s_frame;
    __shared__ unsigned int s_err;
    __shared__ unsigned int s_n;
    if (threadIdx.x == 0)
        {
        s_frame = frame_from_bounds(A.bounds);
        s_err = ld_status(A.error);
        s_n = min(*A.n_items, A.item_capacity);
        }
    __syncthreads();
    if (s_err != 0u) return;
    const QuantFrame f = s_frame;
    const unsigned int n = s_n;
    for (unsigned int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        {
        const uint2 it = A.items[k];
        climb_global<false>(insert, A, f, climb_item(insert, A, f, it), it.y, nullptr);
        }
    }

// The same stage in one block for trees of at most kClimbOneBlockMaxN points: the arrivals are a
// shared bitmap over the splits, so a level of the climb costs a shared atomic and block-scope
// fences instead of a global atomic and two GPU-scope fences.  Whole build: 32,768 points 148 ->
// 125 us, 65,536 points 160 -> 139 us; at 131,072 points one block is slower (198 against 173 us).
constexpr unsigned int kClimbOneBlockMaxN = 1u << 16;
constexpr unsigned int kClimbOneBlockThreads = 1024;

template<class InsertOpT>
__global__ void __launch_bounds__(kClimbOneBlockThreads) k_climb_global_block(const InsertOpT insert, const ClimbArgs A)
    {
    __shared__ unsigned int s_arrived[kClimbOneBlockMaxN / 32];
    __shared__ QuantFrame s_frame;
    __shared__ unsigned int s_err;
    __shared__ unsigned int s_n;
    if (threadIdx.x == 0)
        {
        s_frame = frame_from_bounds(A.bounds);
        s_err = ld_status(A.error);
        s_n = min(*A.n_items, A.item_capacity);
        }
    const unsigned int words = min((A.N + 31u) / 32u, kClimbOneBlockMaxN / 32u);
    for (unsigned int i = threadIdx.x; i < words; i += blockDim.x) s_arrived[i] = 0u;
    __syncthreads();
    if (s_err != 0u || A.N > kClimbOneBlockMaxN) return;
    const QuantFrame f = s_frame;
    const unsigned int n = s_n;
    for (unsigned int k = threadIdx.x; k < n; k += blockDim.x)
        {
        const uint2 it = A.items[k];
        climb_global<true>(insert, A, f, climb_item(insert, A, f, it), it.y, s_arrived);
        }
    }

// ---------------------------------------------------------------------------------------------
// Records in depth-first pre-order.  pre[k] = box records whose first primitive is below k.  Box
// record of node [first, last] with db box records below it on its left spine: slot
// pre[first + 1] - 1 - db + first, skip pre[last + 1] + last + 1.  Point record of sorted leaf s:
// slot pre[s + 1] + s, holding the exact position and kLeafFlag | s.
// ---------------------------------------------------------------------------------------------
struct EmitArgs
    {
    unsigned int N;
    const float4* payload;
    const uint4* nbox;
    const uint2* nmeta;
    const unsigned int* pre;
    uint4* nodes;
    unsigned int node_capacity;
    const unsigned int* error;
    };

static __global__ void __launch_bounds__(256) k_emit(const EmitArgs a)
    {
    __shared__ unsigned int s_err;
    if (threadIdx.x == 0) s_err = ld_status(a.error);
    __syncthreads();
    const unsigned int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.N || s_err != 0u) return;
    const float4 pl = a.payload[k];
    const unsigned int ps = a.pre[k + 1] + k;
    if (ps < a.node_capacity)
        a.nodes[ps] = make_uint4(__float_as_uint(pl.x), __float_as_uint(pl.y), __float_as_uint(pl.z),
                                 kLeafFlag | k);
    if (k + 1u < a.N)
        {
        const uint2 m = a.nmeta[k];
        if (m.y & kMetaLive)
            {
            const uint4 b = a.nbox[k];
            const unsigned int first = b.w;
            const unsigned int last = m.x;
            const unsigned int db = m.y & ~kMetaLive;
            const unsigned int slot = a.pre[first + 1] - 1u - db + first;
            const unsigned int skip = a.pre[last + 1] + last + 1u;
            if (slot < a.node_capacity) a.nodes[slot] = make_uint4(b.x, b.y, b.z, skip);
            }
        }
    }

// ---------------------------------------------------------------------------------------------
// Reference-layout float boxes (the reference's lbvh_bubble_aabbs,
// include/neighbor/kernels/LBVH.cuh:270-327): leaves at N-1+s, internal nodes by bottom-up
// bubbling over the Karras parent/child arrays with one arrival word per node.
// ---------------------------------------------------------------------------------------------
struct RefBubbleArgs
    {
    unsigned int N;
    const int* parent;
    const int* left;
    const int* right;
    float3* lo;
    float3* hi;
    unsigned int* locks;
    unsigned int tag;
    const unsigned int* error;
    };

// Leaf boxes of a point tree: the sorted payload.
struct PayloadLeafBox
    {
    const float4* payload;
    __device__ __forceinline__ BoundingBox operator()(unsigned int s) const
        {
        const float4 p = payload[s];
        const float3 x = make_float3(p.x, p.y, p.z);
        return BoundingBox(x, x);
        }
    };

// The next float above x (x finite, or -inf).
__device__ __forceinline__ float next_float_up(float x)
    {
    const unsigned int u = __float_as_uint(x);
    if (u == 0x80000000u) return __uint_as_float(1u);   // -0: the smallest positive subnormal
    return __uint_as_float((u & 0x80000000u) ? u - 1u : u + 1u);
    }

// Leaf boxes of a double point tree: the payload's lower corner (the point rounded down to FP32)
// and the upper corner it implies.  The point rounded up is the lower corner where the point is a
// float, and the next float above it where it is not (hi_bits), so the box is the one
// BoundingBox(double3, double3) gave at the build.
struct PayloadLeafBoxF64
    {
    const float4* payload;
    const unsigned char* hi_bits;
    __device__ __forceinline__ BoundingBox operator()(unsigned int s) const
        {
        const float4 p = payload[s];
        const unsigned int bits = hi_bits[s];
        const float3 lo = make_float3(p.x, p.y, p.z);
        const float3 hi = make_float3((bits & 1u) ? next_float_up(p.x) : p.x, (bits & 2u) ? next_float_up(p.y) : p.y,
                                      (bits & 4u) ? next_float_up(p.z) : p.z);
        return BoundingBox(lo, hi);
        }
    };

// Leaf boxes from the insert op.
template<class InsertOpT>
struct InsertLeafBox
    {
    InsertOpT insert;
    const unsigned int* primitive;
    __device__ __forceinline__ BoundingBox operator()(unsigned int s) const { return insert.get(primitive[s]); }
    };

__device__ __forceinline__ float3 ld_cg_float3(const float3* p)
    {
    const float* f = reinterpret_cast<const float*>(p);
    return make_float3(__ldcg(f), __ldcg(f + 1), __ldcg(f + 2));
    }

template<class LeafBoxT>
__global__ void k_ref_bubble(const LeafBoxT leaf_box, const RefBubbleArgs a)
    {
    __shared__ unsigned int s_err;
    if (threadIdx.x == 0) s_err = ld_status(a.error);
    __syncthreads();
    const unsigned int s = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned int N = a.N;
    if (s >= N || s_err != 0u) return;
    const BoundingBox b = leaf_box(s);
    const int leaf = (int)(N - 1 + s);
    a.lo[leaf] = b.lo;
    a.hi[leaf] = b.hi;
    int cur = (N == 1) ? LBVHSentinel : a.parent[leaf];
    __threadfence();
    int last = leaf;
    float3 blo = b.lo;
    float3 bhi = b.hi;
    while (cur != LBVHSentinel)
        {
        if (atomicMax(a.locks + cur, a.tag) != a.tag) return;
        __threadfence();
        const int l = a.left[cur];
        const int r = a.right[cur];
        const int sib = (l == last) ? r : l;
        const float3 slo = ld_cg_float3(a.lo + sib);
        const float3 shi = ld_cg_float3(a.hi + sib);
        blo = make_float3(fminf(blo.x, slo.x), fminf(blo.y, slo.y), fminf(blo.z, slo.z));
        bhi = make_float3(fmaxf(bhi.x, shi.x), fmaxf(bhi.y, shi.y), fmaxf(bhi.z, shi.z));
        a.lo[cur] = blo;
        a.hi[cur] = bhi;
        __threadfence();
        last = cur;
        cur = a.parent[cur];
        }
    }

} // namespace gpu
} // namespace neighbor

#endif // NEIGHBOR_KERNELS_BUILD_CUH_
