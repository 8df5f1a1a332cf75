// LBVH build kernels for sm_103a.
//
// Stages (one stream, no host synchronisation):
//   k_codes_histogram  Morton codes of every primitive -> digit histograms of all radix passes
//                      and the scene bounds (root box) in one read of the inputs.
//   k_digit_offsets    exclusive scan of each pass histogram.
//   k_onesweep         one stable LSD radix pass with decoupled look-back (Adinets & Merrill,
//                      "Onesweep", 2022); the first pass computes keys from the insert op.
//   k_gen_hierarchy    Karras 2012 hierarchy (same construction and tie-break as the reference,
//                      include/neighbor/kernels/LBVH.cuh:169-243), plus primitive ranges and
//                      the per-position count of live nodes of the collapsed tree.
//   k_scan_live        chained exclusive scan of those counts (pre-order positions).
//   k_bubble           bottom-up boxes with one atomic per internal node (as the reference's
//                      lbvh_bubble_aabbs, include/neighbor/kernels/LBVH.cuh:270-327), writing the
//                      reference-layout float boxes, the sorted leaf payload and every live
//                      16-bit pre-order node as soon as its box is final.
#ifndef NEIGHBOR_KERNELS_BUILD_CUH_
#define NEIGHBOR_KERNELS_BUILD_CUH_

#include <cfloat>

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
// Morton codes -> histograms of every pass, and the bounds of all leaf boxes.
// bounds[0..2] = max of ~ordered(lo), bounds[3..5] = max of ordered(hi); all start at zero.
// ---------------------------------------------------------------------------------------------
template<class InsertOpT, int RB>
__global__ void __launch_bounds__(256) k_codes_histogram(const InsertOpT insert, unsigned int N,
                                                         float3 scene_lo, float3 scene_ext,
                                                         unsigned int* __restrict__ hist,
                                                         unsigned int* __restrict__ bounds)
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
    for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride)
        {
        const BoundingBox b = insert.get(i);
        bmin.x = fminf(bmin.x, b.lo.x);
        bmin.y = fminf(bmin.y, b.lo.y);
        bmin.z = fminf(bmin.z, b.lo.z);
        bmax.x = fmaxf(bmax.x, b.hi.x);
        bmax.y = fmaxf(bmax.y, b.hi.y);
        bmax.z = fmaxf(bmax.z, b.hi.z);
        const unsigned int code = morton_code(b, scene_lo, scene_ext);
#pragma unroll
        for (int p = 0; p < P; ++p) atomicAdd(&s_hist[p * R + ((code >> (p * RB)) & (R - 1))], 1u);
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
__global__ void __launch_bounds__(BLOCK) k_onesweep(const InsertOpT insert, float3 scene_lo,
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
                keys[j] = morton_code(insert.get(idx), scene_lo, scene_ext);
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
// Karras hierarchy.  One thread per internal node i: direction, range end j by exponential and
// binary search, split by binary search over the longest common prefix with the index tie-break.
// Also writes range[i] = (first, last) and, for the collapsed tree (buckets of <= leaf_size
// primitives), adds 1 to live[first(child)] for both children of every node larger than
// leaf_size (the root's own +1 is set before this kernel).
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ int karras_delta(const unsigned int* __restrict__ codes, unsigned int ci,
                                            long long i, long long j, long long N)
    {
    if (j < 0 || j >= N) return -1;
    const unsigned int cj = __ldg(codes + j);
    if (ci == cj) return 32 + __clz((unsigned int)i ^ (unsigned int)j);
    return __clz(ci ^ cj);
    }

static __global__ void k_gen_hierarchy(const unsigned int* __restrict__ codes,
                                                       unsigned int N, int* __restrict__ left,
                                                       int* __restrict__ right,
                                                       int* __restrict__ parent,
                                                       uint2* __restrict__ ranges,
                                                       unsigned int* __restrict__ live,
                                                       unsigned int leaf_size,
                                                       const unsigned int* __restrict__ error)
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
    ranges[i] = make_uint2((unsigned int)first, (unsigned int)last);
    // Box records of the traversal tree: every node of more than leaf_size primitives, and every
    // bucket (2..leaf_size primitives) whose parent is larger than leaf_size.  Each adds 1 at its
    // first primitive; this node adds its children's.
    if ((unsigned long long)(last - first + 1) > leaf_size)
        {
        if (split > first) atomicAdd(live + first, 1u);
        if (last > split + 1) atomicAdd(live + split + 1, 1u);
        }
    }

// ---------------------------------------------------------------------------------------------
// Chained exclusive scan: out[i] = sum(in[0..i)), out[n] = total, *total_out = total.
// 256 threads x 16 items per tile; tiles taken in launch order; look-back on one status word.
// ---------------------------------------------------------------------------------------------
constexpr int kScanBlock = 256;
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
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        {
        v[k] = (base + k < n) ? in[base + k] : 0u;
        sum += v[k];
        }
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
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        {
        if (base + k <= n) out[base + k] = run;
        if (base + k == n && total_out) *total_out = run;
        run += v[k];
        }
    }

// ---------------------------------------------------------------------------------------------
// Root-box frame of the record bins from the bounds words.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ QuantFrame frame_from_bounds(const unsigned int* bounds)
    {
    QuantFrame f;
    f.lo = make_float3(ordered_to_float(~bounds[0]), ordered_to_float(~bounds[1]), ordered_to_float(~bounds[2]));
    f.hi = make_float3(ordered_to_float(bounds[3]), ordered_to_float(bounds[4]), ordered_to_float(bounds[5]));
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

struct BubbleArgs
    {
    unsigned int N;
    const unsigned int* primitive;
    const int* parent;
    const int* left;
    const int* right;
    const uint2* ranges;
    float3* lo;
    float3* hi;
    unsigned int* locks;
    unsigned int epoch;
    unsigned char* depth_below;
    const unsigned int* pre;  // exclusive scan of live counts, N+1 entries
    uint4* nodes;
    float4* payload;
    const unsigned int* bounds;
    QuantFrame* frame_out;
    unsigned int leaf_size;
    const unsigned int* error;
    unsigned int node_capacity;
    };

__device__ __forceinline__ float3 ld_cg_float3(const float3* p)
    {
    const float* f = reinterpret_cast<const float*>(p);
    return make_float3(__ldcg(f), __ldcg(f + 1), __ldcg(f + 2));
    }

// Pre-order slot of a box record with primitive range [first, last]: the box records that start
// before `first` (pre[first]), the point records before it (first), and the box records above it
// that start at `first` too.  db = number of box records below it on its left spine.
__device__ __forceinline__ void emit_box_record(const BubbleArgs& a, const QuantFrame& f,
                                                unsigned int first, unsigned int last,
                                                unsigned int db, float3 lo, float3 hi)
    {
    const uint3 w = pack_node_box(f, lo, hi);
    const unsigned int skip = a.pre[last + 1] + last + 1u;
    const unsigned int slot = a.pre[first + 1] - 1u - db + first;
    if (slot < a.node_capacity) a.nodes[slot] = make_uint4(w.x, w.y, w.z, skip);
    }

// Point record of sorted primitive s: exact coordinates and the primitive id.
__device__ __forceinline__ void emit_point_record(const BubbleArgs& a, unsigned int s, float3 p,
                                                  unsigned int prim)
    {
    const unsigned int slot = a.pre[s + 1] + s;
    if (slot < a.node_capacity)
        a.nodes[slot] = make_uint4(__float_as_uint(p.x), __float_as_uint(p.y), __float_as_uint(p.z),
                                   kLeafFlag | prim);
    }

template<class InsertOpT>
__global__ void k_bubble(const InsertOpT insert, const BubbleArgs a)
    {
    __shared__ QuantFrame s_frame;
    __shared__ unsigned int s_err;
    if (threadIdx.x == 0)
        {
        const QuantFrame f = frame_from_bounds(a.bounds);
        s_frame = f;
        s_err = ld_status(a.error);
        if (blockIdx.x == 0) *a.frame_out = f;
        }
    __syncthreads();
    const unsigned int s = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned int N = a.N;
    if (s >= N || s_err != 0u) return;
    const QuantFrame f = s_frame;

    const unsigned int prim = a.primitive[s];
    const BoundingBox b = insert.get(prim);
    const int leaf = (int)(N - 1 + s);
    a.lo[leaf] = b.lo;
    a.hi[leaf] = b.hi;
    a.payload[s] = make_float4(b.lo.x, b.lo.y, b.lo.z, __uint_as_float(prim));

    int cur = (N == 1) ? LBVHSentinel : a.parent[leaf];
    emit_point_record(a, s, b.lo, prim);
    __threadfence();

    int last = leaf;
    float3 blo = b.lo;
    float3 bhi = b.hi;
    while (cur != LBVHSentinel)
        {
        // The second thread to reach a node finishes it; both children are final by then.
        if (atomicMax(a.locks + cur, a.epoch) != a.epoch) return;
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
        const uint2 rg = a.ranges[cur];
        const unsigned int size = rg.y - rg.x + 1u;
        // box records below on the left spine: the left child's own count plus itself, unless the
        // left child is a single point (point records are not counted) or this node is a bucket
        unsigned int db = 0;
        if (size > a.leaf_size && (unsigned int)l < N - 1)
            db = 1u + (unsigned int)__ldcg(a.depth_below + l);
        a.depth_below[cur] = (unsigned char)db;
        const int par = a.parent[cur];
        bool live = size > a.leaf_size || par == LBVHSentinel;
        if (!live)
            {
            const uint2 pr = a.ranges[par];
            live = (pr.y - pr.x + 1u) > a.leaf_size;
            }
        if (live) emit_box_record(a, f, rg.x, rg.y, db, blo, bhi);
        __threadfence();
        last = cur;
        cur = par;
        }
    }

} // namespace gpu
} // namespace neighbor

#endif // NEIGHBOR_KERNELS_BUILD_CUH_
