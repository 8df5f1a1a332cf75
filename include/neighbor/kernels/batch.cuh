// Batched ensembles of small periodic systems in one persistent launch (sm_103a).
//
// k_batch_systems runs one block per SM; each block takes the next system from a work counter
// (systems are visited largest first) and does everything for it before taking the next:
//   1. Morton codes of its points (scene [0, L) per axis, the same codes as an LBVH build with
//      lo = 0, hi = L) and the root box by a block reduction;
//   2. a stable sort of the codes: a bitonic sort of (code << 32 | index) keys in shared memory
//      (distinct keys, so the order is the stable order of the codes);
//   3. the radix tree formed bottom-up as in k_climb, with every split's arrival counter in shared
//      memory, packed 15-bit boxes and box-record counts per first primitive;
//   4. an exclusive scan of those counts and the depth-first pre-order records;
//   5. every point's self query over the 27 periodic images of L (exact FP32 minimum-image
//      predicate, the walk of k_traverse_fast): its count and up to max_neigh neighbor ids.
// The result for each system is bit for bit that of LBVH::build + LBVHTraverser::traverseSelf on
// that system alone (rows and ids are global point indices of the batch).  A system's tree data
// lives in global workspace regions of its own, so blocks never share memory.
#ifndef NEIGHBOR_KERNELS_BATCH_CUH_
#define NEIGHBOR_KERNELS_BATCH_CUH_

#include <cfloat>

#include "build.cuh"
#include "traverse.cuh"

namespace neighbor
{
namespace gpu
{

constexpr unsigned int kBatchMaxN = 16384;  // points of one system (the sort runs in shared memory)
constexpr size_t kBatchSmemBytes = kBatchMaxN * sizeof(unsigned long long) + (kBatchMaxN / 2) * sizeof(unsigned int);

enum BatchStatus : unsigned int
    {
    kBatchTooLarge = 1u,  // a system above kBatchMaxN points was skipped
    };

struct BatchArgs
    {
    const float3* points;        // all systems: system s at [start[s], start[s + 1])
    const unsigned int* start;   // S + 1
    const float3* box;           // periodic lengths of each system (its scene is [0, L))
    const float* pad;            // exact-query radius padding of each system
    const unsigned int* order;   // the order systems are taken in
    unsigned int S;
    float rc;
    unsigned int leaf_size;
    unsigned int max_neigh;
    unsigned int* nneigh;        // per point (global index)
    unsigned int* list;          // per point: max_neigh global ids
    // workspace (point counts of the whole batch T)
    uint4* records;              // 2 T
    float4* payload;             // T
    uint4* nbox;                 // T
    uint2* nmeta;                // T
    unsigned int* kids;          // 2 T
    unsigned int* pre;           // T + S (system s at start[s] + s, N + 1 entries)
    unsigned int* next;          // work counter, zero on entry
    unsigned int* status;        // [0] BatchStatus bits, [1] largest count seen
    };

template<int BLOCK>
__device__ __forceinline__ unsigned int batch_block_exclusive_scan(unsigned int v, unsigned int* s_warp,
                                                                   unsigned int& total)
    {
    constexpr int NW = BLOCK / 32;
    const unsigned int lane = threadIdx.x & 31u;
    const unsigned int warp = threadIdx.x >> 5;
    unsigned int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
        {
        const unsigned int x = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (unsigned int)o) incl += x;
        }
    if (lane == 31u) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0)
        {
        const unsigned int w = lane < (unsigned int)NW ? s_warp[lane] : 0u;
        unsigned int wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
            {
            const unsigned int x = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= (unsigned int)o) wi += x;
            }
        if (lane < (unsigned int)NW) s_warp[lane] = wi - w;
        if (lane == 31u) s_warp[NW] = wi;
        }
    __syncthreads();
    const unsigned int r = s_warp[warp] + incl - v;
    total = s_warp[NW];
    __syncthreads();
    return r;
    }

template<int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_batch_systems(const BatchArgs a)
    {
    extern __shared__ __align__(16) unsigned char smem_batch[];
    unsigned long long* skey = reinterpret_cast<unsigned long long*>(smem_batch);
    unsigned int* sflag = reinterpret_cast<unsigned int*>(skey + kBatchMaxN);  // two 16-bit counters per word
    __shared__ unsigned int s_sys;
    __shared__ float s_red[6][BLOCK / 32];
    __shared__ QuantFrame s_frame;
    __shared__ unsigned int s_warp[BLOCK / 32 + 1];
    const unsigned int tid = threadIdx.x;
    const unsigned int lane = tid & 31u;
    const unsigned int warp = tid >> 5;

    while (true)
        {
        if (tid == 0) s_sys = atomicAdd(a.next, 1u);
        __syncthreads();
        const unsigned int k = s_sys;
        __syncthreads();  // every thread has read s_sys before the next write
        if (k >= a.S) break;
        const unsigned int sys = a.order[k];
        const unsigned int o = a.start[sys];
        const unsigned int N = a.start[sys + 1] - o;
        if (N == 0) continue;
        if (N > kBatchMaxN)
            {
            if (tid == 0) atomicOr(a.status, (unsigned int)kBatchTooLarge);
            continue;
            }
        const float3 L = a.box[sys];
        const float3 zero = make_float3(0.f, 0.f, 0.f);

        // 1. codes, keys and the root box
        unsigned int n2 = 1u;
        while (n2 < N) n2 <<= 1;
        float3 bmin = make_float3(FLT_MAX, FLT_MAX, FLT_MAX);
        float3 bmax = make_float3(-FLT_MAX, -FLT_MAX, -FLT_MAX);
        for (unsigned int i = tid; i < n2; i += BLOCK)
            {
            if (i < N)
                {
                const float3 p = a.points[o + i];
                bmin = make_float3(fminf(bmin.x, p.x), fminf(bmin.y, p.y), fminf(bmin.z, p.z));
                bmax = make_float3(fmaxf(bmax.x, p.x), fmaxf(bmax.y, p.y), fmaxf(bmax.z, p.z));
                const unsigned int code = morton_code(BoundingBox(p, p), zero, L);
                skey[i] = ((unsigned long long)code << 32) | i;
                }
            else
                {
                skey[i] = ~0ull;
                }
            }
        for (unsigned int i = tid; i < (N + 1u) / 2u; i += BLOCK) sflag[i] = 0u;
        {
        float vals[6] = {bmin.x, bmin.y, bmin.z, bmax.x, bmax.y, bmax.z};
#pragma unroll
        for (int c = 0; c < 6; ++c)
            {
            float v = vals[c];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1)
                {
                const float x = __shfl_xor_sync(0xffffffffu, v, off);
                v = c < 3 ? fminf(v, x) : fmaxf(v, x);
                }
            if (lane == 0) s_red[c][warp] = v;
            }
        }
        __syncthreads();
        if (tid == 0)
            {
            float r[6];
            for (int c = 0; c < 6; ++c)
                {
                r[c] = s_red[c][0];
                for (int w = 1; w < BLOCK / 32; ++w) r[c] = c < 3 ? fminf(r[c], s_red[c][w]) : fmaxf(r[c], s_red[c][w]);
                }
            s_frame = frame_from_box(make_float3(r[0], r[1], r[2]), make_float3(r[3], r[4], r[5]));
            }

        // 2. bitonic sort of the keys
        for (unsigned int size = 2u; size <= n2; size <<= 1)
            {
            for (unsigned int stride = size >> 1; stride > 0u; stride >>= 1)
                {
                for (unsigned int i = tid; i < n2 / 2u; i += BLOCK)
                    {
                    const unsigned int lo = 2u * i - (i & (stride - 1u));
                    const unsigned int hi = lo + stride;
                    const unsigned long long x = skey[lo];
                    const unsigned long long y = skey[hi];
                    if ((x > y) == ((lo & size) == 0u))
                        {
                        skey[lo] = y;
                        skey[hi] = x;
                        }
                    }
                __syncthreads();
                }
            }
        __syncthreads();
        const QuantFrame f = s_frame;

        // 3. payload, then the climb (every split of the system meets in this block)
        ClimbArgs A;
        A.N = N;
        A.nbox = a.nbox + o;
        A.nmeta = a.nmeta + o;
        A.counts = a.pre + o + sys;
        A.leaf_size = a.leaf_size;
        for (unsigned int s = tid; s < N; s += BLOCK)
            {
            const unsigned int prim = (unsigned int)(skey[s] & 0xffffffffull);
            const float3 p = a.points[o + prim];
            a.payload[o + s] = make_float4(p.x, p.y, p.z, __uint_as_float(prim));
            A.counts[s] = 0u;
            }
        __syncthreads();
        const auto delta = [skey](unsigned int i) {
            return adjacent_delta((unsigned int)(skey[i] >> 32), (unsigned int)(skey[i + 1u] >> 32), i);
        };
        unsigned int* kids = a.kids + 2u * o;
        for (unsigned int s = tid; s < N; s += BLOCK)
            {
            const float4 pl = a.payload[o + s];
            const float3 pp = make_float3(pl.x, pl.y, pl.z);
            ClimbNode X;
            X.box = pack_node_box(f, pp, pp);
            X.l = s;
            X.r = s;
            X.id = s | kNodeLeaf;
            X.db = 0u;
            while (!(X.l == 0u && X.r == N - 1u))
                {
                const unsigned int p = parent_split(X.l, X.r, N, delta);
                const unsigned int side = (p == X.r) ? 0u : 1u;
                kids[2u * p + side] = X.id;
                __threadfence_block();
                const unsigned int sh = 16u * (p & 1u);
                const unsigned int before = (atomicAdd(sflag + (p >> 1), 1u << sh) >> sh) & 0xffffu;
                if (before == 0u) break;  // the sibling finishes p
                __threadfence_block();
                const unsigned int oid = __ldcg(kids + 2u * p + (side ^ 1u));
                ClimbNode S;
                if (oid & kNodeLeaf)
                    {
                    const unsigned int ss = oid & ~kNodeLeaf;
                    const float4 ps = __ldcg(a.payload + o + ss);
                    const float3 q = make_float3(ps.x, ps.y, ps.z);
                    S.box = pack_node_box(f, q, q);
                    S.l = ss;
                    S.r = ss;
                    S.id = oid;
                    S.db = 0u;
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
                }
            }
        __threadfence_block();
        __syncthreads();

        // 4. exclusive scan of the box-record counts (in place: pre[0..N], pre[N] = total)
        unsigned int* pre = A.counts;
        {
        const unsigned int per = (N + BLOCK - 1u) / BLOCK;
        const unsigned int b0 = min(tid * per, N);
        const unsigned int e0 = min(b0 + per, N);
        unsigned int sum = 0u;
        for (unsigned int i = b0; i < e0; ++i) sum += __ldcg(pre + i);
        unsigned int total;
        unsigned int run = batch_block_exclusive_scan<BLOCK>(sum, s_warp, total);
        for (unsigned int i = b0; i < e0; ++i)
            {
            const unsigned int v = __ldcg(pre + i);
            pre[i] = run;
            run += v;
            }
        if (tid == 0) pre[N] = total;
        }
        __threadfence_block();
        __syncthreads();

        // 5. records in pre-order
        uint4* records = a.records + 2u * o;
        const unsigned int n_rec = __ldcg(pre + N) + N;
        for (unsigned int s = tid; s < N; s += BLOCK)
            {
            const float4 pl = __ldcg(a.payload + o + s);
            // point records hold the primitive id (local to the system): the list entries
            records[__ldcg(pre + s + 1u) + s] = make_uint4(__float_as_uint(pl.x), __float_as_uint(pl.y),
                                                          __float_as_uint(pl.z), kLeafFlag | __float_as_uint(pl.w));
            if (s + 1u < N)
                {
                const uint2 m = __ldcg(A.nmeta + s);
                if (m.y & kMetaLive)
                    {
                    const uint4 b = __ldcg(A.nbox + s);
                    const unsigned int first = b.w;
                    const unsigned int last = m.x;
                    const unsigned int db = m.y & ~kMetaLive;
                    const unsigned int slot = __ldcg(pre + first + 1u) - 1u - db + first;
                    const unsigned int skip = __ldcg(pre + last + 1u) + last + 1u;
                    if (slot < 2u * N) records[slot] = make_uint4(b.x, b.y, b.z, skip);
                    }
                }
            }
        __threadfence_block();
        __syncthreads();

        // 6. self queries over the 27 images of L
        const float rc = a.rc;
        const float rs = approx::fadd_ru(rc, a.pad[sys]);
        unsigned int largest = 0u;
        for (unsigned int q = tid; q < N; q += BLOCK)
            {
            const float4 me = __ldcg(a.payload + o + q);
            const float3 P = make_float3(me.x, me.y, me.z);
            const unsigned int row = o + __float_as_uint(me.w);
            const unsigned long long row_first = (unsigned long long)row * a.max_neigh;
            unsigned int flags = lattice_flags(L, f, P, rs);
            const bool multi = __popc(flags) > 1;
            // a query meeting the scene through its own image only needs no minimum-image wrap
            const bool plain = !multi && wrap_free(L, rs);
            const float rc2 = __fmul_rn(rc, rc);
            unsigned int count = 0u;
            while (flags)
                {
                const int bit = __ffs(flags) - 1;
                flags &= flags - 1u;
                const float3 t = PeriodicImagesOp(L).get((unsigned int)bit);
                const float3 c = make_float3(__fadd_rn(P.x, t.x), __fadd_rn(P.y, t.y), __fadd_rn(P.z, t.z));
                const float3 qlo = make_float3(approx::fsub_rd(c.x, rs), approx::fsub_rd(c.y, rs), approx::fsub_rd(c.z, rs));
                const float3 qhi = make_float3(approx::fadd_ru(c.x, rs), approx::fadd_ru(c.y, rs), approx::fadd_ru(c.z, rs));
                const uint3 qb = pack_query_box(f, qlo, qhi);
                // the walk, compiled twice: with the no-wrap predicate and with the general one
                const auto walk = [&](auto plain_tag) {
                    constexpr bool kPlain = decltype(plain_tag)::value;
                    unsigned int i = 0u;
                    while (i < n_rec)
                        {
                        const uint4 n = records[i];
                        if ((int)n.w < 0)
                            {
                            const float3 x = make_float3(__uint_as_float(n.x), __uint_as_float(n.y), __uint_as_float(n.z));
                            const bool accept = kPlain ? plain_pair(P, x, rc2)
                                                       : ((!multi || point_in_box(x, qlo, qhi)) && exact_pair(P, x, rc, L));
                            if (accept)
                                {
                                if (count < a.max_neigh) a.list[row_first + count] = o + (n.w & ~kLeafFlag);
                                ++count;
                                }
                            ++i;
                            }
                        else
                            {
                            i = node_overlaps(n, qb) ? i + 1u : max(n.w, i + 1u);
                            }
                        }
                };
                if (plain)
                    walk(std::true_type());
                else
                    walk(std::false_type());
                }
            a.nneigh[row] = count;
            largest = max(largest, count);
            }
        if (largest) atomicMax(a.status + 1, largest);
        __syncthreads();
        }
    }

} // namespace gpu
} // namespace neighbor

#endif // NEIGHBOR_KERNELS_BATCH_CUH_
