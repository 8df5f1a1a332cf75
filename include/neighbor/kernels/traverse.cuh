// Traversal kernels for sm_103a.
//
// Reference-layout path (any user ops):
//   k_compress_ref10   one int4 per node {lo bins, hi bins from the top, left child or ~prim,
//                      rope}, 10 bits per axis of the root box, rounded outward; the same format
//                      and rounding as the reference's lbvh_compress_ropes
//                      (include/neighbor/kernels/LBVHTraverser.cuh:45-125), so getData() and the
//                      results of user ops with refine() == true match the reference bit for bit.
//   k_traverse_ref10   stackless rope traversal over those nodes, image bitmask against the root
//                      box first (include/neighbor/kernels/LBVHTraverser.cuh:155-252).
//
// Fast path (point trees, exact sphere queries, count / fixed-stride list output):
//   k_traverse_fast    one thread per query walks the 16-bit pre-order nodes: a miss jumps to
//                      the skip link, a hit descends to the next record, a bucket tests its
//                      sorted points against the exact FP32 minimum-image predicate.  A point is
//                      accepted only through the image whose padded query box contains it, so
//                      no pair is reported twice when buckets straddle images.
//   k_traverse_half    self queries with a symmetric image set: each query walks only the records
//                      after its own point record and a pair counts for both rows;
//                      k_half_order_rows gives each list row the reference's order.
#ifndef NEIGHBOR_KERNELS_TRAVERSE_CUH_
#define NEIGHBOR_KERNELS_TRAVERSE_CUH_

#include <type_traits>

#include "../QueryOps.h"
#include "../LBVHTraverserData.h"
#include "common.cuh"

namespace neighbor
{
namespace gpu
{

template<class TransformOpT>
__global__ void k_compress_ref10(const LBVHCompressedData ctree,
                                                        const TransformOpT transform,
                                                        const ConstLBVHData tree,
                                                        unsigned int n_internal,
                                                        unsigned int n_nodes,
                                                        const unsigned int* __restrict__ status)
    {
    __shared__ float3 s_lo, s_hi, s_binv;
    __shared__ unsigned int s_err;
    if (threadIdx.x == 0)
        {
        s_err = ld_status(status);
        const float3 lo = tree.lo[tree.root];
        const float3 hi = tree.hi[tree.root];
        float ex = approx::fsub_ru(hi.x, lo.x);
        float ey = approx::fsub_ru(hi.y, lo.y);
        float ez = approx::fsub_ru(hi.z, lo.z);
        if (ex <= 0.f) ex = 1.0f;
        if (ey <= 0.f) ey = 1.0f;
        if (ez <= 0.f) ez = 1.0f;
        s_lo = lo;
        s_hi = hi;
        // bin count per unit length rounded down: offsets are never overestimated
        s_binv = make_float3(approx::fdiv_rd(1023.f, ex), approx::fdiv_rd(1023.f, ey), approx::fdiv_rd(1023.f, ez));
        }
    __syncthreads();
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int)n_nodes || s_err != 0u) return;
    const float3 tlo = s_lo, thi = s_hi, binv = s_binv;

    // rope: the right sibling of the nearest ancestor-or-self that is a left child
    int rope = LBVHSentinel;
    int cur = idx;
    while (cur != tree.root)
        {
        const int p = tree.parent[cur];
        if (tree.left[p] == cur)
            {
            rope = tree.right[p];
            break;
            }
        cur = p;
        }

    const float3 lo = tree.lo[idx];
    const float3 hi = tree.hi[idx];
    const unsigned int lx = (unsigned int)floorf(approx::fmul_rd(approx::fsub_rd(lo.x, tlo.x), binv.x));
    const unsigned int ly = (unsigned int)floorf(approx::fmul_rd(approx::fsub_rd(lo.y, tlo.y), binv.y));
    const unsigned int lz = (unsigned int)floorf(approx::fmul_rd(approx::fsub_rd(lo.z, tlo.z), binv.z));
    const unsigned int hx = (unsigned int)floorf(approx::fmul_rd(approx::fsub_rd(thi.x, hi.x), binv.x));
    const unsigned int hy = (unsigned int)floorf(approx::fmul_rd(approx::fsub_rd(thi.y, hi.y), binv.y));
    const unsigned int hz = (unsigned int)floorf(approx::fmul_rd(approx::fsub_rd(thi.z, hi.z), binv.z));
    const int z = (idx < (int)n_internal) ? tree.left[idx]
                                          : (int)~transform(tree.primitive[idx - (int)n_internal]);
    ctree.data[idx] = make_int4((int)((lx << 20) | (ly << 10) | lz), (int)((hx << 20) | (hy << 10) | hz), z, rope);
    if (idx == 0)
        {
        *ctree.lo = tlo;
        *ctree.hi = thi;
        *ctree.bins = make_float3(approx::frcp_rd(binv.x), approx::frcp_rd(binv.y), approx::frcp_rd(binv.z));
        }
    }

template<class OutputOpT, class QueryOpT, class TranslateOpT>
__global__ void k_traverse_ref10(const OutputOpT out, const LBVHCompressedData lbvh,
                                 const QueryOpT query, const TranslateOpT images,
                                 const unsigned int* __restrict__ status)
    {
    __shared__ BoundingBox s_box;
    __shared__ float3 s_bins;
    __shared__ unsigned int s_err;
    if (threadIdx.x == 0)
        {
        s_box = BoundingBox(*lbvh.lo, *lbvh.hi);
        s_bins = *lbvh.bins;
        s_err = ld_status(status);
        }
    __syncthreads();
    const unsigned int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= query.size() || s_err != 0u) return;
    const BoundingBox tbox = s_box;
    const float3 bins = s_bins;

    const typename QueryOpT::ThreadData qdata = query.setup(idx);
    typename OutputOpT::ThreadData result = out.setup(idx, qdata);

    unsigned int flags = 0;
    const unsigned int nimg = images.size() < 32u ? images.size() : 32u;
    for (unsigned int i = 0; i < nimg; ++i)
        if (query.overlap(query.get(qdata, images.get(i)), tbox)) flags |= 1u << i;

    while (flags)
        {
        const int bit = __ffs(flags) - 1;
        flags &= flags - 1u;
        const typename QueryOpT::Volume v = query.get(qdata, images.get(bit));
        int node = lbvh.root;
        while (node != LBVHSentinel)
            {
            const int4 n = __ldg(lbvh.data + node);
            const unsigned int lo = (unsigned int)n.x;
            const unsigned int hi = (unsigned int)n.y;
            const float3 blo = make_float3(approx::fadd_rd(tbox.lo.x, approx::fmul_rd((float)((lo >> 20) & 0x3ffu), bins.x)),
                                           approx::fadd_rd(tbox.lo.y, approx::fmul_rd((float)((lo >> 10) & 0x3ffu), bins.y)),
                                           approx::fadd_rd(tbox.lo.z, approx::fmul_rd((float)(lo & 0x3ffu), bins.z)));
            const float3 bhi = make_float3(approx::fsub_ru(tbox.hi.x, approx::fmul_rd((float)((hi >> 20) & 0x3ffu), bins.x)),
                                           approx::fsub_ru(tbox.hi.y, approx::fmul_rd((float)((hi >> 10) & 0x3ffu), bins.y)),
                                           approx::fsub_ru(tbox.hi.z, approx::fmul_rd((float)(hi & 0x3ffu), bins.z)));
            node = n.w;
            if (query.overlap(v, BoundingBox(blo, bhi)))
                {
                if (n.z < 0)
                    {
                    const int prim = ~n.z;
                    if (query.refine(qdata, prim)) out.process(result, prim);
                    }
                else
                    {
                    node = n.z;
                    }
                }
            }
        }
    out.finalize(result);
    }

// Output modes of the fast kernels.
enum FastOutput : int
    {
    kFastCount = 1,
    kFastList = 2,   // fixed stride max_neigh
    kFastCSR = 3,    // per-row offset and capacity
    };

struct FastQueryArgs
    {
    const float4* spheres;    // (x,y,z,cutoff) per query; NULL => self queries
    unsigned int Q;           // number of queries
    float self_rc;            // cutoff of self queries
    int self_rows_sorted;     // self queries: 1 => row s for sorted slot s, 0 => row primitive[s]
    const float3* images;     // image list; NULL => self image only, or the lattice below
    unsigned int n_images;
    int lattice;              // 1 => the 27 periodic images of lattice_L (images ignored)
    float3 lattice_L;
    float3 box;               // periodic lengths for the minimum image (0 = open)
    float pad;                // radius padding of the traversal volume
    unsigned int* nneigh;
    unsigned int* list;
    unsigned int max_neigh;
    const unsigned long long* offsets = nullptr;  // kFastCSR: first slot of each row
    const unsigned int* caps = nullptr;           // kFastCSR: capacity of each row
    const unsigned int* subset = nullptr;         // optional: thread t runs query subset[t] (Q threads)
    unsigned long long* stats = nullptr;  // optional counters: records visited, point tests, walks
    int work_order = 0;                   // CSR fills: a block's rows go to lanes by capacity class
    };

// First slot and capacity of an output row.
template<int OUT>
__device__ __forceinline__ void row_layout(const unsigned long long* offsets, const unsigned int* caps,
                                           unsigned int max_neigh, unsigned int row,
                                           unsigned long long& first, unsigned int& cap)
    {
    if (OUT == kFastCSR)
        {
        first = offsets[row];
        cap = caps[row];
        }
    else
        {
        first = (unsigned long long)row * max_neigh;
        cap = max_neigh;
        }
    }

// Add a thread's (or a packet's) traversal counts to the optional statistics counters.
__device__ __forceinline__ void add_stats(unsigned long long* stats, unsigned long long visits,
                                          unsigned long long tests, unsigned long long walks)
    {
    if (stats)
        {
        atomicAdd(stats + 0, visits);
        atomicAdd(stats + 1, tests);
        atomicAdd(stats + 2, walks);
        }
    }

// Query of a fast traversal: centre, cutoff, output row.
struct FastQuery
    {
    float3 p;
    float rc;
    unsigned int row;
    };

__device__ __forceinline__ FastQuery load_fast_query(const FastLBVHData& tree, const FastQueryArgs& a,
                                                     unsigned int q)
    {
    FastQuery r;
    if (a.spheres)
        {
        const float4 s = a.spheres[q];
        r.p = make_float3(s.x, s.y, s.z);
        r.rc = s.w;
        r.row = q;
        }
    else
        {
        const float4 s = tree.points[q];
        r.p = make_float3(s.x, s.y, s.z);
        r.rc = a.self_rc;
        r.row = a.self_rows_sorted ? q : __float_as_uint(s.w);
        }
    return r;
    }

__device__ __forceinline__ float3 image_vector(const FastQueryArgs& a, int i)
    {
    if (a.lattice) return PeriodicImagesOp(a.lattice_L).get((unsigned int)i);
    return a.images ? a.images[i] : make_float3(0.f, 0.f, 0.f);
    }

// Which of the translations {-L, 0, +L} along one axis bring the padded query interval onto the
// root interval [lo, hi]: bit 0 for -L, bit 1 for 0, bit 2 for +L.  Same rounding as the
// general image test, so the result is the same conservative answer.
__device__ __forceinline__ unsigned int axis_images(float p, float rs, float L, float lo, float hi)
    {
    unsigned int m = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k)
        {
        const float c = __fadd_rn(p, L * (float)(k - 1));
        if (approx::fsub_rd(c, rs) <= hi && approx::fadd_ru(c, rs) >= lo) m |= 1u << k;
        }
    return m;
    }

// Lattice images (bit i = 9*(ix+1) + 3*(iy+1) + (iz+1) of the 27) whose padded query box meets
// the root box: the per-axis masks replicated into 27 bits.
__device__ __forceinline__ unsigned int lattice_flags(const float3& L, const QuantFrame& f, const float3& p, float rs)
    {
    const unsigned int mx = axis_images(p.x, rs, L.x, f.lo.x, f.hi.x);
    const unsigned int my = axis_images(p.y, rs, L.y, f.lo.y, f.hi.y);
    const unsigned int mz = axis_images(p.z, rs, L.z, f.lo.z, f.hi.z);
    const unsigned int X = ((mx & 1u) ? 0x1ffu : 0u) | ((mx & 2u) ? 0x3fe00u : 0u) | ((mx & 4u) ? 0x7fc0000u : 0u);
    const unsigned int Y = (((my & 1u) ? 0x7u : 0u) | ((my & 2u) ? 0x38u : 0u) | ((my & 4u) ? 0x1c0u : 0u)) * 0x40201u;
    const unsigned int Z = mz * 0x1249249u;
    return X & Y & Z;
    }

// Images whose padded query box meets the root box.
__device__ __forceinline__ unsigned int image_flags(const FastQueryArgs& a, const QuantFrame& f,
                                                    const float3& p, float rs)
    {
    if (a.lattice) return lattice_flags(a.lattice_L, f, p, rs);
    const unsigned int nimg = a.images ? min(a.n_images, 32u) : 1u;
    unsigned int flags = 0;
    for (unsigned int i = 0; i < nimg; ++i)
        {
        const float3 t = image_vector(a, i);
        const float3 c = make_float3(__fadd_rn(p.x, t.x), __fadd_rn(p.y, t.y), __fadd_rn(p.z, t.z));
        const bool hit = approx::fsub_rd(c.x, rs) <= f.hi.x && approx::fadd_ru(c.x, rs) >= f.lo.x
                         && approx::fsub_rd(c.y, rs) <= f.hi.y && approx::fadd_ru(c.y, rs) >= f.lo.y
                         && approx::fsub_rd(c.z, rs) <= f.hi.z && approx::fadd_ru(c.z, rs) >= f.lo.z;
        if (hit) flags |= 1u << i;
        }
    return flags;
    }

__device__ __forceinline__ bool point_in_box(const float3& x, const float3& lo, const float3& hi)
    {
    return x.x >= lo.x && x.x <= hi.x && x.y >= lo.y && x.y <= hi.y && x.z >= lo.z && x.z <= hi.z;
    }

// Work order of a block: a counting sort of the block's items (one per thread) by a work class
// in [0, 64).  Returns the item the calling thread takes -- a warp then gets items of similar work
// -- or 0xffffffff when the block has fewer items than threads.  All threads of the block call it.
constexpr unsigned int kWorkClasses = 64;
__device__ __forceinline__ unsigned int block_work_order(unsigned int item, bool valid, unsigned int cls,
                                                         unsigned int* s_class, unsigned int* s_order)
    {
    if (threadIdx.x < kWorkClasses) s_class[threadIdx.x] = 0u;
    __syncthreads();
    unsigned int rank = 0;
    if (valid) rank = atomicAdd(s_class + cls, 1u);
    const unsigned int n = __syncthreads_count(valid ? 1 : 0);
    if (threadIdx.x < 32)
        {
        // exclusive scan of the 64 class sizes, two per lane
        const unsigned int c0 = s_class[2 * threadIdx.x], c1 = s_class[2 * threadIdx.x + 1];
        unsigned int incl = c0 + c1;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
            {
            const unsigned int v = __shfl_up_sync(0xffffffffu, incl, o);
            if ((int)threadIdx.x >= o) incl += v;
            }
        const unsigned int excl = incl - c0 - c1;
        s_class[2 * threadIdx.x] = excl;
        s_class[2 * threadIdx.x + 1] = excl + c0;
        }
    __syncthreads();
    if (valid) s_order[s_class[cls] + rank] = item;
    __syncthreads();
    return threadIdx.x < n ? s_order[threadIdx.x] : 0xffffffffu;
    }

// Work class of a row capacity (or count): about four classes per octave, 0..63.
__device__ __forceinline__ unsigned int capacity_class(unsigned int c)
    {
    const unsigned int bits = __float_as_uint((float)min(c, 65535u) + 1.f);
    return min((bits >> 21) - (127u << 2), kWorkClasses - 1u);
    }

// One thread per query, stackless: a box record is tested against the query's box (hit: the next
// record, miss: the skip link); a point record inside the query's padded box goes to the exact
// predicate.  Images are walked one after the other in the same loop.  When a query visits more
// than one image, a point is found only through the image whose padded box contains it, so each
// pair is reported once.
// One query walked by one thread: the body of k_traverse_fast (and of the thread mode of
// k_traverse_subset).  Writes the row's entries (list outputs) and its count.
template<int OUT, bool STATS, class TransformOpT>
__device__ __forceinline__ void thread_walk(const FastLBVHData& tree, const FastQueryArgs& a,
                                            const TransformOpT& transform, const QuantFrame& f,
                                            unsigned int n_rec, unsigned int q, unsigned int& visits,
                                            unsigned int& tests, unsigned int& walks)
    {
    const FastQuery Q = load_fast_query(tree, a, q);
    const float rs = approx::fadd_ru(Q.rc, a.pad);
    unsigned int flags = n_rec ? image_flags(a, f, Q.p, rs) : 0u;
    // a point inside the padded box of the query's own image needs no minimum-image wrap
    const bool no_wrap = wrap_free(a.box, rs);
    const float rc2 = __fmul_rn(Q.rc, Q.rc);
    unsigned long long row_first = 0;
    unsigned int cap = 0;
    if (OUT != kFastCount) row_layout<OUT>(a.offsets, a.caps, a.max_neigh, Q.row, row_first, cap);

    unsigned int count = 0;
    while (flags)
        {
        const int bit = __ffs(flags) - 1;
        flags &= flags - 1u;
        const float3 t = image_vector(a, bit);
        const float3 c = make_float3(__fadd_rn(Q.p.x, t.x), __fadd_rn(Q.p.y, t.y), __fadd_rn(Q.p.z, t.z));
        const float3 qlo = make_float3(approx::fsub_rd(c.x, rs), approx::fsub_rd(c.y, rs), approx::fsub_rd(c.z, rs));
        const float3 qhi = make_float3(approx::fadd_ru(c.x, rs), approx::fadd_ru(c.y, rs), approx::fadd_ru(c.z, rs));
        const uint3 qb = pack_query_box(f, qlo, qhi);
        const bool plain = no_wrap && t.x == 0.f && t.y == 0.f && t.z == 0.f;
        if (STATS) ++walks;
        // the walk, compiled twice: with the no-wrap predicate and with the general one
        const auto walk = [&](auto plain_tag) {
            constexpr bool kPlain = decltype(plain_tag)::value;
            unsigned int i = 0;
            const auto step = [&]() {
                const uint4 n = __ldg(tree.nodes + i);
                if (STATS) ++visits;
                if ((int)n.w < 0)
                    {
                    const float3 x = make_float3(__uint_as_float(n.x), __uint_as_float(n.y), __uint_as_float(n.z));
                    if (point_in_box(x, qlo, qhi))
                        {
                        if (STATS) ++tests;
                        if (kPlain ? plain_pair(Q.p, x, rc2) : exact_pair(Q.p, x, Q.rc, a.box))
                            {
                            if (OUT != kFastCount && count < cap)
                                a.list[row_first + count] = transform(tree.primitive[n.w & ~kLeafFlag]);
                            ++count;
                            }
                        }
                    ++i;
                    }
                else
                    {
                    // skip links point forward in a valid tree; max() keeps a damaged one from looping
                    i = node_overlaps(n, qb) ? i + 1u : max(n.w, i + 1u);
                    }
            };
            // two records per trip of the loop (clustered 4M plain step, whose CSR fill walks the
            // whole tree: 9.34 -> 9.20 ms)
            while (i < n_rec)
                {
                step();
                if (i >= n_rec) break;
                step();
                }
        };
        if (plain)
            walk(std::true_type());
        else
            walk(std::false_type());
        }
    a.nneigh[Q.row] = count;
    }

// One thread per query, stackless: a box record is tested against the query's box (hit: the next
// record, miss: the skip link); a point record inside the query's padded box goes to the exact
// predicate.  Images are walked one after the other in the same loop.  When a query visits more
// than one image, a point is found only through the image whose padded box contains it, so each
// pair is reported once.
template<int OUT, bool STATS, class TransformOpT>
__global__ void k_traverse_fast(const FastLBVHData tree, const FastQueryArgs a,
                                const TransformOpT transform)
    {
    __shared__ QuantFrame s_frame;
    __shared__ unsigned int s_records;
    __shared__ unsigned int s_class[kWorkClasses];
    __shared__ unsigned int s_order[1024];
    if (threadIdx.x == 0)
        {
        s_frame = *tree.frame;
        // a failed build leaves no tree to walk
        s_records = ld_status(tree.status) != 0u ? 0u : *tree.n_boxes + tree.N;
        }
    unsigned int tq = blockIdx.x * blockDim.x + threadIdx.x;
    if (OUT == kFastCSR && a.work_order)
        {
        // rows with capacities of similar size (their predicted or counted lengths) share warps
        const bool valid = tq < a.Q;
        unsigned int cls = 0;
        if (valid)
            {
            const unsigned int row = a.spheres || a.self_rows_sorted ? tq : __float_as_uint(tree.points[tq].w);
            cls = capacity_class(a.caps[row]);
            }
        tq = block_work_order(tq, valid, cls, s_class, s_order);
        if (tq == 0xffffffffu) return;
        }
    else
        {
        __syncthreads();
        if (tq >= a.Q) return;
        }
    const unsigned int q = a.subset ? a.subset[tq] : tq;
    const QuantFrame f = s_frame;
    unsigned int visits = 0, tests = 0, walks = 0;
    thread_walk<OUT, STATS>(tree, a, transform, f, s_records, q, visits, tests, walks);
    if (STATS) add_stats(a.stats, visits, tests, walks);
    }

// ---------------------------------------------------------------------------------------------
// Double-precision queries (ExactSphereQueryOpF64 on a tree of PointInsertOpF64): the walk of
// k_traverse_fast over the same records, with every pair decided as the double predicate decides
// it and double arithmetic only where FP32 cannot decide.
//
// Records.  A point record holds the leaf box's lower corner, the double point rounded down to
// FP32.  The query box of an image is the double box (centre + image, radius cutoff + pad, the
// op's own rounding) rounded outward to FP32.  A point inside the double box has its rounded-down
// corner inside the FP32 box (the corner is the largest float not above the point, and both box
// faces are floats on the right side of the point), so the record test never drops a pair.  Image
// boxes are separated by box lengths above 2 (cutoff + pad), so each pair is found through one
// image.  Images are chosen in FP32 with a margin (a superset: an extra image finds nothing).
//
// Pairs.  d = minimum image of (record - query) in FP32 differs from the double d of the exact
// predicate by at most 4 ulp(M) per component, M bounding every coordinate and box length: the
// query rounded to nearest (1/2 ulp), the record rounded down (1 ulp), the difference and the wrap
// each rounded (1/2 ulp(2M) = 1 ulp(M) each), the box length rounded (1/2 ulp).  A wrap that
// FP32 and double decide differently leaves |d| near L/2 > cutoff in both.  So |d|_FP32 and |d|
// differ by less than 7 ulp(M), and the squares and sums of FP32 add a relative 3 2^-24.  With
// eps = 16 ulp(M) + 8 2^-24 rc + 2 ulp(rc): |d|^2_FP32 below (rc - eps)^2 is a pair for the double
// predicate, above (rc + eps)^2 is not, and only the band between takes exact_pair_f64 on the
// double positions (read through the reported id, as the op's refine() reads them).
// Rows hold the same entries in the same order as the reference-layout walk of the same op: both
// visit the images in bit order and the points of a subtree in sorted order.
// ---------------------------------------------------------------------------------------------
struct FastQueryArgsF64
    {
    const double4_16a* spheres;  // (x, y, z, cutoff) per query; NULL: self queries (below)
    unsigned int Q;
    const double3* points;       // double positions, indexed by the reported id (self queries: by
                                 // primitive id)
    double3 box;                 // periodic lengths for the minimum image (0 = open)
    float pad;
    const float3* images;        // image list; NULL => self image only, or the lattice below
    unsigned int n_images;
    int lattice;
    float3 lattice_L;
    unsigned int* nneigh;
    unsigned int* list;
    unsigned int max_neigh;
    const unsigned long long* offsets = nullptr;  // kFastCSR
    const unsigned int* caps = nullptr;           // kFastCSR
    // Self queries (spheres == NULL): query s is sorted position s with centre
    // points[primitive[s]] and cutoff self_rc; its row is s (self_rows_sorted) or primitive[s].
    double self_rc = 0.0;
    int self_rows_sorted = 1;
    // Optional: only the queries subset[0 .. *subset_count) (the count read on the device), by a
    // grid-stride loop.
    const unsigned int* subset = nullptr;
    const unsigned int* subset_count = nullptr;
    };

__device__ __forceinline__ float3 image_vector_f64(const FastQueryArgsF64& a, int i)
    {
    if (a.lattice) return PeriodicImagesOp(a.lattice_L).get((unsigned int)i);
    return a.images ? a.images[i] : make_float3(0.f, 0.f, 0.f);
    }

// ulp of a non-negative finite float (the spacing of floats at x's binade; 0 below the normals).
__device__ __forceinline__ float ulp_of(float x)
    {
    return __int_as_float(__float_as_int(x) & 0x7f800000) * 1.1920929e-7f;   // 2^e * 2^-23
    }

__device__ __forceinline__ float wrap_f32(float d, float L)
    {
    if (L > 0.f)
        {
        const float h = __fmul_rn(0.5f, L);
        if (d >= h)
            d = __fsub_rn(d, L);
        else if (d < -h)
            d = __fadd_rn(d, L);
        }
    return d;
    }

// FP32 screen of one double query (centre P, cutoff rc, padded radius rs): the query rounded to
// nearest, the box lengths in FP32, the squared FP32 distances below which a pair is certain (in2)
// and above which it is excluded (out2), and the padded radius that chooses images in FP32.
struct ScreenF64
    {
    float3 Pf;
    float3 Lf;
    float in2;
    float out2;
    float rsf;
    };

__device__ __forceinline__ ScreenF64 screen_f64(const QuantFrame& f, const double3& P, double rc, double rs,
                                                const double3& box)
    {
    ScreenF64 S;
    S.Pf = make_float3(__double2float_rn(P.x), __double2float_rn(P.y), __double2float_rn(P.z));
    S.Lf = make_float3(__double2float_rn(box.x), __double2float_rn(box.y), __double2float_rn(box.z));
    // M bounds every coordinate of the query, the scene and the box lengths (and the images)
    float M = fmaxf(fmaxf(fabsf(S.Pf.x), fabsf(S.Pf.y)), fabsf(S.Pf.z));
    M = fmaxf(M, fmaxf(fmaxf(fabsf(f.lo.x), fabsf(f.lo.y)), fabsf(f.lo.z)));
    M = fmaxf(M, fmaxf(fmaxf(fabsf(f.hi.x), fabsf(f.hi.y)), fabsf(f.hi.z)));
    M = fmaxf(M, fmaxf(fmaxf(S.Lf.x, S.Lf.y), S.Lf.z));
    const float uM = ulp_of(fmaxf(M, 1.17549435e-38f));
    const float rcf = __double2float_ru(rc);
    const float eps = 16.f * uM + 4.7683716e-7f * rcf + 2.f * ulp_of(rcf);
    const float lo_r = approx::fsub_rd(__double2float_rd(rc), eps);
    S.in2 = lo_r > 0.f ? approx::fmul_rd(lo_r, lo_r) : -1.f;   // below: a pair
    const float hi_r = approx::fadd_ru(rcf, eps);
    S.out2 = approx::fmul_ru(hi_r, hi_r);                        // above: not a pair
    // images whose box may meet the scene, in FP32 with a margin for the query's rounding
    S.rsf = approx::fadd_ru(__double2float_ru(rs), 2.f * uM);
    return S;
    }

// Minimum-image squared distance of a record from the screened query, in FP32.  WRAP false: the
// plain difference, for a query that meets the scene through one image with a padded radius below
// 0.45 box lengths (wrap_free): a point that only the wrap brings within the cutoff would lie in
// another image's box, which would then meet the scene too.  The screen then still decides only
// what the double predicate decides the same way: below in2 the plain distance bounds the
// minimum-image one, and above out2 no image but the query's own can hold a pair.
template<bool WRAP = true>
__device__ __forceinline__ float screen_dist2(const ScreenF64& S, const float3& x)
    {
    float dx = __fsub_rn(x.x, S.Pf.x), dy = __fsub_rn(x.y, S.Pf.y), dz = __fsub_rn(x.z, S.Pf.z);
    if (WRAP)
        {
        dx = wrap_f32(dx, S.Lf.x);
        dy = wrap_f32(dy, S.Lf.y);
        dz = wrap_f32(dz, S.Lf.z);
        }
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    }

// Images of a double query whose FP32 box (radius rsf) may meet the root box: the lattice's, or
// those of the image list (the self image when there is none).
__device__ __forceinline__ unsigned int image_flags_f64(const FastQueryArgsF64& a, const QuantFrame& f,
                                                        const float3& Pf, float rsf)
    {
    if (a.lattice) return lattice_flags(a.lattice_L, f, Pf, rsf);
    const unsigned int nimg = a.images ? min(a.n_images, 32u) : 1u;
    unsigned int flags = 0u;
    for (unsigned int k = 0; k < nimg; ++k)
        {
        const float3 t = image_vector_f64(a, (int)k);
        const float3 c = make_float3(__fadd_rn(Pf.x, t.x), __fadd_rn(Pf.y, t.y), __fadd_rn(Pf.z, t.z));
        const float3 lo = make_float3(approx::fsub_rd(c.x, rsf), approx::fsub_rd(c.y, rsf), approx::fsub_rd(c.z, rsf));
        const float3 hi = make_float3(approx::fadd_ru(c.x, rsf), approx::fadd_ru(c.y, rsf), approx::fadd_ru(c.z, rsf));
        if (lo.x <= f.hi.x && hi.x >= f.lo.x && lo.y <= f.hi.y && hi.y >= f.lo.y && lo.z <= f.hi.z && hi.z >= f.lo.z)
            flags |= 1u << k;
        }
    return flags;
    }

// The FP32 query box of image t of a double query: from the query rounded to nearest (S.Pf) and
// the padded radius of the image choice (S.rsf, at least rs + 2 ulp(M)), each step rounded away
// from the box's centre.  Pf lies within ulp(M)/2 of the double centre, so the box holds the exact
// box [P + t - rs, P + t + rs], and a point inside that has its rounded-down record (a float not
// above the point) inside this one.  It is a few ulps wider than the exact box rounded outward,
// which only adds candidates that the predicate turns down, and it keeps the double pipe (about
// 1/64 of the FP32 rate on this GPU) out of the per-image work.
__device__ __forceinline__ void query_box_f32(const ScreenF64& S, const float3& t, float3& qlo, float3& qhi)
    {
    qlo = make_float3(approx::fsub_rd(approx::fadd_rd(S.Pf.x, t.x), S.rsf),
                      approx::fsub_rd(approx::fadd_rd(S.Pf.y, t.y), S.rsf),
                      approx::fsub_rd(approx::fadd_rd(S.Pf.z, t.z), S.rsf));
    qhi = make_float3(approx::fadd_ru(approx::fadd_ru(S.Pf.x, t.x), S.rsf),
                      approx::fadd_ru(approx::fadd_ru(S.Pf.y, t.y), S.rsf),
                      approx::fadd_ru(approx::fadd_ru(S.Pf.z, t.z), S.rsf));
    }

// One double query walked by one thread over the whole tree (images in bit order): the body of
// k_traverse_fast_f64.  Writes the row's entries (list outputs) and its count.
template<int OUT, class TransformOpT>
__device__ __forceinline__ void thread_walk_f64(const FastLBVHData& tree, const FastQueryArgsF64& a,
                                                const TransformOpT& transform, const QuantFrame& f,
                                                unsigned int n_rec, unsigned int q)
    {
    const bool self = a.spheres == nullptr;
    double3 P;
    double rq;
    unsigned int row;
    if (self)
        {
        const unsigned int prim = tree.primitive[q];
        P = a.points[prim];
        rq = a.self_rc;
        row = a.self_rows_sorted ? q : prim;
        }
    else
        {
        const double4_16a s = a.spheres[q];
        P = make_double3(s.x, s.y, s.z);
        rq = s.w;
        row = q;
        }
    const double rs = __dadd_ru(rq, (double)a.pad);
    const ScreenF64 S = screen_f64(f, P, rq, rs, a.box);
    unsigned int flags = n_rec ? image_flags_f64(a, f, S.Pf, S.rsf) : 0u;
    unsigned long long row_first = 0;
    unsigned int cap = 0;
    if (OUT != kFastCount) row_layout<OUT>(a.offsets, a.caps, a.max_neigh, row, row_first, cap);
    // no distance inside the padded box of the query's own image wraps: that image's walk
    // screens without the minimum-image wrap (the same numbers for every point it tests)
    const bool own_plain = wrap_free(S.Lf, S.rsf);
    unsigned int count = 0;
    while (flags)
        {
        const int bit = __ffs(flags) - 1;
        flags &= flags - 1u;
        const float3 t = image_vector_f64(a, bit);
        float3 qlo, qhi;
        query_box_f32(S, t, qlo, qhi);
        const uint3 qb = pack_query_box(f, qlo, qhi);
        // the walk, compiled twice: with the plain screen and with the minimum-image one
        const auto walk = [&](auto plain_tag) {
            constexpr bool kPlain = decltype(plain_tag)::value;
            unsigned int i = 0;
            const auto step = [&]() {
                const uint4 n = __ldg(tree.nodes + i);
                if ((int)n.w < 0)
                    {
                    const float3 x = make_float3(__uint_as_float(n.x), __uint_as_float(n.y), __uint_as_float(n.z));
                    if (point_in_box(x, qlo, qhi))
                        {
                        const float d2 = screen_dist2<!kPlain>(S, x);
                        if (d2 <= S.out2)
                            {
                            const unsigned int prim = tree.primitive[n.w & ~kLeafFlag];
                            const unsigned int id = transform(prim);
                            if (d2 < S.in2 || exact_pair_f64(P, a.points[self ? prim : id], rq, a.box))
                                {
                                if (OUT != kFastCount && count < cap) a.list[row_first + count] = id;
                                ++count;
                                }
                            }
                        }
                    ++i;
                    }
                else
                    {
                    i = node_overlaps(n, qb) ? i + 1u : max(n.w, i + 1u);
                    }
            };
            // two records per trip of the loop (16M double count, whole tree: 7.26 -> 7.03 ms)
            while (i < n_rec)
                {
                step();
                if (i >= n_rec) break;
                step();
                }
        };
        if (own_plain && t.x == 0.f && t.y == 0.f && t.z == 0.f)
            walk(std::true_type());
        else
            walk(std::false_type());
        }
    a.nneigh[row] = count;
    }

// One thread per query (or per listed query, grid-stride, when a.subset is given).
template<int OUT, class TransformOpT>
__global__ void k_traverse_fast_f64(const FastLBVHData tree, const FastQueryArgsF64 a, const TransformOpT transform)
    {
    __shared__ QuantFrame s_frame;
    __shared__ unsigned int s_records;
    __shared__ unsigned int s_n;
    if (threadIdx.x == 0)
        {
        s_frame = *tree.frame;
        s_records = ld_status(tree.status) != 0u ? 0u : *tree.n_boxes + tree.N;
        s_n = a.subset_count ? *a.subset_count : a.Q;
        }
    __syncthreads();
    const QuantFrame f = s_frame;
    const unsigned int n_rec = s_records;
    const unsigned int n = s_n;
    if (a.subset)
        {
        for (unsigned int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
            thread_walk_f64<OUT>(tree, a, transform, f, n_rec, a.subset[t]);
        return;
        }
    const unsigned int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) thread_walk_f64<OUT>(tree, a, transform, f, n_rec, q);
    }

// ---------------------------------------------------------------------------------------------
// One warp per query (long rows, few queries).  The warp takes the records in chunks of 32 in
// pre-order: lane k tests record i + k.  A box that misses covers the records up to its skip link,
// so a record is live when no earlier live-or-not missed box of the chunk covers it (a prefix
// maximum of the missed boxes' skip links over the lanes); live points go to the exact predicate,
// and the accepted ones are written in record order (ballot + rank), which is the order of the
// one-thread walk.  The next chunk starts past the chunk and past every missed subtree (the last
// lane's prefix maximum).  Many lanes test records that a one-thread walk skips, but the walk's
// latency is about 32 times shorter, which is what a handful of long rows needs.
// ---------------------------------------------------------------------------------------------
constexpr unsigned int kWarpWalkBlock = 256;
// Up to this many queries, a traversal walks one group of lanes per query (LBVHTraverser picks the
// group width): one thread per query would leave most of the GPU's SMs idle.
constexpr unsigned int kWarpWalkMaxQueries = 32768;
// self traversals of at most this many points walk the whole tree (no symmetric walk); above it
// the symmetric walk with the pair exchange, whatever the lane-group limit
constexpr unsigned int kSymmetricMinPoints = 4096;

// G < 32: the same walk by groups of G lanes, 32 / G queries per warp (chunks of G records).  A
// group's shuffles and ballots name only its own lanes, so the groups of a warp may be at
// different records or images.
// One query walked by a group of G lanes: the body of k_traverse_warp (and of the group mode of
// k_traverse_subset).  Every lane of the group calls it with the same q; lane 0 writes the count.
template<int OUT, class TransformOpT, int G>
__device__ __forceinline__ void group_walk(const FastLBVHData& tree, const FastQueryArgs& a,
                                           const TransformOpT& transform, const QuantFrame& f,
                                           unsigned int n_rec, unsigned int q, unsigned int lane,
                                           unsigned int gmask, unsigned int lt)
    {
    const FastQuery Q = load_fast_query(tree, a, q);
    const float rs = approx::fadd_ru(Q.rc, a.pad);
    unsigned int flags = n_rec ? image_flags(a, f, Q.p, rs) : 0u;
    const bool no_wrap = wrap_free(a.box, rs);
    const float rc2 = __fmul_rn(Q.rc, Q.rc);
    unsigned long long row_first = 0;
    unsigned int cap = 0;
    if (OUT != kFastCount) row_layout<OUT>(a.offsets, a.caps, a.max_neigh, Q.row, row_first, cap);

    unsigned int count = 0;   // group-uniform
    while (flags)
        {
        const int bit = __ffs(flags) - 1;
        flags &= flags - 1u;
        const float3 t = image_vector(a, bit);
        const float3 c = make_float3(__fadd_rn(Q.p.x, t.x), __fadd_rn(Q.p.y, t.y), __fadd_rn(Q.p.z, t.z));
        const float3 qlo = make_float3(approx::fsub_rd(c.x, rs), approx::fsub_rd(c.y, rs), approx::fsub_rd(c.z, rs));
        const float3 qhi = make_float3(approx::fadd_ru(c.x, rs), approx::fadd_ru(c.y, rs), approx::fadd_ru(c.z, rs));
        const uint3 qb = pack_query_box(f, qlo, qhi);
        const bool plain = no_wrap && t.x == 0.f && t.y == 0.f && t.z == 0.f;
        unsigned int i = 0;
        while (i < n_rec)   // group-uniform
            {
            const unsigned int k = i + lane;
            const bool valid = k < n_rec;
            const uint4 n = valid ? __ldg(tree.nodes + k) : make_uint4(0u, 0u, 0u, 0u);
            const bool is_point = valid && (int)n.w < 0;
            const bool miss = valid && !is_point && !node_overlaps(n, qb);
            const unsigned int kill = miss ? max(n.w, k + 1u) : 0u;   // [k + 1, kill) lies under it
            unsigned int cover = kill;   // inclusive prefix maximum over the group's lanes
#pragma unroll
            for (int o = 1; o < G; o <<= 1)
                {
                const unsigned int v = __shfl_up_sync(gmask, cover, o, G);
                if ((int)lane >= o) cover = max(cover, v);
                }
            const unsigned int before = __shfl_up_sync(gmask, cover, 1, G);
            const bool live = valid && (lane == 0u || before <= k);
            bool accept = false;
            if (live && is_point)
                {
                const float3 x = make_float3(__uint_as_float(n.x), __uint_as_float(n.y), __uint_as_float(n.z));
                if (point_in_box(x, qlo, qhi)) accept = plain ? plain_pair(Q.p, x, rc2) : exact_pair(Q.p, x, Q.rc, a.box);
                }
            const unsigned int hits = __ballot_sync(gmask, accept) & gmask;
            if (OUT != kFastCount && accept)
                {
                const unsigned int pos = count + __popc(hits & lt);
                if (pos < cap) a.list[row_first + pos] = transform(tree.primitive[n.w & ~kLeafFlag]);
                }
            count += __popc(hits);
            // past the chunk and past every missed subtree: the last lane's prefix maximum (a
            // missed box that is not live lies under an earlier one, and so does its skip link)
            const unsigned int next = __shfl_sync(gmask, cover, G - 1, G);
            i = max(i + (unsigned int)G, next);
            }
        }
    if (lane == 0u) a.nneigh[Q.row] = count;
    }

// G < 32: the same walk by groups of G lanes, 32 / G queries per warp (chunks of G records).  A
// group's shuffles and ballots name only its own lanes, so the groups of a warp may be at
// different records or images.
template<int OUT, class TransformOpT, int G = 32>
__global__ void __launch_bounds__(kWarpWalkBlock) k_traverse_warp(const FastLBVHData tree, const FastQueryArgs a,
                                                                  const TransformOpT transform)
    {
    static_assert(G == 4 || G == 8 || G == 16 || G == 32, "lane groups of 4, 8, 16 or 32");
    __shared__ QuantFrame s_frame;
    __shared__ unsigned int s_records;
    if (threadIdx.x == 0)
        {
        s_frame = *tree.frame;
        s_records = ld_status(tree.status) != 0u ? 0u : *tree.n_boxes + tree.N;
        }
    __syncthreads();
    const unsigned int lane = threadIdx.x & (unsigned int)(G - 1);   // lane within the group
    const unsigned int gmask = G == 32 ? 0xffffffffu
                                       : (((1u << (G & 31)) - 1u) << ((threadIdx.x & 31u) & ~(unsigned int)(G - 1)));
    const unsigned int tq = (blockIdx.x * blockDim.x + threadIdx.x) / (unsigned int)G;
    if (tq >= a.Q) return;   // whole groups
    const unsigned int q = a.subset ? a.subset[tq] : tq;
    const QuantFrame f = s_frame;
    group_walk<OUT, TransformOpT, G>(tree, a, transform, f, s_records, q, lane, gmask, lanemask_lt() & gmask);
    }

// ---------------------------------------------------------------------------------------------
// Symmetric (half) self traversal.  When the queries are the tree's own points with one cutoff
// and the image set is symmetric (the self image, or the 27-image lattice), the FP32
// minimum-image predicate is symmetric too (d(j,i) = -d(i,j) exactly, and the wrap keeps |d|), so
// every unordered pair needs to be found once.  Query s starts its walk at its own point record
// (slot pre[s+1] + s) instead of the root: records before it are its ancestors (which contain it)
// and subtrees of smaller sorted positions, so the walk meets exactly the partners j >= s, and
// every record after it is still either visited or excluded by a box it was tested against.
// A pair (s, j) then counts for both rows.
//
// Two ways to turn the pairs into list rows:
//
// Pair exchange (the count keeps the pairs; default).  The count writes, per query, the first
// kHalfCacheSlots keys (image << 27 | sorted position) it found itself, in the order found (own
// keys: ascending), and deposits each pair in the partner's incoming slots: the slot is the old
// value of an atomic increment of the partner's incoming counter, the key the query's position
// with the mirror image (the image through which the partner finds the query; 26 - image on the
// lattice).  k_count_summary then writes each row's count (own + incoming), the largest count and
// the pair total.  A fill over the same tree, cutoff, images and rows walks nothing:
// k_half_assemble sorts each row's incoming keys, merges them with its own keys and writes the
// row, in the order of the reference's rope traversal (images ascending, sorted positions
// ascending within an image).  A row whose own or incoming keys did not fit the slots is
// re-walked whole (k_traverse_subset).
//
// Key ordering pass (when the count did not keep the pairs).  Each entry is first written as a
// key.  The query writes the entries it found itself from the end of its row backwards (already
// in ascending key order) and records how many in own[]; entries found for a row by other queries
// are appended from the front through an atomic cursor (nneigh, zero on entry).
// k_half_order_rows then sorts each row by key and maps keys to transform(primitive) ids.  A row
// with more entries than its capacity (max_neigh, or its own capacity in a CSR list) keeps that
// many of them (which ones is unspecified) and its full count.  Capacities are at most
// kHalfRowThread, so that one thread orders a row; longer rows are filled by the whole-tree walk,
// which writes them in order.
// ---------------------------------------------------------------------------------------------
constexpr unsigned int kHalfKeyBits = 27;
constexpr unsigned int kHalfKeyMask = (1u << kHalfKeyBits) - 1u;
constexpr unsigned int kHalfMaxN = 1u << kHalfKeyBits;   // sorted positions must fit the key
constexpr unsigned int kHalfRowThread = 32;              // longest row a symmetric fill may write

struct HalfArgs
    {
    unsigned int Q;          // number of points (= queries)
    float rc;
    float pad;
    int rows_sorted;         // row of sorted position s: s (1) or primitive[s] (0)
    int lattice;             // 1: the 27 images of lattice_L; 0: the self image only
    float3 lattice_L;
    float3 box;              // periodic lengths of the minimum image (0 = open)
    unsigned int* nneigh;    // zero on entry
    unsigned int* list;      // fill only: rows of max_neigh (kFastList) or offsets/caps (kFastCSR)
    unsigned int max_neigh;
    const unsigned long long* offsets;
    const unsigned int* caps;
    unsigned int* own;       // entries each row found itself (count: for a later fill; fill: for
                             // the ordering pass, with kOwnPlaced)
    unsigned short* walk_out;       // optional: records each query visited (saturated at 65535)
    const unsigned short* walk_in;  // optional: walk lengths of an earlier pass over the same tree
    // fill only, optional: row totals and own counts of a symmetric count over the same tree and
    // rows; a query that met the scene through its own image only then writes its entries as
    // final ids straight after the row's appended entries
    const unsigned int* totals;
    const unsigned int* own_counted;
    // Pair exchange (count only, CACHE): own keys (kHalfCacheSlots per sorted position, in the
    // order found), incoming keys at the slots in_count hands out (in_count zero on entry); own[]
    // is then indexed by sorted position
    unsigned int* cache_out;
    unsigned int* in_cache;
    unsigned int* in_count;
    // rows a partner counted without depositing its key (zero on entry): past the exchange
    unsigned char* in_lost;
    };

constexpr unsigned int kHalfCacheSlots = 16;

// own[] flag of a row whose own entries were written as final ids after its appended entries
constexpr unsigned int kOwnPlaced = 0x80000000u;

constexpr unsigned int kHalfBlock = 128;

// Images (bits of the 27-image lattice, or bit 0 for the self image) whose padded query box
// meets the root box.
__device__ __forceinline__ unsigned int half_image_flags(const HalfArgs& a, const QuantFrame& f,
                                                         const float3& p, float rs)
    {
    if (a.lattice) return lattice_flags(a.lattice_L, f, p, rs);
    const bool hit = approx::fsub_rd(p.x, rs) <= f.hi.x && approx::fadd_ru(p.x, rs) >= f.lo.x
                     && approx::fsub_rd(p.y, rs) <= f.hi.y && approx::fadd_ru(p.y, rs) >= f.lo.y
                     && approx::fsub_rd(p.z, rs) <= f.hi.z && approx::fadd_ru(p.z, rs) >= f.lo.z;
    return hit ? 1u : 0u;
    }

// CACHE (counts only): the pair exchange -- own keys, incoming keys and counters by sorted
// position; compiled separately so that the walk without it carries no test for it.  Blocks of
// 128 queries (16M points: count 3.40 -> 3.35 ms against 256, 3.54 with 512); resident threads
// per SM: 2,048 for counts (3.57 -> 3.14 ms against 1,536), 1,536 for fills (their
// deferred partner stores need the registers).
template<int OUT, class TransformOpT, bool CACHE = false>
__global__ void __launch_bounds__(kHalfBlock, OUT == kFastCount ? 16 : 12) k_traverse_half(const FastLBVHData tree, const HalfArgs a,
                                                                  const TransformOpT transform)
    {
    static_assert(!CACHE || OUT == kFastCount, "the pair exchange is a count's");
    __shared__ QuantFrame s_frame;
    __shared__ unsigned int s_records;
    __shared__ unsigned int s_class[kWorkClasses];
    __shared__ unsigned int s_order[kHalfBlock];
    if (threadIdx.x == 0)
        {
        s_frame = *tree.frame;
        s_records = ld_status(tree.status) != 0u ? 0u : *tree.n_boxes + tree.N;
        }
    unsigned int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (a.walk_in)
        {
        // Work order: the block's queries go to its lanes by walk length (classes of 8 records,
        // from an earlier pass over the same tree), so that a warp's lanes walk about as long as
        // each other.  Results do not depend on which lane takes which query.
        const bool valid = q < a.Q;
        const unsigned int cls = valid ? min((unsigned int)a.walk_in[q] >> 3, kWorkClasses - 1u) : 0u;
        q = block_work_order(q, valid, cls, s_class, s_order);
        if (q == 0xffffffffu) return;
        }
    else
        {
        __syncthreads();
        if (q >= a.Q) return;
        }
    const QuantFrame f = s_frame;
    const unsigned int n_rec = s_records;
    const float4 me = tree.points[q];
    const float3 P = make_float3(me.x, me.y, me.z);
    const unsigned int row = a.rows_sorted ? q : __float_as_uint(me.w);
    const float rs = approx::fadd_ru(a.rc, a.pad);
    unsigned int flags = n_rec ? half_image_flags(a, f, P, rs) : 0u;
    const bool multi = __popc(flags) > 1;
    // a query meeting the scene through its own image only needs no minimum-image wrap
    const bool plain = !multi && wrap_free(a.box, rs);
    const float rc2 = __fmul_rn(a.rc, a.rc);
    const unsigned int start = n_rec ? tree.pre[q + 1] + q : 0u;
    unsigned long long row_first = 0;
    unsigned int cap = 0;
    if (OUT != kFastCount) row_layout<OUT>(a.offsets, a.caps, a.max_neigh, row, row_first, cap);
    // own entries as final ids from slot own_base on (the row's appended entries come first)
    const bool placed = OUT != kFastCount && a.totals != nullptr && !multi;
    const unsigned int own_base = placed ? a.totals[row] - a.own_counted[row] : 0u;
    unsigned int own = 0;
    unsigned int visits = 0;
    // A partner's entry is stored once its slot (the atomic's old value) is known, at the next
    // partner the query finds or after the walk, so the atomic's round trip overlaps the walk.
    bool pending = false;
    unsigned int p_slot = 0, p_cap = 0, p_key = 0;
    unsigned long long p_first = 0;
    // the exchange count's pending deposit: partner (mirror image << 27 | position) and its slot
    // (no slot: 0xffffffff)
    unsigned int x_jm = 0u, x_slot = 0xffffffffu;
    const auto deposit = [&]() {
        if (x_slot < kHalfCacheSlots)
            a.in_cache[(size_t)(x_jm & kHalfKeyMask) * kHalfCacheSlots + x_slot] = (x_jm & ~kHalfKeyMask) | q;
    };
    // one pair (q, j) that the query found through image `bit` (mirror: the partner's image)
    // the query's own entry k (fill): a final id after the row's appended entries, or a key from
    // the end of the row
    const auto own_entry = [&](unsigned int k, unsigned int j, unsigned int bit) {
        if (placed)
            {
            if (own_base + k < cap) a.list[row_first + own_base + k] = transform(tree.primitive[j]);
            }
        else if (k < cap)
            {
            a.list[row_first + (cap - 1u - k)] = (bit << kHalfKeyBits) | j;
            }
    };
    const auto take = [&](unsigned int j, unsigned int bit, unsigned int mirror) {
        if (OUT == kFastCount)
            {
            if (CACHE)
                {
                if (own < kHalfCacheSlots) a.cache_out[(size_t)q * kHalfCacheSlots + own] = (bit << kHalfKeyBits) | j;
                if (j != q)
                    {
                    if (own < kHalfCacheSlots)
                        {
                        // the previous partner's key goes to its slot now that the slot is known
                        deposit();
                        x_slot = atomicAdd(a.in_count + j, 1u);
                        x_jm = (mirror << kHalfKeyBits) | j;
                        }
                    else
                        {
                        // A query with more pairs than its own slots lies in a dense region, where
                        // the partners' slots fill up too (and their counters are contended): the
                        // partner is counted without waiting for a slot and its row is marked for
                        // the fill's re-walk.
                        atomicAdd(a.in_count + j, 1u);
                        a.in_lost[j] = 1u;
                        }
                    }
                }
            else if (j != q)
                {
                atomicAdd(a.nneigh + (a.rows_sorted ? j : tree.primitive[j]), 1u);
                }
            }
        else
            {
            own_entry(own, j, bit);
            if (j != q)
                {
                if (pending && p_slot < p_cap) a.list[p_first + p_slot] = p_key;
                const unsigned int rj = a.rows_sorted ? j : tree.primitive[j];
                p_slot = atomicAdd(a.nneigh + rj, 1u);
                row_layout<OUT>(a.offsets, a.caps, a.max_neigh, rj, p_first, p_cap);
                p_key = (mirror << kHalfKeyBits) | q;
                pending = true;
                }
            }
        ++own;
    };
    while (flags)
        {
        const int bit = __ffs(flags) - 1;
        flags &= flags - 1u;
        const float3 t = a.lattice ? PeriodicImagesOp(a.lattice_L).get((unsigned int)bit) : make_float3(0.f, 0.f, 0.f);
        const unsigned int mirror = a.lattice ? 26u - (unsigned int)bit : 0u;
        const float3 c = make_float3(__fadd_rn(P.x, t.x), __fadd_rn(P.y, t.y), __fadd_rn(P.z, t.z));
        const float3 qlo = make_float3(approx::fsub_rd(c.x, rs), approx::fsub_rd(c.y, rs), approx::fsub_rd(c.z, rs));
        const float3 qhi = make_float3(approx::fadd_ru(c.x, rs), approx::fadd_ru(c.y, rs), approx::fadd_ru(c.z, rs));
        const uint3 qb = pack_query_box(f, qlo, qhi);
        // the walk, compiled twice: with the no-wrap predicate and with the general one
        const auto walk = [&](auto plain_tag) {
            constexpr bool kPlain = decltype(plain_tag)::value;
            unsigned int i = start;
            // one record: a point goes to the predicate, a box that misses jumps to its skip link
            const auto step = [&]() {
                const uint4 n = __ldg(tree.nodes + i);
                if (OUT == kFastCount && !CACHE) ++visits;   // (an exchanged count's fill walks nothing)
                if ((int)n.w < 0)
                    {
                    const float3 x = make_float3(__uint_as_float(n.x), __uint_as_float(n.y), __uint_as_float(n.z));
                    const bool accept = kPlain ? plain_pair(P, x, rc2)
                                               : ((!multi || point_in_box(x, qlo, qhi)) && exact_pair(P, x, a.rc, a.box));
                    if (accept) take(n.w & ~kLeafFlag, (unsigned int)bit, mirror);
                    ++i;
                    }
                else
                    {
                    i = node_overlaps(n, qb) ? i + 1u : max(n.w, i + 1u);
                    }
            };
            while (i < n_rec)
                {
                step();
                // counts take two records per trip of the loop (16M points, the count stage of the
                // step: 3.34 ms with one, 3.26 with two, 3.29 with four)
                if (OUT == kFastCount)
                    {
                    if (i >= n_rec) break;
                    step();
                    }
                }
        };
        if (plain)
            walk(std::true_type());
        else
            walk(std::false_type());
        }
    if (OUT == kFastCount && CACHE)
        {
        deposit();
        a.own[q] = own;
        }
    else if (OUT == kFastCount)
        {
        if (own) atomicAdd(a.nneigh + row, own);
        if (a.own) a.own[row] = own;
        }
    else
        {
        if (pending && p_slot < p_cap) a.list[p_first + p_slot] = p_key;
        a.own[row] = own | (placed ? kOwnPlaced : 0u);
        }
    if (!CACHE && a.walk_out) a.walk_out[q] = (unsigned short)min(visits, 65535u);
    }

// ---------------------------------------------------------------------------------------------
// The exchanging symmetric count of k_traverse_half, one query per group of G lanes: the group
// takes the records after the query's own one in chunks of G, as group_walk does over the whole
// tree (a record is live unless an earlier missed box of the chunk covers it; the next chunk
// starts past the chunk and past every missed subtree), so it meets the same partners in the same
// order.  The accepted pairs of a chunk are ranked by lane (ballot), so the own keys stay in the
// order found; each partner's key goes to the slot its incoming counter hands out.  A pair found
// past the query's own slots marks the partner's row as counted without a key, as the thread walk
// does.  Few queries (small systems) leave most of the GPU idle and the longest walks set the time
// -- a query meeting the scene through up to eight images walks each of them -- and G lanes cut
// each walk's latency about G times.
// ---------------------------------------------------------------------------------------------
template<int G>
__global__ void __launch_bounds__(kWarpWalkBlock) k_traverse_half_group(const FastLBVHData tree, const HalfArgs a)
    {
    static_assert(G == 4 || G == 8 || G == 16 || G == 32, "lane groups of 4, 8, 16 or 32");
    __shared__ QuantFrame s_frame;
    __shared__ unsigned int s_records;
    if (threadIdx.x == 0)
        {
        s_frame = *tree.frame;
        s_records = ld_status(tree.status) != 0u ? 0u : *tree.n_boxes + tree.N;
        }
    __syncthreads();
    const unsigned int lane = threadIdx.x & (unsigned int)(G - 1);
    const unsigned int gmask = G == 32 ? 0xffffffffu
                                       : (((1u << (G & 31)) - 1u) << ((threadIdx.x & 31u) & ~(unsigned int)(G - 1)));
    const unsigned int lt = lanemask_lt() & gmask;
    const unsigned int q = (blockIdx.x * blockDim.x + threadIdx.x) / (unsigned int)G;
    if (q >= a.Q) return;   // whole groups
    const QuantFrame f = s_frame;
    const unsigned int n_rec = s_records;
    const float4 me = tree.points[q];
    const float3 P = make_float3(me.x, me.y, me.z);
    const float rs = approx::fadd_ru(a.rc, a.pad);
    unsigned int flags = n_rec ? half_image_flags(a, f, P, rs) : 0u;
    const bool multi = __popc(flags) > 1;
    const bool plain = !multi && wrap_free(a.box, rs);
    const float rc2 = __fmul_rn(a.rc, a.rc);
    const unsigned int start = n_rec ? tree.pre[q + 1] + q : 0u;
    unsigned int own = 0;   // group-uniform: own pairs found so far
    while (flags)
        {
        const int bit = __ffs(flags) - 1;
        flags &= flags - 1u;
        const float3 t = a.lattice ? PeriodicImagesOp(a.lattice_L).get((unsigned int)bit) : make_float3(0.f, 0.f, 0.f);
        const unsigned int mirror = a.lattice ? 26u - (unsigned int)bit : 0u;
        const float3 c = make_float3(__fadd_rn(P.x, t.x), __fadd_rn(P.y, t.y), __fadd_rn(P.z, t.z));
        const float3 qlo = make_float3(approx::fsub_rd(c.x, rs), approx::fsub_rd(c.y, rs), approx::fsub_rd(c.z, rs));
        const float3 qhi = make_float3(approx::fadd_ru(c.x, rs), approx::fadd_ru(c.y, rs), approx::fadd_ru(c.z, rs));
        const uint3 qb = pack_query_box(f, qlo, qhi);
        unsigned int i = start;
        while (i < n_rec)   // group-uniform
            {
            const unsigned int k = i + lane;
            const bool valid = k < n_rec;
            const uint4 n = valid ? __ldg(tree.nodes + k) : make_uint4(0u, 0u, 0u, 0u);
            const bool is_point = valid && (int)n.w < 0;
            const bool miss = valid && !is_point && !node_overlaps(n, qb);
            const unsigned int kill = miss ? max(n.w, k + 1u) : 0u;   // [k + 1, kill) lies under it
            unsigned int cover = kill;   // inclusive prefix maximum over the group's lanes
#pragma unroll
            for (int o = 1; o < G; o <<= 1)
                {
                const unsigned int v = __shfl_up_sync(gmask, cover, o, G);
                if ((int)lane >= o) cover = max(cover, v);
                }
            const unsigned int before = __shfl_up_sync(gmask, cover, 1, G);
            const bool live = valid && (lane == 0u || before <= k);
            bool accept = false;
            if (live && is_point)
                {
                const float3 x = make_float3(__uint_as_float(n.x), __uint_as_float(n.y), __uint_as_float(n.z));
                accept = plain ? plain_pair(P, x, rc2)
                               : ((!multi || point_in_box(x, qlo, qhi)) && exact_pair(P, x, a.rc, a.box));
                }
            const unsigned int hits = __ballot_sync(gmask, accept) & gmask;
            if (accept)
                {
                const unsigned int j = n.w & ~kLeafFlag;
                const unsigned int pos = own + __popc(hits & lt);   // this pair's place among the own keys
                if (pos < kHalfCacheSlots) a.cache_out[(size_t)q * kHalfCacheSlots + pos] = ((unsigned int)bit << kHalfKeyBits) | j;
                if (j != q)
                    {
                    const unsigned int slot = atomicAdd(a.in_count + j, 1u);
                    if (pos >= kHalfCacheSlots)
                        a.in_lost[j] = 1u;
                    else if (slot < kHalfCacheSlots)
                        a.in_cache[(size_t)j * kHalfCacheSlots + slot] = (mirror << kHalfKeyBits) | q;
                    }
                }
            own += __popc(hits);
            const unsigned int next = __shfl_sync(gmask, cover, G - 1, G);
            i = max(i + (unsigned int)G, next);
            }
        }
    if (lane == 0u) a.own[q] = own;
    }

// ---------------------------------------------------------------------------------------------
// Symmetric count of double self queries with the pair exchange: the exchanging count of
// k_traverse_half with the double predicate of k_traverse_fast_f64 (FP32 screen, exact_pair_f64 in
// the band).  The double predicate is symmetric -- the minimum-image difference of (j, q) is the
// exact negation of that of (q, j), component by component, so both have the same squared length
// -- and the screen only decides pairs that the double predicate decides the same way, so a pair
// found from the smaller sorted position counts for both rows.  A point inside a query's padded
// double box has its rounded-down record inside the FP32 box of that image, and the partner's
// record lies in the mirror image's box of the partner, as in the FP32 walk.  Own keys, incoming
// keys and counters are those of k_traverse_half: k_count_summary and k_half_assemble take them
// unchanged.
// ---------------------------------------------------------------------------------------------
struct HalfArgsF64
    {
    unsigned int Q;              // number of points (= queries)
    const double3* points;       // double positions, by primitive id
    double rc;
    double3 box;                 // periodic lengths of the minimum image (0 = open)
    float pad;
    int lattice;                 // 1: the 27 images of lattice_L; 0: the self image only
    float3 lattice_L;
    unsigned int* own;           // pairs each query found itself, by sorted position
    unsigned int* cache_out;     // own keys, kHalfCacheSlots per sorted position
    unsigned int* in_cache;      // incoming keys, kHalfCacheSlots per sorted position
    unsigned int* in_count;      // zero on entry
    unsigned char* in_lost;      // zero on entry
    };

// MINB: resident blocks per SM.  16M points, count alone: 16 blocks (32 registers, a few spilled)
// 3.75 ms, 12 blocks 4.20, 10 blocks 4.66, 8 blocks 5.30.
template<int MINB = 16>
__global__ void __launch_bounds__(kHalfBlock, MINB) k_traverse_half_f64(const FastLBVHData tree, const HalfArgsF64 a)
    {
    __shared__ QuantFrame s_frame;
    __shared__ unsigned int s_records;
    if (threadIdx.x == 0)
        {
        s_frame = *tree.frame;
        s_records = ld_status(tree.status) != 0u ? 0u : *tree.n_boxes + tree.N;
        }
    __syncthreads();
    const unsigned int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= a.Q) return;
    const QuantFrame f = s_frame;
    const unsigned int n_rec = s_records;
    const double3* P = a.points + tree.primitive[q];   // read again only for the band's exact test
    const double3 Pq = *P;
    const double rs = __dadd_ru(a.rc, (double)a.pad);
    const ScreenF64 S = screen_f64(f, Pq, a.rc, rs, a.box);

    unsigned int flags = 0u;
    if (n_rec)
        {
        if (a.lattice)
            flags = lattice_flags(a.lattice_L, f, S.Pf, S.rsf);
        else
            flags = (approx::fsub_rd(S.Pf.x, S.rsf) <= f.hi.x && approx::fadd_ru(S.Pf.x, S.rsf) >= f.lo.x
                     && approx::fsub_rd(S.Pf.y, S.rsf) <= f.hi.y && approx::fadd_ru(S.Pf.y, S.rsf) >= f.lo.y
                     && approx::fsub_rd(S.Pf.z, S.rsf) <= f.hi.z && approx::fadd_ru(S.Pf.z, S.rsf) >= f.lo.z)
                        ? 1u : 0u;
        }
    const bool multi = __popc(flags) > 1;
    const bool plain = !multi && wrap_free(S.Lf, S.rsf);
    const unsigned int start = n_rec ? tree.pre[q + 1] + q : 0u;
    unsigned int own = 0;
    // the pending deposit: partner (mirror image << 27 | position) and its slot (none: 0xffffffff)
    unsigned int x_jm = 0u, x_slot = 0xffffffffu;
    const auto deposit = [&]() {
        if (x_slot < kHalfCacheSlots)
            a.in_cache[(size_t)(x_jm & kHalfKeyMask) * kHalfCacheSlots + x_slot] = (x_jm & ~kHalfKeyMask) | q;
    };
    const auto take = [&](unsigned int j, unsigned int bit, unsigned int mirror) {
        if (own < kHalfCacheSlots) a.cache_out[(size_t)q * kHalfCacheSlots + own] = (bit << kHalfKeyBits) | j;
        if (j != q)
            {
            if (own < kHalfCacheSlots)
                {
                deposit();
                x_slot = atomicAdd(a.in_count + j, 1u);
                x_jm = (mirror << kHalfKeyBits) | j;
                }
            else
                {
                atomicAdd(a.in_count + j, 1u);
                a.in_lost[j] = 1u;
                }
            }
        ++own;
    };
    while (flags)
        {
        const int bit = __ffs(flags) - 1;
        flags &= flags - 1u;
        const float3 t = a.lattice ? PeriodicImagesOp(a.lattice_L).get((unsigned int)bit) : make_float3(0.f, 0.f, 0.f);
        const unsigned int mirror = a.lattice ? 26u - (unsigned int)bit : 0u;
        float3 qlo, qhi;
        query_box_f32(S, t, qlo, qhi);
        const uint3 qb = pack_query_box(f, qlo, qhi);
        // the walk, compiled twice: with the plain screen and with the minimum-image one
        const auto walk = [&](auto plain_tag) {
            constexpr bool kPlain = decltype(plain_tag)::value;
            unsigned int i = start;
            const auto step = [&]() {
                const uint4 n = __ldg(tree.nodes + i);
                if ((int)n.w < 0)
                    {
                    // with one image the predicate alone decides (a pair lies inside its box); with
                    // several, a point is taken only through the image whose box holds its record
                    const float3 x = make_float3(__uint_as_float(n.x), __uint_as_float(n.y), __uint_as_float(n.z));
                    if (kPlain || !multi || point_in_box(x, qlo, qhi))
                        {
                        const float d2 = screen_dist2<!kPlain>(S, x);
                        if (d2 <= S.out2)
                            {
                            const unsigned int j = n.w & ~kLeafFlag;
                            if (d2 < S.in2 || exact_pair_f64(*P, a.points[tree.primitive[j]], a.rc, a.box))
                                take(j, (unsigned int)bit, mirror);
                            }
                        }
                    ++i;
                    }
                else
                    {
                    i = node_overlaps(n, qb) ? i + 1u : max(n.w, i + 1u);
                    }
            };
            // two records per trip of the loop (16M points, count alone: 3.75 -> 3.67 ms; four: 3.72)
            while (i < n_rec)
                {
                step();
                if (i >= n_rec) break;
                step();
                }
        };
        if (plain)
            walk(std::true_type());
        else
            walk(std::false_type());
        }
    deposit();
    a.own[q] = own;
    }

// A row is past the pair exchange -- its row is walked again by the fill -- when its own or its
// incoming keys did not fit their slots, or when a partner counted it without depositing a key.
__device__ __forceinline__ bool past_exchange(unsigned int own, unsigned int in, unsigned char lost)
    {
    return own > kHalfCacheSlots || in > kHalfCacheSlots || lost != 0u;
    }

// Summary of a count, in four device words: [0] the largest row count, [1] rows whose own or
// incoming keys did not fit the pair exchange's slots (EXCHANGE) or rows longer than both slot
// sets together (otherwise), [2..3] the pair total (64-bit, ordered pairs, self included).  The
// words are zero on entry.
//   EXCHANGE: the rows of a pair-exchange count: nneigh[row(s)] = own[s] + in_count[s].
//   otherwise: the counts already in nneigh[0..N) (any count route).
constexpr unsigned int kSummaryWords = 4;
constexpr unsigned int kSummaryBlock = 256;

template<bool EXCHANGE>
__global__ void __launch_bounds__(kSummaryBlock) k_count_summary(unsigned int N, const unsigned int* __restrict__ own,
                                                                 const unsigned int* __restrict__ in_count,
                                                                 const unsigned char* __restrict__ lost,
                                                                 const unsigned int* __restrict__ primitive,
                                                                 int rows_sorted, unsigned int* nneigh,
                                                                 unsigned int* words, const unsigned int* status)
    {
    // a grid of a few blocks per SM strides over the rows; one atomic per word and block (the
    // words are shared by the whole grid: an atomic per warp measured 0.7 ms at 16M rows)
    __shared__ unsigned int s_max[kSummaryBlock / 32], s_past[kSummaryBlock / 32];
    __shared__ unsigned long long s_sum[kSummaryBlock / 32];
    const bool failed = status != nullptr && ld_status(status) != 0u;
    unsigned int mx = 0, past = 0;
    unsigned long long sum = 0;
    unsigned int first_scalar = 0u;
    if (EXCHANGE && !failed && rows_sorted
        && ((reinterpret_cast<uintptr_t>(own) | reinterpret_cast<uintptr_t>(in_count) | reinterpret_cast<uintptr_t>(nneigh)) & 15u) == 0u
        && (reinterpret_cast<uintptr_t>(lost) & 3u) == 0u)
        {
        // rows in sorted order: four per thread, as 16-byte loads and one 16-byte store
        const unsigned int groups = N / 4u;
        for (unsigned int g = blockIdx.x * blockDim.x + threadIdx.x; g < groups; g += gridDim.x * blockDim.x)
            {
            const uint4 o = reinterpret_cast<const uint4*>(own)[g];
            const uint4 i = reinterpret_cast<const uint4*>(in_count)[g];
            const uchar4 l = reinterpret_cast<const uchar4*>(lost)[g];
            const uint4 t = make_uint4(o.x + i.x, o.y + i.y, o.z + i.z, o.w + i.w);
            reinterpret_cast<uint4*>(nneigh)[g] = t;
            past += (past_exchange(o.x, i.x, l.x) ? 1u : 0u) + (past_exchange(o.y, i.y, l.y) ? 1u : 0u)
                    + (past_exchange(o.z, i.z, l.z) ? 1u : 0u) + (past_exchange(o.w, i.w, l.w) ? 1u : 0u);
            mx = max(max(mx, max(t.x, t.y)), max(t.z, t.w));
            sum += (unsigned long long)t.x + t.y + t.z + t.w;
            }
        first_scalar = groups * 4u;
        }
    for (unsigned int s = first_scalar + blockIdx.x * blockDim.x + threadIdx.x; s < N; s += gridDim.x * blockDim.x)
        {
        if (failed)
            {
            if (EXCHANGE) nneigh[s] = 0u;   // a failed build has no pairs
            continue;
            }
        unsigned int total;
        if (EXCHANGE)
            {
            const unsigned int o = own[s], i = in_count[s];
            total = o + i;
            nneigh[rows_sorted ? s : primitive[s]] = total;
            past += past_exchange(o, i, lost[s]) ? 1u : 0u;
            }
        else
            {
            total = nneigh[s];
            past += total > 2u * kHalfCacheSlots ? 1u : 0u;   // too long for any exchange
            }
        mx = max(mx, total);
        sum += total;
        }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        {
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        past += __shfl_xor_sync(0xffffffffu, past, o);
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
        }
    const unsigned int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31u) == 0u)
        {
        s_max[w] = mx;
        s_past[w] = past;
        s_sum[w] = sum;
        }
    __syncthreads();
    if (threadIdx.x == 0)
        {
        for (unsigned int k = 1; k < kSummaryBlock / 32; ++k)
            {
            mx = max(mx, s_max[k]);
            past += s_past[k];
            sum += s_sum[k];
            }
        if (mx) atomicMax(words + 0, mx);
        if (past) atomicAdd(words + 1, past);
        if (sum) atomicAdd(reinterpret_cast<unsigned long long*>(words + 2), sum);
        }
    }

// Rows re-walked whole after an assembly (the rows past the pair exchange; their number is known
// only on the device, *subset_count).  A persistent grid.  With at most kSubsetGroupMax rows, the
// rows listed in subset[] each get a warp (a few long walks set the time, and 32 lanes shorten
// each about 32 times).  With more, the grid scans all rows in sorted order in chunks of a block
// (handed out by a ticket) and gives each row past the exchange one thread, in order of the
// rows' counts within the block: neighboring queries keep walking neighboring records, and a
// warp's lanes walk about as long as each other (the total work sets the time).
constexpr unsigned int kSubsetBlock = 256;
constexpr unsigned int kSubsetGroupMax = 32768;

// What tells the scan which rows are past the exchange.
struct SubsetScan
    {
    const unsigned int* own;        // own keys found, by sorted position
    const unsigned int* in_count;   // incoming keys counted, by sorted position
    const unsigned char* lost;      // rows counted without a deposited key
    unsigned int* ticket;           // zero on entry
    };

template<int OUT, class TransformOpT>
__global__ void __launch_bounds__(kSubsetBlock) k_traverse_subset(const FastLBVHData tree, const FastQueryArgs a,
                                                                  const TransformOpT transform,
                                                                  const unsigned int* __restrict__ subset_count,
                                                                  const SubsetScan scan)
    {
    __shared__ QuantFrame s_frame;
    __shared__ unsigned int s_records;
    __shared__ unsigned int s_n;
    __shared__ unsigned int s_chunk;
    __shared__ unsigned int s_class[kWorkClasses];
    __shared__ unsigned int s_order[kSubsetBlock];
    if (threadIdx.x == 0)
        {
        s_frame = *tree.frame;
        s_records = ld_status(tree.status) != 0u ? 0u : *tree.n_boxes + tree.N;
        s_n = *subset_count;
        }
    __syncthreads();
    const unsigned int n = s_n;
    const unsigned int n_rec = s_records;
    if (n == 0u || n_rec == 0u) return;
    const QuantFrame f = s_frame;
    if (n <= kSubsetGroupMax)
        {
        const unsigned int gid = blockIdx.x * blockDim.x + threadIdx.x;
        const unsigned int lane = threadIdx.x & 31u;
        const unsigned int lt = lanemask_lt();
        for (unsigned int t = gid >> 5; t < n; t += (gridDim.x * blockDim.x) >> 5)
            group_walk<OUT, TransformOpT, 32>(tree, a, transform, f, n_rec, a.subset[t], lane, 0xffffffffu, lt);
        return;
        }
    unsigned int visits = 0, tests = 0, walks = 0;
    const unsigned int N = tree.N;
    while (true)
        {
        if (threadIdx.x == 0) s_chunk = atomicAdd(scan.ticket, 1u);
        __syncthreads();
        const unsigned int b0 = s_chunk * blockDim.x;
        if (b0 >= N) break;   // block-uniform
        const unsigned int item = b0 + threadIdx.x;
        const bool valid = item < N && past_exchange(scan.own[item], scan.in_count[item], scan.lost[item]);
        unsigned int cls = 0;
        if (valid)
            {
            const unsigned int row = a.self_rows_sorted ? item : __float_as_uint(tree.points[item].w);
            cls = capacity_class(a.nneigh[row]);
            }
        const unsigned int t = block_work_order(item, valid, cls, s_class, s_order);
        if (t != 0xffffffffu) thread_walk<OUT, false>(tree, a, transform, f, n_rec, t, visits, tests, walks);
        __syncthreads();   // s_chunk and s_order are rewritten by the next round
        }
    }

// ---------------------------------------------------------------------------------------------
// Assembly of list rows from a pair-exchange count (no walk, no atomics on rows).  One thread per
// sorted position s: its own keys (ascending: found in pre-order from its own record) and its
// incoming keys (in the order the partners' atomics arrived) go to registers, the incoming keys
// are sorted with a sorting network, and the row is written in key order (image, then sorted
// position) as transform(primitive) ids -- the order of the reference's rope traversal.  When
// every key has the query's own image (`center`), each incoming key (a partner before s) sorts
// before each own key (s and partners after it), so the row is the sorted incoming keys followed
// by the own keys; otherwise the two sorted halves are merged (bitonic).  The first min(count,
// capacity) entries are written, which is what the reference's NeighborListOp keeps of a row that
// overflows.  Rows whose keys did not fit the slots are appended to subset[] for a whole walk.
// ---------------------------------------------------------------------------------------------
struct AssembleArgs
    {
    unsigned int N;
    int rows_sorted;
    unsigned int center;                 // image field of pairs through the query's own image
    const unsigned int* own;             // own keys found, by sorted position
    const unsigned int* in_count;        // incoming keys deposited, by sorted position
    const unsigned char* lost;           // rows counted without a deposited key
    const unsigned int* own_keys;        // kHalfCacheSlots per sorted position
    const unsigned int* in_keys;         // kHalfCacheSlots per sorted position
    const unsigned int* primitive;
    unsigned int* nneigh;
    unsigned int* list;
    unsigned int max_neigh;              // stride of a fixed-stride list
    const unsigned long long* offsets;   // CSR rows (kFastCSR)
    const unsigned int* caps;
    unsigned int* subset;                // rows to re-walk (sorted positions)
    unsigned int* subset_count;          // zero on entry
    const unsigned int* status;
    };

// Compare-exchange of two registers into ascending (UP) or descending order.
template<bool UP>
__device__ __forceinline__ void cas(unsigned int& x, unsigned int& y)
    {
    const unsigned int lo = min(x, y), hi = max(x, y);
    x = UP ? lo : hi;
    y = UP ? hi : lo;
    }

// Bitonic sort of v[B .. B+M) into ascending order (M a power of two; indices resolve at compile
// time, so the keys stay in registers).
template<int M, int B, int K>
__device__ __forceinline__ void bitonic_sort(unsigned int (&v)[K])
    {
#pragma unroll
    for (int k = 2; k <= M; k <<= 1)
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1)
#pragma unroll
            for (int i = 0; i < M; ++i)
                {
                const int l = i ^ j;
                if (l > i)
                    {
                    if ((i & k) == 0)
                        cas<true>(v[B + i], v[B + l]);
                    else
                        cas<false>(v[B + i], v[B + l]);
                    }
                }
    }

template<int OUT, class TransformOpT>
__global__ void __launch_bounds__(256) k_half_assemble(const AssembleArgs a, const TransformOpT transform)
    {
    constexpr int S = (int)kHalfCacheSlots;
    static_assert(S == 16, "16 own and 16 incoming slots");
    const unsigned int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.N) return;
    if (ld_status(a.status) != 0u)
        {
        a.nneigh[s] = 0u;   // a failed build has no pairs
        return;
        }
    const unsigned int o = a.own[s], ni = a.in_count[s];
    const unsigned int total = o + ni;
    const unsigned int row = a.rows_sorted ? s : a.primitive[s];
    a.nneigh[row] = total;
    const bool past = past_exchange(o, ni, a.lost[s]);
    // rows past the exchange join the re-walk list (one atomic per warp); past kSubsetGroupMax
    // rows the re-walk scans all rows instead and the list is not needed
    const unsigned int active = __activemask();
    const unsigned int ballot = __ballot_sync(active, past);
    if (past)
        {
        const unsigned int leader = __ffs(ballot) - 1u;
        unsigned int base = 0u;
        if ((threadIdx.x & 31u) == leader) base = atomicAdd(a.subset_count, __popc(ballot));
        base = __shfl_sync(ballot, base, leader);
        const unsigned int k = base + __popc(ballot & lanemask_lt());
        if (k < kSubsetGroupMax) a.subset[k] = s;
        return;
        }
    unsigned long long first = 0;
    unsigned int cap = 0;
    row_layout<OUT>(a.offsets, a.caps, a.max_neigh, row, first, cap);
    // v[0..16): own keys, v[16..32): incoming keys; unused slots hold 0xffffffff, above every key
    unsigned int v[2 * S];
    const uint4* ok = reinterpret_cast<const uint4*>(a.own_keys + (size_t)s * S);
    const uint4* ik = reinterpret_cast<const uint4*>(a.in_keys + (size_t)s * S);
#pragma unroll
    for (int w = 0; w < S / 4; ++w)
        {
        const uint4 x = 4u * w < o ? ok[w] : make_uint4(~0u, ~0u, ~0u, ~0u);
        const uint4 y = 4u * w < ni ? ik[w] : make_uint4(~0u, ~0u, ~0u, ~0u);
        v[4 * w + 0] = x.x;
        v[4 * w + 1] = x.y;
        v[4 * w + 2] = x.z;
        v[4 * w + 3] = x.w;
        v[S + 4 * w + 0] = y.x;
        v[S + 4 * w + 1] = y.y;
        v[S + 4 * w + 2] = y.z;
        v[S + 4 * w + 3] = y.w;
        }
    bool single = true;
#pragma unroll
    for (int k = 0; k < S; ++k)
        {
        if ((unsigned int)k >= o) v[k] = ~0u;
        else single = single && (v[k] >> kHalfKeyBits) == a.center;
        if ((unsigned int)k >= ni) v[S + k] = ~0u;
        else single = single && (v[S + k] >> kHalfKeyBits) == a.center;
        }
    if (ni > 1u)
        {
        if (ni <= 4u)
            bitonic_sort<4, S>(v);
        else if (ni <= 8u)
            bitonic_sort<8, S>(v);
        else
            bitonic_sort<16, S>(v);
        }
    unsigned int* out = a.list + first;
    // ids are gathered before any entry is stored, so that the gathers are in flight together
    // (a store to the list could otherwise alias the next gather)
    if (single)
        {
#pragma unroll
        for (int k = 0; k < S; ++k)
            {
            if ((unsigned int)k < ni) v[S + k] = transform(__ldg(a.primitive + (v[S + k] & kHalfKeyMask)));
            if ((unsigned int)k < o) v[k] = transform(__ldg(a.primitive + (v[k] & kHalfKeyMask)));
            }
#pragma unroll
        for (int k = 0; k < S; ++k)
            if ((unsigned int)k < ni && (unsigned int)k < cap) out[k] = v[S + k];
#pragma unroll
        for (int k = 0; k < S; ++k)
            if ((unsigned int)k < o && ni + k < cap) out[ni + k] = v[k];
        return;
        }
    // own ascending then incoming descending is a bitonic sequence: merge it (reversing the
    // incoming half is a renaming of registers)
#pragma unroll
    for (int k = 0; k < S / 2; ++k)
        {
        const unsigned int t = v[S + k];
        v[S + k] = v[2 * S - 1 - k];
        v[2 * S - 1 - k] = t;
        }
#pragma unroll
    for (int j = S; j > 0; j >>= 1)
#pragma unroll
        for (int i = 0; i < 2 * S; ++i)
            {
            const int l = i ^ j;
            if (l > i) cas<true>(v[i], v[l]);
            }
#pragma unroll
    for (int k = 0; k < 2 * S; ++k)
        if ((unsigned int)k < total) v[k] = transform(__ldg(a.primitive + (v[k] & kHalfKeyMask)));
#pragma unroll
    for (int k = 0; k < 2 * S; ++k)
        if ((unsigned int)k < total && (unsigned int)k < cap) out[k] = v[k];
    }

struct HalfOrderArgs
    {
    unsigned int Q;
    unsigned int* nneigh;       // in: entries appended by other queries; out: row totals
    unsigned int* list;
    unsigned int max_neigh;
    const unsigned long long* offsets;  // CSR rows (null: stride max_neigh)
    const unsigned int* caps;
    const unsigned int* own;
    const unsigned int* primitive;
    const unsigned int* status;
    };

// Key k of a row (0 <= k < m): the appended entries first, then the query's own entries in the
// order it found them (stored backwards from the end of the row).  Rows that overflowed hold
// max_neigh keys in no particular order.
__device__ __forceinline__ unsigned int half_row_key(const unsigned int* row, unsigned int k,
                                                     unsigned int appended, unsigned int total,
                                                     unsigned int max_neigh)
    {
    if (total > max_neigh || k < appended) return row[k];
    return row[max_neigh - 1u - (k - appended)];
    }

template<class TransformOpT>
__global__ void __launch_bounds__(256) k_half_order_rows(const HalfOrderArgs a, const TransformOpT transform)
    {
    const unsigned int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= a.Q || ld_status(a.status) != 0u) return;
    const unsigned int appended = a.nneigh[r];
    const unsigned int own_word = a.own[r];
    const unsigned int total = appended + (own_word & ~kOwnPlaced);
    a.nneigh[r] = total;
    const unsigned long long first = a.offsets ? a.offsets[r] : (unsigned long long)r * a.max_neigh;
    const unsigned int cap = a.offsets ? a.caps[r] : a.max_neigh;
    if (own_word & kOwnPlaced)
        {
        // own entries are final ids already (after the appended ones): order the appended keys
        const unsigned int ma = min(appended, min(cap, kHalfRowThread));
        if (ma == 0u) return;
        unsigned int* row = a.list + first;
        unsigned int key[kHalfRowThread];
#pragma unroll 8
        for (unsigned int k = 0; k < ma; ++k) key[k] = row[k];
        for (unsigned int k = 1; k < ma; ++k)
            {
            const unsigned int v = key[k];
            unsigned int j = k;
            while (j > 0u && key[j - 1u] > v)
                {
                key[j] = key[j - 1u];
                --j;
                }
            key[j] = v;
            }
#pragma unroll 8
        for (unsigned int k = 0; k < ma; ++k) key[k] = a.primitive[key[k] & kHalfKeyMask];
#pragma unroll 8
        for (unsigned int k = 0; k < ma; ++k) row[k] = transform(key[k]);
        return;
        }
    const unsigned int m = min(total, cap);
    if (m == 0u) return;
    // callers route fills with rows longer than kHalfRowThread to the whole-tree walk
    if (m > kHalfRowThread) return;
    unsigned int* row = a.list + first;
    unsigned int key[kHalfRowThread];
    // loads first (independent, several in flight), then the insertion sort, then the ids
#pragma unroll 8
    for (unsigned int k = 0; k < m; ++k) key[k] = half_row_key(row, k, appended, total, cap);
    for (unsigned int k = 1; k < m; ++k)
        {
        const unsigned int v = key[k];
        unsigned int j = k;
        while (j > 0u && key[j - 1u] > v)
            {
            key[j] = key[j - 1u];
            --j;
            }
        key[j] = v;
        }
#pragma unroll 8
    for (unsigned int k = 0; k < m; ++k) key[k] = a.primitive[key[k] & kHalfKeyMask];
#pragma unroll 8
    for (unsigned int k = 0; k < m; ++k) row[k] = transform(key[k]);
    }

// ---------------------------------------------------------------------------------------------
// Warp-cooperative (packet) traversal.  The 32 queries of a warp are consecutive in the query
// order (Morton order when the queries are the tree's own points).  The warp walks the tree once
// with the union of their padded boxes: record loads are one broadcast address and every branch
// is warp-uniform; at a point record every lane applies the exact predicate to its own query.
// Where the Morton curve jumps the union box is much larger than its halves' boxes and the packet
// is split (recursively).  Measured slower than one thread per query on uniform inputs (the
// union box makes a warp visit several times more records than its lanes need); kept as a mode.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ float warp_min(float v)
    {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
    }
__device__ __forceinline__ float warp_max(float v)
    {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
    }

struct PacketBox
    {
    float3 lo;
    float3 hi;
    };

// Union over the lanes in [a, b) with on == true of their boxes (empty box if none).
__device__ __forceinline__ PacketBox packet_union(const float3& lo, const float3& hi, bool on,
                                                  int lane, int a, int b)
    {
    const bool in = on && lane >= a && lane < b;
    PacketBox r;
    r.lo = make_float3(warp_min(in ? lo.x : 3.0e38f), warp_min(in ? lo.y : 3.0e38f), warp_min(in ? lo.z : 3.0e38f));
    r.hi = make_float3(warp_max(in ? hi.x : -3.0e38f), warp_max(in ? hi.y : -3.0e38f), warp_max(in ? hi.z : -3.0e38f));
    return r;
    }

__device__ __forceinline__ float packet_volume(const PacketBox& b)
    {
    const float dx = fmaxf(b.hi.x - b.lo.x, 0.f);
    const float dy = fmaxf(b.hi.y - b.lo.y, 0.f);
    const float dz = fmaxf(b.hi.z - b.lo.z, 0.f);
    return dx * dy * dz;
    }

constexpr float kPacketSplitRatio = 1.5f;

template<int OUT, class TransformOpT>
__global__ void k_traverse_packet(const FastLBVHData tree, const FastQueryArgs a,
                                  const TransformOpT transform)
    {
    __shared__ QuantFrame s_frame;
    __shared__ unsigned int s_records;
    if (threadIdx.x == 0)
        {
        s_frame = *tree.frame;
        s_records = ld_status(tree.status) != 0u ? 0u : *tree.n_boxes + tree.N;
        }
    __syncthreads();
    const QuantFrame f = s_frame;
    const unsigned int n_rec = s_records;
    const unsigned int q = blockIdx.x * blockDim.x + threadIdx.x;
    if ((q & ~31u) >= a.Q) return;  // whole warp idle
    const bool valid = q < a.Q;
    const int lane = threadIdx.x & 31;

    FastQuery Q;
    Q.p = make_float3(0.f, 0.f, 0.f);
    Q.rc = 0.f;
    Q.row = 0;
    if (valid) Q = load_fast_query(tree, a, q);
    const float rs = approx::fadd_ru(Q.rc, a.pad);
    const unsigned int flags = valid ? image_flags(a, f, Q.p, rs) : 0u;
    unsigned int wflags = __reduce_or_sync(0xffffffffu, flags);
    const bool multi = __popc(wflags) > 1;
    const unsigned long long row_first = (unsigned long long)Q.row * a.max_neigh;

    unsigned int count = 0;
    unsigned int visits = 0, tests = 0, walks = 0;  // per packet (warp-uniform)
    while (wflags)
        {
        const int bit = __ffs(wflags) - 1;
        wflags &= wflags - 1u;
        const float3 t = image_vector(a, bit);
        const float3 c = make_float3(__fadd_rn(Q.p.x, t.x), __fadd_rn(Q.p.y, t.y), __fadd_rn(Q.p.z, t.z));
        const bool lane_on = valid && ((flags >> bit) & 1u);
        const float3 qlo = make_float3(approx::fsub_rd(c.x, rs), approx::fsub_rd(c.y, rs), approx::fsub_rd(c.z, rs));
        const float3 qhi = make_float3(approx::fadd_ru(c.x, rs), approx::fadd_ru(c.y, rs), approx::fadd_ru(c.z, rs));

        int stack_lo[8], stack_hi[8];
        stack_lo[0] = 0;
        stack_hi[0] = 32;
        int sp = 1;
        while (sp > 0)
            {
            --sp;
            const int ra = stack_lo[sp];
            const int rb = stack_hi[sp];
            const PacketBox g = packet_union(qlo, qhi, lane_on, lane, ra, rb);
            if (g.lo.x > g.hi.x) continue;  // no active lane in this range
            if (rb - ra > 1)
                {
                const int m = (ra + rb) >> 1;
                const PacketBox ga = packet_union(qlo, qhi, lane_on, lane, ra, m);
                const PacketBox gb = packet_union(qlo, qhi, lane_on, lane, m, rb);
                if (packet_volume(g) > kPacketSplitRatio * (packet_volume(ga) + packet_volume(gb)))
                    {
                    stack_lo[sp] = m;
                    stack_hi[sp] = rb;
                    ++sp;
                    stack_lo[sp] = ra;
                    stack_hi[sp] = m;
                    ++sp;
                    continue;
                    }
                }
            const bool mine = lane_on && lane >= ra && lane < rb;
            const uint3 qb = pack_query_box(f, g.lo, g.hi);
            ++walks;
            unsigned int i = 0;
            while (i < n_rec)
                {
                const uint4 n = __ldg(tree.nodes + i);
                ++visits;
                if (n.w & kLeafFlag)
                    {
                    ++tests;
                    const float3 x = make_float3(__uint_as_float(n.x), __uint_as_float(n.y), __uint_as_float(n.z));
                    bool ok = mine && exact_pair(Q.p, x, Q.rc, a.box);
                    if (multi) ok = ok && point_in_box(x, qlo, qhi);
                    if (ok)
                        {
                        if (OUT == kFastList && count < a.max_neigh)
                            a.list[row_first + count] = transform(tree.primitive[n.w & ~kLeafFlag]);
                        ++count;
                        }
                    ++i;
                    }
                else
                    {
                    i = node_overlaps(n, qb) ? i + 1u : max(n.w, i + 1u);
                    }
                }
            }
        }
    if (valid) a.nneigh[Q.row] = count;
    if (lane == 0) add_stats(a.stats, visits, tests, walks);
    }

} // namespace gpu
} // namespace neighbor

#endif // NEIGHBOR_KERNELS_TRAVERSE_CUH_
