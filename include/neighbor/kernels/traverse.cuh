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
#ifndef NEIGHBOR_KERNELS_TRAVERSE_CUH_
#define NEIGHBOR_KERNELS_TRAVERSE_CUH_

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

// Output modes of the fast kernel.
enum FastOutput : int
    {
    kFastCount = 1,
    kFastList = 2,
    };

struct FastQueryArgs
    {
    const float4* spheres;    // (x,y,z,cutoff) per query; NULL => self queries
    unsigned int Q;           // number of queries
    float self_rc;            // cutoff of self queries
    int self_rows_sorted;     // self queries: 1 => row s for sorted slot s, 0 => row primitive[s]
    const float3* images;     // NULL => self image only
    unsigned int n_images;
    float3 box;               // periodic lengths for the minimum image (0 = open)
    float pad;                // radius padding of the traversal volume
    unsigned int* nneigh;
    unsigned int* list;
    unsigned int max_neigh;
    };

template<int OUT, class TransformOpT>
__global__ void k_traverse_fast(const FastLBVHData tree, const FastQueryArgs a,
                                                       const TransformOpT transform)
    {
    __shared__ QuantFrame s_frame;
    __shared__ unsigned int s_nodes;
    if (threadIdx.x == 0)
        {
        s_frame = *tree.frame;
        // a failed build leaves no tree to walk
        s_nodes = ld_status(tree.status) != 0u ? 0u : *tree.n_nodes;
        }
    __syncthreads();
    const unsigned int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= a.Q) return;
    const QuantFrame f = s_frame;
    const unsigned int n_nodes = s_nodes;

    float3 p;
    float rc;
    unsigned int row;
    if (a.spheres)
        {
        const float4 s = a.spheres[q];
        p = make_float3(s.x, s.y, s.z);
        rc = s.w;
        row = q;
        }
    else
        {
        const float4 s = tree.points[q];
        p = make_float3(s.x, s.y, s.z);
        rc = a.self_rc;
        row = a.self_rows_sorted ? q : __float_as_uint(s.w);
        }
    const float rs = approx::fadd_ru(rc, a.pad);
    const unsigned int nimg = a.images ? min(a.n_images, 32u) : 1u;

    // images whose padded query box meets the root box
    unsigned int flags = 0;
    for (unsigned int i = 0; i < nimg; ++i)
        {
        const float3 t = a.images ? a.images[i] : make_float3(0.f, 0.f, 0.f);
        const float3 c = make_float3(__fadd_rn(p.x, t.x), __fadd_rn(p.y, t.y), __fadd_rn(p.z, t.z));
        const bool hit = approx::fsub_rd(c.x, rs) <= f.hi.x && approx::fadd_ru(c.x, rs) >= f.lo.x
                         && approx::fsub_rd(c.y, rs) <= f.hi.y && approx::fadd_ru(c.y, rs) >= f.lo.y
                         && approx::fsub_rd(c.z, rs) <= f.hi.z && approx::fadd_ru(c.z, rs) >= f.lo.z;
        if (hit) flags |= 1u << i;
        }

    const unsigned long long row_first = (unsigned long long)row * a.max_neigh;
    const unsigned int cmask = (1u << tree.count_bits) - 1u;
    unsigned int count = 0;
    while (flags)
        {
        const int bit = __ffs(flags) - 1;
        flags &= flags - 1u;
        const float3 t = a.images ? a.images[bit] : make_float3(0.f, 0.f, 0.f);
        const float3 c = make_float3(__fadd_rn(p.x, t.x), __fadd_rn(p.y, t.y), __fadd_rn(p.z, t.z));
        const float3 qlo = make_float3(approx::fsub_rd(c.x, rs), approx::fsub_rd(c.y, rs), approx::fsub_rd(c.z, rs));
        const float3 qhi = make_float3(approx::fadd_ru(c.x, rs), approx::fadd_ru(c.y, rs), approx::fadd_ru(c.z, rs));
        const uint3 qb = pack_query_box(f, qlo, qhi);
        unsigned int i = 0;
        while (i < n_nodes)
            {
            const uint4 n = __ldg(tree.nodes + i);
            const bool hit = node_overlaps(n, qb);
            if (n.w & kLeafFlag)
                {
                if (hit)
                    {
                    const unsigned int first = (n.w & ~kLeafFlag) >> tree.count_bits;
                    const unsigned int end = min(first + (n.w & cmask) + 1u, tree.N);
                    for (unsigned int k = first; k < end; ++k)
                        {
                        const float4 pt = __ldg(tree.points + k);
                        const bool inside = pt.x >= qlo.x && pt.x <= qhi.x && pt.y >= qlo.y
                                            && pt.y <= qhi.y && pt.z >= qlo.z && pt.z <= qhi.z;
                        if (inside && exact_pair(p, make_float3(pt.x, pt.y, pt.z), rc, a.box))
                            {
                            if (OUT == kFastList && count < a.max_neigh)
                                a.list[row_first + count] = transform(__float_as_uint(pt.w));
                            ++count;
                            }
                        }
                    }
                ++i;
                }
            else
                {
                // skip links always point forward in a valid tree; max() keeps even a damaged
                // one from looping
                i = hit ? i + 1u : max(n.w, i + 1u);
                }
            }
        }
    a.nneigh[row] = count;
    }

} // namespace gpu
} // namespace neighbor

#endif // NEIGHBOR_KERNELS_TRAVERSE_CUH_
