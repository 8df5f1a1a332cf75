// Query operations: the search volume of each query and its narrow-phase test.
//
// Interface as in the reference (include/neighbor/QueryOps.h:32-120): typedefs ThreadData and
// Volume; setup(idx), get(qdata, image), overlap(volume, box), refine(qdata, primitive), size().
//
// SphereQueryOp is the reference's stock op: refine() accepts every primitive whose (compressed)
// leaf box the sphere overlaps, so the result is a conservative superset of the true neighbors.
//
// ExactSphereQueryOp (new in this library) makes the neighbor set exact: the traversal volume is
// the sphere padded by a few ulps (so it never misses), and refine() applies the FP32 minimum-image
// distance predicate exact_pair() below.  That predicate is the brute force of the reference's
// validation test (test/lbvh_test.cu:469-482) with its arithmetic order pinned and no contraction,
// so two implementations that both traverse conservatively return bit-identical sets.
#ifndef NEIGHBOR_QUERY_OPS_H_
#define NEIGHBOR_QUERY_OPS_H_

#include <cmath>

#include <cuda_runtime.h>

#include "BoundingVolumes.h"

namespace neighbor
{

struct SphereQueryOp
    {
    SphereQueryOp(float4* spheres_, unsigned int N_) : spheres(spheres_), N(N_) {}

    typedef float4 ThreadData;
    typedef BoundingSphere Volume;

    __device__ __forceinline__ ThreadData setup(const unsigned int idx) const { return spheres[idx]; }

    __device__ __forceinline__ Volume get(const ThreadData& q, const float3& image) const
        {
        const float3 t = make_float3(__fadd_rn(q.x, image.x), __fadd_rn(q.y, image.y),
                                     __fadd_rn(q.z, image.z));
        return BoundingSphere(t, q.w);
        }

    __device__ __forceinline__ bool overlap(const Volume& v, const BoundingBox& box) const
        {
        return v.overlap(box);
        }

    __device__ __forceinline__ bool refine(const ThreadData&, const int) const { return true; }

    __host__ __device__ __forceinline__ unsigned int size() const { return N; }

    const float4* spheres;
    const unsigned int N;
    };

// FP32 minimum-image distance predicate.  d = pj - pi per component, wrapped once by L when
// |d| reaches L/2 (only where L > 0), then ((dx*dx + dy*dy) + dz*dz) <= rc*rc, every operation
// rounded to nearest and never fused.
__device__ __forceinline__ float min_image_component(float d, float L)
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

__device__ __forceinline__ float exact_dist2(const float3& pi, const float3& pj, const float3& L)
    {
    const float dx = min_image_component(__fsub_rn(pj.x, pi.x), L.x);
    const float dy = min_image_component(__fsub_rn(pj.y, pi.y), L.y);
    const float dz = min_image_component(__fsub_rn(pj.z, pi.z), L.z);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    }

__device__ __forceinline__ bool exact_pair(const float3& pi, const float3& pj, float rc,
                                           const float3& L)
    {
    return exact_dist2(pi, pj, L) <= __fmul_rn(rc, rc);
    }

// exact_pair() without the minimum-image wrap (rc2 = rc * rc rounded).  It gives the same answer
// for a query whose only periodic image meeting the scene is the query itself: a point accepted
// through a wrap lies within rc of another image of the query, whose padded box would then meet
// the scene too; and where no axis wraps both compute the same numbers.  Valid while no distance
// inside the padded query box can wrap: wrap_free(L, rs) with rs the padded radius.
__device__ __forceinline__ bool plain_pair(const float3& pi, const float3& pj, float rc2)
    {
    const float dx = __fsub_rn(pj.x, pi.x);
    const float dy = __fsub_rn(pj.y, pi.y);
    const float dz = __fsub_rn(pj.z, pi.z);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)) <= rc2;
    }

__device__ __forceinline__ bool wrap_free(const float3& L, float rs)
    {
    const float r = fabsf(rs);
    return (L.x == 0.f || r < 0.45f * L.x) && (L.y == 0.f || r < 0.45f * L.y) && (L.z == 0.f || r < 0.45f * L.z);
    }

// Radius padding that keeps a conservative traversal from missing any pair the predicate
// accepts: 16 ulps of twice the largest coordinate magnitude (query centres, points and image
// translations included) plus 1e-6 relative to the cutoff.
inline float exact_query_pad(float rc, float coord_max)
    {
    const float m = std::fmax(std::fabs(coord_max), 1.0f) * 2.0f + std::fabs(rc);
    int e;
    std::frexp(m, &e);
    return 16.0f * std::ldexp(1.0f, e - 24) + std::fabs(rc) * 1.0e-6f;
    }

// Addition: the exact predicate in double precision -- d = pj - pi, wrapped once by +-L when
// |d| >= L/2, ((dx*dx + dy*dy) + dz*dz) <= rc*rc, every operation rounded to nearest and none
// contracted -- for double positions (PointInsertOpF64 trees).
__device__ __forceinline__ double min_image_component_f64(double d, double L)
    {
    if (L > 0.0)
        {
        const double h = __dmul_rn(0.5, L);
        if (d >= h)
            d = __dsub_rn(d, L);
        else if (d < -h)
            d = __dadd_rn(d, L);
        }
    return d;
    }

__device__ __forceinline__ bool exact_pair_f64(const double3& pi, const double3& pj, double rc, const double3& L)
    {
    const double dx = min_image_component_f64(__dsub_rn(pj.x, pi.x), L.x);
    const double dy = min_image_component_f64(__dsub_rn(pj.y, pi.y), L.y);
    const double dz = min_image_component_f64(__dsub_rn(pj.z, pi.z), L.z);
    const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    return d2 <= __dmul_rn(rc, rc);
    }

// Addition: exact sphere query on double positions.  The traversal volume is the double sphere
// (radius + pad) enclosed by an FP32 sphere (BoundingSphere(double3, double)); refine applies
// exact_pair_f64.  Image translations are FP32 (the translate ops' type), so pad must cover their
// rounding as well: exact_query_pad(rc, 2 * largest coordinate) does.  With box lengths above
// 2 (rc + pad) every neighbor is found through exactly one image.
struct ExactSphereQueryOpF64
    {
    ExactSphereQueryOpF64(const double4_16a* spheres_, unsigned int N_, const double3* points_, double3 box_,
                          float pad_)
        : spheres(spheres_), N(N_), points(points_), box(box_), pad(pad_)
        {}

    typedef double4_16a ThreadData;
    typedef BoundingSphere Volume;

    __device__ __forceinline__ ThreadData setup(const unsigned int idx) const { return spheres[idx]; }

    __device__ __forceinline__ Volume get(const ThreadData& q, const float3& image) const
        {
        const double3 t = make_double3(__dadd_rn(q.x, (double)image.x), __dadd_rn(q.y, (double)image.y),
                                       __dadd_rn(q.z, (double)image.z));
        return BoundingSphere(t, __dadd_ru(q.w, (double)pad));
        }

    __device__ __forceinline__ bool overlap(const Volume& v, const BoundingBox& box_) const
        {
        return v.overlap(box_);
        }

    __device__ __forceinline__ bool refine(const ThreadData& q, const int primitive) const
        {
        return exact_pair_f64(make_double3(q.x, q.y, q.z), points[primitive], q.w, box);
        }

    __host__ __device__ __forceinline__ unsigned int size() const { return N; }

    const double4_16a* spheres;
    const unsigned int N;
    const double3* points;
    const double3 box;
    const float pad;
    };

struct ExactSphereQueryOp
    {
    // spheres: (x, y, z, cutoff) per query.  points: positions indexed by the primitive id that
    // the traversal reports (the transformed id when a TransformOp is used).  box: periodic box
    // lengths (0 = not periodic).  pad: see exact_query_pad().
    ExactSphereQueryOp(const float4* spheres_, unsigned int N_, const float3* points_,
                       float3 box_, float pad_)
        : spheres(spheres_), N(N_), points(points_), box(box_), pad(pad_)
        {}

    typedef float4 ThreadData;
    typedef BoundingSphere Volume;

    __device__ __forceinline__ ThreadData setup(const unsigned int idx) const { return spheres[idx]; }

    __device__ __forceinline__ Volume get(const ThreadData& q, const float3& image) const
        {
        const float3 t = make_float3(__fadd_rn(q.x, image.x), __fadd_rn(q.y, image.y),
                                     __fadd_rn(q.z, image.z));
        return BoundingSphere(t, approx::fadd_ru(q.w, pad));
        }

    __device__ __forceinline__ bool overlap(const Volume& v, const BoundingBox& box_) const
        {
        return v.overlap(box_);
        }

    __device__ __forceinline__ bool refine(const ThreadData& q, const int primitive) const
        {
        return exact_pair(make_float3(q.x, q.y, q.z), points[primitive], q.w, box);
        }

    __host__ __device__ __forceinline__ unsigned int size() const { return N; }

    const float4* spheres;
    const unsigned int N;
    const float3* points;
    const float3 box;
    const float pad;
    };

} // namespace neighbor

#endif // NEIGHBOR_QUERY_OPS_H_
