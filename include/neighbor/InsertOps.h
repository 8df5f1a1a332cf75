// Insert operations: turn primitive i into the FP32 box of leaf i.
//
// Same interface as the reference's insert ops (include/neighbor/InsertOps.h:18-96):
// `BoundingBox get(unsigned int) const` on the device and `unsigned int size() const` on both sides.
// A user-written insert op with that interface works with LBVH::build.
#ifndef NEIGHBOR_INSERT_OPS_H_
#define NEIGHBOR_INSERT_OPS_H_

#include <cuda_runtime.h>

#include "BoundingVolumes.h"

namespace neighbor
{

// Points: degenerate boxes [p, p].
struct PointInsertOp
    {
    PointInsertOp(const float3* points_, unsigned int N_) : points(points_), N(N_) {}

    __device__ __forceinline__ BoundingBox get(const unsigned int idx) const
        {
        const float3 p = points[idx];
        return BoundingBox(p, p);
        }

    __host__ __device__ __forceinline__ unsigned int size() const { return N; }

    const float3* points;
    const unsigned int N;
    };

// Spheres of one constant radius: boxes [p - r, p + r] (round to nearest).
struct SphereInsertOp
    {
    SphereInsertOp(const float3* points_, const float r_, unsigned int N_)
        : points(points_), r(r_), N(N_)
        {}

    __device__ __forceinline__ BoundingBox get(unsigned int idx) const
        {
        const float3 p = points[idx];
        return BoundingBox(make_float3(__fsub_rn(p.x, r), __fsub_rn(p.y, r), __fsub_rn(p.z, r)),
                           make_float3(__fadd_rn(p.x, r), __fadd_rn(p.y, r), __fadd_rn(p.z, r)));
        }

    __host__ __device__ __forceinline__ unsigned int size() const { return N; }

    const float3* points;
    const float r;
    const unsigned int N;
    };

// Addition: points given in double precision (HOOMD-blue's Scalar = double); each leaf box is
// the point rounded outward to FP32 (BoundingBox(double3, double3),
// include/neighbor/BoundingVolumes.h:54-58 of the reference), so it always contains the point.
struct PointInsertOpF64
    {
    PointInsertOpF64(const double3* points_, unsigned int N_) : points(points_), N(N_) {}

    __device__ __forceinline__ BoundingBox get(const unsigned int idx) const
        {
        const double3 p = points[idx];
        return BoundingBox(p, p);
        }

    __host__ __device__ __forceinline__ unsigned int size() const { return N; }

    const double3* points;
    const unsigned int N;
    };

// Trait: does this insert op store bare points, so that the leaf payload (sorted positions) can
// serve the exact-sphere fast traversal?  User ops default to "no".
template<class InsertOpT>
struct is_point_insert { static constexpr bool value = false; };
template<>
struct is_point_insert<PointInsertOp> { static constexpr bool value = true; };

} // namespace neighbor

#endif // NEIGHBOR_INSERT_OPS_H_
