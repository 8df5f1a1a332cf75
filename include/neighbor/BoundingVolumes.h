// Bounding volumes used by insert and query ops.
//
// Interface and rounding contract follow the reference (include/neighbor/BoundingVolumes.h:28-175):
// a BoundingBox stores FP32 bounds (double inputs are rounded outward), and a BoundingSphere
// stores its centre and an outward-rounded squared radius; the sphere-box test computes the
// closest-point distance rounding down, so it never reports a miss for a true overlap.
#ifndef NEIGHBOR_BOUNDING_VOLUMES_H_
#define NEIGHBOR_BOUNDING_VOLUMES_H_

#include <cuda_runtime.h>

#include "ApproximateMath.h"

namespace neighbor
{

struct BoundingBox
    {
    // Left uninitialised on purpose: kernels construct boxes in registers.
    __device__ BoundingBox() {}

    __device__ BoundingBox(const float3& lo_, const float3& hi_) : lo(lo_), hi(hi_) {}

    // Double-precision bounds rounded outward to FP32.
    __device__ BoundingBox(const double3& lo_, const double3& hi_)
        {
        lo = make_float3(approx::double2float_rd(lo_.x), approx::double2float_rd(lo_.y),
                         approx::double2float_rd(lo_.z));
        hi = make_float3(approx::double2float_ru(hi_.x), approx::double2float_ru(hi_.y),
                         approx::double2float_ru(hi_.z));
        }

    // Arithmetic mean of the bounds, round-to-nearest (used for Morton binning).
    __device__ __forceinline__ float3 getCenter() const
        {
        return make_float3(__fmul_rn(0.5f, __fadd_rn(lo.x, hi.x)),
                           __fmul_rn(0.5f, __fadd_rn(lo.y, hi.y)),
                           __fmul_rn(0.5f, __fadd_rn(lo.z, hi.z)));
        }

    __device__ __forceinline__ bool overlap(const BoundingBox& box) const
        {
        const bool sep = (hi.x < box.lo.x) | (lo.x > box.hi.x) | (hi.y < box.lo.y)
                         | (lo.y > box.hi.y) | (hi.z < box.lo.z) | (lo.z > box.hi.z);
        return !sep;
        }

    float3 lo;
    float3 hi;
    };

struct BoundingSphere
    {
    __device__ BoundingSphere() {}

    // Squared radius rounded up.
    __device__ BoundingSphere(const float3& o, const float r)
        {
        origin = o;
        Rsq = approx::fmul_ru(r, r);
        }

    // Double-precision centre: the FP32 centre is the rounded-down corner and the radius grows
    // by the widest rounding gap, so the FP32 sphere encloses the double one.
    __device__ BoundingSphere(const double3& o, const double r)
        {
        const float3 dn = make_float3(approx::double2float_rd(o.x), approx::double2float_rd(o.y),
                                      approx::double2float_rd(o.z));
        const float3 up = make_float3(approx::double2float_ru(o.x), approx::double2float_ru(o.y),
                                      approx::double2float_ru(o.z));
        const float gap = fmaxf(fmaxf(approx::fsub_ru(up.x, dn.x), approx::fsub_ru(up.y, dn.y)),
                                approx::fsub_ru(up.z, dn.z));
        const float R = approx::fadd_ru(approx::double2float_ru(r), gap);
        origin = dn;
        Rsq = approx::fmul_ru(R, R);
        }

    // Closest point of the box to the centre, squared distance rounded down, compared with the
    // rounded-up squared radius.
    __device__ __forceinline__ bool overlap(const BoundingBox& box) const
        {
        const float dx = approx::fsub_rd(fminf(fmaxf(origin.x, box.lo.x), box.hi.x), origin.x);
        const float dy = approx::fsub_rd(fminf(fmaxf(origin.y, box.lo.y), box.hi.y), origin.y);
        const float dz = approx::fsub_rd(fminf(fmaxf(origin.z, box.lo.z), box.hi.z), origin.z);
        const float d2 = approx::fmaf_rd(dx, dx, approx::fmaf_rd(dy, dy, approx::fmul_rd(dz, dz)));
        return d2 <= Rsq;
        }

    float3 origin;
    float Rsq;
    };

} // namespace neighbor

#endif // NEIGHBOR_BOUNDING_VOLUMES_H_
