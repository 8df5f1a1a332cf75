// The reference's own device kernels (mphowardlab/neighbor v0.3.2, include/neighbor/kernels/
// LBVH.cuh and LBVHTraverser.cuh), compiled from its headers where they lie into a cubin for the
// reference harness (TEST / MEASUREMENT INFRASTRUCTURE ONLY; see ref_driver.cu).  Nothing of the
// reference is copied here: this unit only instantiates its templates with the ops the harness
// runs, and defines one plugin query op through the reference's public operator interface.
#include <cstddef>

#include <neighbor/neighbor.h>

// Exact sphere query written against the reference's QueryOp interface
// (include/neighbor/QueryOps.h:32-120): traversal volume = sphere padded by `pad`, refine() =
// the FP32 minimum-image predicate with the operation order pinned (same as the library's
// ExactSphereQueryOp and the oracle's orc_exact_pair).
struct RefExactQueryOp
    {
    const float4* spheres;
    unsigned int N;
    const float3* points;
    float3 box;
    float pad;

    typedef float4 ThreadData;
    typedef neighbor::BoundingSphere Volume;

    __device__ __forceinline__ ThreadData setup(const unsigned int idx) const { return spheres[idx]; }
    __device__ __forceinline__ Volume get(const ThreadData& q, const float3& image) const
        {
        const float3 t = make_float3(__fadd_rn(q.x, image.x), __fadd_rn(q.y, image.y), __fadd_rn(q.z, image.z));
        return neighbor::BoundingSphere(t, __fadd_ru(q.w, pad));
        }
    __device__ __forceinline__ bool overlap(const Volume& v, const neighbor::BoundingBox& b) const { return v.overlap(b); }
    __device__ __forceinline__ static float wrap(float d, float L)
        {
        if (L > 0.f)
            {
            const float h = __fmul_rn(0.5f, L);
            if (d >= h) d = __fsub_rn(d, L);
            else if (d < -h) d = __fadd_rn(d, L);
            }
        return d;
        }
    __device__ __forceinline__ bool refine(const ThreadData& q, const int primitive) const
        {
        const float3 p = points[primitive];
        const float dx = wrap(__fsub_rn(p.x, q.x), box.x);
        const float dy = wrap(__fsub_rn(p.y, q.y), box.y);
        const float dz = wrap(__fsub_rn(p.z, q.z), box.z);
        const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
        return d2 <= __fmul_rn(q.w, q.w);
        }
    __host__ __device__ __forceinline__ unsigned int size() const { return N; }
    };

// Kernel-parameter layouts the driver mirrors (ref_driver.cu asserts the same numbers).
static_assert(sizeof(neighbor::PointInsertOp) == 16 && offsetof(neighbor::PointInsertOp, N) == 8, "PointInsertOp layout");
static_assert(sizeof(neighbor::SphereInsertOp) == 16 && offsetof(neighbor::SphereInsertOp, r) == 8
              && offsetof(neighbor::SphereInsertOp, N) == 12, "SphereInsertOp layout");
static_assert(sizeof(neighbor::LBVHData) == 56 && offsetof(neighbor::LBVHData, root) == 48, "LBVHData layout");
static_assert(sizeof(neighbor::ConstLBVHData) == 56 && offsetof(neighbor::ConstLBVHData, root) == 48, "ConstLBVHData layout");
static_assert(sizeof(neighbor::LBVHCompressedData) == 40 && offsetof(neighbor::LBVHCompressedData, data) == 8, "LBVHCompressedData layout");
static_assert(sizeof(neighbor::CountNeighborsOp) == 8, "CountNeighborsOp layout");
static_assert(sizeof(neighbor::NeighborListOp) == 24 && offsetof(neighbor::NeighborListOp, max_neigh) == 16, "NeighborListOp layout");
static_assert(sizeof(neighbor::ImageListOp<float3>) == 16 && offsetof(neighbor::ImageListOp<float3>, N) == 8, "ImageListOp layout");
static_assert(sizeof(neighbor::SphereQueryOp) == 16, "SphereQueryOp layout");
static_assert(sizeof(neighbor::NullTransformOp) == 1, "NullTransformOp layout");
static_assert(sizeof(RefExactQueryOp) == 40 && offsetof(RefExactQueryOp, points) == 16 && offsetof(RefExactQueryOp, box) == 24
              && offsetof(RefExactQueryOp, pad) == 36, "RefExactQueryOp layout");

namespace neighbor
{
namespace gpu
{
namespace kernel
{
template __global__ void lbvh_gen_codes<PointInsertOp>(unsigned int*, unsigned int*, const PointInsertOp, const float3,
                                                       const float3, const unsigned int);
template __global__ void lbvh_bubble_aabbs<PointInsertOp>(const LBVHData, const PointInsertOp, unsigned int*,
                                                          const unsigned int);
template __global__ void lbvh_one_primitive<PointInsertOp>(const LBVHData, const PointInsertOp);
template __global__ void lbvh_gen_codes<SphereInsertOp>(unsigned int*, unsigned int*, const SphereInsertOp, const float3,
                                                        const float3, const unsigned int);
template __global__ void lbvh_bubble_aabbs<SphereInsertOp>(const LBVHData, const SphereInsertOp, unsigned int*,
                                                           const unsigned int);
template __global__ void lbvh_one_primitive<SphereInsertOp>(const LBVHData, const SphereInsertOp);
template __global__ void lbvh_compress_ropes<NullTransformOp>(const LBVHCompressedData, const NullTransformOp,
                                                              const ConstLBVHData, const unsigned int, const unsigned int);
template __global__ void lbvh_traverse_ropes<CountNeighborsOp, SphereQueryOp, ImageListOp<float3>>(
    const CountNeighborsOp, const LBVHCompressedData, const SphereQueryOp, const ImageListOp<float3>);
template __global__ void lbvh_traverse_ropes<CountNeighborsOp, RefExactQueryOp, ImageListOp<float3>>(
    const CountNeighborsOp, const LBVHCompressedData, const RefExactQueryOp, const ImageListOp<float3>);
template __global__ void lbvh_traverse_ropes<NeighborListOp, RefExactQueryOp, ImageListOp<float3>>(
    const NeighborListOp, const LBVHCompressedData, const RefExactQueryOp, const ImageListOp<float3>);
template __global__ void lbvh_traverse_ropes<NeighborListOp, SphereQueryOp, ImageListOp<float3>>(
    const NeighborListOp, const LBVHCompressedData, const SphereQueryOp, const ImageListOp<float3>);
} // namespace kernel
} // namespace gpu
} // namespace neighbor
