// The reference's own device kernels (mphowardlab/neighbor v0.3.2, include/neighbor/kernels/
// LBVH.cuh and LBVHTraverser.cuh), compiled from its headers where they lie into a cubin for the
// reference harness (TEST / MEASUREMENT INFRASTRUCTURE ONLY; see ref_driver.cu).  Nothing of the
// reference is copied here: this unit only instantiates its templates with the ops the harness
// runs, and defines plugin ops through the reference's public operator interface (an FP32 exact
// sphere query, and a double-precision point insert op and exact sphere query).
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

// Double-precision points (HOOMD-blue's Scalar = double positions, as in the reference's own
// benchmark ops, benchmark/lbvh_benchmark.cuh:25-92) through the reference's InsertOp interface:
// each leaf box is the point rounded outward by the reference's BoundingBox(double3, double3).
struct RefPointInsertOpF64
    {
    const double3* points;
    unsigned int N;

    __device__ __forceinline__ neighbor::BoundingBox get(const unsigned int idx) const
        {
        const double3 p = points[idx];
        return neighbor::BoundingBox(p, p);
        }
    __host__ __device__ __forceinline__ unsigned int size() const { return N; }
    };

struct __align__(16) RefSphereF64
    {
    double x, y, z, w;
    };

// Exact sphere query on double positions: volume = the reference's BoundingSphere(double3,
// double) of the imaged centre with radius cutoff + pad; refine() = the double minimum-image
// predicate with the operation order pinned (the library's exact_pair_f64).
struct RefExactQueryOpF64
    {
    const RefSphereF64* spheres;
    unsigned int N;
    const double3* points;
    double3 box;
    float pad;

    typedef RefSphereF64 ThreadData;
    typedef neighbor::BoundingSphere Volume;

    __device__ __forceinline__ ThreadData setup(const unsigned int idx) const { return spheres[idx]; }
    __device__ __forceinline__ Volume get(const ThreadData& q, const float3& image) const
        {
        const double3 t = make_double3(__dadd_rn(q.x, (double)image.x), __dadd_rn(q.y, (double)image.y),
                                       __dadd_rn(q.z, (double)image.z));
        return neighbor::BoundingSphere(t, __dadd_ru(q.w, (double)pad));
        }
    __device__ __forceinline__ bool overlap(const Volume& v, const neighbor::BoundingBox& b) const { return v.overlap(b); }
    __device__ __forceinline__ static double wrap(double d, double L)
        {
        if (L > 0.0)
            {
            const double h = __dmul_rn(0.5, L);
            if (d >= h) d = __dsub_rn(d, L);
            else if (d < -h) d = __dadd_rn(d, L);
            }
        return d;
        }
    __device__ __forceinline__ bool refine(const ThreadData& q, const int primitive) const
        {
        const double3 p = points[primitive];
        const double dx = wrap(__dsub_rn(p.x, q.x), box.x);
        const double dy = wrap(__dsub_rn(p.y, q.y), box.y);
        const double dz = wrap(__dsub_rn(p.z, q.z), box.z);
        const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
        return d2 <= __dmul_rn(q.w, q.w);
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
static_assert(sizeof(RefPointInsertOpF64) == 16 && offsetof(RefPointInsertOpF64, N) == 8, "RefPointInsertOpF64 layout");
static_assert(sizeof(RefExactQueryOpF64) == 56 && offsetof(RefExactQueryOpF64, N) == 8
              && offsetof(RefExactQueryOpF64, points) == 16 && offsetof(RefExactQueryOpF64, box) == 24
              && offsetof(RefExactQueryOpF64, pad) == 48, "RefExactQueryOpF64 layout");

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
template __global__ void lbvh_gen_codes<RefPointInsertOpF64>(unsigned int*, unsigned int*, const RefPointInsertOpF64,
                                                             const float3, const float3, const unsigned int);
template __global__ void lbvh_bubble_aabbs<RefPointInsertOpF64>(const LBVHData, const RefPointInsertOpF64, unsigned int*,
                                                                const unsigned int);
template __global__ void lbvh_one_primitive<RefPointInsertOpF64>(const LBVHData, const RefPointInsertOpF64);
template __global__ void lbvh_traverse_ropes<CountNeighborsOp, RefExactQueryOpF64, ImageListOp<float3>>(
    const CountNeighborsOp, const LBVHCompressedData, const RefExactQueryOpF64, const ImageListOp<float3>);
template __global__ void lbvh_traverse_ropes<NeighborListOp, RefExactQueryOpF64, ImageListOp<float3>>(
    const NeighborListOp, const LBVHCompressedData, const RefExactQueryOpF64, const ImageListOp<float3>);
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
