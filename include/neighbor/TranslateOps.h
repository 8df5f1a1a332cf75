// Translate operations: the image vectors a query volume is moved through (periodic images).
//
// Interface as in the reference (include/neighbor/TranslateOps.h:19-91): `typedef ... type`,
// device get(i), host/device size().  At most 32 images per traversal.
#ifndef NEIGHBOR_TRANSLATE_OPS_H_
#define NEIGHBOR_TRANSLATE_OPS_H_

#include <cstddef>

#include <cuda_runtime.h>

namespace neighbor
{

// Only the zero translation.
struct SelfOp
    {
    typedef float3 type;
    SelfOp() {}
    __device__ __forceinline__ float3 get(const unsigned int) const { return make_float3(0.f, 0.f, 0.f); }
    __host__ __device__ __forceinline__ unsigned int size() const { return 1; }
    };

// A device array of image vectors.
template<typename Real3>
struct ImageListOp
    {
    typedef Real3 type;
    ImageListOp() : images(NULL), N(0) {}
    ImageListOp(const Real3* images_, unsigned int N_) : images(images_), N(N_) {}
    __device__ __forceinline__ Real3 get(const unsigned int idx) const { return images[idx]; }
    __host__ __device__ __forceinline__ unsigned int size() const { return N; }
    const Real3* images;
    const unsigned int N;
    };

// The 27 periodic images of an orthorhombic box: translations (ix*L.x, iy*L.y, iz*L.z) for
// ix, iy, iz in {-1, 0, 1}, image i = 9*(ix+1) + 3*(iy+1) + (iz+1) -- the list the reference's
// tests build by hand (test/lbvh_test.cu:427-440).  The fast traversal recognises it and decides
// which images a query needs with three per-axis tests instead of 27 box tests.
struct PeriodicImagesOp
    {
    typedef float3 type;
    __host__ __device__ explicit PeriodicImagesOp(float3 L_) : L(L_) {}
    __host__ __device__ __forceinline__ float3 get(const unsigned int idx) const
        {
        const float ix = (float)((int)(idx / 9u) - 1);
        const float iy = (float)((int)((idx / 3u) % 3u) - 1);
        const float iz = (float)((int)(idx % 3u) - 1);
        return make_float3(L.x * ix, L.y * iy, L.z * iz);
        }
    __host__ __device__ __forceinline__ unsigned int size() const { return 27; }
    float3 L;
    };

} // namespace neighbor

#endif // NEIGHBOR_TRANSLATE_OPS_H_
