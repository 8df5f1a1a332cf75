// Transform operations: map the primitive id cached in a leaf to the id the traversal reports.
//
// Interface as in the reference (include/neighbor/TransformOps.h:25-64): `unsigned int
// operator()(unsigned int) const` on host and device.
#ifndef NEIGHBOR_TRANSFORM_OPS_H_
#define NEIGHBOR_TRANSFORM_OPS_H_

#include <cuda_runtime.h>

namespace neighbor
{

struct MapTransformOp
    {
    MapTransformOp(const unsigned int* map_) : map(map_) {}
    __host__ __device__ __forceinline__ unsigned int operator()(unsigned int primitive) const
        {
        return map[primitive];
        }
    const unsigned int* map;
    };

struct NullTransformOp
    {
    __host__ __device__ __forceinline__ unsigned int operator()(unsigned int primitive) const
        {
        return primitive;
        }
    };

} // namespace neighbor

#endif // NEIGHBOR_TRANSFORM_OPS_H_
