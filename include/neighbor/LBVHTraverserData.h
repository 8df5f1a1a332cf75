// Compressed-tree view for rope traversal in the reference's int4 layout.
//
// LBVHCompressedData keeps the reference's fields (include/neighbor/LBVHTraverserData.h:14-21):
// one int4 per node {lo bins, hi bins (from the top), left child or ~primitive, rope}, 10 bits per
// axis relative to the root box, plus the root bounds and the bin width.
#ifndef NEIGHBOR_LBVH_TRAVERSER_DATA_H_
#define NEIGHBOR_LBVH_TRAVERSER_DATA_H_

#include <cuda_runtime.h>

namespace neighbor
{

struct LBVHCompressedData
    {
    int root;
    int4* data;
    float3* lo;
    float3* hi;
    float3* bins;
    };

} // namespace neighbor

#endif // NEIGHBOR_LBVH_TRAVERSER_DATA_H_
