// Raw-pointer views of an LBVH for use inside kernels.
//
// LBVHSentinel, LBVHData and ConstLBVHData keep the reference's names and fields
// (include/neighbor/LBVHData.h:14-43): node 0 is the root, internal nodes 0..N-2 precede leaves
// N-1..2N-2, leaf N-1+i holds sorted primitive i.
//
// FastLBVHData (new) is the traversal form this library builds alongside: the tree after
// collapsing every subtree of at most leaf_size primitives into a bucket, as 16-byte records in
// depth-first pre-order.  A box record {lo.x|lo.y<<16, lo.z|~hi.x<<16, ~hi.y|~hi.z<<16, skip}
// (15-bit bins of the root box in 16-bit fields, rounded outward, ~h = 32767-h) covers an internal node or a
// bucket; the next record is its first child (or its bucket's first point) and skip is the index
// just past its subtree.  A point record {x, y, z as float bits, 0x80000000 | primitive id}
// holds one primitive with exact coordinates.
#ifndef NEIGHBOR_LBVH_DATA_H_
#define NEIGHBOR_LBVH_DATA_H_

#include <cuda_runtime.h>

namespace neighbor
{

const int LBVHSentinel = 0x7fffffff;

struct LBVHData
    {
    int* parent;
    int* left;
    int* right;
    unsigned int* primitive;
    float3* lo;
    float3* hi;
    int root;
    };

struct ConstLBVHData
    {
    const int* parent;
    const int* left;
    const int* right;
    const unsigned int* primitive;
    const float3* lo;
    const float3* hi;
    int root;
    };

// Quantisation frame of the box records: bins = (x - lo) * scale, scale = 32767 / extent
// rounded down.
struct QuantFrame
    {
    float3 lo;
    float3 hi;
    float3 scale;
    };

struct FastLBVHData
    {
    const uint4* nodes;          // records in pre-order
    const unsigned int* n_boxes; // device scalar: number of box records (records = boxes + N)
    const float4* points;        // sorted leaf payload: (x, y, z, primitive id as bits)
    const unsigned int* primitive; // primitive id of each sorted position
    const unsigned int* pre;     // box records whose first primitive is below s (N+1 entries)
    const QuantFrame* frame;     // device scalar
    const unsigned int* status;  // build status word; traversals do nothing when it is set
    unsigned int N;              // primitives (= point records)
    unsigned int leaf_size;
    };

} // namespace neighbor

#endif // NEIGHBOR_LBVH_DATA_H_
