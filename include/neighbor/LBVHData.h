// Raw-pointer views of an LBVH for use inside kernels.
//
// LBVHSentinel, LBVHData and ConstLBVHData keep the reference's names and fields
// (include/neighbor/LBVHData.h:14-43): node 0 is the root, internal nodes 0..N-2 precede leaves
// N-1..2N-2, leaf N-1+i holds sorted primitive i.
//
// FastLBVHData (new) is the traversal form this library builds alongside: live nodes of the tree
// after collapsing every subtree of at most leaf_size primitives into one leaf bucket, stored in
// depth-first pre-order as 16-byte records {lo.x|lo.y<<16, lo.z|~hi.x<<16, ~hi.y|~hi.z<<16, link}.
// Bounds are 16-bit bins of the root box rounded outward (~h = 65535-h).  The left child of an
// internal node is the next record; link is the skip index past its subtree, or for a bucket
// 0x80000000 | first<<count_bits | (count-1) over the sorted primitives.
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

// 16-bit quantisation frame of the fast nodes: bins = (x - lo) * scale, scale = 65535 / extent
// rounded down.
struct QuantFrame
    {
    float3 lo;
    float3 hi;
    float3 scale;
    };

struct FastLBVHData
    {
    const uint4* nodes;          // live nodes in pre-order
    const unsigned int* n_nodes; // device scalar: number of live nodes
    const float4* points;        // sorted leaf payload: (x, y, z, primitive id as bits)
    const QuantFrame* frame;     // device scalar
    const unsigned int* status;  // build status word; traversals do nothing when it is set
    unsigned int N;              // primitives
    unsigned int count_bits;     // bits of (count-1) in a bucket link
    unsigned int leaf_size;
    };

} // namespace neighbor

#endif // NEIGHBOR_LBVH_DATA_H_
