// Output operations: what the traversal does with each accepted primitive.
//
// Interface as in the reference (include/neighbor/OutputOps.h:28-176): a ThreadData type,
// setup(idx, qdata), process(threaddata, primitive) and finalize(threaddata).
//
// CountNeighborsOp writes the number of accepted primitives per query.  NeighborListOp writes
// them into a fixed-stride list (row idx starts at max_neigh*idx), stores only the first
// max_neigh, and always writes the full count -- so nneigh[i] > max_neigh signals overflow.
// CSRNeighborListOp (an addition) gives every row its own offset and capacity.
#ifndef NEIGHBOR_OUTPUT_OPS_H_
#define NEIGHBOR_OUTPUT_OPS_H_

#include <cuda_runtime.h>

namespace neighbor
{

struct CountNeighborsOp
    {
    CountNeighborsOp(unsigned int* nneigh_) : nneigh(nneigh_) {}

    struct ThreadData
        {
        __device__ ThreadData(const unsigned int idx_) : idx(idx_), num_neigh(0) {}
        const int idx;
        unsigned int num_neigh;
        };

    template<class QueryDataT>
    __device__ __forceinline__ ThreadData setup(const unsigned int idx, const QueryDataT&) const
        {
        return ThreadData(idx);
        }

    __device__ __forceinline__ void process(ThreadData& t, const int) const { ++t.num_neigh; }

    __device__ __forceinline__ void finalize(const ThreadData& t) const { nneigh[t.idx] = t.num_neigh; }

    unsigned int* nneigh;
    };

struct NeighborListOp
    {
    NeighborListOp(unsigned int* neigh_list_, unsigned int* nneigh_, unsigned int max_neigh_)
        : neigh_list(neigh_list_), nneigh(nneigh_), max_neigh(max_neigh_)
        {}

    struct ThreadData
        {
        __device__ ThreadData(const unsigned int idx_, unsigned long long first_)
            : idx(idx_), first(first_), num_neigh(0)
            {}
        const int idx;
        const unsigned long long first;
        unsigned int num_neigh;
        };

    template<class QueryDataT>
    __device__ __forceinline__ ThreadData setup(const unsigned int idx, const QueryDataT&) const
        {
        return ThreadData(idx, (unsigned long long)max_neigh * idx);
        }

    __device__ __forceinline__ void process(ThreadData& t, const int primitive) const
        {
        if (t.num_neigh < max_neigh)
            neigh_list[t.first + t.num_neigh] = primitive;
        ++t.num_neigh;
        }

    __device__ __forceinline__ void finalize(const ThreadData& t) const { nneigh[t.idx] = t.num_neigh; }

    unsigned int* neigh_list;
    unsigned int* nneigh;
    const unsigned int max_neigh;
    };

// Addition: rows of individual capacity in one array.  Row idx occupies
// [offsets[idx], offsets[idx] + capacity[idx]); entries past the capacity are dropped and the full
// count is always written, so nneigh[idx] > capacity[idx] signals that the row overflowed.  With
// capacity = the exact counts and offsets = their exclusive scan this is a compact CSR list.
// max_capacity, when known (an upper bound of every capacity), lets self traversals take the
// symmetric kernels; 0 means unknown.
struct CSRNeighborListOp
    {
    CSRNeighborListOp(unsigned int* neigh_list_, unsigned int* nneigh_,
                      const unsigned long long* offsets_, const unsigned int* capacity_,
                      unsigned int max_capacity_ = 0)
        : neigh_list(neigh_list_), nneigh(nneigh_), offsets(offsets_), capacity(capacity_),
          max_capacity(max_capacity_)
        {}

    struct ThreadData
        {
        __device__ ThreadData(const unsigned int idx_, unsigned long long first_, unsigned int cap_)
            : idx(idx_), first(first_), cap(cap_), num_neigh(0)
            {}
        const int idx;
        const unsigned long long first;
        const unsigned int cap;
        unsigned int num_neigh;
        };

    template<class QueryDataT>
    __device__ __forceinline__ ThreadData setup(const unsigned int idx, const QueryDataT&) const
        {
        return ThreadData(idx, offsets[idx], capacity[idx]);
        }

    __device__ __forceinline__ void process(ThreadData& t, const int primitive) const
        {
        if (t.num_neigh < t.cap)
            neigh_list[t.first + t.num_neigh] = primitive;
        ++t.num_neigh;
        }

    __device__ __forceinline__ void finalize(const ThreadData& t) const { nneigh[t.idx] = t.num_neigh; }

    unsigned int* neigh_list;
    unsigned int* nneigh;
    const unsigned long long* offsets;
    const unsigned int* capacity;
    unsigned int max_capacity;
    };

// Trait used to route a traversal to the specialised fast kernels.  0 = generic op.
template<class OutputOpT> struct output_kind { static constexpr int value = 0; };
template<> struct output_kind<CountNeighborsOp> { static constexpr int value = 1; };
template<> struct output_kind<NeighborListOp> { static constexpr int value = 2; };
template<> struct output_kind<CSRNeighborListOp> { static constexpr int value = 3; };

} // namespace neighbor

#endif // NEIGHBOR_OUTPUT_OPS_H_
