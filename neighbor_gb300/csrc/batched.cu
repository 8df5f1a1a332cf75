// C ABI of batched ensembles (include/neighbor_gb300.h): the one-launch batched form and, for
// comparison, the same work as one plain two-pass call per system.
#include <algorithm>
#include <vector>

#include <cuda_runtime.h>

#include "capi_internal.h"
#include "neighbor/Batched.h"

struct nbr_batch_s
    {
    neighbor::BatchedNeighborList batch;
    };

namespace
{
using neighbor_capi::as_stream;
using neighbor_capi::fail;
using neighbor_capi::guarded;
using neighbor_capi::valid_block;

// Largest value of counts[0..n) into *out (one block).
__global__ void k_max_u32(const unsigned int* __restrict__ counts, unsigned int n, unsigned int* __restrict__ out)
    {
    __shared__ unsigned int s_max[32];
    unsigned int m = 0u;
    for (unsigned int i = threadIdx.x; i < n; i += blockDim.x) m = max(m, counts[i]);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31u) == 0u) s_max[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0)
        {
        unsigned int r = 0u;
        for (unsigned int w = 0; w < blockDim.x / 32u; ++w) r = max(r, s_max[w]);
        *out = r;
        }
    }
} // namespace

extern "C" {

int nbr_batch_create(nbr_batch* out)
    {
    if (!out) return fail(NBR_ERR_INVALID, "null output handle");
    return guarded([&] { *out = new nbr_batch_s(); });
    }

int nbr_batch_destroy(nbr_batch b)
    {
    return guarded([&] { delete b; });
    }

int nbr_batch_setup(nbr_batch b, const unsigned int* start, const float* box, unsigned int S, float rc,
                    unsigned int max_neigh)
    {
    if (!b || !start || (S > 0 && !box)) return fail(NBR_ERR_INVALID, "null argument");
    return guarded([&] { b->batch.setup(start, box, S, rc, max_neigh); });
    }

int nbr_batch_set_config(nbr_batch b, unsigned int leaf_size, unsigned int block)
    {
    if (!b) return fail(NBR_ERR_INVALID, "null handle");
    if (block != 512 && block != 1024) return fail(NBR_ERR_INVALID, "batch block must be 512 or 1024");
    if (leaf_size < 1 || leaf_size > 64) return fail(NBR_ERR_INVALID, "leaf size must be in [1, 64]");
    b->batch.setConfig(neighbor::BatchedNeighborList::Config{leaf_size, block});
    return NBR_OK;
    }

int nbr_batch_get_config(nbr_batch b, unsigned int* leaf_size, unsigned int* block)
    {
    if (!b) return fail(NBR_ERR_INVALID, "null handle");
    const auto c = b->batch.getConfig();
    if (leaf_size) *leaf_size = c.leaf_size;
    if (block) *block = c.block;
    return NBR_OK;
    }

int nbr_batch_run(nbr_batch b, const float* points, unsigned int* nneigh, unsigned int* list, void* stream)
    {
    if (!b) return fail(NBR_ERR_INVALID, "null handle");
    if (b->batch.numPoints() > 0 && (!points || !nneigh || !list)) return fail(NBR_ERR_INVALID, "null argument");
    return guarded([&] {
        b->batch.run(reinterpret_cast<const float3*>(points), nneigh, list, as_stream(stream));
    });
    }

int nbr_batch_tune(nbr_batch b, const float* points, unsigned int* nneigh, unsigned int* list, void* stream,
                   unsigned int* leaf_size, unsigned int* block)
    {
    if (!b) return fail(NBR_ERR_INVALID, "null handle");
    if (b->batch.numPoints() > 0 && (!points || !nneigh || !list)) return fail(NBR_ERR_INVALID, "null argument");
    return guarded([&] {
        const auto c = b->batch.tune(reinterpret_cast<const float3*>(points), nneigh, list, as_stream(stream));
        if (leaf_size) *leaf_size = c.leaf_size;
        if (block) *block = c.block;
    });
    }

int nbr_batch_capture(nbr_batch b, const float* points, unsigned int* nneigh, unsigned int* list, void* stream)
    {
    if (!b || !stream) return fail(NBR_ERR_INVALID, "capture needs a handle and a stream other than the default");
    return guarded([&] {
        b->batch.capture(reinterpret_cast<const float3*>(points), nneigh, list, as_stream(stream));
    });
    }

int nbr_batch_replay(nbr_batch b, void* stream)
    {
    if (!b) return fail(NBR_ERR_INVALID, "null handle");
    return guarded([&] { b->batch.replay(as_stream(stream)); });
    }

int nbr_batch_status(nbr_batch b, unsigned int* bits, unsigned int* largest, void* stream)
    {
    if (!b) return fail(NBR_ERR_INVALID, "null handle");
    return guarded([&] { b->batch.status(as_stream(stream), bits, largest); });
    }

int nbr_batch_sequential_plain(nbr_lbvh h, nbr_traverser t, const float* points, const unsigned int* start,
                               const float* box, unsigned int S, float rc, unsigned int* nneigh, unsigned int* list,
                               unsigned int max_neigh, unsigned int block_size, void* stream)
    {
    if (!h || !t || !start || (S > 0 && (!box || !points || !nneigh || !list)))
        return fail(NBR_ERR_INVALID, "null argument");
    if (!valid_block(block_size)) return fail(NBR_ERR_INVALID, "Invalid tuning parameter.");
    return guarded([&] {
        cudaStream_t st = as_stream(stream);
        const neighbor::LBVH::LaunchParameters p(block_size, st);
        neighbor::device_array<unsigned int> dmax;
        dmax.reserve(1);
        for (unsigned int s = 0; s < S; ++s)
            {
            const unsigned int o = start[s];
            const unsigned int N = start[s + 1] - o;
            if (N == 0) continue;
            const float3 L = make_float3(box[3 * s], box[3 * s + 1], box[3 * s + 2]);
            const float pad = neighbor::exact_query_pad(rc, 2.f * std::max(L.x, std::max(L.y, L.z)));
            const float3* pts = reinterpret_cast<const float3*>(points) + o;
            h->lbvh.build(p, neighbor::PointInsertOp(pts, N), make_float3(0.f, 0.f, 0.f), L);
            // count, read the largest count, fill (the reference's two-pass pattern)
            t->trav.traverseSelf(p, h->lbvh, rc, L, pad, neighbor::CountNeighborsOp(nneigh + o),
                                 neighbor::PeriodicImagesOp(L), neighbor::NullTransformOp(), false);
            k_max_u32<<<1, 256, 0, st>>>(nneigh + o, N, dmax.get());
            unsigned int mx = 0;
            neighbor::detail::check_cuda(cudaMemcpyAsync(&mx, dmax.get(), sizeof(mx), cudaMemcpyDeviceToHost, st), "copy");
            neighbor::detail::check_cuda(cudaStreamSynchronize(st), "sync");
            if (mx > max_neigh) throw std::runtime_error("sequential batch: a count exceeds max_neigh");
            t->trav.traverseSelf(p, h->lbvh, rc, L, pad,
                                 neighbor::NeighborListOp(list + (size_t)o * max_neigh, nneigh + o, max_neigh),
                                 neighbor::PeriodicImagesOp(L), neighbor::NullTransformOp(), false);
            }
    });
    }

} // extern "C"
