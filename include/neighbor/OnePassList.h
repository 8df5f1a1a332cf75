// One-pass self neighbor list with per-row capacities (an addition of this library).
//
// The reference fills a neighbor list in two traversals: count, read the largest count on the
// host, then fill rows of that fixed stride.  Here the rows get individual capacities before any
// traversal -- predicted by a CapacityModel, or given by the caller -- and one traversal fills a
// CSR list (row r at offsets[r], capacity caps[r]).  Every count is exact even when a row
// overflows, so the rows that overflowed are re-run with exactly their count of slots, appended
// after the main list, by a whole-tree walk of just those queries.  The result is always the
// exact list, in the same row order as every other self traversal of this library.
#ifndef NEIGHBOR_ONE_PASS_LIST_H_
#define NEIGHBOR_ONE_PASS_LIST_H_

#include <cuda_runtime.h>

#include "CapacityModel.h"
#include "LBVH.h"
#include "LBVHTraverser.h"
#include "Memory.h"
#include "Trace.h"
#include "OutputOps.h"
#include "TransformOps.h"
#include "TranslateOps.h"
#include "kernels/capacity.cuh"

namespace neighbor
{
namespace gpu
{
// Sorted positions whose row overflowed, with their exact counts, in ascending order (so the
// appended space is laid out the same way on every run): k_overflow_count counts them per block,
// k_scan64_sums turns the counts into block offsets, k_overflow_write writes them in order.
constexpr int kOverflowBlock = 256;

__device__ __forceinline__ bool row_overflows(unsigned int q, unsigned int N, int rows_sorted,
                                              const unsigned int* __restrict__ primitive,
                                              const unsigned int* __restrict__ nneigh,
                                              const unsigned int* __restrict__ caps, unsigned int& count)
    {
    if (q >= N) return false;
    const unsigned int row = rows_sorted ? q : primitive[q];
    count = nneigh[row];
    return count > caps[row];
    }

static __global__ void __launch_bounds__(kOverflowBlock) k_overflow_count(unsigned int N, int rows_sorted,
                                                                          const unsigned int* __restrict__ primitive,
                                                                          const unsigned int* __restrict__ nneigh,
                                                                          const unsigned int* __restrict__ caps,
                                                                          unsigned long long* __restrict__ block_count)
    {
    __shared__ unsigned int s_n;
    if (threadIdx.x == 0) s_n = 0u;
    __syncthreads();
    unsigned int c;
    const bool ovf = row_overflows(blockIdx.x * blockDim.x + threadIdx.x, N, rows_sorted, primitive, nneigh, caps, c);
    const unsigned int w = __ballot_sync(0xffffffffu, ovf);
    if ((threadIdx.x & 31u) == 0u && w) atomicAdd(&s_n, (unsigned int)__popc(w));
    __syncthreads();
    if (threadIdx.x == 0) block_count[blockIdx.x] = s_n;
    }

static __global__ void __launch_bounds__(kOverflowBlock) k_overflow_write(unsigned int N, int rows_sorted,
                                                                          const unsigned int* __restrict__ primitive,
                                                                          const unsigned int* __restrict__ nneigh,
                                                                          const unsigned int* __restrict__ caps,
                                                                          const unsigned long long* __restrict__ block_base,
                                                                          unsigned int* __restrict__ ovf_q,
                                                                          unsigned int* __restrict__ ovf_count)
    {
    __shared__ unsigned int s_warp[kOverflowBlock / 32];
    const unsigned int q = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned int c = 0;
    const bool ovf = row_overflows(q, N, rows_sorted, primitive, nneigh, caps, c);
    const unsigned int w = __ballot_sync(0xffffffffu, ovf);
    const unsigned int lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    if (lane == 0u) s_warp[warp] = __popc(w);
    __syncthreads();
    unsigned int before = 0;
    for (unsigned int k = 0; k < warp; ++k) before += s_warp[k];
    if (ovf)
        {
        const unsigned int k = (unsigned int)block_base[blockIdx.x] + before + __popc(w & lanemask_lt());
        ovf_q[k] = q;
        ovf_count[k] = c;
        }
    }

// Re-point the overflowed rows at their exact space after the main list.
static __global__ void __launch_bounds__(256) k_overflow_assign(unsigned int n, int rows_sorted,
                                                                const unsigned int* __restrict__ primitive,
                                                                const unsigned int* __restrict__ ovf_q,
                                                                const unsigned int* __restrict__ ovf_count,
                                                                const unsigned long long* __restrict__ ovf_off,
                                                                unsigned long long base,
                                                                unsigned long long* __restrict__ offsets,
                                                                unsigned int* __restrict__ caps)
    {
    const unsigned int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const unsigned int q = ovf_q[k];
    const unsigned int row = rows_sorted ? q : primitive[q];
    offsets[row] = base + ovf_off[k];
    caps[row] = ovf_count[k];
    }
} // namespace gpu

class OnePassNeighborList
    {
    public:
        struct Stats
            {
            unsigned long long slots;           // slots of the main list (sum of capacities)
            unsigned int overflow_rows;         // rows re-run
            unsigned long long overflow_slots;  // slots appended for them
            };

        OnePassNeighborList() : m_N(0), m_total(0), m_side(nullptr), m_pred_done(nullptr) {}
        ~OnePassNeighborList()
            {
            if (m_pred_done) cudaEventDestroy(m_pred_done);
            if (m_side) cudaStreamDestroy(m_side);
            }
        OnePassNeighborList(const OnePassNeighborList&) = delete;
        OnePassNeighborList& operator=(const OnePassNeighborList&) = delete;

        // Capacity array of N rows for the caller (or a CapacityModel) to fill before build().
        unsigned int* capacity(unsigned int N)
            {
            m_caps.reserve(N);
            return m_caps.get();
            }

        // Exclusive scan of n 32-bit values into 64-bit offsets; returns the total (synchronises)
        // unless read_total is false (the total then stays on the device).
        unsigned long long scan(const unsigned int* in, unsigned int n, unsigned long long* out, cudaStream_t stream,
                                bool read_total = true)
            {
            const unsigned int tiles = detail::ceil_div(n, gpu::kScan64Tile);
            m_tiles.reserve((size_t)tiles + 1);
            gpu::k_scan64_tiles<<<tiles, gpu::kScan64Block, 0, stream>>>(in, n, m_tiles.get());
            gpu::k_scan64_sums<<<1, 1024, 0, stream>>>(m_tiles.get(), tiles, m_tiles.get() + tiles);
            gpu::k_scan64_apply<<<tiles, gpu::kScan64Block, 0, stream>>>(in, n, m_tiles.get(), out);
            detail::check_cuda(cudaGetLastError(), "scan launch");
            if (!read_total) return 0ull;
            unsigned long long total = 0;
            detail::check_cuda(cudaMemcpyAsync(&total, m_tiles.get() + tiles, sizeof(total), cudaMemcpyDeviceToHost,
                                               stream), "copy");
            detail::check_cuda(cudaStreamSynchronize(stream), "sync");
            return total;
            }

        // Fill the list of every point of `lbvh` (self queries, cutoff rc, periodic box or open),
        // rows sized by capacity(); cap_max bounds every capacity (for the symmetric traversal).
        template<class TransformOpT = NullTransformOp>
        Stats build(const LBVHTraverser::LaunchParameters& params, const LBVH& lbvh, LBVHTraverser& trav, float rc, float3 box,
                    float pad, bool periodic, bool rows_sorted, unsigned int cap_max,
                    const TransformOpT& transform = TransformOpT())
            {
            const detail::TraceRange trace_range("neighbor::OnePassNeighborList::build");
            Stats st = {0, 0, 0};
            const unsigned int N = lbvh.getN();
            m_N = N;
            if (N == 0) return st;
            cudaStream_t stream = params.stream;
            m_caps.reserve(N);
            m_nneigh.reserve(N);
            m_offsets.reserve(N);
            // With small capacities the list is sized N * cap_max up front and the total stays on the
            // device until the overflow check (no wait for the GPU before the traversal).
            const unsigned long long bound = (unsigned long long)N * cap_max;
            const bool presized = bound <= kPresizeSlots;
            if (presized) m_list.grow(bound + 1, 0, stream);
            st.slots = scan(m_caps.get(), N, m_offsets.get(), stream, !presized);
            if (!presized) m_list.grow(st.slots + 1, 0, stream);
            const CSRNeighborListOp out(m_list.get(), m_nneigh.get(), m_offsets.get(), m_caps.get(), cap_max);
            if (periodic)
                trav.traverseSelf(params, lbvh, rc, box, pad, out, PeriodicImagesOp(box), transform, rows_sorted);
            else
                trav.traverseSelf(params, lbvh, rc, make_float3(0.f, 0.f, 0.f), pad, out, SelfOp(), transform,
                                  rows_sorted);

            // rows that overflowed: exact counts are known, re-run them into appended space
            m_ovf_q.reserve(N);
            m_ovf_count.reserve(N);
            m_ovf_off.reserve(N);
            const unsigned int blocks = detail::ceil_div(N, gpu::kOverflowBlock);
            m_ovf_blocks.reserve((size_t)blocks + 1);
            gpu::k_overflow_count<<<blocks, gpu::kOverflowBlock, 0, stream>>>(
                N, rows_sorted ? 1 : 0, lbvh.fastData().primitive, m_nneigh.get(), m_caps.get(), m_ovf_blocks.get());
            gpu::k_scan64_sums<<<1, 1024, 0, stream>>>(m_ovf_blocks.get(), blocks, m_ovf_blocks.get() + blocks);
            gpu::k_overflow_write<<<blocks, gpu::kOverflowBlock, 0, stream>>>(
                N, rows_sorted ? 1 : 0, lbvh.fastData().primitive, m_nneigh.get(), m_caps.get(), m_ovf_blocks.get(),
                m_ovf_q.get(), m_ovf_count.get());
            detail::check_cuda(cudaGetLastError(), "overflow launch");
            unsigned long long n_ovf64 = 0;
            detail::check_cuda(cudaMemcpyAsync(&n_ovf64, m_ovf_blocks.get() + blocks, sizeof(n_ovf64),
                                               cudaMemcpyDeviceToHost, stream), "copy");
            detail::check_cuda(cudaStreamSynchronize(stream), "sync");
            const unsigned int n_ovf = (unsigned int)n_ovf64;
            st.overflow_rows = n_ovf;
            if (presized)
                {
                // the stream is idle here (synchronised above)
                const unsigned int tiles = detail::ceil_div(N, gpu::kScan64Tile);
                detail::check_cuda(cudaMemcpy(&st.slots, m_tiles.get() + tiles, sizeof(st.slots),
                                              cudaMemcpyDeviceToHost), "copy");
                }
            m_total = st.slots;
            if (n_ovf)
                {
                st.overflow_slots = scan(m_ovf_count.get(), n_ovf, m_ovf_off.get(), stream);
                m_list.grow(st.slots + st.overflow_slots + 1, st.slots, stream);
                gpu::k_overflow_assign<<<detail::ceil_div(n_ovf, 256), 256, 0, stream>>>(
                    n_ovf, rows_sorted ? 1 : 0, lbvh.fastData().primitive, m_ovf_q.get(), m_ovf_count.get(),
                    m_ovf_off.get(), st.slots, m_offsets.get(), m_caps.get());
                detail::check_cuda(cudaGetLastError(), "overflow assign launch");
                const CSRNeighborListOp exact(m_list.get(), m_nneigh.get(), m_offsets.get(), m_caps.get(), 0u);
                if (periodic)
                    trav.traverseSelfSubset(params, lbvh, rc, box, pad, exact, PeriodicImagesOp(box), transform,
                                            rows_sorted, m_ovf_q.get(), n_ovf);
                else
                    trav.traverseSelfSubset(params, lbvh, rc, make_float3(0.f, 0.f, 0.f), pad, exact, SelfOp(),
                                            transform, rows_sorted, m_ovf_q.get(), n_ovf);
                m_total += st.overflow_slots;
                }
            return st;
            }

        // The learned one-pass step in one call: build the tree of `points`, predict every row's
        // capacity with `model`, fill the list.  The prediction needs only the sort's output: the
        // warp-tile kernel runs on a second stream from LBVH::sortedEvent() on, alongside the rest
        // of the build; the tcgen05 kernel runs after the build on the caller's stream (16M
        // points: 9.01 ms per step there against 9.48 ms beside the build, where its blocks hold
        // back the climb's; the warp-tile kernel 9.07 beside, 9.10 after).
        template<class TransformOpT = NullTransformOp>
        Stats buildLearned(const LBVHTraverser::LaunchParameters& params, LBVH& lbvh, LBVHTraverser& trav,
                           CapacityModel& model, const float3* points, unsigned int N, const float3& lo,
                           const float3& hi, float rc, float3 box, float pad, bool periodic, bool rows_sorted,
                           unsigned int cap_max, const TransformOpT& transform = TransformOpT())
            {
            const detail::TraceRange trace_range("neighbor::OnePassNeighborList::buildLearned");
            cudaStream_t stream = params.stream;
            lbvh.build(params, PointInsertOp(points, N), lo, hi);
            if (N == 0) return build(params, lbvh, trav, rc, box, pad, periodic, rows_sorted, cap_max, transform);
            unsigned int* caps = capacity(N);
            if (N < 2)
                {
                const unsigned int one = 1u;
                detail::check_cuda(cudaMemcpy(caps, &one, sizeof(one), cudaMemcpyHostToDevice), "copy");
                return build(params, lbvh, trav, rc, box, pad, periodic, rows_sorted, cap_max, transform);
                }
            if (model.getInferKernel() == CapacityModel::InferKernel::TensorMemory)
                {
                model.predictSorted(lbvh.getCodes().get(), lbvh.getPrimitives().get(), points, N,
                                    CapacityModel::frame(lo, hi, rc, periodic), rows_sorted, cap_max, caps, nullptr,
                                    stream);
                return build(params, lbvh, trav, rc, box, pad, periodic, rows_sorted, cap_max, transform);
                }
            if (!m_side)
                {
                // highest priority: the prediction's blocks take SMs as soon as blocks of the build's
                // later kernels retire, instead of queueing behind all of them
                int least = 0, greatest = 0;
                detail::check_cuda(cudaDeviceGetStreamPriorityRange(&least, &greatest), "priority range");
                detail::check_cuda(cudaStreamCreateWithPriority(&m_side, cudaStreamNonBlocking, greatest),
                                   "stream create");
                detail::check_cuda(cudaEventCreateWithFlags(&m_pred_done, cudaEventDisableTiming), "event create");
                }
            detail::check_cuda(cudaStreamWaitEvent(m_side, lbvh.sortedEvent(), 0), "wait");
            model.predictSorted(lbvh.getCodes().get(), lbvh.getPrimitives().get(), points, N,
                                CapacityModel::frame(lo, hi, rc, periodic), rows_sorted, cap_max, caps, nullptr,
                                m_side);
            detail::check_cuda(cudaEventRecord(m_pred_done, m_side), "event record");
            detail::check_cuda(cudaStreamWaitEvent(stream, m_pred_done, 0), "wait");
            return build(params, lbvh, trav, rc, box, pad, periodic, rows_sorted, cap_max, transform);
            }

        const unsigned int* list() const { return m_list.get(); }
        const unsigned long long* offsets() const { return m_offsets.get(); }
        const unsigned int* capacities() const { return m_caps.get(); }
        const unsigned int* nneigh() const { return m_nneigh.get(); }
        unsigned long long totalSlots() const { return m_total; }

    private:
        static constexpr unsigned long long kPresizeSlots = 1ull << 29;  // 2 GB of entries
        unsigned int m_N;
        unsigned long long m_total;
        device_array<unsigned int> m_caps;
        device_array<unsigned int> m_nneigh;
        device_array<unsigned long long> m_offsets;
        device_array<unsigned int> m_list;
        device_array<unsigned int> m_ovf_q;
        device_array<unsigned int> m_ovf_count;
        device_array<unsigned long long> m_ovf_off;
        device_array<unsigned long long> m_tiles;
        device_array<unsigned long long> m_ovf_blocks;
        cudaStream_t m_side;
        cudaEvent_t m_pred_done;
    };

} // namespace neighbor

#endif // NEIGHBOR_ONE_PASS_LIST_H_
