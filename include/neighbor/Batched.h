// Batched ensembles of independent small periodic systems (an addition of this library).
//
// A simulation ensemble, a parameter sweep or a set of replicas gives thousands of small systems
// (tens to tens of thousands of points each).  Building and traversing them one by one costs a
// dozen launches and a host synchronisation per system; here one persistent kernel
// (kernels/batch.cuh) does every system's build and self neighbor list, each system inside one
// block.  The launch can be captured once in a CUDA graph and replayed every step.  A small
// autotuner picks the leaf size and block shape by timing the candidates on the actual batch.
// Results per system are those of LBVH::build + LBVHTraverser::traverseSelf on that system
// alone (27 periodic images of its box, exact predicate), with global row and id numbering.
#ifndef NEIGHBOR_BATCHED_H_
#define NEIGHBOR_BATCHED_H_

#include <algorithm>
#include <numeric>
#include <stdexcept>
#include <vector>

#include <cuda_runtime.h>

#include "LBVH.h"
#include "Memory.h"
#include "Trace.h"
#include "QueryOps.h"
#include "kernels/batch.cuh"

namespace neighbor
{

class BatchedNeighborList
    {
    public:
        struct Config
            {
            unsigned int leaf_size;
            unsigned int block;  // threads per block: 512 or 1024
            };

        BatchedNeighborList() : m_S(0), m_total(0), m_rc(0.f), m_max_neigh(0), m_graph(nullptr), m_exec(nullptr)
            {
            m_cfg.leaf_size = 4;
            m_cfg.block = 512;
            }
        ~BatchedNeighborList() { release_graph(); }
        BatchedNeighborList(const BatchedNeighborList&) = delete;
        BatchedNeighborList& operator=(const BatchedNeighborList&) = delete;

        static unsigned int maxSystemSize() { return gpu::kBatchMaxN; }

        // Describe the batch: system s holds points [start[s], start[s+1]) (host array of S + 1),
        // periodic box lengths box[3 s .. 3 s + 2] (host), cutoff rc, list capacity per point.
        void setup(const unsigned int* start, const float* box, unsigned int S, float rc, unsigned int max_neigh)
            {
            release_graph();
            std::vector<unsigned int> st(start, start + S + 1);
            std::vector<float3> bx(S);
            std::vector<float> pad(S);
            for (unsigned int s = 0; s < S; ++s)
                {
                if (st[s + 1] < st[s]) throw std::runtime_error("Batch offsets must not decrease.");
                if (st[s + 1] - st[s] > gpu::kBatchMaxN)
                    throw std::runtime_error("A batched system must have at most 16384 points.");
                bx[s] = make_float3(box[3 * s], box[3 * s + 1], box[3 * s + 2]);
                pad[s] = exact_query_pad(rc, 2.f * std::max(bx[s].x, std::max(bx[s].y, bx[s].z)));
                }
            // largest systems first: the last systems to finish are the small ones
            std::vector<unsigned int> order(S);
            std::iota(order.begin(), order.end(), 0u);
            std::stable_sort(order.begin(), order.end(), [&st](unsigned int x, unsigned int y) {
                return st[x + 1] - st[x] > st[y + 1] - st[y];
            });
            m_S = S;
            m_total = st[S];
            m_rc = rc;
            m_max_neigh = max_neigh;
            m_start.reserve(S + 1);
            m_box.reserve(std::max(S, 1u));
            m_pad.reserve(std::max(S, 1u));
            m_order.reserve(std::max(S, 1u));
            detail::check_cuda(cudaMemcpy(m_start.get(), st.data(), (S + 1) * sizeof(unsigned int), cudaMemcpyHostToDevice), "copy");
            if (S)
                {
                detail::check_cuda(cudaMemcpy(m_box.get(), bx.data(), S * sizeof(float3), cudaMemcpyHostToDevice), "copy");
                detail::check_cuda(cudaMemcpy(m_pad.get(), pad.data(), S * sizeof(float), cudaMemcpyHostToDevice), "copy");
                detail::check_cuda(cudaMemcpy(m_order.get(), order.data(), S * sizeof(unsigned int), cudaMemcpyHostToDevice), "copy");
                }
            const size_t T = std::max(m_total, 1u);
            m_records.reserve(2 * T);
            m_payload.reserve(T);
            m_nbox.reserve(T);
            m_nmeta.reserve(T);
            m_kids.reserve(2 * T);
            m_pre.reserve(T + S + 1);
            m_small.reserve(4);
            detail::check_cuda(cudaFuncSetAttribute(gpu::k_batch_systems<512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)gpu::kBatchSmemBytes), "batch attribute");
            detail::check_cuda(cudaFuncSetAttribute(gpu::k_batch_systems<1024>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)gpu::kBatchSmemBytes), "batch attribute");
            int dev = 0;
            detail::check_cuda(cudaGetDevice(&dev), "device");
            detail::check_cuda(cudaDeviceGetAttribute(&m_sms, cudaDevAttrMultiProcessorCount, dev), "attribute");
            }

        // Every system's build and self list in one launch (plus one memset of its counters).
        void run(const float3* points, unsigned int* nneigh, unsigned int* list, cudaStream_t stream, const Config& cfg)
            {
            const detail::TraceRange trace_range("neighbor::BatchedNeighborList::run");
            if (cfg.block != 512 && cfg.block != 1024) throw std::runtime_error("Batch block must be 512 or 1024.");
            if (cfg.leaf_size < 1 || cfg.leaf_size > 64) throw std::runtime_error("Leaf size must be in [1, 64].");
            detail::check_cuda(cudaMemsetAsync(m_small.get(), 0, 4 * sizeof(unsigned int), stream), "memset");
            if (m_S == 0) return;
            gpu::BatchArgs a;
            a.points = points;
            a.start = m_start.get();
            a.box = m_box.get();
            a.pad = m_pad.get();
            a.order = m_order.get();
            a.S = m_S;
            a.rc = m_rc;
            unsigned int leaf = 1;
            while (leaf < cfg.leaf_size) leaf <<= 1;
            a.leaf_size = leaf;
            a.max_neigh = m_max_neigh;
            a.nneigh = nneigh;
            a.list = list;
            a.records = m_records.get();
            a.payload = m_payload.get();
            a.nbox = m_nbox.get();
            a.nmeta = m_nmeta.get();
            a.kids = m_kids.get();
            a.pre = m_pre.get();
            a.next = m_small.get();
            a.status = m_small.get() + 1;
            const unsigned int grid = (unsigned int)std::min<long long>(m_sms, (long long)m_S);
            if (cfg.block == 1024)
                gpu::k_batch_systems<1024><<<grid, 1024, gpu::kBatchSmemBytes, stream>>>(a);
            else
                gpu::k_batch_systems<512><<<grid, 512, gpu::kBatchSmemBytes, stream>>>(a);
            detail::check_cuda(cudaGetLastError(), "batch launch");
            }
        void run(const float3* points, unsigned int* nneigh, unsigned int* list, cudaStream_t stream)
            {
            run(points, nneigh, list, stream, m_cfg);
            }

        // Time every candidate configuration on this batch (one untimed and two timed runs each)
        // and keep the fastest; returns it.
        Config tune(const float3* points, unsigned int* nneigh, unsigned int* list, cudaStream_t stream)
            {
            cudaEvent_t e0, e1;
            detail::check_cuda(cudaEventCreate(&e0), "event");
            detail::check_cuda(cudaEventCreate(&e1), "event");
            float best = 1e30f;
            Config best_cfg = m_cfg;
            for (unsigned int block : {512u, 1024u})
                for (unsigned int leaf : {1u, 2u, 4u, 8u})
                    {
                    const Config c{leaf, block};
                    run(points, nneigh, list, stream, c);
                    detail::check_cuda(cudaEventRecord(e0, stream), "record");
                    run(points, nneigh, list, stream, c);
                    run(points, nneigh, list, stream, c);
                    detail::check_cuda(cudaEventRecord(e1, stream), "record");
                    detail::check_cuda(cudaEventSynchronize(e1), "sync");
                    float ms = 0.f;
                    detail::check_cuda(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
                    if (ms < best)
                        {
                        best = ms;
                        best_cfg = c;
                        }
                    }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            m_cfg = best_cfg;
            return best_cfg;
            }

        void setConfig(const Config& cfg) { m_cfg = cfg; }
        Config getConfig() const { return m_cfg; }

        // Capture run() with the current configuration into a CUDA graph on `stream` (which must
        // not be the legacy default stream); replay() launches it.
        void capture(const float3* points, unsigned int* nneigh, unsigned int* list, cudaStream_t stream)
            {
            release_graph();
            detail::check_cuda(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "begin capture");
            run(points, nneigh, list, stream, m_cfg);
            detail::check_cuda(cudaStreamEndCapture(stream, &m_graph), "end capture");
            detail::check_cuda(cudaGraphInstantiate(&m_exec, m_graph, 0), "instantiate");
            }
        void replay(cudaStream_t stream)
            {
            if (!m_exec) throw std::runtime_error("No captured batch to replay.");
            detail::check_cuda(cudaGraphLaunch(m_exec, stream), "graph launch");
            }

        // Status of the last run (synchronises the stream): BatchStatus bits and the largest count.
        void status(cudaStream_t stream, unsigned int* bits, unsigned int* largest) const
            {
            unsigned int h[2] = {0u, 0u};
            detail::check_cuda(cudaMemcpyAsync(h, m_small.get() + 1, sizeof(h), cudaMemcpyDeviceToHost, stream), "copy");
            detail::check_cuda(cudaStreamSynchronize(stream), "sync");
            if (bits) *bits = h[0];
            if (largest) *largest = h[1];
            }

        unsigned int numSystems() const { return m_S; }
        unsigned int numPoints() const { return m_total; }

    private:
        unsigned int m_S;
        unsigned int m_total;
        float m_rc;
        unsigned int m_max_neigh;
        int m_sms = 1;
        Config m_cfg;
        cudaGraph_t m_graph;
        cudaGraphExec_t m_exec;
        device_array<unsigned int> m_start;
        device_array<float3> m_box;
        device_array<float> m_pad;
        device_array<unsigned int> m_order;
        device_array<uint4> m_records;
        device_array<float4> m_payload;
        device_array<uint4> m_nbox;
        device_array<uint2> m_nmeta;
        device_array<unsigned int> m_kids;
        device_array<unsigned int> m_pre;
        device_array<unsigned int> m_small;

        void release_graph()
            {
            if (m_exec) cudaGraphExecDestroy(m_exec);
            if (m_graph) cudaGraphDestroy(m_graph);
            m_exec = nullptr;
            m_graph = nullptr;
            }
    };

} // namespace neighbor

#endif // NEIGHBOR_BATCHED_H_
