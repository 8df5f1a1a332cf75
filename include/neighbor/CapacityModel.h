// Learned neighbor capacity (an addition of this library; the reference has no counterpart).
//
// A small network predicts, for every point of a tree, how many neighbors its self query will
// find, from the occupancy of the coarse Morton cells around it (kernels/capacity.cuh has the
// features, the network and its kernels).  The predictions size the rows of a one-pass neighbor
// list (OnePassNeighborList): one traversal instead of count-then-fill, and rows that turn out
// too small are re-run exactly, so the list is always exact.  The network is trained on the GPU
// by this library's own forward/backward kernels on exact counts from the plain method.
#ifndef NEIGHBOR_CAPACITY_MODEL_H_
#define NEIGHBOR_CAPACITY_MODEL_H_

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "LBVH.h"
#include "Memory.h"
#include "Trace.h"
#include "kernels/capacity.cuh"

namespace neighbor
{

class CapacityModel
    {
    public:
        static constexpr int kParams = gpu::kCapParams;
        static constexpr int kFeatures = gpu::kCapIn;

        explicit CapacityModel(unsigned long long seed = 1) : m_step(0), m_infer(InferKernel::TensorMemory)
            {
            setMargin(0.f);
            m_status.reserve(1);
            m_tiles.reserve(1);
            detail::check_cuda(cudaMemset(m_status.get(), 0, sizeof(unsigned int)), "memset");
            m_p.reserve(kParams);
            m_m.reserve(kParams);
            m_v.reserve(kParams);
            m_grad.reserve(kParams);
            m_loss.reserve(1);
            m_w.reserve(gpu::kCapBfWeights);
            reset(seed);
            }

        // He-uniform weights from a fixed generator, zero biases, output bias 2; Adam state cleared.
        void reset(unsigned long long seed)
            {
            std::vector<float> p(kParams, 0.f);
            unsigned long long s = seed * 0x9e3779b97f4a7c15ull + 0x632be59bd9b4e019ull;
            const auto uniform = [&s]() {
                s ^= s >> 12;
                s ^= s << 25;
                s ^= s >> 27;
                return (double)((s * 0x2545f4914f6cdd1dull) >> 11) * (1.0 / 9007199254740992.0);
            };
            const auto fill = [&](int off, int n, int fan_in) {
                const double r = std::sqrt(6.0 / fan_in);
                for (int i = 0; i < n; ++i) p[off + i] = (float)((2.0 * uniform() - 1.0) * r);
            };
            fill(gpu::kCapOffW1, gpu::kCapHidden * gpu::kCapIn, gpu::kCapIn);
            fill(gpu::kCapOffW2, gpu::kCapHidden * gpu::kCapHidden, gpu::kCapHidden);
            fill(gpu::kCapOffW3, gpu::kCapHidden, gpu::kCapHidden);
            p[gpu::kCapOffB3] = 2.f;
            setParams(p.data());
            m_step = 0;
            }

        // Coarse level for cutoff rc: the smallest shift whose cells are at least rc wide.
        static unsigned int levelFor(float rc, const float3& ext)
            {
            const float w = std::fmax(ext.x, std::fmax(ext.y, ext.z)) / 1024.f;
            unsigned int sh = 0;
            while (sh < 9 && w * (float)(1u << sh) < rc) ++sh;
            return sh;
            }

        // Frame of the features: the scene box the tree was built with.
        static gpu::CapFrame frame(const float3& lo, const float3& hi, float rc, bool periodic)
            {
            gpu::CapFrame f;
            f.lo = lo;
            f.ext = make_float3(hi.x - lo.x, hi.y - lo.y, hi.z - lo.z);
            f.shift = levelFor(rc, f.ext);
            f.periodic = periodic ? 1 : 0;
            return f;
            }

        // Occupancy grid of the tree's points at the frame's level.
        void occupancy(const LBVH& lbvh, const gpu::CapFrame& fr, cudaStream_t stream)
            {
            occupancy(lbvh.getCodes().get(), lbvh.getN(), fr, stream);
            }
        void occupancy(const unsigned int* codes, unsigned int N, const gpu::CapFrame& fr, cudaStream_t stream)
            {
            const size_t G = 1024u >> fr.shift;
            m_occ.reserve(G * G * G);
            detail::check_cuda(cudaMemsetAsync(m_occ.get(), 0, G * G * G * sizeof(unsigned int), stream), "memset");
            if (N < 2) return;
            gpu::k_cap_occupancy<<<detail::ceil_div(N, 256), 256, 0, stream>>>(codes, N, fr.shift, m_occ.get());
            detail::check_cuda(cudaGetLastError(), "occupancy launch");
            }

        // Features of every sorted point ([N][32] FP32).
        void features(const LBVH& lbvh, const gpu::CapFrame& fr, float* out, cudaStream_t stream)
            {
            const unsigned int N = lbvh.getN();
            if (N < 2) throw std::runtime_error("capacity features need a tree of at least two points");
            occupancy(lbvh, fr, stream);
            gpu::k_cap_features<<<detail::ceil_div(N, 256), 256, 0, stream>>>(
                fr, lbvh.getCodes().get(), lbvh.fastData().points, N, m_occ.get(), out);
            detail::check_cuda(cudaGetLastError(), "features launch");
            }

        // Capacity of every row (and optionally the network output y): features and network in
        // one kernel.  Rows are sorted positions (rows_sorted) or primitive ids.
        void predict(const LBVH& lbvh, const gpu::CapFrame& fr, bool rows_sorted, unsigned int cap_max,
                     unsigned int* caps, float* y, cudaStream_t stream)
            {
            const detail::TraceRange trace_range("neighbor::CapacityModel::predict");
            const unsigned int N = lbvh.getN();
            if (N < 2) throw std::runtime_error("capacity prediction needs a tree of at least two points");
            occupancy(lbvh, fr, stream);
            gpu::CapInferArgs a;
            a.frame = fr;
            a.codes = lbvh.getCodes().get();
            a.points = lbvh.fastData().points;
            a.points3 = nullptr;
            a.primitive = nullptr;
            a.N = N;
            infer(a, rows_sorted, cap_max, caps, y, stream);
            }

        // The same prediction from the sort's output alone (sorted codes, primitive order, the
        // original points), so that it can run while the rest of a build is still forming the
        // tree (LBVH::sortedEvent()).
        void predictSorted(const unsigned int* codes, const unsigned int* primitive, const float3* points,
                           unsigned int N, const gpu::CapFrame& fr, bool rows_sorted, unsigned int cap_max,
                           unsigned int* caps, float* y, cudaStream_t stream)
            {
            const detail::TraceRange trace_range("neighbor::CapacityModel::predictSorted");
            if (N < 2) throw std::runtime_error("capacity prediction needs a tree of at least two points");
            occupancy(codes, N, fr, stream);
            gpu::CapInferArgs a;
            a.frame = fr;
            a.codes = codes;
            a.points = nullptr;
            a.points3 = points;
            a.primitive = primitive;
            a.N = N;
            infer(a, rows_sorted, cap_max, caps, y, stream);
            }

    private:
        void infer(gpu::CapInferArgs& a, bool rows_sorted, unsigned int cap_max, unsigned int* caps, float* y,
                   cudaStream_t stream)
            {
            const unsigned int N = a.N;
            a.occ = m_occ.get();
            a.w = m_w.get();
            a.p = m_p.get();
            for (int b = 0; b < gpu::kCapMarginBins; ++b) a.margins[b] = m_margins[b];
            a.cap_max = cap_max;
            a.rows_sorted = rows_sorted ? 1 : 0;
            a.y_out = y;
            a.cap_out = caps;
            a.status = m_status.get();
            a.tile_counter = nullptr;
            int dev = 0, sms = 152;
            detail::check_cuda(cudaGetDevice(&dev), "device");
            detail::check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "attribute");
            if (m_infer == InferKernel::TensorMemory)
                {
                static bool attr = false;
                if (!attr)
                    {
                    detail::check_cuda(cudaFuncSetAttribute(gpu::k_cap_infer_tc,
                                                            cudaFuncAttributePreferredSharedMemoryCarveout,
                                                            (int)cudaSharedmemCarveoutMaxShared),
                                       "inference attribute");
                    attr = true;
                    }
                // persistent: kCapTcMinBlocks blocks of 128 queries per SM take the tiles from a
                // ticket counter
                const unsigned int tiles = detail::ceil_div(N, (unsigned int)gpu::kCapTcRows);
                const unsigned int grid = std::min(tiles, (unsigned int)sms * (unsigned int)gpu::kCapTcMinBlocks);
                detail::check_cuda(cudaMemsetAsync(m_tiles.get(), 0, sizeof(unsigned int), stream), "memset");
                a.tile_counter = m_tiles.get();
                gpu::k_cap_infer_tc<<<grid, gpu::kCapTcRows, 0, stream>>>(a);
                }
            else
                {
                // persistent: two blocks per SM (the kernel's register budget) walk all tiles
                const unsigned int tiles = detail::ceil_div(N, 32);
                const unsigned int grid =
                    std::min(detail::ceil_div(tiles, gpu::kCapInferWarps), (unsigned int)sms * 2u);
                gpu::k_cap_infer<<<grid, gpu::kCapInferWarps * 32, 0, stream>>>(a);
                }
            detail::check_cuda(cudaGetLastError(), "capacity inference launch");
            }

    public:
        // The inference kernel: warp tiles of mma.sync m16n8k16 (k_cap_infer) or 128-query tiles
        // on tcgen05 with Tensor Memory accumulators (k_cap_infer_tc).  Both give the same
        // capacities up to FP32 summation order.
        enum class InferKernel : int
            {
            WarpTiles = 0,
            TensorMemory = 1,
            };
        void setInferKernel(InferKernel k) { m_infer = k; }
        InferKernel getInferKernel() const { return m_infer; }

        // Device status word of the inference (gpu::kStatusTensorWait: a tensor-core wait gave up
        // and that prediction is incomplete).  Reads it and clears it; synchronises the device.
        unsigned int takeStatus()
            {
            unsigned int v = 0;
            detail::check_cuda(cudaMemcpy(&v, m_status.get(), sizeof(v), cudaMemcpyDeviceToHost), "copy");
            detail::check_cuda(cudaMemset(m_status.get(), 0, sizeof(v)), "memset");
            return v;
            }
        // Throws if a wait of the inference gave up.
        void checkStatus()
            {
            const unsigned int v = takeStatus();
            if (v & gpu::kStatusTensorWait)
                throw std::runtime_error("capacity inference: a wait for a tensor-core MMA gave up (output incomplete)");
            }

    public:
        // log1p(count) targets from exact counts.
        static void targets(const unsigned int* counts, unsigned int N, float* out, cudaStream_t stream)
            {
            gpu::k_cap_targets<<<detail::ceil_div(N, 256), 256, 0, stream>>>(counts, N, out);
            detail::check_cuda(cudaGetLastError(), "targets launch");
            }

        // Summed gradient and loss of one batch (rows offset + b*stride mod N), no update.
        void gradient(const float* features, const float* targets, unsigned int N, unsigned int batch,
                      unsigned int offset, unsigned int stride, float* grad, float* loss, cudaStream_t stream)
            {
            detail::check_cuda(cudaMemsetAsync(grad, 0, kParams * sizeof(float), stream), "memset");
            detail::check_cuda(cudaMemsetAsync(loss, 0, sizeof(float), stream), "memset");
            launch_train(features, targets, N, batch, offset, stride, grad, loss, stream);
            }

        // `steps` Adam steps on batches of `batch` rows drawn from (features, targets); the
        // learning rate decays on a cosine from lr to lr/20.  Returns the mean loss of the last step.
        float train(const float* features, const float* targets, unsigned int N, unsigned int steps,
                    unsigned int batch, float lr, unsigned long long seed, cudaStream_t stream)
            {
            const detail::TraceRange trace_range("neighbor::CapacityModel::train");
            if (N == 0 || batch == 0) return 0.f;
            unsigned long long s = seed * 0xbf58476d1ce4e5b9ull + 1;
            const auto next = [&s]() {
                s += 0x9e3779b97f4a7c15ull;
                unsigned long long z = s;
                z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
                z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
                return z ^ (z >> 31);
            };
            const auto gcd = [](unsigned long long a, unsigned long long b) {
                while (b) { const unsigned long long t = a % b; a = b; b = t; }
                return a;
            };
            for (unsigned int k = 0; k < steps; ++k)
                {
                const unsigned int offset = (unsigned int)(next() % N);
                unsigned int stride = 1;
                if (N > 1)
                    {
                    for (int tries = 0; tries < 64; ++tries)
                        {
                        stride = 1u + (unsigned int)(next() % (N - 1));
                        if (gcd(stride, N) == 1) break;
                        stride = 1;
                        }
                    }
                gradient(features, targets, N, batch, offset, stride, m_grad.get(), m_loss.get(), stream);
                const double phase = steps > 1 ? (double)k / (double)(steps - 1) : 1.0;
                const float rate = (float)(lr * (0.05 + 0.95 * 0.5 * (1.0 + std::cos(3.141592653589793 * phase))));
                adam(rate, 1.f / (float)batch, stream);
                }
            float loss = 0.f;
            detail::check_cuda(cudaMemcpyAsync(&loss, m_loss.get(), sizeof(float), cudaMemcpyDeviceToHost, stream), "copy");
            detail::check_cuda(cudaStreamSynchronize(stream), "sync");
            return loss / (float)batch;
            }

        // One Adam step from the gradient buffer (scaled by `scale`).
        void adam(float lr, float scale, cudaStream_t stream)
            {
            ++m_step;
            gpu::CapAdamArgs a;
            a.p = m_p.get();
            a.m = m_m.get();
            a.v = m_v.get();
            a.grad = m_grad.get();
            a.w = m_w.get();
            a.scale = scale;
            a.lr = lr;
            a.beta1 = 0.9f;
            a.beta2 = 0.999f;
            a.eps = 1e-8f;
            a.bias1 = (float)(1.0 - std::pow(0.9, (double)m_step));
            a.bias2 = (float)(1.0 - std::pow(0.999, (double)m_step));
            gpu::k_cap_adam<<<detail::ceil_div(kParams, 256), 256, 0, stream>>>(a);
            detail::check_cuda(cudaGetLastError(), "adam launch");
            }

        // One margin for every output (capacity = ceil(expm1(y + margin))).
        void setMargin(float margin)
            {
            for (int b = 0; b < gpu::kCapMarginBins; ++b) m_margins[b] = margin;
            }
        // The largest margin of the table.
        float getMargin() const
            {
            float m = m_margins[0];
            for (int b = 1; b < gpu::kCapMarginBins; ++b) m = std::fmax(m, m_margins[b]);
            return m;
            }
        // Calibration table: margin of the outputs y in [b/2, (b+1)/2) for b < kMarginBins - 1, the
        // last bin open-ended.
        static constexpr int kMarginBins = gpu::kCapMarginBins;
        void setMargins(const float* margins)
            {
            for (int b = 0; b < gpu::kCapMarginBins; ++b) m_margins[b] = margins[b];
            }
        void getMargins(float* margins) const
            {
            for (int b = 0; b < gpu::kCapMarginBins; ++b) margins[b] = m_margins[b];
            }

        void getParams(float* host) const
            {
            detail::check_cuda(cudaMemcpy(host, m_p.get(), kParams * sizeof(float), cudaMemcpyDeviceToHost), "copy");
            }
        // New FP32 parameters (and their BF16 copies); Adam state cleared.
        void setParams(const float* host)
            {
            detail::check_cuda(cudaMemcpy(m_p.get(), host, kParams * sizeof(float), cudaMemcpyHostToDevice), "copy");
            detail::check_cuda(cudaMemset(m_m.get(), 0, kParams * sizeof(float)), "memset");
            detail::check_cuda(cudaMemset(m_v.get(), 0, kParams * sizeof(float)), "memset");
            gpu::k_cap_cast<<<detail::ceil_div(gpu::kCapBfWeights, 256), 256>>>(m_p.get(), m_w.get());
            detail::check_cuda(cudaGetLastError(), "cast launch");
            detail::check_cuda(cudaDeviceSynchronize(), "sync");
            m_step = 0;
            }

        // Weights file (little-endian): the 8 bytes "NBRCAPMD", u32 version (1), u32 parameters,
        // u32 inputs, u32 hidden units, u32 margin bins, the FP32 parameters, the FP32 margin
        // table, and a u64 FNV-1a hash of all the bytes before it.  load() rejects a file whose
        // magic, version, shapes, size or hash differ.
        void save(const char* path) const
            {
            std::vector<unsigned char> b = file_image();
            const unsigned long long h = fnv1a(b.data(), b.size());
            append(b, &h, sizeof(h));
            FILE* f = std::fopen(path, "wb");
            if (!f) throw std::runtime_error(std::string("Invalid path: cannot write capacity model file ") + path);
            const size_t w = std::fwrite(b.data(), 1, b.size(), f);
            const bool ok = std::fclose(f) == 0 && w == b.size();
            if (!ok) throw std::runtime_error(std::string("Invalid path: cannot write capacity model file ") + path);
            }
        void load(const char* path)
            {
            FILE* f = std::fopen(path, "rb");
            if (!f) throw std::runtime_error(std::string("Invalid capacity model file (cannot open) ") + path);
            std::vector<unsigned char> b;
            unsigned char chunk[4096];
            size_t r;
            while ((r = std::fread(chunk, 1, sizeof(chunk), f)) > 0) b.insert(b.end(), chunk, chunk + r);
            std::fclose(f);
            const std::vector<unsigned char> shape = file_image(false);
            const size_t body = shape.size() + (size_t)kParams * 4 + (size_t)kMarginBins * 4;
            if (b.size() != body + 8 || std::memcmp(b.data(), shape.data(), shape.size()) != 0)
                throw std::runtime_error("Invalid capacity model file: magic, version or shapes differ");
            unsigned long long h = 0;
            std::memcpy(&h, b.data() + body, sizeof(h));
            if (h != fnv1a(b.data(), body)) throw std::runtime_error("Invalid capacity model file: hash mismatch");
            std::vector<float> p(kParams);
            float margins[kMarginBins];
            std::memcpy(p.data(), b.data() + shape.size(), (size_t)kParams * 4);
            std::memcpy(margins, b.data() + shape.size() + (size_t)kParams * 4, sizeof(margins));
            setParams(p.data());
            setMargins(margins);
            }

        const float* params() const { return m_p.get(); }
        const __nv_bfloat16* weights() const { return m_w.get(); }

    private:
        device_array<float> m_p;
        device_array<float> m_m;
        device_array<float> m_v;
        device_array<float> m_grad;
        device_array<float> m_loss;
        device_array<__nv_bfloat16> m_w;
        device_array<unsigned int> m_occ;
        device_array<unsigned int> m_status;
        device_array<unsigned int> m_tiles;
        unsigned int m_step;
        InferKernel m_infer;
        float m_margins[gpu::kCapMarginBins];

        static void append(std::vector<unsigned char>& b, const void* p, size_t n)
            {
            const unsigned char* c = static_cast<const unsigned char*>(p);
            b.insert(b.end(), c, c + n);
            }
        static unsigned long long fnv1a(const unsigned char* p, size_t n)
            {
            unsigned long long h = 0xcbf29ce484222325ull;
            for (size_t i = 0; i < n; ++i)
                {
                h ^= p[i];
                h *= 0x100000001b3ull;
                }
            return h;
            }
        // header, and (with_body) the parameters and margins
        std::vector<unsigned char> file_image(bool with_body = true) const
            {
            std::vector<unsigned char> b;
            append(b, "NBRCAPMD", 8);
            const uint32_t head[5] = {1u, (uint32_t)kParams, (uint32_t)gpu::kCapIn, (uint32_t)gpu::kCapHidden,
                                      (uint32_t)gpu::kCapMarginBins};
            append(b, head, sizeof(head));
            if (with_body)
                {
                std::vector<float> p(kParams);
                getParams(p.data());
                append(b, p.data(), p.size() * sizeof(float));
                append(b, m_margins, sizeof(m_margins));
                }
            return b;
            }

        void launch_train(const float* features, const float* targets, unsigned int N, unsigned int batch,
                          unsigned int offset, unsigned int stride, float* grad, float* loss, cudaStream_t stream)
            {
            static bool attr = false;
            if (!attr)
                {
                detail::check_cuda(cudaFuncSetAttribute(gpu::k_cap_train_step, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                        (int)sizeof(gpu::CapTrainSmem)), "train attribute");
                attr = true;
                }
            gpu::CapTrainArgs a;
            a.features = features;
            a.target = targets;
            a.N = N;
            a.batch = batch;
            a.offset = offset;
            a.stride = stride;
            a.w = m_w.get();
            a.p = m_p.get();
            a.grad = grad;
            a.loss_out = loss;
            const unsigned int tiles = detail::ceil_div(batch, gpu::kCapTrainTile);
            const unsigned int grid = std::min(tiles, 152u * 2u);
            gpu::k_cap_train_step<<<grid, gpu::kCapTrainTile, sizeof(gpu::CapTrainSmem), stream>>>(a);
            detail::check_cuda(cudaGetLastError(), "train launch");
            }
    };

} // namespace neighbor

#endif // NEIGHBOR_CAPACITY_MODEL_H_
