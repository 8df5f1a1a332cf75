// Autotuner of the single-system self neighbor list.  No counterpart in the reference, whose
// Tunable (include/neighbor/Tunable.h:28-118) only lists the valid block sizes of each launcher
// and leaves the choice to its caller (HOOMD-blue's autotuner).
//
// SelfListTuner times the step a caller repeats -- LBVH::build, the counting self traversal, the
// host read of its summary, the list fill -- on the caller's own points, for every combination of
// the knobs that change its speed but never its result:
//   leaf size (box records of up to 1, 2, 4 or 8 points), sort digit width (8 or 10 bits), and
//   climb block (256 or 512 sorted leaves per block of the agglomerative build).
// The fastest combination is applied to the LBVH and cached for the workload's class:
// (N rounded up to a power of two, cutoff, number density in bins of a quarter octave), so that
// later calls for the same class reuse it without timing.  Results of every combination are the
// same lists, bit for bit.
#ifndef NEIGHBOR_SELF_LIST_TUNER_H_
#define NEIGHBOR_SELF_LIST_TUNER_H_

#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include <cuda_runtime.h>

#include "InsertOps.h"
#include "LBVH.h"
#include "LBVHTraverser.h"
#include "Memory.h"
#include "OutputOps.h"
#include "TranslateOps.h"

namespace neighbor
{

struct SelfListConfig
    {
    unsigned int leaf_size = 4;
    unsigned int radix_bits = 8;
    unsigned int climb_block = 512;
    float ms = 0.f;   // measured milliseconds per step (0 when taken from the cache)
    };

class SelfListTuner
    {
    public:
        // Tune (or look up) the configuration for `points` and apply it to `lbvh`.  images: the
        // 27 periodic images of `box` (periodic) or the self image.  reps timed steps per
        // combination after one untimed step.  `timings` (optional) receives every measured
        // combination.
        SelfListConfig tune(LBVH& lbvh, LBVHTraverser& trav, const float3* points, unsigned int N, float3 lo,
                            float3 hi, float rc, float3 box, float pad, bool periodic, unsigned int reps,
                            cudaStream_t stream, std::vector<SelfListConfig>* timings = nullptr)
            {
            const Key key = make_key(N, lo, hi, rc);
                {
                std::lock_guard<std::mutex> lock(cache_mutex());
                auto it = cache().find(key);
                if (it != cache().end())
                    {
                    SelfListConfig c = it->second;
                    c.ms = 0.f;
                    apply(lbvh, c);
                    return c;
                    }
                }
            m_nneigh.reserve(N);
            SelfListConfig best;
            best.ms = -1.f;
            cudaEvent_t e0, e1;
            detail::check_cuda(cudaEventCreate(&e0), "event");
            detail::check_cuda(cudaEventCreate(&e1), "event");
            for (unsigned int leaf : {1u, 2u, 4u, 8u})
                for (unsigned int bits : {8u, 10u})
                    for (unsigned int climb : {256u, 512u})
                        {
                        SelfListConfig c;
                        c.leaf_size = leaf;
                        c.radix_bits = bits;
                        c.climb_block = climb;
                        apply(lbvh, c);
                        step(lbvh, trav, points, N, lo, hi, rc, box, pad, periodic, stream);   // untimed
                        float total = 0.f;
                        for (unsigned int r = 0; r < reps; ++r)
                            {
                            detail::check_cuda(cudaEventRecord(e0, stream), "event");
                            step(lbvh, trav, points, N, lo, hi, rc, box, pad, periodic, stream);
                            detail::check_cuda(cudaEventRecord(e1, stream), "event");
                            detail::check_cuda(cudaEventSynchronize(e1), "event");
                            float ms = 0.f;
                            detail::check_cuda(cudaEventElapsedTime(&ms, e0, e1), "event");
                            total += ms;
                            }
                        c.ms = total / (float)(reps ? reps : 1);
                        if (timings) timings->push_back(c);
                        if (best.ms < 0.f || c.ms < best.ms) best = c;
                        }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            lbvh.checkStatus(stream);
            apply(lbvh, best);
                {
                std::lock_guard<std::mutex> lock(cache_mutex());
                cache()[key] = best;
                }
            return best;
            }

        // Forget every cached configuration (process-wide).
        static void clearCache()
            {
            std::lock_guard<std::mutex> lock(cache_mutex());
            cache().clear();
            }

        static void apply(LBVH& lbvh, const SelfListConfig& c)
            {
            lbvh.setLeafSize(c.leaf_size);
            lbvh.setRadixBits(c.radix_bits);
            lbvh.setClimbBlock(c.climb_block);
            }

    private:
        // (log2 of N rounded up, cutoff, number density in quarter octaves)
        typedef std::tuple<int, float, int> Key;

        static Key make_key(unsigned int N, float3 lo, float3 hi, float rc)
            {
            const double vol = std::fabs((double)(hi.x - lo.x) * (double)(hi.y - lo.y) * (double)(hi.z - lo.z));
            const double rho = vol > 0.0 ? (double)N / vol : 0.0;
            const int nbin = (int)std::ceil(std::log2((double)(N > 1 ? N : 1)));
            const int dbin = rho > 0.0 ? (int)std::floor(4.0 * std::log2(rho)) : -1000;
            return Key(nbin, rc, dbin);
            }

        static std::map<Key, SelfListConfig>& cache()
            {
            static std::map<Key, SelfListConfig> c;
            return c;
            }
        static std::mutex& cache_mutex()
            {
            static std::mutex m;
            return m;
            }

        // The timed step: build, count, host read of the largest count, fill of a list of that
        // stride (rows by sorted position).
        void step(LBVH& lbvh, LBVHTraverser& trav, const float3* points, unsigned int N, float3 lo, float3 hi,
                  float rc, float3 box, float pad, bool periodic, cudaStream_t stream)
            {
            const LBVH::LaunchParameters bp(256, stream);
            const LBVHTraverser::LaunchParameters tp(256, stream);
            lbvh.build(bp, PointInsertOp(points, N), lo, hi);
            unsigned int mx = 0, past = 0;
            unsigned long long total = 0;
            if (periodic)
                trav.traverseSelf(tp, lbvh, rc, box, pad, CountNeighborsOp(m_nneigh.get()), PeriodicImagesOp(box),
                                  NullTransformOp(), true);
            else
                trav.traverseSelf(tp, lbvh, rc, box, pad, CountNeighborsOp(m_nneigh.get()), SelfOp(), NullTransformOp(),
                                  true);
            trav.readCountSummary(stream, mx, total, past);
            if (mx == 0) return;
            m_list.reserve((size_t)N * mx);
            if (periodic)
                trav.traverseSelf(tp, lbvh, rc, box, pad, NeighborListOp(m_list.get(), m_nneigh.get(), mx),
                                  PeriodicImagesOp(box), NullTransformOp(), true);
            else
                trav.traverseSelf(tp, lbvh, rc, box, pad, NeighborListOp(m_list.get(), m_nneigh.get(), mx), SelfOp(),
                                  NullTransformOp(), true);
            }

        device_array<unsigned int> m_nneigh;
        device_array<unsigned int> m_list;
    };

} // namespace neighbor

#endif // NEIGHBOR_SELF_LIST_TUNER_H_
