// Stackless LBVH traversal.
//
// Public interface as in the reference (include/neighbor/LBVHTraverser.h:60-355): setup() with an
// optional TransformOp (compress once, replay later), reset(), the nine traverse() overloads
// (LaunchParameters | stream | neither) x (with/without images) x (with/without transform),
// getData() returning the int4 nodes in the reference's 10-bit layout, std::runtime_error for more
// than 32 images or an invalid tunable.
//
// Routing.  An ExactSphereQueryOp with CountNeighborsOp or NeighborListOp on a tree built from
// points runs the fast kernel over the LBVH's 16-bit pre-order nodes (no compression step; the
// transform is applied to the reported ids); an ExactSphereQueryOpF64 on a tree of
// PointInsertOpF64 runs the same walk with the double predicate (k_traverse_fast_f64).  Any other combination of ops -- including the
// stock SphereQueryOp, whose superset result depends on the node format -- runs the
// reference-layout rope kernel, so it returns exactly what the reference returns.
#ifndef NEIGHBOR_LBVH_TRAVERSER_H_
#define NEIGHBOR_LBVH_TRAVERSER_H_

#include <algorithm>
#include <memory>
#include <stdexcept>
#include <type_traits>

#include <cuda_runtime.h>

#include "LBVH.h"
#include "LBVHTraverserData.h"
#include "Memory.h"
#include "Trace.h"
#include "OutputOps.h"
#include "QueryOps.h"
#include "TransformOps.h"
#include "TranslateOps.h"
#include "Tunable.h"
#include "kernels/traverse.cuh"

namespace neighbor
{

class LBVHTraverser : public Tunable<unsigned int>
    {
    public:
        LBVHTraverser()
            : Tunable<unsigned int>(32, 1024, 32), m_root(0), m_lbvh_lo(1), m_lbvh_hi(1), m_bins(1),
              m_replay(false), m_fast_enabled(true), m_mode(kThreadTraversal),
              m_stats(nullptr), m_symmetric(true)
            {}

        template<class TransformOpT>
        void setup(const LaunchParameters& params, const LBVH& lbvh, const TransformOpT& transform)
            {
            reset();
            if (lbvh.getN() != 0)
                {
                compress(params, lbvh, transform);
                m_replay = true;
                }
            }
        void setup(const LaunchParameters& params, const LBVH& lbvh) { setup(params, lbvh, NullTransformOp()); }
        template<class TransformOpT>
        void setup(cudaStream_t stream, const LBVH& lbvh, const TransformOpT& transform)
            {
            setup(LaunchParameters(32, stream), lbvh, transform);
            }
        void setup(cudaStream_t stream, const LBVH& lbvh) { setup(stream, lbvh, NullTransformOp()); }
        template<class TransformOpT>
        void setup(const LBVH& lbvh, const TransformOpT& transform) { setup(cudaStream_t(0), lbvh, transform); }
        void setup(const LBVH& lbvh) { setup(cudaStream_t(0), lbvh, NullTransformOp()); }

        void reset() { m_replay = false; }

        template<class QueryOpT, class OutputOpT, class TranslateOpT, class TransformOpT>
        void traverse(const LaunchParameters& params, const LBVH& lbvh, const QueryOpT& query,
                      const OutputOpT& out, const TranslateOpT& images, const TransformOpT& transform);

        template<class QueryOpT, class OutputOpT, class TranslateOpT>
        void traverse(const LaunchParameters& params, const LBVH& lbvh, const QueryOpT& query,
                      const OutputOpT& out, const TranslateOpT& images)
            {
            traverse(params, lbvh, query, out, images, NullTransformOp());
            }

        template<class QueryOpT, class OutputOpT>
        void traverse(const LaunchParameters& params, const LBVH& lbvh, const QueryOpT& query, const OutputOpT& out)
            {
            traverse(params, lbvh, query, out, SelfOp(), NullTransformOp());
            }

        template<class QueryOpT, class OutputOpT, class TranslateOpT, class TransformOpT>
        void traverse(cudaStream_t stream, const LBVH& lbvh, const QueryOpT& query, const OutputOpT& out,
                      const TranslateOpT& images, const TransformOpT& transform)
            {
            traverse(LaunchParameters(32, stream), lbvh, query, out, images, transform);
            }

        template<class QueryOpT, class OutputOpT, class TranslateOpT>
        void traverse(cudaStream_t stream, const LBVH& lbvh, const QueryOpT& query, const OutputOpT& out,
                      const TranslateOpT& images)
            {
            traverse(stream, lbvh, query, out, images, NullTransformOp());
            }

        template<class QueryOpT, class OutputOpT>
        void traverse(cudaStream_t stream, const LBVH& lbvh, const QueryOpT& query, const OutputOpT& out)
            {
            traverse(stream, lbvh, query, out, SelfOp(), NullTransformOp());
            }

        template<class QueryOpT, class OutputOpT, class TranslateOpT, class TransformOpT>
        void traverse(const LBVH& lbvh, const QueryOpT& query, const OutputOpT& out, const TranslateOpT& images,
                      const TransformOpT& transform)
            {
            traverse(cudaStream_t(0), lbvh, query, out, images, transform);
            }

        template<class QueryOpT, class OutputOpT, class TranslateOpT>
        void traverse(const LBVH& lbvh, const QueryOpT& query, const OutputOpT& out, const TranslateOpT& images)
            {
            traverse(cudaStream_t(0), lbvh, query, out, images, NullTransformOp());
            }

        template<class QueryOpT, class OutputOpT>
        void traverse(const LBVH& lbvh, const QueryOpT& query, const OutputOpT& out)
            {
            traverse(cudaStream_t(0), lbvh, query, out, SelfOp(), NullTransformOp());
            }

        // Reference-layout nodes written by the last compression (setup(), or a traversal that
        // took the reference-layout path without a setup()).
        const shared_array<int4>& getData() const { return m_data; }

        // ---- additions of this library ----

        // Compression frame of getData(): root lower/upper bounds and bin width (managed float[3]).
        const float* getFrameLo() const { return reinterpret_cast<const float*>(m_lbvh_lo.get()); }
        const float* getFrameHi() const { return reinterpret_cast<const float*>(m_lbvh_hi.get()); }
        const float* getFrameBins() const { return reinterpret_cast<const float*>(m_bins.get()); }

        // Route eligible traversals to the fast kernel (default) or always use the
        // reference-layout kernel.
        void setFastPath(bool enabled) { m_fast_enabled = enabled; }
        bool getFastPath() const { return m_fast_enabled; }

        // Fast-path kernel: kThreadTraversal (one thread walks the tree per query; default) or
        // kPacketTraversal (a warp walks it once for 32 consecutive queries).
        enum Mode { kThreadTraversal = 0, kPacketTraversal = 1 };
        void setMode(int mode)
            {
            if (mode != kThreadTraversal && mode != kPacketTraversal)
                throw std::runtime_error("Traversal mode must be 0 (thread) or 1 (packet).");
            m_mode = mode;
            }
        int getMode() const { return m_mode; }

        // Optional device counters (3 x uint64: node visits, point tests, packets walked) that
        // the fast kernels add to; NULL disables them.
        void setStats(unsigned long long* counters) { m_stats = counters; }

        // Self traversals with the self image or PeriodicImagesOp find each unordered pair once
        // and write it to both rows (default); off: every query walks the whole tree.  Counts,
        // neighbor sets and the order of each row are the same either way.
        void setSymmetric(bool enabled) { m_symmetric = enabled; }
        bool getSymmetric() const { return m_symmetric; }

        // Work order of fills (true, default): a symmetric count without the pair cache records
        // how many records each query visited, and a symmetric fill over the same tree with the
        // same cutoff hands each block's queries to its lanes in order of those lengths; a
        // whole-tree CSR fill orders them by row capacity.  false: sorted order.  Results do not
        // depend on it.
        void setWorkOrder(bool enabled) { m_work_order = enabled; }
        bool getWorkOrder() const { return m_work_order; }

        // Pair exchange (true, default): a symmetric count also keeps, per point, the first 16
        // pairs it found itself and the first 16 pairs other points found with it (128 bytes per
        // point), and a fill over the same tree, cutoff, images and rows assembles every row from
        // them without walking (rows with more re-walk the tree).  false: the fill walks again.
        // Results do not depend on it.
        void setPairCache(bool enabled) { m_pair_cache = enabled; }
        bool getPairCache() const { return m_pair_cache; }

        // Summary of the last counting traversal (traverse or traverseSelf with
        // CountNeighborsOp), four device words: [0] the largest count, [1] rows whose pairs did
        // not fit the pair exchange (exchanging self counts) or, for other counts, rows of more
        // than 32 entries (which no exchange could hold), [2..3] the total of the counts (64-bit).
        // Written on the traversal's stream.
        const unsigned int* getCountSummary() const { return m_words.get(); }
        // The same, read on the host: synchronises `stream` (the reference's two-pass pattern
        // reads the largest count here before the fill, benchmark/lbvh_benchmark.cc:177-196).
        void readCountSummary(cudaStream_t stream, unsigned int& max_count, unsigned long long& total,
                              unsigned int& past_exchange)
            {
            if (!m_host_words)
                {
                void* p = nullptr;
                detail::check_cuda(cudaMallocHost(&p, gpu::kSummaryWords * sizeof(unsigned int)), "host alloc");
                m_host_words.reset(static_cast<unsigned int*>(p));
                }
            unsigned int* h = m_host_words.get();
            if (m_words.size() < kWordCount)
                {
                h[0] = h[1] = h[2] = h[3] = 0u;
                }
            else
                {
                detail::check_cuda(cudaMemcpyAsync(h, m_words.get(), gpu::kSummaryWords * sizeof(unsigned int),
                                                   cudaMemcpyDeviceToHost, stream), "copy");
                detail::check_cuda(cudaStreamSynchronize(stream), "sync");
                }
            max_count = h[0];
            past_exchange = h[1];
            total = (unsigned long long)h[2] | ((unsigned long long)h[3] << 32);
            // a self count's summary read on the host also steers the following fill and the
            // next counts (results never depend on it): with more than a quarter of the rows past
            // the exchange, the exchange costs more than it saves
            if (m_summary_self && m_words.size() >= kWordCount)
                {
                // an exchanging count measures its rows past the exchange (dense above a quarter of
                // the rows); another counts only rows longer than 32, a lower bound (dense above
                // an eighth, so that the choice does not flip back and forth between frames)
                m_summary_read = true;
                const unsigned long long n = m_summary_n, p = past_exchange;
                m_dense = m_summary_exchange ? p * 4ull > n : p * 8ull > n;
                }
            }

        // Routing by size (results do not depend on it).  With few queries the GPU is mostly idle
        // and the longest walks set the time.  Self traversals of more than
        // getSymmetricMinPoints() points take the symmetric walk with the pair exchange; other
        // traversals of at most getWarpWalkMaxQueries() queries walk one group of lanes per query
        // (getWalkLanes()), which shortens a walk about as many times as the group has lanes, and
        // larger ones one thread per query.  Build + count + max + fill driven from C++, median of
        // 200 steps (the symmetric count by lane groups up to 65,536 points): 4,096 points lane
        // groups 150 us, symmetric 155; 8,192 points 182 / 174; 16,384 points 226 / 194; 32,768
        // points 295 / 210; 65,536 points 436 / 285.  Larger (python-driven, median of 30):
        // 262,144 points 558 / 427 (thread walk 556); 524,288 points thread 773, symmetric 548.
        // 0 turns a limit off.
        void setWarpWalkMaxQueries(unsigned int q) { m_warp_walk_max = q; }
        unsigned int getWarpWalkMaxQueries() const { return m_warp_walk_max; }
        void setSymmetricMinPoints(unsigned int n) { m_symmetric_min = n; }
        unsigned int getSymmetricMinPoints() const { return m_symmetric_min; }
        // Lanes per query of those small traversals: 4, 8, 16 or 32; 0 (default) picks by size.
        void setWalkLanes(unsigned int lanes)
            {
            if (lanes != 0 && lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32)
                throw std::runtime_error("Invalid walk lanes (0, 4, 8, 16 or 32).");
            m_walk_lanes = lanes;
            }
        unsigned int getWalkLanes() const { return m_walk_lanes; }
        // Lanes per query of the symmetric count with the pair exchange: 1 (one thread per
        // query), 4, 8, 16 or 32; 0 (default) picks by size.  Results do not depend on it.
        void setHalfWalkLanes(unsigned int lanes)
            {
            if (lanes != 0 && lanes != 1 && lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32)
                throw std::runtime_error("Invalid half-walk lanes (0, 1, 4, 8, 16 or 32).");
            m_half_lanes = lanes;
            }
        unsigned int getHalfWalkLanes() const { return m_half_lanes; }

        // Self queries on the fast path: every primitive of the tree queries the tree with cutoff
        // rc.  Queries run in the tree's sorted order; rows_sorted selects whether row s of the
        // output belongs to sorted slot s (the reference benchmark's layout) or to the original
        // primitive index.  OutputOpT is CountNeighborsOp or NeighborListOp.
        template<class OutputOpT, class TranslateOpT, class TransformOpT>
        void traverseSelf(const LaunchParameters& params, const LBVH& lbvh, float rc, float3 box,
                          float pad, const OutputOpT& out, const TranslateOpT& images,
                          const TransformOpT& transform, bool rows_sorted);

        // Self queries of the sorted positions subset[0..count) only, each walking the whole tree
        // (rows as in traverseSelf); used to re-run rows whose one-pass capacity was too small.
        template<class OutputOpT, class TranslateOpT, class TransformOpT>
        void traverseSelfSubset(const LaunchParameters& params, const LBVH& lbvh, float rc, float3 box,
                                float pad, const OutputOpT& out, const TranslateOpT& images,
                                const TransformOpT& transform, bool rows_sorted, const unsigned int* subset,
                                unsigned int count);

        // Self queries of a tree of double points (built with PointInsertOpF64 from `points`,
        // indexed by primitive id), exact double predicate: the results of traverse() with
        // ExactSphereQueryOpF64 over the spheres (points[primitive[s]], rc) in sorted order, with
        // row s (rows_sorted) or primitive[s].  Counts above getSymmetricMinPoints() points with
        // SelfOp or PeriodicImagesOp take the symmetric walk with the pair exchange, and a fill
        // over the same tree, points, cutoff, images and rows assembles the rows from it; other
        // traversals walk the whole tree per query.  Results do not depend on the route.
        template<class OutputOpT, class TranslateOpT, class TransformOpT>
        void traverseSelfF64(const LaunchParameters& params, const LBVH& lbvh, const double3* points, double rc,
                             double3 box, float pad, const OutputOpT& out, const TranslateOpT& images,
                             const TransformOpT& transform, bool rows_sorted);

    private:
        int m_root;
        shared_array<int4> m_data;
        shared_array<float3> m_lbvh_lo;
        shared_array<float3> m_lbvh_hi;
        shared_array<float3> m_bins;
        bool m_replay;
        bool m_fast_enabled;
        int m_mode;
        unsigned long long* m_stats;
        bool m_symmetric;
        bool m_work_order = true;
        unsigned int m_warp_walk_max = gpu::kWarpWalkMaxQueries;
        unsigned int m_symmetric_min = gpu::kSymmetricMinPoints;
        unsigned int m_walk_lanes = 0;
        unsigned int m_half_lanes = 0;
        bool m_pair_cache = true;
        bool m_count_cached = false;
        // the summary words come from a self count (m_summary_self); its summary was read on the
        // host (m_summary_read); that summary found more than a quarter of the rows past the
        // exchange, or too long for it (m_dense)
        bool m_summary_self = false;
        bool m_summary_read = false;
        bool m_dense = false;
        bool m_summary_exchange = false;   // the summary's count used the exchange
        unsigned int m_summary_n = 0;      // rows of the summary's count
        // pair exchange of the last symmetric count: own keys and incoming keys (16 per sorted
        // position each) and the incoming counters
        device_array<unsigned int> m_cache;
        device_array<unsigned int> m_in_cache;
        device_array<unsigned int> m_in_count;
        device_array<unsigned char> m_lost;   // rows counted without a deposited key
        // [0..4) count summary, [4] rows left to re-walk after an assembly, [5] the re-walk's ticket
        static constexpr size_t kWordCount = 8;
        device_array<unsigned int> m_words;
        device_array<unsigned int> m_subset;
        struct host_free { void operator()(unsigned int* p) const { if (p) cudaFreeHost(p); } };
        std::unique_ptr<unsigned int, host_free> m_host_words;
        int m_sms = 0;
        unsigned int sm_count()
            {
            if (!m_sms)
                {
                int dev = 0;
                detail::check_cuda(cudaGetDevice(&dev), "device");
                detail::check_cuda(cudaDeviceGetAttribute(&m_sms, cudaDevAttrMultiProcessorCount, dev), "attribute");
                }
            return (unsigned int)m_sms;
            }
        // blocks of the count summary: enough per SM to keep its loads in flight, each adding its
        // rows to the words once (16M rows: 4 blocks per SM 0.111 ms)
        unsigned int summary_grid(unsigned int N)
            {
            return std::max(1u, std::min(detail::ceil_div(N, gpu::kSummaryBlock), 16u * sm_count()));
            }
        // the summary (largest count, total) of counts already written to nneigh[0..Q)
        void summarize_counts(cudaStream_t stream, unsigned int* nneigh, unsigned int Q, const unsigned int* status)
            {
            clear_summary(stream);
            gpu::k_count_summary<false><<<summary_grid(Q), gpu::kSummaryBlock, 0, stream>>>(
                Q, nullptr, nullptr, nullptr, nullptr, 0, nneigh, m_words.get(), status);
            detail::check_cuda(cudaGetLastError(), "summary launch");
            }
        // zero the summary words before a count
        void clear_summary(cudaStream_t stream)
            {
            m_words.reserve(kWordCount);
            detail::check_cuda(cudaMemsetAsync(m_words.get(), 0, gpu::kSummaryWords * sizeof(unsigned int), stream),
                               "memset");
            }
        // self traversal, count + fill: 4,096 points 63 us with 32 lanes (16: 85, 8: 110);
        // 16,384 points 120 us with 32 (8: 124, 4: 172); 32,768 points 185 us with 16 (8: 188,
        // 32: 195, 4: 193; one thread per query 269)
        unsigned int walk_lanes(unsigned int Q) const
            {
            if (m_walk_lanes) return m_walk_lanes;
            return Q <= 16384u ? 32u : 16u;
            }
        // the symmetric count alone (exchange, kernel only): 32,768 points one thread per query
        // 149 us, lane groups of 4 / 8 / 16 / 32: 114 / 88 / 71 / 57 us; 65,536 points 127 us,
        // 114 / 90 / 100 / 92 us; 131,072 points 133 us, 159 / 133 / 168 / 178 us; above that one
        // thread per query leads (262,144 points 147 against 237 us with 8 lanes)
        unsigned int half_lanes(unsigned int N) const
            {
            if (m_half_lanes) return m_half_lanes;
            return N <= 32768u ? 32u : (N <= 65536u ? 8u : 1u);
            }
        // What a symmetric count ran on (the tree's address and process-unique build id, cutoff,
        // images, box and rows); a fill with the same tag reuses its results.
        struct PassTag
            {
            const LBVH* tree = nullptr;
            unsigned long long build = 0;
            unsigned int N = 0;
            float rc = 0.f, pad = 0.f;
            int lattice = -1;
            float3 L = make_float3(0.f, 0.f, 0.f);
            float3 box = make_float3(0.f, 0.f, 0.f);
            int rows_sorted = -1;
            // double self queries: their points, cutoff and box (an FP32 count leaves them zero)
            const void* points64 = nullptr;
            double rc64 = 0.0;
            double3 box64 = make_double3(0.0, 0.0, 0.0);
            bool operator==(const PassTag& o) const
                {
                return tree == o.tree && build == o.build && N == o.N && rc == o.rc && pad == o.pad
                       && lattice == o.lattice && L.x == o.L.x && L.y == o.L.y && L.z == o.L.z && box.x == o.box.x
                       && box.y == o.box.y && box.z == o.box.z && rows_sorted == o.rows_sorted
                       && points64 == o.points64 && rc64 == o.rc64 && box64.x == o.box64.x && box64.y == o.box64.y
                       && box64.z == o.box64.z;
                }
            };
        // results of the last symmetric count: walk lengths (by sorted position), own counts and
        // row totals (by row)
        PassTag m_count_tag;
        device_array<unsigned short> m_walk;
        device_array<unsigned int> m_count_own;
        device_array<unsigned int> m_totals;
        device_array<unsigned int> m_own;

        template<class TransformOpT>
        void compress(const LaunchParameters& params, const LBVH& lbvh, const TransformOpT& transform)
            {
            checkParameter(params);
            const unsigned int n = lbvh.getNNodes();
            if (n > m_data.size())
                {
                shared_array<int4> tmp(n);
                m_data.swap(tmp);
                }
            m_root = lbvh.getRoot();
            const unsigned int bs = params.tunable;
            gpu::k_compress_ref10<TransformOpT><<<detail::ceil_div(n, bs), bs, 0, params.stream>>>(
                data(), transform, lbvh.data(params.stream), lbvh.getNInternal(), n, lbvh.getStatusPointer());
            detail::check_cuda(cudaGetLastError(), "compress launch");
            }

        LBVHCompressedData data()
            {
            LBVHCompressedData c;
            c.root = m_root;
            c.data = m_data.get();
            c.lo = m_lbvh_lo.get();
            c.hi = m_lbvh_hi.get();
            c.bins = m_bins.get();
            return c;
            }

        template<class OutputOpT, class TransformOpT>
        void launch_fast(const LaunchParameters& params, const LBVH& lbvh, gpu::FastQueryArgs a,
                         const OutputOpT& out, const TransformOpT& transform, unsigned int Q);

        template<class OutputOpT, class TransformOpT>
        void launch_half(const LaunchParameters& params, const LBVH& lbvh, const gpu::FastQueryArgs& a,
                         const OutputOpT& out, const TransformOpT& transform);

        template<class OutputOpT, class TransformOpT>
        void launch_assemble(const LaunchParameters& params, const LBVH& lbvh, const gpu::FastQueryArgs& a,
                             const OutputOpT& out, const TransformOpT& transform);

        // the assembly of a fill from the last exchanging count (rows, images and outputs from a);
        // the rows past the exchange are listed for a re-walk
        template<int kind, class TransformOpT>
        void assemble_rows(cudaStream_t stream, const LBVH& lbvh, const gpu::FastQueryArgs& a,
                           const TransformOpT& transform);

        PassTag self_tag(const LBVH& lbvh, const gpu::FastQueryArgs& a) const
            {
            return PassTag{&lbvh, lbvh.getBuildId(), lbvh.getN(), a.self_rc, a.pad, a.lattice, a.lattice_L, a.box,
                           a.self_rows_sorted};
            }
        PassTag self_tag_f64(const LBVH& lbvh, const gpu::FastQueryArgsF64& a) const
            {
            PassTag t{&lbvh, lbvh.getBuildId(), lbvh.getN(), 0.f, a.pad, a.lattice, a.lattice_L,
                      make_float3(0.f, 0.f, 0.f), a.self_rows_sorted};
            t.points64 = a.points;
            t.rc64 = a.self_rc;
            t.box64 = a.box;
            return t;
            }
    };

namespace detail
{
template<class T> struct is_float3_images : std::false_type {};
template<> struct is_float3_images<ImageListOp<float3>> : std::true_type {};
template<> struct is_float3_images<SelfOp> : std::true_type {};
template<> struct is_float3_images<PeriodicImagesOp> : std::true_type {};

inline const float3* image_pointer(const SelfOp&) { return nullptr; }
inline const float3* image_pointer(const ImageListOp<float3>& op) { return op.images; }
inline const float3* image_pointer(const PeriodicImagesOp&) { return nullptr; }
template<class T> inline int image_lattice(const T&) { return 0; }
inline int image_lattice(const PeriodicImagesOp&) { return 1; }
template<class T> inline float3 lattice_box(const T&, float3 box) { return box; }
inline float3 lattice_box(const PeriodicImagesOp& op, float3) { return op.L; }
template<class T> inline const float3* image_pointer(const T&) { return nullptr; }
template<class T> struct is_symmetric_images : std::false_type {};
template<> struct is_symmetric_images<SelfOp> : std::true_type {};
template<> struct is_symmetric_images<PeriodicImagesOp> : std::true_type {};

inline void set_output(gpu::FastQueryArgs& a, const CountNeighborsOp& out)
    {
    a.nneigh = out.nneigh;
    a.list = nullptr;
    a.max_neigh = 0;
    }
inline void set_output(gpu::FastQueryArgs& a, const NeighborListOp& out)
    {
    a.nneigh = out.nneigh;
    a.list = out.neigh_list;
    a.max_neigh = out.max_neigh;
    }
inline void set_output(gpu::FastQueryArgs& a, const CSRNeighborListOp& out)
    {
    a.nneigh = out.nneigh;
    a.list = out.neigh_list;
    a.max_neigh = out.max_capacity;  // 0 = unknown
    a.offsets = out.offsets;
    a.caps = out.capacity;
    }
inline void set_output_f64(gpu::FastQueryArgsF64& a, const CountNeighborsOp& out)
    {
    a.nneigh = out.nneigh;
    a.list = nullptr;
    a.max_neigh = 0;
    }
inline void set_output_f64(gpu::FastQueryArgsF64& a, const NeighborListOp& out)
    {
    a.nneigh = out.nneigh;
    a.list = out.neigh_list;
    a.max_neigh = out.max_neigh;
    }
inline void set_output_f64(gpu::FastQueryArgsF64& a, const CSRNeighborListOp& out)
    {
    a.nneigh = out.nneigh;
    a.list = out.neigh_list;
    a.max_neigh = out.max_capacity;
    a.offsets = out.offsets;
    a.caps = out.capacity;
    }
// Longest row a traversal may write (0 = unknown).
inline unsigned int max_row(const CountNeighborsOp&) { return 0u; }
inline unsigned int max_row(const NeighborListOp& out) { return out.max_neigh; }
inline unsigned int max_row(const CSRNeighborListOp& out) { return out.max_capacity; }
} // namespace detail

template<class OutputOpT, class TransformOpT>
void LBVHTraverser::launch_fast(const LaunchParameters& params, const LBVH& lbvh, gpu::FastQueryArgs a,
                                const OutputOpT& out, const TransformOpT& transform, unsigned int Q)
    {
    detail::set_output(a, out);
    a.stats = m_stats;
    a.work_order = (output_kind<OutputOpT>::value == gpu::kFastCSR && !a.subset && m_work_order) ? 1 : 0;
    const unsigned int bs = params.tunable;
    constexpr int kind = output_kind<OutputOpT>::value;
    if (m_mode == kPacketTraversal && kind != gpu::kFastCSR && !a.subset)
        gpu::k_traverse_packet<kind == gpu::kFastCSR ? gpu::kFastList : kind, TransformOpT><<<detail::ceil_div(Q, bs), bs, 0, params.stream>>>(
            lbvh.fastData(), a, transform);
    else if (m_stats)
        gpu::k_traverse_fast<kind, true, TransformOpT><<<detail::ceil_div(Q, bs), bs, 0, params.stream>>>(
            lbvh.fastData(), a, transform);
    else if (a.subset || Q <= m_warp_walk_max)
        {
        // few queries (a subset is the rows that overflowed a one-pass list): a group of lanes
        // walks each, so the walks' latency, not the GPU's width, sets the time
        const unsigned int G = a.subset ? 32u : walk_lanes(Q);
        const unsigned int grid = (unsigned int)(((unsigned long long)Q * G + gpu::kWarpWalkBlock - 1u)
                                                 / gpu::kWarpWalkBlock);
        if (G == 4)
            gpu::k_traverse_warp<kind, TransformOpT, 4><<<grid, gpu::kWarpWalkBlock, 0, params.stream>>>(
                lbvh.fastData(), a, transform);
        else if (G == 8)
            gpu::k_traverse_warp<kind, TransformOpT, 8><<<grid, gpu::kWarpWalkBlock, 0, params.stream>>>(
                lbvh.fastData(), a, transform);
        else if (G == 16)
            gpu::k_traverse_warp<kind, TransformOpT, 16><<<grid, gpu::kWarpWalkBlock, 0, params.stream>>>(
                lbvh.fastData(), a, transform);
        else
            gpu::k_traverse_warp<kind, TransformOpT, 32><<<grid, gpu::kWarpWalkBlock, 0, params.stream>>>(
                lbvh.fastData(), a, transform);
        }
    else
        gpu::k_traverse_fast<kind, false, TransformOpT><<<detail::ceil_div(Q, bs), bs, 0, params.stream>>>(
            lbvh.fastData(), a, transform);
    detail::check_cuda(cudaGetLastError(), "fast traversal launch");
    }

template<class QueryOpT, class OutputOpT, class TranslateOpT, class TransformOpT>
void LBVHTraverser::traverse(const LaunchParameters& params, const LBVH& lbvh, const QueryOpT& query,
                             const OutputOpT& out, const TranslateOpT& images, const TransformOpT& transform)
    {
    const detail::TraceRange trace_range("neighbor::LBVHTraverser::traverse");
    if (lbvh.getN() == 0) return;
    if (query.size() == 0 || images.size() == 0) return;
    if (images.size() > 32)
        throw std::runtime_error("A maximum of 32 image vectors are supported by LBVH traversers.");
    checkParameter(params);

    if constexpr (std::is_same<QueryOpT, ExactSphereQueryOp>::value && output_kind<OutputOpT>::value != 0
                  && detail::is_float3_images<TranslateOpT>::value)
        {
        if (m_fast_enabled && lbvh.hasFastData())
            {
            gpu::FastQueryArgs a;
            a.spheres = query.spheres;
            a.Q = query.size();
            a.self_rc = 0.f;
            a.self_rows_sorted = 1;
            a.images = detail::image_pointer(images);
            a.n_images = images.size();
            a.lattice = detail::image_lattice(images);
            a.lattice_L = detail::lattice_box(images, query.box);
            a.box = query.box;
            a.pad = query.pad;
            launch_fast(params, lbvh, a, out, transform, query.size());
            if constexpr (std::is_same<OutputOpT, CountNeighborsOp>::value)
                {
                summarize_counts(params.stream, out.nneigh, query.size(), lbvh.getStatusPointer());
                m_summary_self = false;
                }
            return;
            }
        }

    if constexpr (std::is_same<QueryOpT, ExactSphereQueryOpF64>::value && output_kind<OutputOpT>::value != 0
                  && detail::is_float3_images<TranslateOpT>::value)
        {
        if (m_fast_enabled && lbvh.hasFastF64Data())
            {
            gpu::FastQueryArgsF64 a;
            a.spheres = query.spheres;
            a.Q = query.size();
            a.points = query.points;
            a.box = query.box;
            a.pad = query.pad;
            a.images = detail::image_pointer(images);
            a.n_images = images.size();
            a.lattice = detail::image_lattice(images);
            a.lattice_L = detail::lattice_box(images, make_float3((float)query.box.x, (float)query.box.y,
                                                                  (float)query.box.z));
            detail::set_output_f64(a, out);
            constexpr int kind = output_kind<OutputOpT>::value;
            const unsigned int bs = params.tunable;
            gpu::k_traverse_fast_f64<kind, TransformOpT><<<detail::ceil_div(query.size(), bs), bs, 0, params.stream>>>(
                lbvh.fastData(), a, transform);
            detail::check_cuda(cudaGetLastError(), "double traversal launch");
            if constexpr (std::is_same<OutputOpT, CountNeighborsOp>::value)
                {
                summarize_counts(params.stream, out.nneigh, query.size(), lbvh.getStatusPointer());
                m_summary_self = false;
                }
            return;
            }
        }

    if (!m_replay) compress(params, lbvh, transform);
    const unsigned int bs = params.tunable;
    gpu::k_traverse_ref10<OutputOpT, QueryOpT, TranslateOpT>
        <<<detail::ceil_div(query.size(), bs), bs, 0, params.stream>>>(out, data(), query, images,
                                                                        lbvh.getStatusPointer());
    detail::check_cuda(cudaGetLastError(), "traversal launch");
    if constexpr (std::is_same<OutputOpT, CountNeighborsOp>::value)
        {
        summarize_counts(params.stream, out.nneigh, query.size(), lbvh.getStatusPointer());
        m_summary_self = false;
        }
    }

template<class OutputOpT, class TranslateOpT, class TransformOpT>
void LBVHTraverser::traverseSelf(const LaunchParameters& params, const LBVH& lbvh, float rc, float3 box,
                                 float pad, const OutputOpT& out, const TranslateOpT& images,
                                 const TransformOpT& transform, bool rows_sorted)
    {
    const detail::TraceRange trace_range("neighbor::LBVHTraverser::traverseSelf");
    static_assert(output_kind<OutputOpT>::value != 0,
                  "traverseSelf needs CountNeighborsOp, NeighborListOp or CSRNeighborListOp");
    static_assert(detail::is_float3_images<TranslateOpT>::value,
                  "traverseSelf needs SelfOp, ImageListOp<float3> or PeriodicImagesOp");
    if (lbvh.getN() == 0 || images.size() == 0) return;
    if (images.size() > 32)
        throw std::runtime_error("A maximum of 32 image vectors are supported by LBVH traversers.");
    if (!lbvh.hasFastData()) throw std::runtime_error("traverseSelf needs a tree built from points.");
    checkParameter(params);
    gpu::FastQueryArgs a;
    a.spheres = nullptr;
    a.Q = lbvh.getN();
    a.self_rc = rc;
    a.self_rows_sorted = rows_sorted ? 1 : 0;
    a.images = detail::image_pointer(images);
    a.n_images = images.size();
    a.lattice = detail::image_lattice(images);
    a.lattice_L = detail::lattice_box(images, box);
    a.box = box;
    a.pad = pad;
    detail::set_output(a, out);
    const unsigned int longest = detail::max_row(out);
    constexpr int kind = output_kind<OutputOpT>::value;
    const bool symmetric = detail::is_symmetric_images<TranslateOpT>::value && m_symmetric
                           && m_mode == kThreadTraversal && !m_stats && lbvh.getN() < gpu::kHalfMaxN
                           && lbvh.getN() > m_symmetric_min;
    // Counts take the symmetric kernel above the size limits.  A fill after a count that exchanged
    // the pairs (same tree, cutoff, images and rows) assembles the rows; other fills walk
    // symmetrically only while every row also fits the one-thread ordering (longer rows cost
    // more to order than the whole-tree walk costs, and that walk writes every row in order).
    // (a fill after an exchanging count whose summary showed most work past the exchange walks
    // the whole tree: the assembly would re-walk those rows anyway, in a less coherent order)
    if (symmetric && kind != gpu::kFastCount && m_count_cached && m_pair_cache && self_tag(lbvh, a) == m_count_tag
        && !(m_summary_read && m_dense))
        launch_assemble(params, lbvh, a, out, transform);
    else if (symmetric
             && (kind == gpu::kFastCount || (longest > 0u && longest <= gpu::kHalfRowThread)
                 || (kind == gpu::kFastList && longest == 0u)))
        launch_half(params, lbvh, a, out, transform);
    else
        {
        launch_fast(params, lbvh, a, out, transform, lbvh.getN());
        if (kind == gpu::kFastCount)
            {
            summarize_counts(params.stream, a.nneigh, lbvh.getN(), lbvh.getStatusPointer());
            m_summary_self = true;
            m_summary_read = false;
            m_summary_exchange = false;
            m_summary_n = lbvh.getN();
            }
        }
    }

template<class OutputOpT, class TranslateOpT, class TransformOpT>
void LBVHTraverser::traverseSelfSubset(const LaunchParameters& params, const LBVH& lbvh, float rc, float3 box,
                                       float pad, const OutputOpT& out, const TranslateOpT& images,
                                       const TransformOpT& transform, bool rows_sorted,
                                       const unsigned int* subset, unsigned int count)
    {
    const detail::TraceRange trace_range("neighbor::LBVHTraverser::traverseSelfSubset");
    static_assert(output_kind<OutputOpT>::value != 0,
                  "traverseSelfSubset needs CountNeighborsOp, NeighborListOp or CSRNeighborListOp");
    static_assert(detail::is_float3_images<TranslateOpT>::value,
                  "traverseSelfSubset needs SelfOp, ImageListOp<float3> or PeriodicImagesOp");
    if (lbvh.getN() == 0 || images.size() == 0 || count == 0) return;
    if (images.size() > 32)
        throw std::runtime_error("A maximum of 32 image vectors are supported by LBVH traversers.");
    if (!lbvh.hasFastData()) throw std::runtime_error("traverseSelfSubset needs a tree built from points.");
    checkParameter(params);
    gpu::FastQueryArgs a;
    a.spheres = nullptr;
    a.Q = count;
    a.self_rc = rc;
    a.self_rows_sorted = rows_sorted ? 1 : 0;
    a.images = detail::image_pointer(images);
    a.n_images = images.size();
    a.lattice = detail::image_lattice(images);
    a.lattice_L = detail::lattice_box(images, box);
    a.box = box;
    a.pad = pad;
    a.subset = subset;
    launch_fast(params, lbvh, a, out, transform, count);
    }

template<class OutputOpT, class TransformOpT>
void LBVHTraverser::launch_half(const LaunchParameters& params, const LBVH& lbvh, const gpu::FastQueryArgs& a,
                                const OutputOpT& out, const TransformOpT& transform)
    {
    constexpr int kind = output_kind<OutputOpT>::value;
    const unsigned int N = lbvh.getN();
    cudaStream_t stream = params.stream;
    gpu::HalfArgs h;
    h.Q = N;
    h.rc = a.self_rc;
    h.pad = a.pad;
    h.rows_sorted = a.self_rows_sorted;
    h.lattice = a.lattice;
    h.lattice_L = a.lattice_L;
    h.box = a.box;
    h.nneigh = a.nneigh;
    h.list = a.list;
    h.max_neigh = a.max_neigh;
    h.offsets = a.offsets;
    h.caps = a.caps;
    h.own = nullptr;
    if (kind != gpu::kFastCount)
        {
        m_own.reserve(N);
        h.own = m_own.get();
        }
    h.walk_out = nullptr;
    h.walk_in = nullptr;
    h.totals = nullptr;
    h.own_counted = nullptr;
    h.cache_out = nullptr;
    h.in_cache = nullptr;
    h.in_count = nullptr;
    h.in_lost = nullptr;
    // what the last symmetric count ran on: this tree and build, cutoff, images, box and rows
    const PassTag tag = self_tag(lbvh, a);
    const unsigned int grid = detail::ceil_div(N, gpu::kHalfBlock);
    if (kind == gpu::kFastCount)
        {
        m_count_own.reserve(N);
        h.own = m_count_own.get();
        m_count_tag = tag;
        // the exchange unless the last read summary of a self count found a dense workload
        m_count_cached = m_pair_cache && !m_dense;
        m_summary_self = true;
        m_summary_read = false;
        m_summary_exchange = m_count_cached;
        m_summary_n = N;
        clear_summary(stream);
        if (m_count_cached)
            {
            // pair exchange: own keys, incoming keys, incoming counters (by sorted position)
            m_cache.reserve((size_t)N * gpu::kHalfCacheSlots);
            m_in_cache.reserve((size_t)N * gpu::kHalfCacheSlots);
            m_in_count.reserve(N);
            m_lost.reserve(N);
            h.cache_out = m_cache.get();
            h.in_cache = m_in_cache.get();
            h.in_count = m_in_count.get();
            h.in_lost = m_lost.get();
            detail::check_cuda(cudaMemsetAsync(m_in_count.get(), 0, (size_t)N * sizeof(unsigned int), stream), "memset");
            detail::check_cuda(cudaMemsetAsync(m_lost.get(), 0, N, stream), "memset");
            if constexpr (kind == gpu::kFastCount)
                {
                const unsigned int G = half_lanes(N);
                const unsigned int ggrid = (unsigned int)(((unsigned long long)N * G + gpu::kWarpWalkBlock - 1u)
                                                          / gpu::kWarpWalkBlock);
                if (G == 4)
                    gpu::k_traverse_half_group<4><<<ggrid, gpu::kWarpWalkBlock, 0, stream>>>(lbvh.fastData(), h);
                else if (G == 8)
                    gpu::k_traverse_half_group<8><<<ggrid, gpu::kWarpWalkBlock, 0, stream>>>(lbvh.fastData(), h);
                else if (G == 16)
                    gpu::k_traverse_half_group<16><<<ggrid, gpu::kWarpWalkBlock, 0, stream>>>(lbvh.fastData(), h);
                else if (G == 32)
                    gpu::k_traverse_half_group<32><<<ggrid, gpu::kWarpWalkBlock, 0, stream>>>(lbvh.fastData(), h);
                else
                    gpu::k_traverse_half<kind, TransformOpT, true><<<grid, gpu::kHalfBlock, 0, stream>>>(
                        lbvh.fastData(), h, transform);
                }
            gpu::k_count_summary<true><<<summary_grid(N), gpu::kSummaryBlock, 0, stream>>>(
                N, m_count_own.get(), m_in_count.get(), m_lost.get(), lbvh.fastData().primitive, a.self_rows_sorted, a.nneigh,
                m_words.get(), lbvh.getStatusPointer());
            detail::check_cuda(cudaGetLastError(), "half traversal launch");
            return;
            }
        // no exchange: row counters by atomics, walk lengths and row totals for a walking fill
        m_walk.reserve(N);
        m_totals.reserve(N);
        h.walk_out = m_walk.get();
        }
    else if (tag == m_count_tag && !m_count_cached)
        {
        h.totals = m_totals.get();
        h.own_counted = m_count_own.get();
        if (m_work_order) h.walk_in = m_walk.get();
        }
    detail::check_cuda(cudaMemsetAsync(a.nneigh, 0, (size_t)N * sizeof(unsigned int), stream), "memset");
    gpu::k_traverse_half<kind, TransformOpT, false><<<grid, gpu::kHalfBlock, 0, stream>>>(lbvh.fastData(), h,
                                                                                          transform);
    if (kind == gpu::kFastCount)
        {
        detail::check_cuda(cudaMemcpyAsync(m_totals.get(), a.nneigh, (size_t)N * sizeof(unsigned int),
                                           cudaMemcpyDeviceToDevice, stream), "copy");
        gpu::k_count_summary<false><<<summary_grid(N), gpu::kSummaryBlock, 0, stream>>>(
            N, nullptr, nullptr, nullptr, nullptr, 0, a.nneigh, m_words.get(), lbvh.getStatusPointer());
        }
    if (kind != gpu::kFastCount)
        {
        gpu::HalfOrderArgs o;
        o.Q = N;
        o.nneigh = a.nneigh;
        o.list = a.list;
        o.max_neigh = a.max_neigh;
        o.offsets = kind == gpu::kFastCSR ? a.offsets : nullptr;
        o.caps = a.caps;
        o.own = m_own.get();
        o.primitive = lbvh.fastData().primitive;
        o.status = lbvh.getStatusPointer();
        gpu::k_half_order_rows<TransformOpT><<<detail::ceil_div(N, 256), 256, 0, stream>>>(o, transform);
        }
    detail::check_cuda(cudaGetLastError(), "half traversal launch");
    }

template<int kind, class TransformOpT>
void LBVHTraverser::assemble_rows(cudaStream_t stream, const LBVH& lbvh, const gpu::FastQueryArgs& a,
                                  const TransformOpT& transform)
    {
    const unsigned int N = lbvh.getN();
    m_words.reserve(kWordCount);
    m_subset.reserve(N);
    // the re-walk list's length and the re-walk's ticket start at zero
    detail::check_cuda(cudaMemsetAsync(m_words.get() + gpu::kSummaryWords, 0, 2 * sizeof(unsigned int), stream),
                       "memset");
    gpu::AssembleArgs g;
    g.N = N;
    g.rows_sorted = a.self_rows_sorted;
    g.center = a.lattice ? 13u : 0u;
    g.own = m_count_own.get();
    g.in_count = m_in_count.get();
    g.lost = m_lost.get();
    g.own_keys = m_cache.get();
    g.in_keys = m_in_cache.get();
    g.primitive = lbvh.fastData().primitive;
    g.nneigh = a.nneigh;
    g.list = a.list;
    g.max_neigh = a.max_neigh;
    g.offsets = a.offsets;
    g.caps = a.caps;
    g.subset = m_subset.get();
    g.subset_count = m_words.get() + gpu::kSummaryWords;
    g.status = lbvh.getStatusPointer();
    gpu::k_half_assemble<kind, TransformOpT><<<detail::ceil_div(N, 256), 256, 0, stream>>>(g, transform);
    detail::check_cuda(cudaGetLastError(), "assembly launch");
    }

template<class OutputOpT, class TransformOpT>
void LBVHTraverser::launch_assemble(const LaunchParameters& params, const LBVH& lbvh, const gpu::FastQueryArgs& a,
                                    const OutputOpT& out, const TransformOpT& transform)
    {
    constexpr int kind = output_kind<OutputOpT>::value;
    const unsigned int N = lbvh.getN();
    cudaStream_t stream = params.stream;
    assemble_rows<kind>(stream, lbvh, a, transform);
    // rows whose pairs did not fit the exchange: walked whole (their count is known on the device)
    gpu::FastQueryArgs b = a;
    b.Q = N;
    b.subset = m_subset.get();
    b.stats = nullptr;
    b.work_order = 0;
    const unsigned int blocks = std::max(1u, std::min(detail::ceil_div(N, gpu::kSubsetBlock), 8u * sm_count()));
    gpu::SubsetScan scan;
    scan.own = m_count_own.get();
    scan.in_count = m_in_count.get();
    scan.lost = m_lost.get();
    scan.ticket = m_words.get() + gpu::kSummaryWords + 1;
    gpu::k_traverse_subset<kind, TransformOpT><<<blocks, gpu::kSubsetBlock, 0, stream>>>(
        lbvh.fastData(), b, transform, m_words.get() + gpu::kSummaryWords, scan);
    detail::check_cuda(cudaGetLastError(), "assembly launch");
    (void)out;
    }

template<class OutputOpT, class TranslateOpT, class TransformOpT>
void LBVHTraverser::traverseSelfF64(const LaunchParameters& params, const LBVH& lbvh, const double3* points,
                                    double rc, double3 box, float pad, const OutputOpT& out,
                                    const TranslateOpT& images, const TransformOpT& transform, bool rows_sorted)
    {
    const detail::TraceRange trace_range("neighbor::LBVHTraverser::traverseSelfF64");
    static_assert(output_kind<OutputOpT>::value != 0,
                  "traverseSelfF64 needs CountNeighborsOp, NeighborListOp or CSRNeighborListOp");
    static_assert(detail::is_float3_images<TranslateOpT>::value,
                  "traverseSelfF64 needs SelfOp, ImageListOp<float3> or PeriodicImagesOp");
    const unsigned int N = lbvh.getN();
    if (N == 0 || images.size() == 0) return;
    if (images.size() > 32)
        throw std::runtime_error("A maximum of 32 image vectors are supported by LBVH traversers.");
    if (!lbvh.hasFastF64Data())
        throw std::runtime_error("traverseSelfF64 needs a tree built from double points (PointInsertOpF64).");
    if (!points) throw std::runtime_error("traverseSelfF64 needs the tree's double points.");
    checkParameter(params);
    constexpr int kind = output_kind<OutputOpT>::value;
    cudaStream_t stream = params.stream;
    gpu::FastQueryArgsF64 a;
    a.spheres = nullptr;
    a.Q = N;
    a.points = points;
    a.box = box;
    a.pad = pad;
    a.images = detail::image_pointer(images);
    a.n_images = images.size();
    a.lattice = detail::image_lattice(images);
    a.lattice_L = detail::lattice_box(images, make_float3((float)box.x, (float)box.y, (float)box.z));
    detail::set_output_f64(a, out);
    a.self_rc = rc;
    a.self_rows_sorted = rows_sorted ? 1 : 0;
    const bool symmetric = detail::is_symmetric_images<TranslateOpT>::value && m_symmetric
                           && m_mode == kThreadTraversal && !m_stats && N < gpu::kHalfMaxN && N > m_symmetric_min;
    const PassTag tag = self_tag_f64(lbvh, a);
    const unsigned int bs = params.tunable;
    if (kind == gpu::kFastCount)
        {
        m_count_tag = tag;
        m_count_cached = symmetric && m_pair_cache && !m_dense;
        m_summary_self = true;
        m_summary_read = false;
        m_summary_exchange = m_count_cached;
        m_summary_n = N;
        if (m_count_cached)
            {
            clear_summary(stream);
            m_count_own.reserve(N);
            m_cache.reserve((size_t)N * gpu::kHalfCacheSlots);
            m_in_cache.reserve((size_t)N * gpu::kHalfCacheSlots);
            m_in_count.reserve(N);
            m_lost.reserve(N);
            detail::check_cuda(cudaMemsetAsync(m_in_count.get(), 0, (size_t)N * sizeof(unsigned int), stream), "memset");
            detail::check_cuda(cudaMemsetAsync(m_lost.get(), 0, N, stream), "memset");
            gpu::HalfArgsF64 h;
            h.Q = N;
            h.points = points;
            h.rc = rc;
            h.box = box;
            h.pad = pad;
            h.lattice = a.lattice;
            h.lattice_L = a.lattice_L;
            h.own = m_count_own.get();
            h.cache_out = m_cache.get();
            h.in_cache = m_in_cache.get();
            h.in_count = m_in_count.get();
            h.in_lost = m_lost.get();
            gpu::k_traverse_half_f64<><<<detail::ceil_div(N, gpu::kHalfBlock), gpu::kHalfBlock, 0, stream>>>(
                lbvh.fastData(), h);
            gpu::k_count_summary<true><<<summary_grid(N), gpu::kSummaryBlock, 0, stream>>>(
                N, m_count_own.get(), m_in_count.get(), m_lost.get(), lbvh.fastData().primitive, a.self_rows_sorted,
                a.nneigh, m_words.get(), lbvh.getStatusPointer());
            detail::check_cuda(cudaGetLastError(), "double half traversal launch");
            return;
            }
        gpu::k_traverse_fast_f64<kind, TransformOpT><<<detail::ceil_div(N, bs), bs, 0, stream>>>(lbvh.fastData(), a,
                                                                                                 transform);
        detail::check_cuda(cudaGetLastError(), "double traversal launch");
        summarize_counts(stream, a.nneigh, N, lbvh.getStatusPointer());
        return;
        }
    if (symmetric && m_count_cached && m_pair_cache && tag == m_count_tag && !(m_summary_read && m_dense))
        {
        // rows from the exchange; the rows past it walk the whole tree (listed by the assembly,
        // their number read on the device)
        gpu::FastQueryArgs g{};
        g.self_rows_sorted = a.self_rows_sorted;
        g.lattice = a.lattice;
        g.nneigh = a.nneigh;
        g.list = a.list;
        g.max_neigh = a.max_neigh;
        g.offsets = a.offsets;
        g.caps = a.caps;
        assemble_rows<kind>(stream, lbvh, g, transform);
        gpu::FastQueryArgsF64 b = a;
        b.subset = m_subset.get();
        b.subset_count = m_words.get() + gpu::kSummaryWords;
        const unsigned int blocks = std::max(1u, std::min(detail::ceil_div(N, bs), 8u * sm_count()));
        gpu::k_traverse_fast_f64<kind, TransformOpT><<<blocks, bs, 0, stream>>>(lbvh.fastData(), b, transform);
        detail::check_cuda(cudaGetLastError(), "double traversal launch");
        return;
        }
    gpu::k_traverse_fast_f64<kind, TransformOpT><<<detail::ceil_div(N, bs), bs, 0, stream>>>(lbvh.fastData(), a,
                                                                                             transform);
    detail::check_cuda(cudaGetLastError(), "double traversal launch");
    }

} // namespace neighbor

#endif // NEIGHBOR_LBVH_TRAVERSER_H_
