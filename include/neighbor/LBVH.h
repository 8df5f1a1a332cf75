// Linear bounding volume hierarchy built on the GPU.
//
// Public interface as in the reference (include/neighbor/LBVH.h:47-219): setup()/build() with
// LaunchParameters, a stream, or neither; getRoot/getN/getNInternal/getNNodes; getters for
// parents, children, bounds and the sorted primitive order as host-indexable shared_arrays;
// data() for kernels.  The tree produced is the reference's: same Morton codes, same stable order,
// same Karras hierarchy, same boxes.
//
// What differs is how it is built (all hand-written sm_103a kernels, no CUB): a fused Morton /
// histogram / bounds pass, a onesweep radix sort, a block-local agglomerative climb that forms
// the radix tree with packed 15-bit boxes, and one pass that writes the 16-bit pre-order
// traversal tree (fastData()) with leaf buckets of up to getLeafSize() primitives.  Every
// spin-wait in those kernels is bounded; checkStatus() reports a wait that gave up.
//
// The reference-layout arrays (parents, children, float boxes) are not needed by the traversal
// tree.  For trees of points they are computed when first asked for after a build (a getter,
// data(), or a traversal with user ops), on the build's stream, so a build that only feeds the
// fast traversal does not write them; hold no reference to them across builds without calling
// the getter again.  For every other insert op they are computed during build().
#ifndef NEIGHBOR_LBVH_H_
#define NEIGHBOR_LBVH_H_

#include <atomic>
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <type_traits>

#include <cuda_runtime.h>

#include "InsertOps.h"
#include "LBVHData.h"
#include "Memory.h"
#include "Trace.h"
#include "Tunable.h"
#include "kernels/build.cuh"

namespace neighbor
{

namespace detail
{
inline void check_cuda(cudaError_t code, const char* what)
    {
    if (code != cudaSuccess)
        {
        (void)cudaGetLastError();
        throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(code));
        }
    }

inline unsigned int ceil_div(unsigned long long a, unsigned long long b)
    {
    return (unsigned int)((a + b - 1) / b);
    }

inline unsigned int bits_for_count(unsigned int leaf_size)
    {
    unsigned int b = 0;
    while ((1u << b) < leaf_size) ++b;
    return b;
    }
} // namespace detail

class LBVH : public Tunable<unsigned int>
    {
    public:
        LBVH()
            : Tunable<unsigned int>(32, 1024, 32), m_root(LBVHSentinel), m_N(0), m_N_internal(0),
              m_N_nodes(0), m_capacity(0), m_leaf_size(4), m_radix_bits(8), m_fast_points(false), m_fast_f64(false),
              m_epoch(0), m_block(256), m_climb_block(512), m_stream(0), m_ref_valid(true),
              m_sorted_event(nullptr)
            {}

        ~LBVH()
            {
            if (m_sorted_event) cudaEventDestroy(m_sorted_event);
            }
        LBVH(const LBVH&) = delete;
        LBVH& operator=(const LBVH&) = delete;

        template<class InsertOpT>
        void setup(const LaunchParameters& params, const InsertOpT& insert)
            {
            (void)params;
            allocate(insert.size());
            }

        template<class InsertOpT>
        void setup(cudaStream_t stream, const InsertOpT& insert)
            {
            setup(LaunchParameters(32, stream), insert);
            }

        template<class InsertOpT>
        void setup(const InsertOpT& insert)
            {
            setup(cudaStream_t(0), insert);
            }

        template<class InsertOpT>
        void build(const LaunchParameters& params, const InsertOpT& insert, const float3& lo, const float3& hi);

        template<class InsertOpT>
        void build(cudaStream_t stream, const InsertOpT& insert, const float3& lo, const float3& hi)
            {
            build(LaunchParameters(32, stream), insert, lo, hi);
            }

        template<class InsertOpT>
        void build(const InsertOpT& insert, const float3& lo, const float3& hi)
            {
            build(cudaStream_t(0), insert, lo, hi);
            }

        int getRoot() const { return m_root; }
        unsigned int getN() const { return m_N; }
        unsigned int getNInternal() const { return m_N_internal; }
        unsigned int getNNodes() const { return m_N_nodes; }

        const shared_array<int>& getParents() const { materialize(m_stream); return m_parent; }
        const shared_array<int>& getLeftChildren() const { materialize(m_stream); return m_left; }
        const shared_array<int>& getRightChildren() const { materialize(m_stream); return m_right; }
        const shared_array<float3>& getLowerBounds() const { materialize(m_stream); return m_lo; }
        const shared_array<float3>& getUpperBounds() const { materialize(m_stream); return m_hi; }
        const shared_array<unsigned int>& getPrimitives() const { return m_indexes.current(); }
        const shared_array<unsigned int>& getCodes() const { return m_codes.current(); }

        const ConstLBVHData data() const { return data(m_stream); }

        // data() with the reference-layout arrays made current on `stream` (for callers whose
        // kernels run on a stream other than the build's).
        const ConstLBVHData data(cudaStream_t stream) const
            {
            materialize(stream);
            ConstLBVHData t;
            t.parent = m_parent.get();
            t.left = m_left.get();
            t.right = m_right.get();
            t.primitive = m_indexes.current().get();
            t.lo = m_lo.get();
            t.hi = m_hi.get();
            t.root = m_root;
            return t;
            }

        // ---- additions of this library ----

        // Identifier of the current tree: unique in the process (every build of any LBVH takes the
        // next one), so that a traverser's results of an earlier pass are never taken for another
        // tree's, even one built in the same memory after this object was destroyed.
        unsigned long long getBuildId() const { return m_build_id; }

        // Primitives per leaf bucket of the traversal tree (1..64; rounded to a power of two).
        void setLeafSize(unsigned int leaf_size)
            {
            if (leaf_size < 1 || leaf_size > 64) throw std::runtime_error("Leaf size must be in [1, 64].");
            unsigned int b = 1;
            while (b < leaf_size) b <<= 1;
            m_leaf_size = b;
            }
        unsigned int getLeafSize() const { return m_leaf_size; }

        // Radix digit width of the sort: 8 (4 passes over 30-bit codes) or 10 (3 passes).
        void setRadixBits(unsigned int bits)
            {
            if (bits != 8 && bits != 10) throw std::runtime_error("Radix bits must be 8 or 10.");
            m_radix_bits = bits;
            }
        unsigned int getRadixBits() const { return m_radix_bits; }

        // Sorted leaves per block of the agglomerative climb: 128, 256 or 512.
        void setClimbBlock(unsigned int leaves)
            {
            if (leaves != 128 && leaves != 256 && leaves != 512)
                throw std::runtime_error("Climb block must be 128, 256 or 512.");
            m_climb_block = leaves;
            }
        unsigned int getClimbBlock() const { return m_climb_block; }

        // True when the last build used a point insert op, so fastData() holds point positions.
        bool hasFastData() const { return m_fast_points && m_N > 0; }
        // True when the last build used PointInsertOpF64: fastData()'s point records hold each
        // double point rounded down to FP32 (its leaf box's lower corner), for the double walk.
        bool hasFastF64Data() const { return m_fast_f64 && m_N > 0; }

        FastLBVHData fastData() const
            {
            FastLBVHData f;
            f.nodes = m_nodes.get();
            f.n_boxes = m_small.get() + kSmallLiveCount;
            f.points = m_payload.get();
            f.primitive = m_indexes.current().get();
            f.pre = m_live.get();
            f.frame = reinterpret_cast<const QuantFrame*>(m_small.get() + kSmallFrame);
            f.status = m_small.get() + kSmallStatus;
            f.N = m_N;
            f.leaf_size = m_leaf_size;
            return f;
            }

        // Event recorded on the build's stream once the sorted codes and primitive order of the
        // last build are final (before the tree is formed): work that needs only those -- such as
        // capacity prediction -- can start on another stream while the rest of the build runs.
        cudaEvent_t sortedEvent() const { return m_sorted_event; }

        // Device status word (0 = all waits completed).
        const unsigned int* getStatusPointer() const { return m_small.get() + kSmallStatus; }

        // Wait for the stream and throw if a bounded wait in the last build gave up.
        unsigned int checkStatus(cudaStream_t stream = 0) const
            {
            if (m_capacity == 0) return 0;
            unsigned int s = 0;
            detail::check_cuda(cudaMemcpyAsync(&s, getStatusPointer(), sizeof(unsigned int),
                                               cudaMemcpyDeviceToHost, stream), "status copy");
            detail::check_cuda(cudaStreamSynchronize(stream), "status sync");
            if (s != gpu::kStatusOk)
                throw std::runtime_error("LBVH build: a bounded device wait gave up (status "
                                         + std::to_string(s) + ")");
            return s;
            }

        // Number of traversal records (box + point) of the last build (synchronises the stream).
        unsigned int getNumFastNodes(cudaStream_t stream = 0) const
            {
            if (m_N == 0) return 0;
            unsigned int n = 0;
            detail::check_cuda(cudaMemcpyAsync(&n, fastData().n_boxes, sizeof(unsigned int),
                                               cudaMemcpyDeviceToHost, stream), "node count copy");
            detail::check_cuda(cudaStreamSynchronize(stream), "node count sync");
            return n + m_N;
            }

    private:
        // tile shape of the onesweep sort: threads per block, keys per thread
        static constexpr int kSortBlock = 256;
        static constexpr int kSortItems = 16;
        // below kSortSmallN keys the passes take tiles of kSortItemsSmall keys per thread: more
        // tiles, so that a small sort spreads over more SMs
        static constexpr int kSortItemsSmall = 4;
        static constexpr unsigned int kSortSmallN = 1u << 20;
        // layout of the small scratch buffer (uint32 words)
        static constexpr size_t kSmallHist = 0;            // 4 passes x 1024
        static constexpr size_t kSmallOffsets = 4096;      // 4 passes x 1024
        static constexpr size_t kSmallCounters = 8192;     // tile tickets (passes, scan at +7), climb items at +6
        static constexpr size_t kSmallBounds = 8200;       // 6 words
        static constexpr size_t kSmallStatus = 8206;       // 1 word
        static constexpr size_t kSmallZeroEnd = 8208;      // words cleared before every build
        static constexpr size_t kSmallLiveCount = 8208;    // 1 word
        static constexpr size_t kSmallFrame = 8212;        // QuantFrame (9 floats), 16-byte aligned
        static constexpr size_t kSmallWords = 8224;

        int m_root;
        unsigned int m_N;
        unsigned int m_N_internal;
        unsigned int m_N_nodes;
        unsigned int m_capacity;
        unsigned int m_leaf_size;
        unsigned int m_radix_bits;
        bool m_fast_points;
        bool m_fast_f64;
        unsigned int m_epoch;
        unsigned long long m_build_id = 0;
        unsigned int m_block;
        unsigned int m_climb_block;
        cudaStream_t m_stream;
        mutable bool m_ref_valid;
        cudaEvent_t m_sorted_event;  // reference-layout arrays match the last build

        mutable shared_array<int> m_parent;
        mutable shared_array<int> m_left;
        mutable shared_array<int> m_right;
        mutable shared_array<float3> m_lo;
        mutable shared_array<float3> m_hi;
        buffered_array<unsigned int> m_codes;
        buffered_array<unsigned int> m_indexes;

        device_array<uint4> m_nbox;            // per internal node: packed box, first primitive
        device_array<uint2> m_nmeta;           // per internal node: last primitive, db | live
        device_array<unsigned int> m_kids;     // child ids met at splits across blocks
        device_array<uint2> m_items;           // nodes whose climb continues across blocks
        device_array<unsigned int> m_live;     // box records per first primitive, then their scan
        mutable device_array<unsigned int> m_locks;
        device_array<uint4> m_nodes;
        device_array<float4> m_payload;
        device_array<unsigned char> m_hi_bits;   // double point trees: upper-corner bits per leaf
        device_array<unsigned int> m_small;
        device_array<unsigned long long> m_sort_status;
        device_array<unsigned long long> m_scan_status;

        void allocate(unsigned int N);

        // Reference-layout arrays of the last build (Karras children/parents, float boxes).
        template<class LeafBoxT>
        void reference_layout(const LeafBoxT& leaf_box, cudaStream_t stream) const;
        void materialize(cudaStream_t stream) const
            {
            if (m_ref_valid) return;
            if (m_fast_f64)
                reference_layout(gpu::PayloadLeafBoxF64{m_payload.get(), m_hi_bits.get()}, stream);
            else
                reference_layout(gpu::PayloadLeafBox{m_payload.get()}, stream);
            }

        unsigned int next_epoch()
            {
            static std::atomic<unsigned long long> s_next_build_id{0};
            m_build_id = ++s_next_build_id;
            ++m_epoch;
            if (m_epoch >= (1u << 27))
                {
                // tags would repeat: clear every tagged buffer once and restart
                m_epoch = 1;
                if (m_sort_status.size())
                    cudaMemset(m_sort_status.get(), 0, m_sort_status.size() * sizeof(unsigned long long));
                if (m_scan_status.size())
                    cudaMemset(m_scan_status.get(), 0, m_scan_status.size() * sizeof(unsigned long long));
                if (m_locks.size()) cudaMemset(m_locks.get(), 0, m_locks.size() * sizeof(unsigned int));
                }
            return m_epoch;
            }

        template<class InsertOpT, int RB, int ITEMS>
        void sort_codes(const InsertOpT& insert, const float3& lo, const float3& ext,
                        cudaStream_t stream, unsigned int epoch);
    };

namespace gpu
{
// Single-primitive tree (the reference's lbvh_one_primitive case): identity order, sentinel
// parent, and a traversal tree of one point record (no box records).
static __global__ void k_single_init(unsigned int* primitive, int* parent, unsigned int* live)
    {
    if (threadIdx.x == 0 && blockIdx.x == 0)
        {
        primitive[0] = 0u;
        parent[0] = LBVHSentinel;
        live[0] = 0u;
        }
    }
} // namespace gpu

inline void LBVH::allocate(unsigned int N)
    {
    if (N >= (1u << 30)) throw std::runtime_error("LBVH supports fewer than 2^30 primitives.");
    m_root = 0;
    m_N = N;
    m_N_internal = N > 0 ? N - 1 : 0;
    m_N_nodes = N + m_N_internal;
    if (m_small.size() == 0)
        {
        m_small.reserve(kSmallWords);
        detail::check_cuda(cudaMemset(m_small.get(), 0, kSmallWords * sizeof(unsigned int)), "memset");
        }
    if (N == 0 || N <= m_capacity) return;

    const size_t nodes = 2 * (size_t)N - 1;
    if (m_parent.size() < nodes)
        {
        shared_array<int> parent(nodes);
        m_parent.swap(parent);
        shared_array<float3> lo(nodes), hi(nodes);
        m_lo.swap(lo);
        m_hi.swap(hi);
        }
    if (N > 1 && m_left.size() < (size_t)N - 1)
        {
        shared_array<int> left(N - 1), right(N - 1);
        m_left.swap(left);
        m_right.swap(right);
        }
    if (m_codes.size() < N)
        {
        buffered_array<unsigned int> codes(N), indexes(N);
        m_codes.swap(codes);
        m_indexes.swap(indexes);
        }
    m_nbox.reserve(N);
    m_nmeta.reserve(N);
    m_kids.reserve(2 * (size_t)N);
    // at most one pending node per split of a block plus two per block edge
    m_items.reserve((size_t)N + 2 * (size_t)detail::ceil_div(N, 128) + 16);
    m_live.reserve((size_t)N + 1 + gpu::kScanTile);
    if (m_locks.size() < N)
        {
        m_locks.reserve(N);
        detail::check_cuda(cudaMemset(m_locks.get(), 0, m_locks.size() * sizeof(unsigned int)), "memset");
        }
    m_nodes.reserve(nodes);
    m_payload.reserve(N);
    // one status word per (tile, digit, pass), enough for the widest configuration (4 passes x 256
    // digits, or 3 passes x 1024 digits) of the sort's tiles
    // the most tiles any size up to this capacity sorts in: small tiles below kSortSmallN keys
    const size_t tiles = std::max(detail::ceil_div((size_t)std::min(N, kSortSmallN - 1u), (size_t)kSortBlock * kSortItemsSmall),
                                  detail::ceil_div((size_t)N, (size_t)kSortBlock * kSortItems));
    const size_t need = tiles * 4 * 1024;
    if (m_sort_status.size() < need)
        {
        m_sort_status.reserve(need);
        detail::check_cuda(cudaMemset(m_sort_status.get(), 0, need * sizeof(unsigned long long)), "memset");
        }
    const size_t scan_tiles = detail::ceil_div((size_t)N + 1, gpu::kScanTile);
    if (m_scan_status.size() < scan_tiles)
        {
        m_scan_status.reserve(scan_tiles);
        detail::check_cuda(cudaMemset(m_scan_status.get(), 0, scan_tiles * sizeof(unsigned long long)), "memset");
        }
    m_capacity = N;
    }

template<class InsertOpT, int RB, int ITEMS>
void LBVH::sort_codes(const InsertOpT& insert, const float3& lo, const float3& ext,
                      cudaStream_t stream, unsigned int epoch)
    {
    constexpr int R = gpu::RadixConfig<RB>::kRadix;
    constexpr int P = gpu::RadixConfig<RB>::kPasses;
    constexpr int BLOCK = kSortBlock;
    typedef gpu::OnesweepConfig<RB, BLOCK, ITEMS> Cfg;
    const unsigned int N = m_N;
    unsigned int* small = m_small.get();
    unsigned int* error = small + kSmallStatus;

    // digit histograms of every pass + bounds
    {
    const unsigned int grid = std::min(detail::ceil_div(N, 256), 152u * 8u);
    // the codes also go to the buffer the first sort pass reads
    gpu::k_codes_histogram<InsertOpT, RB><<<grid, 256, 0, stream>>>(insert, N, lo, ext, small + kSmallHist,
                                                                    small + kSmallBounds, m_codes.current().get());
    gpu::k_digit_offsets<RB><<<P, 1024, 0, stream>>>(small + kSmallHist, small + kSmallOffsets);
    }

    static bool attr_set[2] = {false, false};
    if (!attr_set[0])
        {
        detail::check_cuda(cudaFuncSetAttribute(gpu::k_onesweep<InsertOpT, RB, BLOCK, ITEMS, true>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)Cfg::kSmemBytes), "onesweep attribute");
        detail::check_cuda(cudaFuncSetAttribute(gpu::k_onesweep<InsertOpT, RB, BLOCK, ITEMS, false>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)Cfg::kSmemBytes), "onesweep attribute");
        // all of L1 that can be shared memory: tiles are staged there, several blocks per SM
        detail::check_cuda(cudaFuncSetAttribute(gpu::k_onesweep<InsertOpT, RB, BLOCK, ITEMS, true>,
                                                cudaFuncAttributePreferredSharedMemoryCarveout,
                                                (int)cudaSharedmemCarveoutMaxShared), "onesweep attribute");
        detail::check_cuda(cudaFuncSetAttribute(gpu::k_onesweep<InsertOpT, RB, BLOCK, ITEMS, false>,
                                                cudaFuncAttributePreferredSharedMemoryCarveout,
                                                (int)cudaSharedmemCarveoutMaxShared), "onesweep attribute");
        attr_set[0] = true;
        }

    const unsigned int tiles = detail::ceil_div(N, Cfg::kTile);
    for (int p = 0; p < P; ++p)
        {
        const unsigned int* kin = m_codes.current().get();
        const unsigned int* vin = m_indexes.current().get();
        unsigned int* kout = m_codes.alternate().get();
        unsigned int* vout = m_indexes.alternate().get();
        unsigned long long* status = m_sort_status.get() + (size_t)p * tiles * R;
        const unsigned int tag = (epoch * 4u + (unsigned int)p) & 0x3fffffffu;
        if (p == 0)
            gpu::k_onesweep<InsertOpT, RB, BLOCK, ITEMS, true><<<tiles, BLOCK, Cfg::kSmemBytes, stream>>>(
                insert, lo, ext, kin, vin, kout, vout, N, p * RB, small + kSmallOffsets + p * R, status,
                tag, small + kSmallCounters + p, error);
        else
            gpu::k_onesweep<InsertOpT, RB, BLOCK, ITEMS, false><<<tiles, BLOCK, Cfg::kSmemBytes, stream>>>(
                insert, lo, ext, kin, vin, kout, vout, N, p * RB, small + kSmallOffsets + p * R, status,
                tag, small + kSmallCounters + p, error);
        m_codes.flip();
        m_indexes.flip();
        }
    }

template<class LeafBoxT>
void LBVH::reference_layout(const LeafBoxT& leaf_box, cudaStream_t stream) const
    {
    m_ref_valid = true;
    const unsigned int N = m_N;
    if (N == 0) return;
    const unsigned int* status = getStatusPointer();
    const unsigned int bs = m_block;
    if (N > 1)
        gpu::k_gen_hierarchy<<<detail::ceil_div(N - 1, bs), bs, 0, stream>>>(
            m_codes.current().get(), N, m_left.get(), m_right.get(), m_parent.get(), status);
    gpu::RefBubbleArgs a;
    a.N = N;
    a.parent = m_parent.get();
    a.left = m_left.get();
    a.right = m_right.get();
    a.lo = m_lo.get();
    a.hi = m_hi.get();
    a.locks = m_locks.get();
    a.tag = 2u * m_epoch + 1u;
    a.error = status;
    gpu::k_ref_bubble<LeafBoxT><<<detail::ceil_div(N, bs), bs, 0, stream>>>(leaf_box, a);
    detail::check_cuda(cudaGetLastError(), "LBVH reference layout launch");
    }

template<class InsertOpT>
void LBVH::build(const LaunchParameters& params, const InsertOpT& insert, const float3& lo, const float3& hi)
    {
    const detail::TraceRange trace_range("neighbor::LBVH::build");
    setup(params, insert);
    m_fast_points = is_point_insert<InsertOpT>::value;
    m_fast_f64 = std::is_same<InsertOpT, PointInsertOpF64>::value;
    m_ref_valid = true;
    if (m_N == 0) return;
    checkParameter(params);
    cudaStream_t stream = params.stream;
    m_stream = stream;
    m_block = params.tunable;
    const unsigned int N = m_N;
    const unsigned int epoch = next_epoch();
    unsigned int* small = m_small.get();

    detail::check_cuda(cudaMemsetAsync(small, 0, kSmallZeroEnd * sizeof(unsigned int), stream), "memset");
    // counts past the last position stay zero for the scan
    detail::check_cuda(cudaMemsetAsync(m_live.get() + N, 0, sizeof(unsigned int), stream), "memset");

    const float3 ext = make_float3(hi.x - lo.x, hi.y - lo.y, hi.z - lo.z);
    if (N == 1)
        {
        // bounds for the quantisation frame (no sort needed)
        gpu::k_codes_histogram<InsertOpT, 8><<<1, 256, 0, stream>>>(insert, N, lo, ext, small + kSmallHist,
                                                                    small + kSmallBounds);
        gpu::k_single_init<<<1, 32, 0, stream>>>(m_indexes.current().get(), m_parent.get(), m_live.get());
        }
    else if (m_radix_bits == 10)
        {
        if (N < kSortSmallN)
            sort_codes<InsertOpT, 10, kSortItemsSmall>(insert, lo, ext, stream, epoch);
        else
            sort_codes<InsertOpT, 10, kSortItems>(insert, lo, ext, stream, epoch);
        }
    else
        {
        if (N < kSortSmallN)
            sort_codes<InsertOpT, 8, kSortItemsSmall>(insert, lo, ext, stream, epoch);
        else
            sort_codes<InsertOpT, 8, kSortItems>(insert, lo, ext, stream, epoch);
        }
    if (!m_sorted_event)
        detail::check_cuda(cudaEventCreateWithFlags(&m_sorted_event, cudaEventDisableTiming), "event create");
    detail::check_cuda(cudaEventRecord(m_sorted_event, stream), "event record");

    // radix tree, packed boxes, box-record counts
    gpu::ClimbArgs c;
    c.N = N;
    c.codes = m_codes.current().get();
    c.primitive = m_indexes.current().get();
    c.payload = m_payload.get();
    c.nbox = m_nbox.get();
    c.nmeta = m_nmeta.get();
    c.kids = m_kids.get();
    c.locks = m_locks.get();
    c.tag = 2u * epoch;
    c.counts = m_live.get();
    c.items = m_items.get();
    c.n_items = small + kSmallCounters + 6;
    c.item_capacity = (unsigned int)m_items.size();
    c.bounds = small + kSmallBounds;
    c.frame_out = reinterpret_cast<QuantFrame*>(small + kSmallFrame);
    c.leaf_size = m_leaf_size;
    c.error = small + kSmallStatus;
    if (m_fast_f64)
        {
        m_hi_bits.reserve(N);
        c.hi_bits = m_hi_bits.get();
        }
    const unsigned int T = m_climb_block;
    if (T == 128)
        gpu::k_climb<InsertOpT, 128><<<detail::ceil_div(N, 128), 128, 0, stream>>>(insert, c);
    else if (T == 256)
        gpu::k_climb<InsertOpT, 256><<<detail::ceil_div(N, 256), 256, 0, stream>>>(insert, c);
    else
        gpu::k_climb<InsertOpT, 512><<<detail::ceil_div(N, 512), 512, 0, stream>>>(insert, c);
    if (N > T && N <= gpu::kClimbOneBlockMaxN)
        gpu::k_climb_global_block<InsertOpT><<<1, gpu::kClimbOneBlockThreads, 0, stream>>>(insert, c);
    else if (N > T)
        gpu::k_climb_global<InsertOpT><<<std::min(detail::ceil_div(N, 2048), 152u * 8u), 256, 0, stream>>>(insert, c);

    // pre-order positions of the box records
    gpu::k_scan_exclusive<<<detail::ceil_div((size_t)N + 1, gpu::kScanTile), gpu::kScanBlock, 0, stream>>>(
        m_live.get(), m_live.get(), N, m_scan_status.get(), epoch & 0x3fffffffu, small + kSmallCounters + 7,
        small + kSmallLiveCount, small + kSmallStatus);

    gpu::EmitArgs e;
    e.N = N;
    e.payload = m_payload.get();
    e.nbox = m_nbox.get();
    e.nmeta = m_nmeta.get();
    e.pre = m_live.get();
    e.nodes = m_nodes.get();
    e.node_capacity = (unsigned int)m_nodes.size();
    e.error = small + kSmallStatus;
    gpu::k_emit<<<detail::ceil_div(N, 256), 256, 0, stream>>>(e);
    detail::check_cuda(cudaGetLastError(), "LBVH build launch");

    // point trees form the reference-layout arrays on first access (from the payload); other
    // insert ops here, while their inputs are known to be valid
    m_ref_valid = false;
    if (!is_point_insert<InsertOpT>::value && !m_fast_f64)
        reference_layout(gpu::InsertLeafBox<InsertOpT>{insert, m_indexes.current().get()}, stream);
    }

} // namespace neighbor

#endif // NEIGHBOR_LBVH_H_
