// Morton-code sort of a point set that allocates no memory.
//
// Some callers cannot call cudaMalloc: code that runs inside a host framework which owns every
// device allocation (and forbids side allocations), code that must not add allocator
// synchronisation to a latency-critical loop, and code that runs while the device memory budget
// is fully committed.  nbr_morton_sort_noalloc gives them the first stage of the LBVH build --
// 30-bit Morton codes of the points and their stable sort -- with all working memory in one
// file-scope device array of fixed size (NBR_NOALLOC_MAX_POINTS points).  The caller passes only
// inputs and outputs.
//
// The array lives as long as the library is loaded, on every GPU that loads it.  Its address is
// looked up once per device (cudaGetSymbolAddress with that device current) on the first call
// there; make that first call before any stream capture.  Every call shares the array: calls that
// overlap on the GPU (two streams, two host threads) race and must be serialised by the caller.
// The counters that must start at zero are cleared at the start of every call.
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "neighbor/neighbor.h"
#include "neighbor_gb300.h"

namespace
{
namespace gpu = neighbor::gpu;

constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kPasses = gpu::RadixConfig<kRadixBits>::kPasses;  // 4 passes over 30 bits
constexpr int kBlock = 256;
constexpr int kItems = 16;
typedef gpu::OnesweepConfig<kRadixBits, kBlock, kItems> Cfg;

constexpr unsigned int kMaxPoints = NBR_NOALLOC_MAX_POINTS;
constexpr unsigned int kMaxTiles = (kMaxPoints + Cfg::kTile - 1) / Cfg::kTile;

// Word layout of the scratch array.
constexpr size_t kHistWords = (size_t)kPasses * kRadix;       // digit histograms
constexpr size_t kOffsetWords = (size_t)kPasses * kRadix;     // their exclusive scans
constexpr size_t kTicketWords = 8;                            // tile tickets, one per pass
constexpr size_t kBoundsWords = 8;                            // scene bounds (6 used)
constexpr size_t kStatusWords = 8;                            // wait status (1 used)
constexpr size_t kZeroWords = kHistWords + kOffsetWords + kTicketWords + kBoundsWords + kStatusWords;
constexpr size_t kLookbackWords = 2 * (size_t)kPasses * kMaxTiles * kRadix;  // uint64 words
constexpr size_t kBufferWords = 2 * (size_t)kMaxPoints;       // one ping-pong pair (keys, values)
constexpr size_t kScratchWords = kZeroWords + kLookbackWords + kBufferWords;

// ~10 MB: 8 MB ping-pong buffer + 2 MB look-back words + a few KB of counters.
static __device__ __align__(256) unsigned int g_noalloc_scratch[kScratchWords];

std::mutex g_mutex;
constexpr int kMaxDevices = 64;
unsigned int* g_scratch_ptr[kMaxDevices] = {};
unsigned int g_calls[kMaxDevices] = {};
bool g_attr_set[kMaxDevices] = {};

} // namespace

// Message of the last failed call (kept by the C-ABI layer in capi.cu).
namespace neighbor_capi
{
void set_last_error(const std::string& msg);
}

static int noalloc_fail(int code, const std::string& msg)
    {
    neighbor_capi::set_last_error(msg);
    return code;
    }

extern "C" int nbr_morton_sort_noalloc(const float* points, unsigned int N, const float lo[3],
                                       const float hi[3], unsigned int* codes_out,
                                       unsigned int* order_out, void* stream)
    {
    if (N == 0) return NBR_OK;
    if (!points || !lo || !hi || !codes_out || !order_out) return noalloc_fail(NBR_ERR_INVALID, "null argument");
    if (N > kMaxPoints)
        return noalloc_fail(NBR_ERR_INVALID, "nbr_morton_sort_noalloc: " + std::to_string(N)
                                                 + " points exceed its fixed scratch of "
                                                 + std::to_string(kMaxPoints) + " points");

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        {
        (void)cudaGetLastError();
        return noalloc_fail(NBR_ERR_CUDA, "nbr_morton_sort_noalloc: no current device");
        }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    unsigned int* scratch = nullptr;
    unsigned int epoch = 0;
        {
        std::lock_guard<std::mutex> lock(g_mutex);
        if (!g_scratch_ptr[dev])
            {
            // One-time set-up on this device (the device is current): the host-side name of
            // the array is not a device address, so look the address up.
            void* ptr = nullptr;
            const cudaError_t rc = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (rc != cudaSuccess || !ptr)
                {
                (void)cudaGetLastError();
                return noalloc_fail(NBR_ERR_CUDA, std::string("nbr_morton_sort_noalloc: scratch address: ")
                                                      + cudaGetErrorString(rc));
                }
            g_scratch_ptr[dev] = static_cast<unsigned int*>(ptr);
            }
        if (!g_attr_set[dev])
            {
            if (cudaFuncSetAttribute(gpu::k_onesweep<neighbor::PointInsertOp, kRadixBits, kBlock, kItems, true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::kSmemBytes) != cudaSuccess
                || cudaFuncSetAttribute(gpu::k_onesweep<neighbor::PointInsertOp, kRadixBits, kBlock, kItems, false>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::kSmemBytes) != cudaSuccess)
                {
                (void)cudaGetLastError();
                return NBR_ERR_CUDA;
                }
            g_attr_set[dev] = true;
            }
        scratch = g_scratch_ptr[dev];
        // distinct look-back tags per call: the array keeps the previous call's words
        epoch = ++g_calls[dev];
        if (epoch >= (1u << 27))
            {
            g_calls[dev] = epoch = 1;
            if (cudaMemsetAsync(scratch + kZeroWords, 0, kLookbackWords * sizeof(unsigned int), st) != cudaSuccess)
                {
                (void)cudaGetLastError();
                return NBR_ERR_CUDA;
                }
            }
        }

    unsigned int* hist = scratch;
    unsigned int* offsets = hist + kHistWords;
    unsigned int* tickets = offsets + kOffsetWords;
    unsigned int* bounds = tickets + kTicketWords;
    unsigned int* status_word = bounds + kBoundsWords;
    unsigned long long* lookback = reinterpret_cast<unsigned long long*>(scratch + kZeroWords);
    unsigned int* buf_keys = scratch + kZeroWords + kLookbackWords;
    unsigned int* buf_vals = buf_keys + kMaxPoints;

    // histograms, tickets, bounds and the status word start at zero
    if (cudaMemsetAsync(scratch, 0, kZeroWords * sizeof(unsigned int), st) != cudaSuccess)
        {
        (void)cudaGetLastError();
        return NBR_ERR_CUDA;
        }
    const neighbor::PointInsertOp insert(reinterpret_cast<const float3*>(points), N);
    const float3 slo = make_float3(lo[0], lo[1], lo[2]);
    const float3 ext = make_float3(hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]);
    const unsigned int grid = (N + 255) / 256 < 152u * 8u ? (N + 255) / 256 : 152u * 8u;
    gpu::k_codes_histogram<neighbor::PointInsertOp, kRadixBits><<<grid, 256, 0, st>>>(insert, N, slo, ext, hist, bounds);
    gpu::k_digit_offsets<kRadixBits><<<kPasses, 1024, 0, st>>>(hist, offsets);

    // four passes: points -> scratch -> out -> scratch -> out
    const unsigned int tiles = (N + Cfg::kTile - 1) / Cfg::kTile;
    const unsigned int* kin = nullptr;
    const unsigned int* vin = nullptr;
    for (int p = 0; p < kPasses; ++p)
        {
        unsigned int* kout = (p % 2 == 0) ? buf_keys : codes_out;
        unsigned int* vout = (p % 2 == 0) ? buf_vals : order_out;
        unsigned long long* stat = lookback + (size_t)p * kMaxTiles * kRadix;
        const unsigned int tag = (epoch * 4u + (unsigned int)p) & 0x3fffffffu;
        if (p == 0)
            gpu::k_onesweep<neighbor::PointInsertOp, kRadixBits, kBlock, kItems, true>
                <<<tiles, kBlock, Cfg::kSmemBytes, st>>>(insert, slo, ext, kin, vin, kout, vout, N, 0,
                                                         offsets, stat, tag, tickets, status_word);
        else
            gpu::k_onesweep<neighbor::PointInsertOp, kRadixBits, kBlock, kItems, false>
                <<<tiles, kBlock, Cfg::kSmemBytes, st>>>(insert, slo, ext, kin, vin, kout, vout, N,
                                                         p * kRadixBits, offsets + p * kRadix, stat, tag,
                                                         tickets + p, status_word);
        kin = kout;
        vin = vout;
        }
    const cudaError_t rc = cudaGetLastError();
    if (rc != cudaSuccess)
        return noalloc_fail(NBR_ERR_CUDA, std::string("nbr_morton_sort_noalloc: ") + cudaGetErrorString(rc));
    neighbor_capi::set_last_error("");
    return NBR_OK;
    }
