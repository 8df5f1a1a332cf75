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
//
// The sort's decoupled look-back waits are bounded: a wait that gives up sets a status word in
// the array (and the later passes then write nothing), so the outputs of that call are not valid.
// nbr_morton_sort_noalloc_status reads the word of the last call on the current device.
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
int g_sms[kMaxDevices] = {};

// Words of the array, in order.
constexpr size_t kHistAt = 0;
constexpr size_t kOffsetsAt = kHistAt + kHistWords;
constexpr size_t kTicketsAt = kOffsetsAt + kOffsetWords;
constexpr size_t kBoundsAt = kTicketsAt + kTicketWords;
constexpr size_t kStatusAt = kBoundsAt + kBoundsWords;

// Test hook only: the first tile ticket of pass 0 starts at 1, so tile 0 never runs.
__global__ void k_noalloc_skip_first_tile(unsigned int* tickets) { tickets[0] = 1u; }

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

namespace
{
// The current device's array and per-device set-up (address, kernel attributes, SM count), done
// once per device with that device current.  Returns NBR_OK or an error code.
int noalloc_setup(int& dev, unsigned int*& scratch)
    {
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        {
        (void)cudaGetLastError();
        return noalloc_fail(NBR_ERR_CUDA, "nbr_morton_sort_noalloc: no current device");
        }
    if (!g_scratch_ptr[dev])
        {
        // the host-side name of the array is not a device address: look the address up
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
        // the build's settings for the sort passes: their tile in dynamic shared memory, and all
        // of L1 that can be shared memory (several blocks per SM)
        const void* k1 = (const void*)gpu::k_onesweep<neighbor::PointInsertOp, kRadixBits, kBlock, kItems, true>;
        const void* k0 = (const void*)gpu::k_onesweep<neighbor::PointInsertOp, kRadixBits, kBlock, kItems, false>;
        if (cudaFuncSetAttribute(k1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::kSmemBytes) != cudaSuccess
            || cudaFuncSetAttribute(k0, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::kSmemBytes) != cudaSuccess
            || cudaFuncSetAttribute(k1, cudaFuncAttributePreferredSharedMemoryCarveout,
                                    (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess
            || cudaFuncSetAttribute(k0, cudaFuncAttributePreferredSharedMemoryCarveout,
                                    (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess
            || cudaDeviceGetAttribute(&g_sms[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            {
            (void)cudaGetLastError();
            return noalloc_fail(NBR_ERR_CUDA, "nbr_morton_sort_noalloc: kernel set-up failed");
            }
        g_attr_set[dev] = true;
        }
    scratch = g_scratch_ptr[dev];
    return NBR_OK;
    }

// True when ptr is device-accessible memory of device `dev` (or managed memory).
bool on_device(const void* ptr, int dev)
    {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess)
        {
        (void)cudaGetLastError();
        return false;
        }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == dev;
    }

// The sort itself; skip_first_tile (test hook) never runs pass 0's first tile, so that the
// look-back of the next tile waits for a tile that never comes and gives up.
int noalloc_sort(const float* points, unsigned int N, const float lo[3], const float hi[3], unsigned int* codes_out,
                 unsigned int* order_out, void* stream, bool skip_first_tile)
    {
    if (N == 0) return NBR_OK;
    if (!points || !lo || !hi || !codes_out || !order_out) return noalloc_fail(NBR_ERR_INVALID, "null argument");
    if (N > kMaxPoints)
        return noalloc_fail(NBR_ERR_INVALID, "nbr_morton_sort_noalloc: " + std::to_string(N)
                                                 + " points exceed its fixed scratch of "
                                                 + std::to_string(kMaxPoints) + " points");

    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    unsigned int* scratch = nullptr;
    unsigned int epoch = 0;
    int dev = 0;
    int sms = 0;
        {
        std::lock_guard<std::mutex> lock(g_mutex);
        const int rc = noalloc_setup(dev, scratch);
        if (rc != NBR_OK) return rc;
        sms = g_sms[dev];
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
    // the kernels run on the current device: inputs and outputs must live there
    if (!on_device(points, dev) || !on_device(codes_out, dev) || !on_device(order_out, dev))
        return noalloc_fail(NBR_ERR_INVALID, "nbr_morton_sort_noalloc: points and outputs must be memory of the "
                                             "current device");

    unsigned int* hist = scratch + kHistAt;
    unsigned int* offsets = scratch + kOffsetsAt;
    unsigned int* tickets = scratch + kTicketsAt;
    unsigned int* bounds = scratch + kBoundsAt;
    unsigned int* status_word = scratch + kStatusAt;
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
    const unsigned int cap = 8u * (unsigned int)(sms > 0 ? sms : 1);
    const unsigned int grid = (N + 255) / 256 < cap ? (N + 255) / 256 : cap;
    gpu::k_codes_histogram<neighbor::PointInsertOp, kRadixBits><<<grid, 256, 0, st>>>(insert, N, slo, ext, hist, bounds);
    gpu::k_digit_offsets<kRadixBits><<<kPasses, 1024, 0, st>>>(hist, offsets);

    // four passes: points -> scratch -> out -> scratch -> out
    const unsigned int tiles = (N + Cfg::kTile - 1) / Cfg::kTile;
    if (skip_first_tile) k_noalloc_skip_first_tile<<<1, 1, 0, st>>>(tickets);
    const unsigned int* kin = nullptr;
    const unsigned int* vin = nullptr;
    for (int p = 0; p < kPasses; ++p)
        {
        unsigned int* kout = (p % 2 == 0) ? buf_keys : codes_out;
        unsigned int* vout = (p % 2 == 0) ? buf_vals : order_out;
        unsigned long long* stat = lookback + (size_t)p * kMaxTiles * kRadix;
        const unsigned int tag = (epoch * 4u + (unsigned int)p) & 0x3fffffffu;
        if (p == 0)
            {
            // (test hook: one block fewer, taking tiles 1 .. tiles-1)
            const unsigned int blocks = skip_first_tile ? tiles - 1u : tiles;
            if (blocks > 0)
                gpu::k_onesweep<neighbor::PointInsertOp, kRadixBits, kBlock, kItems, true>
                    <<<blocks, kBlock, Cfg::kSmemBytes, st>>>(insert, slo, ext, kin, vin, kout, vout, N, 0,
                                                              offsets, stat, tag, tickets, status_word);
            }
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
} // namespace

extern "C" int nbr_morton_sort_noalloc(const float* points, unsigned int N, const float lo[3],
                                       const float hi[3], unsigned int* codes_out,
                                       unsigned int* order_out, void* stream)
    {
    return noalloc_sort(points, N, lo, hi, codes_out, order_out, stream, false);
    }

// Status of the last nbr_morton_sort_noalloc call on the current device: one copy of the array's
// status word to the host on `stream` (after that call's work), then a synchronisation.
extern "C" int nbr_morton_sort_noalloc_status(unsigned int* status_out, void* stream)
    {
    int dev = 0;
    unsigned int* scratch = nullptr;
        {
        std::lock_guard<std::mutex> lock(g_mutex);
        const int rc = noalloc_setup(dev, scratch);
        if (rc != NBR_OK) return rc;
        }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    unsigned int word = 0;
    if (cudaMemcpyAsync(&word, scratch + kStatusAt, sizeof(word), cudaMemcpyDeviceToHost, st) != cudaSuccess
        || cudaStreamSynchronize(st) != cudaSuccess)
        {
        const cudaError_t e = cudaGetLastError();
        return noalloc_fail(NBR_ERR_CUDA, std::string("nbr_morton_sort_noalloc_status: ") + cudaGetErrorString(e));
        }
    if (status_out) *status_out = word;
    if (word != 0u)
        return noalloc_fail(NBR_ERR_DEVICE_WAIT, "nbr_morton_sort_noalloc: a bounded look-back wait of the sort gave "
                                                 "up (status " + std::to_string(word) + "); the outputs of that call "
                                                 "are not valid");
    neighbor_capi::set_last_error("");
    return NBR_OK;
    }

// Test hook for the status above (no counterpart in the reference): the same sort with pass 0's
// first tile never run, so the look-back of the next tile gives up after its bounded wait (well
// under a second) and sets the status word.  Outputs are not valid afterwards; the array and the
// context stay usable.
extern "C" int nbr_debug_noalloc_wait_timeout(const float* points, unsigned int N, const float lo[3],
                                              const float hi[3], unsigned int* codes_out,
                                              unsigned int* order_out, void* stream)
    {
    if (N <= kBlock * kItems) return noalloc_fail(NBR_ERR_INVALID, "the hook needs more than one sort tile");
    return noalloc_sort(points, N, lo, hi, codes_out, order_out, stream, true);
    }
