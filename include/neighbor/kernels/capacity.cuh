// Learned per-query neighbor capacity (sm_103a).
//
// A query's neighbor count is predicted from the occupancy of the coarse Morton cells around it:
// the 10-bit Morton bins of the build, shifted right by `shift` bits per axis, give a G^3 grid
// (G = 1024 >> shift) whose cells are indexed by the coarse Morton code (code >> 3*shift).
//
// Features of a query (32, FP32):
//   0..26  log1p(occupancy) of the 27 cells (dx, dy, dz) in {-1,0,1}^3 around its own cell,
//          k = 9(dx+1) + 3(dy+1) + (dz+1); neighbors wrap around the grid for periodic boxes and
//          count 0 outside it otherwise
//   27..29 position inside its own cell along x, y, z, in [0, 1]
//   30     log1p(sum of the 27 occupancies)
//   31     1
// Network: 32 -> 64 (ReLU) -> 64 (ReLU) -> 1 (softplus), weights in BF16, inputs and first
// hidden activations rounded to BF16 (the operands of the two tensor-core layers), the second
// hidden layer kept in FP32 for the output dot product, every product accumulated in FP32,
// biases FP32.  The output
// approximates log1p(count); capacity = ceil(expm1(y + margin(y))), clamped to [1, cap_max], where
// margin(y) is a calibration table over bins of 0.5 in y (kCapMarginBins bins, the last open).
//
//   k_cap_occupancy      occupancy grid from the sorted Morton codes (warp-aggregated atomics)
//   k_cap_features       the 32 features of every sorted point (training data, tests)
//   k_cap_infer          features + network + capacity fused, one warp per 32 queries; the two
//                        hidden layers are BF16 mma.sync m16n8k16 tiles with FP32 accumulators (a
//                        layer's accumulator fragments are the next layer's A fragments) and the
//                        output layer is folded into the second layer's accumulators
//   k_cap_infer_tc       the same on the fifth-generation tensor cores: 128-query tiles, tcgen05.mma
//                        from shared-memory operands into Tensor Memory, tcgen05.ld epilogues
//   k_cap_train_step     forward + backward of a mini-batch on CUDA cores (one thread per sample,
//                        block tiles in shared memory), gradients summed in FP32
//   k_cap_adam           Adam update of the FP32 master weights and their BF16 copies
#ifndef NEIGHBOR_KERNELS_CAPACITY_CUH_
#define NEIGHBOR_KERNELS_CAPACITY_CUH_

#include <cuda_bf16.h>

#include "common.cuh"
#include "tcgen05.cuh"

namespace neighbor
{
namespace gpu
{

constexpr int kCapIn = 32;
constexpr int kCapHidden = 64;
// FP32 parameter vector: W1 [64][32], b1 [64], W2 [64][64], b2 [64], W3 [64], b3
constexpr int kCapOffW1 = 0;
constexpr int kCapOffB1 = kCapOffW1 + kCapHidden * kCapIn;
constexpr int kCapOffW2 = kCapOffB1 + kCapHidden;
constexpr int kCapOffB2 = kCapOffW2 + kCapHidden * kCapHidden;
constexpr int kCapOffW3 = kCapOffB2 + kCapHidden;
constexpr int kCapOffB3 = kCapOffW3 + kCapHidden;
constexpr int kCapParams = kCapOffB3 + 1;
// BF16 weight vector: W1, W2, W3 (same order, no biases)
constexpr int kCapBfW1 = 0;
constexpr int kCapBfW2 = kCapBfW1 + kCapHidden * kCapIn;
constexpr int kCapBfW3 = kCapBfW2 + kCapHidden * kCapHidden;
constexpr int kCapBfWeights = kCapBfW3 + kCapHidden;

struct CapFrame
    {
    float3 lo;          // Morton frame of the build (scene lower corner and extent)
    float3 ext;
    unsigned int shift; // coarse level: bins >> shift
    int periodic;       // neighbor cells wrap around the grid
    };

__device__ __forceinline__ unsigned int compact1by2(unsigned int v)
    {
    v &= 0x09249249u;
    v = (v | (v >> 2)) & 0x030c30c3u;
    v = (v | (v >> 4)) & 0x0300f00fu;
    v = (v | (v >> 8)) & 0x030000ffu;
    v = (v | (v >> 16)) & 0x000003ffu;
    return v;
    }

__device__ __forceinline__ float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// Occupancy of every coarse cell: occ[code >> 3*shift] += 1 (occ zero on entry).
__global__ void __launch_bounds__(256) k_cap_occupancy(const unsigned int* __restrict__ codes, unsigned int N,
                                                       unsigned int shift, unsigned int* __restrict__ occ)
    {
    const unsigned int s = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = s < N;
    const unsigned int c = valid ? (codes[s] >> (3u * shift)) : 0xffffffffu;
    const unsigned int peers = __match_any_sync(0xffffffffu, c);
    if (valid && (threadIdx.x & 31u) == 31u - __clz(peers)) atomicAdd(occ + c, __popc(peers));
    }

// log1pf of small occupancies, shared by a block (the same values log1pf gives).
constexpr int kCapLogTable = 256;
__device__ __forceinline__ void cap_fill_log_table(float* table)
    {
    for (int i = threadIdx.x; i < kCapLogTable; i += blockDim.x) table[i] = log1pf((float)i);
    }
__device__ __forceinline__ float cap_log1p(const float* table, unsigned int o)
    {
    return o < (unsigned int)kCapLogTable ? table[o] : log1pf((float)o);
    }

// Spread Morton bits of the three cells c-1, c, c+1 of one axis (wrapped around the grid when
// periodic; a cell outside an open grid gets valid = 0).
__device__ __forceinline__ void cap_axis(int c, int G, int periodic, unsigned int (&part)[3], unsigned int (&valid)[3])
    {
#pragma unroll
    for (int d = 0; d < 3; ++d)
        {
        int n = c + d - 1;
        bool ok = true;
        if (periodic)
            {
            if (n < 0) n += G;
            if (n >= G) n -= G;
            }
        else
            {
            ok = n >= 0 && n < G;
            }
        part[d] = ok ? part1by2((unsigned int)n) : 0u;
        valid[d] = ok ? 1u : 0u;
        }
    }

// Occupancy of neighbor cell k = 9(dx+1) + 3(dy+1) + (dz+1).
__device__ __forceinline__ unsigned int cap_occ(const unsigned int* __restrict__ occ, int k,
                                                const unsigned int (&px)[3], const unsigned int (&vx)[3],
                                                const unsigned int (&py)[3], const unsigned int (&vy)[3],
                                                const unsigned int (&pz)[3], const unsigned int (&vz)[3])
    {
    const int a = k / 9, b = (k / 3) % 3, c = k % 3;
    return (vx[a] & vy[b] & vz[c]) ? __ldg(occ + ((px[a] << 2) | (py[b] << 1) | pz[c])) : 0u;
    }

// Position of a point inside its coarse cell along the three axes (features 27..29).
__device__ __forceinline__ void cap_frac(const CapFrame& fr, const float3& p, int cx, int cy, int cz, float* f)
    {
    const unsigned int sh = fr.shift;
    const float inv = 1.0f / (float)(1u << sh);
    const float tx = fminf(fmaxf(__fmul_rn(__fdiv_rn(__fsub_rn(p.x, fr.lo.x), fr.ext.x), 1023.f), 0.f), 1023.f);
    const float ty = fminf(fmaxf(__fmul_rn(__fdiv_rn(__fsub_rn(p.y, fr.lo.y), fr.ext.y), 1023.f), 0.f), 1023.f);
    const float tz = fminf(fmaxf(__fmul_rn(__fdiv_rn(__fsub_rn(p.z, fr.lo.z), fr.ext.z), 1023.f), 0.f), 1023.f);
    f[0] = fminf(fmaxf((tx - (float)(cx << sh)) * inv, 0.f), 1.f);
    f[1] = fminf(fmaxf((ty - (float)(cy << sh)) * inv, 0.f), 1.f);
    f[2] = fminf(fmaxf((tz - (float)(cz << sh)) * inv, 0.f), 1.f);
    }

// Features of sorted point s (see the file comment); `table` is a block's log1p table.  emit(k, v)
// receives feature k.
template<class EmitF>
__device__ __forceinline__ void cap_features(const CapFrame& fr, unsigned int code, const float3& p,
                                             const unsigned int* __restrict__ occ, const float* table,
                                             const EmitF& emit)
    {
    const unsigned int sh = fr.shift;
    const int G = 1024 >> sh;
    const unsigned int c = code >> (3u * sh);
    const int cx = (int)compact1by2(c >> 2);
    const int cy = (int)compact1by2(c >> 1);
    const int cz = (int)compact1by2(c);
    unsigned int px[3], py[3], pz[3], vx[3], vy[3], vz[3];
    cap_axis(cx, G, fr.periodic, px, vx);
    cap_axis(cy, G, fr.periodic, py, vy);
    cap_axis(cz, G, fr.periodic, pz, vz);
    unsigned int sum = 0u;
#pragma unroll
    for (int k = 0; k < 27; ++k)
        {
        const unsigned int o = cap_occ(occ, k, px, vx, py, vy, pz, vz);
        sum += o;
        emit(k, cap_log1p(table, o));
        }
    float fr3[3];
    cap_frac(fr, p, cx, cy, cz, fr3);
    emit(27, fr3[0]);
    emit(28, fr3[1]);
    emit(29, fr3[2]);
    emit(30, log1pf((float)sum));
    emit(31, 1.f);
    }

__global__ void __launch_bounds__(256) k_cap_features(const CapFrame fr, const unsigned int* __restrict__ codes,
                                                      const float4* __restrict__ points, unsigned int N,
                                                      const unsigned int* __restrict__ occ, float* __restrict__ out)
    {
    __shared__ float s_log[kCapLogTable];
    cap_fill_log_table(s_log);
    __syncthreads();
    const unsigned int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    const float4 p = points[s];
    float f[kCapIn];
    cap_features(fr, codes[s], make_float3(p.x, p.y, p.z), occ, s_log, [&f](int k, float v) { f[k] = v; });
    float4* o = reinterpret_cast<float4*>(out + (size_t)s * kCapIn);
#pragma unroll
    for (int k = 0; k < kCapIn / 4; ++k) o[k] = make_float4(f[4 * k], f[4 * k + 1], f[4 * k + 2], f[4 * k + 3]);
    }

// Numerically stable softplus and its derivative.
__device__ __forceinline__ float cap_softplus(float z) { return fmaxf(z, 0.f) + log1pf(expf(-fabsf(z))); }
__device__ __forceinline__ float cap_sigmoid(float z) { return 1.f / (1.f + expf(-z)); }

constexpr int kCapMarginBins = 16;
__host__ __device__ __forceinline__ int cap_margin_bin(float y)
    {
    const float b = floorf(y * 2.f);
    return b <= 0.f ? 0 : (b >= (float)(kCapMarginBins - 1) ? kCapMarginBins - 1 : (int)b);
    }

__device__ __forceinline__ unsigned int cap_from_output(float y, float margin, unsigned int cap_max)
    {
    const float c = ceilf(expm1f(y + margin));
    if (!(c >= 1.f)) return 1u;
    if (c >= (float)cap_max) return cap_max;
    return (unsigned int)c;
    }

// ---------------------------------------------------------------------------------------------
// Inference: features, network and capacity fused.  A warp takes 32 consecutive queries (two
// m16 tiles): each lane writes one query's features to shared memory (BF16), then the warp runs
// H1 = relu(X W1^T + b1) and H2 = relu(H1 W2^T + b2) as mma.sync m16n8k16 BF16 tiles with FP32
// accumulators.  The accumulator fragment of N-tiles 2t and 2t+1 is exactly the A fragment of
// K-tile t of the next layer (rows: groupID, groupID + 8; columns: 2*tig + {0,1} (+8)), so H1
// never leaves registers; each H2 fragment is multiplied into the output weights at once, and the
// four lanes of a group add their columns with two shuffles, after which each of the four
// finishes one of the group's four rows.  Accumulators start at the bias (the sum is still FP32).
// ---------------------------------------------------------------------------------------------
struct CapInferArgs
    {
    CapFrame frame;
    const unsigned int* codes;      // sorted Morton codes
    const float4* points;           // sorted payload (x, y, z, primitive id), or NULL and then:
    const float3* points3;          //   the original points, gathered through
    const unsigned int* primitive;  //   the sorted primitive order
    unsigned int N;
    const unsigned int* occ;
    const __nv_bfloat16* w;         // BF16 weights (kCapBfWeights)
    const float* p;                 // FP32 parameters (biases read from here)
    float margins[kCapMarginBins];  // calibration: margin of each bin of y
    unsigned int cap_max;
    int rows_sorted;                // row of sorted position s: s or primitive id
    float* y_out;                   // optional: network output per row
    unsigned int* cap_out;          // capacity per row
    unsigned int* status;           // device status word (k_cap_infer_tc: kStatusTensorWait)
    unsigned int* tile_counter;     // k_cap_infer_tc: zero on entry; blocks take tiles from it
    };

__device__ __forceinline__ unsigned int pack_bf16x2(float lo, float hi)
    {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const unsigned int*>(&v);
    }

// pack_bf16x2(max(lo, 0), max(hi, 0)) in one conversion: rounding to nearest keeps the sign, so
// clamping after the rounding gives the same values (a negative input becomes +0).
__device__ __forceinline__ unsigned int pack_relu_bf16x2(float lo, float hi)
    {
    unsigned int d;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
    }

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const unsigned int (&a)[4], unsigned int b0,
                                               unsigned int b1)
    {
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
    }

// Position and output row of sorted point s.
__device__ __forceinline__ float3 cap_position(const CapInferArgs& a, unsigned int s)
    {
    if (a.points) {
        const float4 p = a.points[s];
        return make_float3(p.x, p.y, p.z);
    }
    return a.points3[a.primitive[s]];
    }
__device__ __forceinline__ unsigned int cap_row(const CapInferArgs& a, unsigned int s)
    {
    if (a.rows_sorted) return s;
    return a.points ? __float_as_uint(a.points[s].w) : a.primitive[s];
    }

// Features of a warp's 32 sorted points s (one per lane) as cap_features() gives them, gathered
// once per distinct coarse cell: sorted points of one cell are consecutive, so the 32 points lie in
// m (typically a few) cells, and the warp's lanes share the 27 m occupancy lookups.  Writes the BF16
// feature row of each distinct cell to cell[k * STRIDE ..] (features 0..26, 30, 31; `part` is
// scratch of 32 x 9 words) and returns, per lane, the row k of its cell and its two point-specific
// words: word 13 = (feature 26 of its cell, x fraction), word 14 = (y, z fractions).
template<int STRIDE>
__device__ __forceinline__ void cap_warp_features(const CapInferArgs& a, const float* s_log, unsigned int s,
                                                  unsigned int lane, unsigned int* part, unsigned short* cell,
                                                  unsigned int& ci_out, uint2& pt_out)
    {
    const unsigned int sh = a.frame.shift;
    const int G = 1024 >> sh;
    const unsigned int lane_le = lanemask_lt() | (1u << lane);
    // lane nb < 27 gathers neighbor cell nb = 9(dx+1) + 3(dy+1) + (dz+1) of every distinct cell
    const unsigned int nb_x = lane / 9u, nb_y = 3u + (lane / 3u) % 3u, nb_z = 6u + lane % 3u;
    const unsigned int c = a.codes[s] >> (3u * sh);
    const float3 pos = cap_position(a, s);   // loaded early: used after the occupancy gather
    const unsigned int c_prev = __shfl_up_sync(0xffffffffu, c, 1);
    const unsigned int heads = __ballot_sync(0xffffffffu, lane == 0u || c != c_prev);
    const unsigned int m = __popc(heads);
    const unsigned int ci = __popc(heads & lane_le) - 1u;
    const int cx = (int)compact1by2(c >> 2);
    const int cy = (int)compact1by2(c >> 1);
    const int cz = (int)compact1by2(c);
    ci_out = ci;
    if ((heads >> lane) & 1u)
        {
        unsigned int p[3], v[3];
        cap_axis(cx, G, a.frame.periodic, p, v);
#pragma unroll
        for (int d = 0; d < 3; ++d) part[ci * 9 + d] = v[d] ? p[d] : 0xffffffffu;
        cap_axis(cy, G, a.frame.periodic, p, v);
#pragma unroll
        for (int d = 0; d < 3; ++d) part[ci * 9 + 3 + d] = v[d] ? p[d] : 0xffffffffu;
        cap_axis(cz, G, a.frame.periodic, p, v);
#pragma unroll
        for (int d = 0; d < 3; ++d) part[ci * 9 + 6 + d] = v[d] ? p[d] : 0xffffffffu;
        }
    __syncwarp();
    // one distinct cell per step: lanes 0..26 its 27 occupancies (a spread part of 0xffffffff,
    // outside an open grid, makes the index >= 2^30), lane 30 the log of their sum (a warp
    // reduction), lane 31 the constant; the loads of four cells are issued before their sums
    for (unsigned int k0 = 0; k0 < m; k0 += 4u)
        {
        unsigned int o[4];
#pragma unroll
        for (unsigned int j = 0; j < 4u; ++j)
            {
            const unsigned int* pk = part + (k0 + j) * 9u;
            o[j] = 0u;
            if (lane < 27u && k0 + j < m)
                {
                const unsigned int idx = (pk[nb_x] << 2) | (pk[nb_y] << 1) | pk[nb_z];
                if (idx < (1u << 30)) o[j] = __ldg(a.occ + idx);
                }
            }
#pragma unroll
        for (unsigned int j = 0; j < 4u; ++j)
            {
            const unsigned int k = k0 + j;
            if (k >= m) break;   // uniform over the warp
            const unsigned int sum = __reduce_add_sync(0xffffffffu, o[j]);
            const float f = lane < 27u ? cap_log1p(s_log, o[j]) : (lane == 31u ? 1.f : cap_log1p(s_log, sum));
            if (lane < 27u || lane >= 30u)
                cell[k * STRIDE + lane] = __bfloat16_as_ushort(__float2bfloat16_rn(f));
            }
        }
    __syncwarp();
    {
    // the point's own words: 13 = (feature 26 of its cell, x fraction), 14 = (y, z fractions)
    float fr3[3];
    cap_frac(a.frame, pos, cx, cy, cz, fr3);
    const unsigned int f26 = cell[ci * STRIDE + 26];
    pt_out = make_uint2(f26 | ((unsigned int)__bfloat16_as_ushort(__float2bfloat16_rn(fr3[0])) << 16),
                        pack_bf16x2(fr3[1], fr3[2]));
    }
    }

constexpr int kCapInferWarps = 8;
// Row stride (BF16 values) of a warp's per-cell feature rows: 32 features + 2 of padding, so that
// rows of different cells start in different banks (17 words apart).
constexpr int kCapCellStride = 34;
// Weights in shared memory in fragment order: for output row n, k-tile kt and thread-in-group t
// the two words of the B fragment (B[2t..2t+1][n], B[8+2t..8+2t+1][n]) are one 64-bit word at
// (kt * 4 + t) * kCapWStride + n; the stride of 72 spreads a warp's words over all bank pairs.
constexpr int kCapWStride = 72;
// m16 row tiles that go through the layers together, and the kernel's resident blocks per SM
// (16M points: 2 tiles at 2 blocks 1.18 ms; 1 tile at 3 blocks (80 registers) 1.35 ms, at 4
// blocks (64) 1.42 ms)
constexpr int kCapInferTiles = 2;
constexpr int kCapInferMinBlocks = 2;

__global__ void __launch_bounds__(kCapInferWarps * 32, kCapInferMinBlocks) k_cap_infer(const CapInferArgs a)
    {
    __shared__ uint2 s_w1[2 * 4 * kCapWStride];   // 2 k-tiles x 4 x 64 rows (+pad)
    __shared__ uint2 s_w2[4 * 4 * kCapWStride];   // 4 k-tiles x 4 x 64 rows (+pad)
    __shared__ float2 s_w3[kCapHidden / 2];        // (w3[2c], w3[2c + 1])
    __shared__ float2 s_b1[kCapHidden / 2];        // (b1[2c], b1[2c + 1])
    __shared__ float2 s_b2[kCapHidden / 2];
    __shared__ float s_log[kCapLogTable];
    // per warp: the distinct coarse cells of its 32 points -- spread Morton parts of the 3 x 3
    // neighbor coordinates (0xffffffff outside an open grid), BF16 feature rows -- and per point
    // its cell and its two point-specific feature words
    __shared__ unsigned int s_part[kCapInferWarps][32 * 9];
    __shared__ unsigned short s_cell[kCapInferWarps][32 * kCapCellStride];
    __shared__ unsigned int s_ci[kCapInferWarps][32];
    __shared__ uint2 s_pt[kCapInferWarps][32];
    const unsigned int* wsrc = reinterpret_cast<const unsigned int*>(a.w);
    for (int i = threadIdx.x; i < kCapHidden * 2 * 4; i += blockDim.x)
        {
        const int n = i % kCapHidden, t = (i / kCapHidden) % 4, kt = i / (kCapHidden * 4);
        s_w1[(kt * 4 + t) * kCapWStride + n] = make_uint2(wsrc[kCapBfW1 / 2 + n * (kCapIn / 2) + kt * 8 + t],
                                                          wsrc[kCapBfW1 / 2 + n * (kCapIn / 2) + kt * 8 + 4 + t]);
        }
    for (int i = threadIdx.x; i < kCapHidden * 4 * 4; i += blockDim.x)
        {
        const int n = i % kCapHidden, t = (i / kCapHidden) % 4, kt = i / (kCapHidden * 4);
        s_w2[(kt * 4 + t) * kCapWStride + n] = make_uint2(wsrc[kCapBfW2 / 2 + n * (kCapHidden / 2) + kt * 8 + t],
                                                          wsrc[kCapBfW2 / 2 + n * (kCapHidden / 2) + kt * 8 + 4 + t]);
        }
    for (int i = threadIdx.x; i < kCapHidden / 2; i += blockDim.x)
        {
        s_w3[i] = make_float2(__bfloat162float(a.w[kCapBfW3 + 2 * i]), __bfloat162float(a.w[kCapBfW3 + 2 * i + 1]));
        s_b1[i] = make_float2(a.p[kCapOffB1 + 2 * i], a.p[kCapOffB1 + 2 * i + 1]);
        s_b2[i] = make_float2(a.p[kCapOffB2 + 2 * i], a.p[kCapOffB2 + 2 * i + 1]);
        }
    cap_fill_log_table(s_log);
    __syncthreads();
    const float b3 = a.p[kCapOffB3];
    const unsigned int lane = threadIdx.x & 31u;
    const unsigned int warp = threadIdx.x >> 5;
    const unsigned int g = lane >> 2;   // groupID
    const unsigned int t = lane & 3u;   // thread in group
    unsigned int* part = s_part[warp];
    unsigned short* cell = s_cell[warp];
    unsigned int* cidx = s_ci[warp];
    uint2* pt = s_pt[warp];
    const unsigned int n_tiles = (a.N + 31u) / 32u;
    for (unsigned int tile = blockIdx.x * kCapInferWarps + warp; tile < n_tiles; tile += gridDim.x * kCapInferWarps)
        {
        const unsigned int base = tile * 32u;
        // lanes past the end repeat the last point (their outputs are not written)
        const unsigned int s = base + min(lane, a.N - 1u - base);
        unsigned int ci;
        uint2 ptw;
        cap_warp_features<kCapCellStride>(a, s_log, s, lane, part, cell, ci, ptw);
        cidx[lane] = ci;
        pt[lane] = ptw;
        __syncwarp();
        // The two m16 tiles (rows g, g + 8 and g + 16, g + 24 of this lane) go through the layers
        // kCapInferTiles at a time: every B fragment read from shared memory feeds that many MMAs.
        float z[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
#pragma unroll 1
        for (int m0 = 0; m0 < 2; m0 += kCapInferTiles)
            {
            float zc[kCapInferTiles][2];
#pragma unroll
            for (int i = 0; i < kCapInferTiles; ++i) zc[i][0] = zc[i][1] = 0.f;
            unsigned int a1[kCapInferTiles][2][4];
#pragma unroll
            for (int i = 0; i < kCapInferTiles; ++i)
                {
                const unsigned int r0 = (m0 + i) * 16u + g;
                // feature words of rows r0 and r0 + 8: the cell's row, except words 13 and 14
                const unsigned int* x0 = reinterpret_cast<const unsigned int*>(cell + cidx[r0] * kCapCellStride);
                const unsigned int* x1 = reinterpret_cast<const unsigned int*>(cell + cidx[r0 + 8u] * kCapCellStride);
                a1[i][0][0] = x0[t];
                a1[i][0][1] = x1[t];
                a1[i][0][2] = x0[4 + t];
                a1[i][0][3] = x1[4 + t];
                a1[i][1][0] = x0[8 + t];
                a1[i][1][1] = x1[8 + t];
                a1[i][1][2] = t == 1u ? pt[r0].x : (t == 2u ? pt[r0].y : x0[12 + t]);
                a1[i][1][3] = t == 1u ? pt[r0 + 8u].x : (t == 2u ? pt[r0 + 8u].y : x1[12 + t]);
                }
            // layer 1 -> BF16 A fragments of layer 2 (k-tile j = n-tiles 2j, 2j+1); the accumulators
            // start at the bias, and one conversion applies the ReLU and packs two columns
            unsigned int a2[kCapInferTiles][4][4];
#pragma unroll
            for (int nt = 0; nt < 8; ++nt)
                {
                const float2 bias = s_b1[nt * 4 + t];
                float acc[kCapInferTiles][4];
#pragma unroll
                for (int i = 0; i < kCapInferTiles; ++i)
                    {
                    acc[i][0] = bias.x; acc[i][1] = bias.y; acc[i][2] = bias.x; acc[i][3] = bias.y;
                    }
#pragma unroll
                for (int kt = 0; kt < 2; ++kt)
                    {
                    const uint2 b = s_w1[(kt * 4 + t) * kCapWStride + nt * 8 + g];
#pragma unroll
                    for (int i = 0; i < kCapInferTiles; ++i) mma_bf16_16816(acc[i], a1[i][kt], b.x, b.y);
                    }
#pragma unroll
                for (int i = 0; i < kCapInferTiles; ++i)
                    {
                    a2[i][nt >> 1][(nt & 1) * 2 + 0] = pack_relu_bf16x2(acc[i][0], acc[i][1]);
                    a2[i][nt >> 1][(nt & 1) * 2 + 1] = pack_relu_bf16x2(acc[i][2], acc[i][3]);
                    }
                }
            // layer 2 with the output layer folded in: z(row) = sum over columns of relu(h2) * w3
#pragma unroll
            for (int nt = 0; nt < 8; ++nt)
                {
                const float2 bias = s_b2[nt * 4 + t];
                float acc[kCapInferTiles][4];
#pragma unroll
                for (int i = 0; i < kCapInferTiles; ++i)
                    {
                    acc[i][0] = bias.x; acc[i][1] = bias.y; acc[i][2] = bias.x; acc[i][3] = bias.y;
                    }
#pragma unroll
                for (int kt = 0; kt < 4; ++kt)
                    {
                    const uint2 b = s_w2[(kt * 4 + t) * kCapWStride + nt * 8 + g];
#pragma unroll
                    for (int i = 0; i < kCapInferTiles; ++i) mma_bf16_16816(acc[i], a2[i][kt], b.x, b.y);
                    }
                const float2 w = s_w3[nt * 4 + t];
#pragma unroll
                for (int i = 0; i < kCapInferTiles; ++i)
                    {
                    zc[i][0] = fmaf(fmaxf(acc[i][0], 0.f), w.x, zc[i][0]);
                    zc[i][0] = fmaf(fmaxf(acc[i][1], 0.f), w.y, zc[i][0]);
                    zc[i][1] = fmaf(fmaxf(acc[i][2], 0.f), w.x, zc[i][1]);
                    zc[i][1] = fmaf(fmaxf(acc[i][3], 0.f), w.y, zc[i][1]);
                    }
                }
            // (the loop is not unrolled, so that one pass's fragments are all that is live: the
            // partial sums leave through selects, not through an index)
#pragma unroll
            for (int i = 0; i < kCapInferTiles; ++i)
#pragma unroll
                for (int mt = 0; mt < 2; ++mt)
                    if (m0 + i == mt)
                        {
                        z[mt][0] = zc[i][0];
                        z[mt][1] = zc[i][1];
                        }
            }
        // the four lanes of a group hold disjoint columns of rows g, g + 8 (tile 0) and g + 16,
        // g + 24 (tile 1): after the sums lane t of the group finishes row g + 8t
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int h = 0; h < 2; ++h)
                {
                z[mt][h] += __shfl_xor_sync(0xffffffffu, z[mt][h], 1);
                z[mt][h] += __shfl_xor_sync(0xffffffffu, z[mt][h], 2);
                }
        {
        const float zr = t == 0u ? z[0][0] : (t == 1u ? z[0][1] : (t == 2u ? z[1][0] : z[1][1]));
        const unsigned int s = base + g + 8u * t;
        if (s < a.N)
            {
            const float y = cap_softplus(zr + b3);
            const unsigned int row = cap_row(a, s);
            if (a.y_out) a.y_out[row] = y;
            a.cap_out[row] = cap_from_output(y, a.margins[cap_margin_bin(y)], a.cap_max);
            }
        }
        __syncwarp();
        }
    }

// ---------------------------------------------------------------------------------------------
// Inference on the fifth-generation tensor cores (tcgen05).  A block of four warps takes 128
// consecutive queries per step -- the M of one MMA.  Each warp gathers the features of its 32
// queries as k_cap_infer does, and each lane writes its query's BF16 feature row into the A tile
// of layer 1 (shared memory, K-major core matrices).  One thread issues H1 = X W1^T as two
// tcgen05.mma (M 128, N 64, K 16) into 64 Tensor Memory columns; their completion arrives on an
// mbarrier.  Each warp reads its 32 TMEM lanes (lane = query, a row per thread) with tcgen05.ld,
// adds b1, applies the ReLU, rounds to BF16 and writes the A tile of layer 2; H2 = H1 W2^T (four
// MMAs into the same columns) follows, and the output layer is a per-thread FP32 dot product of
// relu(H2 + b2) with w3.  The rounding points are those of k_cap_infer: BF16 inputs, weights and
// first hidden layer, FP32 accumulation and biases.  Accumulators start at zero and the bias is
// added after the MMA (k_cap_infer starts them at the bias): outputs agree to FP32 summation
// order.  Every mbarrier wait is bounded: one that gives up sets kStatusTensorWait, waits once
// more (bounded) for the MMA in flight, frees the block's Tensor Memory and ends the block.
// ---------------------------------------------------------------------------------------------
constexpr int kCapTcWarps = 4;
constexpr int kCapTcRows = kCapTcWarps * 32;   // 128 queries = the MMA's M = the TMEM lanes
constexpr unsigned int kCapTcCols = 64;        // TMEM columns: H1, then H2 (N = 64)
// ~39 KB of shared memory per block: five blocks per SM (20 warps, 320 of the 512 TMEM columns)
constexpr int kCapTcMinBlocks = 5;
// BF16 values per gathered cell row: 80 bytes, so that a row is read as five 16-byte words
constexpr int kCapTcCellStride = 40;
constexpr unsigned int kCapTcWaitLimit = 1u << 22;

__global__ void __launch_bounds__(kCapTcRows, kCapTcMinBlocks) k_cap_infer_tc(const CapInferArgs a)
    {
    // A of layer 1: 128 rows x 32 BF16 (K-major core matrices, SBO 512)
    __shared__ __align__(1024) unsigned char s_x[kCapTcRows * kCapIn * 2];
    // A of layer 2: 128 rows x 64 BF16 (SBO 1024).  Warp w's rows are bytes [4096 w, 4096 w + 4096),
    // which also hold its gather scratch (cell parts, cell rows) while its features are formed.
    __shared__ __align__(1024) unsigned char s_h[kCapTcRows * kCapHidden * 2];
    // B operands: W1 (64 x 32) and W2 (64 x 64), rows = output units, K-major like A
    __shared__ __align__(1024) unsigned char s_w1[kCapHidden * kCapIn * 2];
    __shared__ __align__(1024) unsigned char s_w2[kCapHidden * kCapHidden * 2];
    __shared__ float s_b1[kCapHidden];
    __shared__ float s_b2[kCapHidden];
    __shared__ float s_w3[kCapHidden];
    __shared__ float s_log[kCapLogTable];
    __shared__ __align__(8) unsigned long long s_bar;
    __shared__ unsigned int s_tmem;
    __shared__ unsigned int s_tile;

    const unsigned int lane = threadIdx.x & 31u;
    const unsigned int warp = threadIdx.x >> 5;
    // 16-byte chunk (n, kg) of a weight matrix = W[n][8 kg .. 8 kg + 7]
    const uint4* wsrc = reinterpret_cast<const uint4*>(a.w);
    for (unsigned int i = threadIdx.x; i < (unsigned int)(kCapHidden * kCapIn / 8); i += blockDim.x)
        *reinterpret_cast<uint4*>(s_w1 + tc::kmajor_offset(i / (kCapIn / 8), (i % (kCapIn / 8)) * 8u, kCapIn)) =
            wsrc[kCapBfW1 / 8 + i];
    for (unsigned int i = threadIdx.x; i < (unsigned int)(kCapHidden * kCapHidden / 8); i += blockDim.x)
        *reinterpret_cast<uint4*>(s_w2 + tc::kmajor_offset(i / (kCapHidden / 8), (i % (kCapHidden / 8)) * 8u,
                                                           kCapHidden)) = wsrc[kCapBfW2 / 8 + i];
    for (unsigned int i = threadIdx.x; i < (unsigned int)kCapHidden; i += blockDim.x)
        {
        s_b1[i] = a.p[kCapOffB1 + i];
        s_b2[i] = a.p[kCapOffB2 + i];
        s_w3[i] = __bfloat162float(a.w[kCapBfW3 + i]);
        }
    cap_fill_log_table(s_log);
    if (warp == 0) tc::tmem_alloc(&s_tmem, kCapTcCols);
    if (threadIdx.x == 0) tc::mbar_init(&s_bar, 1u);
    tc::fence_proxy_async();   // the weights are read by the tensor core
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const unsigned int tmem = s_tmem;
    const unsigned int t_rows = tmem + ((warp * 32u) << 16);   // this warp's 32 TMEM lanes
    const float b3 = a.p[kCapOffB3];
    unsigned int* part = reinterpret_cast<unsigned int*>(s_h + warp * 4096u);
    unsigned short* cell = reinterpret_cast<unsigned short*>(s_h + warp * 4096u + 32u * 9u * 4u);
    const unsigned int r = warp * 32u + lane;   // the thread's row of the tile
    constexpr unsigned int idesc = tc::idesc_bf16_f32(kCapTcRows, kCapHidden);
    const unsigned int x_addr = tc::smem_addr(s_x);
    const unsigned int h_addr = tc::smem_addr(s_h);
    const unsigned int w1_addr = tc::smem_addr(s_w1);
    const unsigned int w2_addr = tc::smem_addr(s_w2);
    unsigned int phase = 0u;
    bool failed = false;
    const unsigned int n_tiles = (a.N + (unsigned int)kCapTcRows - 1u) / (unsigned int)kCapTcRows;
    // Each block takes its first tile by its index and the next ones from a ticket counter, so that
    // blocks that start late (the kernel may share the GPU with a build still running) take fewer.
    for (unsigned int it = 0;; ++it)
        {
        if (threadIdx.x == 0)
            s_tile = it == 0 ? blockIdx.x
                             : (a.tile_counter ? gridDim.x + atomicAdd(a.tile_counter, 1u) : blockIdx.x + it * gridDim.x);
        __syncthreads();
        const unsigned int tile = s_tile;
        if (tile >= n_tiles) break;
        // rows past the end repeat the last query (their outputs are not written)
        const unsigned int q = tile * (unsigned int)kCapTcRows + r;
        unsigned int ci;
        uint2 ptw;
        cap_warp_features<kCapTcCellStride>(a, s_log, min(q, a.N - 1u), lane, part, cell, ci, ptw);
        {
        // the query's feature row: its cell's row with words 13 and 14 its own
        const uint4* src = reinterpret_cast<const uint4*>(cell + ci * kCapTcCellStride);
        const uint4 v0 = src[0], v1 = src[1], v2 = src[2];
        uint4 v3 = src[3];
        v3.y = ptw.x;
        v3.z = ptw.y;
        *reinterpret_cast<uint4*>(s_x + tc::kmajor_offset(r, 0u, kCapIn)) = v0;
        *reinterpret_cast<uint4*>(s_x + tc::kmajor_offset(r, 8u, kCapIn)) = v1;
        *reinterpret_cast<uint4*>(s_x + tc::kmajor_offset(r, 16u, kCapIn)) = v2;
        *reinterpret_cast<uint4*>(s_x + tc::kmajor_offset(r, 24u, kCapIn)) = v3;
        }
        tc::fence_proxy_async();
        __syncthreads();
        if (threadIdx.x == 0)
            {
            tc::fence_after_sync();
#pragma unroll
            for (unsigned int k = 0; k < (unsigned int)kCapIn / 16u; ++k)
                tc::mma_bf16(tmem, tc::smem_desc(x_addr + k * 256u, 128u, kCapIn * 16u),
                             tc::smem_desc(w1_addr + k * 256u, 128u, kCapIn * 16u), idesc, k > 0u);
            tc::mma_commit(&s_bar);
            }
        bool ok = tc::mbar_wait_bounded(&s_bar, phase, kCapTcWaitLimit);
        if (__syncthreads_or(!ok))
            {
            failed = true;
            break;
            }
        phase ^= 1u;
        tc::fence_after_sync();
        {
        // H1 = relu(acc + b1) rounded to BF16 -> the thread's row of the A tile of layer 2
        unsigned int v[4][16];
#pragma unroll
        for (int c = 0; c < 4; ++c) tc::ld_32x32b_x16(t_rows + 16u * c, v[c]);
#pragma unroll
        for (int c = 0; c < 4; ++c) tc::wait_ld(v[c]);
#pragma unroll
        for (int c = 0; c < 4; ++c)
#pragma unroll
            for (int h = 0; h < 2; ++h)
                {
                const int n0 = 16 * c + 8 * h;
                unsigned int o[4];
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    o[j] = pack_relu_bf16x2(__uint_as_float(v[c][8 * h + 2 * j]) + s_b1[n0 + 2 * j],
                                            __uint_as_float(v[c][8 * h + 2 * j + 1]) + s_b1[n0 + 2 * j + 1]);
                *reinterpret_cast<uint4*>(s_h + tc::kmajor_offset(r, (unsigned int)n0, kCapHidden)) =
                    make_uint4(o[0], o[1], o[2], o[3]);
                }
        }
        tc::fence_proxy_async();
        tc::fence_before_sync();
        __syncthreads();
        if (threadIdx.x == 0)
            {
            tc::fence_after_sync();
#pragma unroll
            for (unsigned int k = 0; k < (unsigned int)kCapHidden / 16u; ++k)
                tc::mma_bf16(tmem, tc::smem_desc(h_addr + k * 256u, 128u, kCapHidden * 16u),
                             tc::smem_desc(w2_addr + k * 256u, 128u, kCapHidden * 16u), idesc, k > 0u);
            tc::mma_commit(&s_bar);
            }
        ok = tc::mbar_wait_bounded(&s_bar, phase, kCapTcWaitLimit);
        if (__syncthreads_or(!ok))
            {
            failed = true;
            break;
            }
        phase ^= 1u;
        tc::fence_after_sync();
        float z = 0.f;
        {
        unsigned int v[4][16];
#pragma unroll
        for (int c = 0; c < 4; ++c) tc::ld_32x32b_x16(t_rows + 16u * c, v[c]);
#pragma unroll
        for (int c = 0; c < 4; ++c) tc::wait_ld(v[c]);
#pragma unroll
        for (int c = 0; c < 4; ++c)
#pragma unroll
            for (int j = 0; j < 16; ++j)
                z = fmaf(fmaxf(__uint_as_float(v[c][j]) + s_b2[16 * c + j], 0.f), s_w3[16 * c + j], z);
        }
        // the next tile's MMA (after the next barrier) overwrites the columns just read
        tc::fence_before_sync();
        if (q < a.N)
            {
            const float y = cap_softplus(z + b3);
            const unsigned int row = cap_row(a, q);
            if (a.y_out) a.y_out[row] = y;
            a.cap_out[row] = cap_from_output(y, a.margins[cap_margin_bin(y)], a.cap_max);
            }
        }
    if (failed)
        {
        if (threadIdx.x == 0 && a.status) atomicOr(a.status, kStatusTensorWait);
        // the MMA may still be in flight: give it one more bounded wait before its columns go
        tc::mbar_wait_bounded(&s_bar, phase, kCapTcWaitLimit);
        }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, kCapTcCols);
    }

// ---------------------------------------------------------------------------------------------
// Training.  One mini-batch step: sample b of the batch is row (offset + b * stride) mod N of the
// feature matrix.  Each block runs tiles of kCapTrainTile samples, one thread per sample, with
// the same BF16 rounding points as inference; per-sample activations and deltas go to shared
// memory, and the block adds the tile's weight gradients (FP32) into its shared accumulator,
// then into the global gradient with atomics.  grad = sum over the batch of dL/dp with
// L = 0.5 (y - target)^2; loss_out += sum of L.
// ---------------------------------------------------------------------------------------------
constexpr int kCapTrainTile = 64;

struct CapTrainArgs
    {
    const float* features;   // [N][32]
    const float* target;     // [N] log1p(count)
    unsigned int N;
    unsigned int batch;
    unsigned int offset;
    unsigned int stride;
    const __nv_bfloat16* w;
    const float* p;
    float* grad;             // [kCapParams], zero on entry
    float* loss_out;
    };

struct CapTrainSmem
    {
    float w1[kCapHidden * kCapIn];
    float w2[kCapHidden * kCapHidden];
    float w3[kCapHidden];
    float b1[kCapHidden];
    float b2[kCapHidden];
    float x[kCapTrainTile][kCapIn + 1];
    float h1[kCapTrainTile][kCapHidden + 1];
    float h2[kCapTrainTile][kCapHidden + 1];
    float d2[kCapTrainTile][kCapHidden + 1];
    float d1[kCapTrainTile][kCapHidden + 1];
    float dz[kCapTrainTile];
    float g[kCapParams];
    };

__global__ void __launch_bounds__(kCapTrainTile) k_cap_train_step(const CapTrainArgs a)
    {
    extern __shared__ __align__(16) unsigned char smem_cap[];
    CapTrainSmem& S = *reinterpret_cast<CapTrainSmem*>(smem_cap);
    const int tid = threadIdx.x;
    for (int i = tid; i < kCapHidden * kCapIn; i += blockDim.x) S.w1[i] = __bfloat162float(a.w[kCapBfW1 + i]);
    for (int i = tid; i < kCapHidden * kCapHidden; i += blockDim.x) S.w2[i] = __bfloat162float(a.w[kCapBfW2 + i]);
    for (int i = tid; i < kCapHidden; i += blockDim.x)
        {
        S.w3[i] = __bfloat162float(a.w[kCapBfW3 + i]);
        S.b1[i] = a.p[kCapOffB1 + i];
        S.b2[i] = a.p[kCapOffB2 + i];
        }
    for (int i = tid; i < kCapParams; i += blockDim.x) S.g[i] = 0.f;
    const float b3 = a.p[kCapOffB3];
    __syncthreads();
    float loss = 0.f;
    const unsigned int n_tiles = (a.batch + kCapTrainTile - 1) / kCapTrainTile;
    for (unsigned int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x)
        {
        const unsigned int b = tile * kCapTrainTile + tid;
        const bool on = b < a.batch;
        float dz = 0.f;
        if (on)
            {
            const unsigned int row = (unsigned int)(((unsigned long long)a.offset + (unsigned long long)b * a.stride) % a.N);
            const float* xf = a.features + (size_t)row * kCapIn;
            for (int k = 0; k < kCapIn; ++k) S.x[tid][k] = bf16_round(xf[k]);
            for (int j = 0; j < kCapHidden; ++j)
                {
                float acc = 0.f;
                for (int k = 0; k < kCapIn; ++k) acc = fmaf(S.w1[j * kCapIn + k], S.x[tid][k], acc);
                S.h1[tid][j] = bf16_round(fmaxf(acc + S.b1[j], 0.f));
                }
            for (int j = 0; j < kCapHidden; ++j)
                {
                float acc = 0.f;
                for (int k = 0; k < kCapHidden; ++k) acc = fmaf(S.w2[j * kCapHidden + k], S.h1[tid][k], acc);
                S.h2[tid][j] = fmaxf(acc + S.b2[j], 0.f);
                }
            float z = 0.f;
            for (int k = 0; k < kCapHidden; ++k) z = fmaf(S.w3[k], S.h2[tid][k], z);
            z += b3;
            const float y = cap_softplus(z);
            const float dy = y - a.target[row];
            loss += 0.5f * dy * dy;
            dz = dy * cap_sigmoid(z);
            for (int j = 0; j < kCapHidden; ++j) S.d2[tid][j] = S.h2[tid][j] > 0.f ? dz * S.w3[j] : 0.f;
            for (int k = 0; k < kCapHidden; ++k)
                {
                float acc = 0.f;
                for (int j = 0; j < kCapHidden; ++j) acc = fmaf(S.w2[j * kCapHidden + k], S.d2[tid][j], acc);
                S.d1[tid][k] = S.h1[tid][k] > 0.f ? acc : 0.f;
                }
            }
        else
            {
            for (int k = 0; k < kCapIn; ++k) S.x[tid][k] = 0.f;
            for (int j = 0; j < kCapHidden; ++j)
                {
                S.h1[tid][j] = 0.f;
                S.h2[tid][j] = 0.f;
                S.d2[tid][j] = 0.f;
                S.d1[tid][j] = 0.f;
                }
            }
        S.dz[tid] = dz;
        __syncthreads();
        // tile gradients: thread tid owns rows j = tid (and tid + 64 ...) of each weight matrix
        for (int j = tid; j < kCapHidden; j += blockDim.x)
            {
            float gb1 = 0.f, gb2 = 0.f, gw3 = 0.f;
            for (int s = 0; s < kCapTrainTile; ++s)
                {
                gb1 += S.d1[s][j];
                gb2 += S.d2[s][j];
                gw3 += S.dz[s] * S.h2[s][j];
                }
            S.g[kCapOffB1 + j] += gb1;
            S.g[kCapOffB2 + j] += gb2;
            S.g[kCapOffW3 + j] += gw3;
            for (int k = 0; k < kCapIn; ++k)
                {
                float acc = 0.f;
                for (int s = 0; s < kCapTrainTile; ++s) acc = fmaf(S.d1[s][j], S.x[s][k], acc);
                S.g[kCapOffW1 + j * kCapIn + k] += acc;
                }
            for (int k = 0; k < kCapHidden; ++k)
                {
                float acc = 0.f;
                for (int s = 0; s < kCapTrainTile; ++s) acc = fmaf(S.d2[s][j], S.h1[s][k], acc);
                S.g[kCapOffW2 + j * kCapHidden + k] += acc;
                }
            }
        if (tid == 0)
            {
            float gb3 = 0.f;
            for (int s = 0; s < kCapTrainTile; ++s) gb3 += S.dz[s];
            S.g[kCapOffB3] += gb3;
            }
        __syncthreads();
        }
    for (int i = tid; i < kCapParams; i += blockDim.x)
        if (S.g[i] != 0.f) atomicAdd(a.grad + i, S.g[i]);
    if (loss != 0.f) atomicAdd(a.loss_out, loss);
    }

struct CapAdamArgs
    {
    float* p;
    float* m;
    float* v;
    const float* grad;
    __nv_bfloat16* w;
    float scale;      // 1 / batch
    float lr;
    float beta1, beta2, eps;
    float bias1, bias2;  // 1 - beta^t
    };

__global__ void __launch_bounds__(256) k_cap_adam(const CapAdamArgs a)
    {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kCapParams) return;
    const float g = a.grad[i] * a.scale;
    const float m = a.beta1 * a.m[i] + (1.f - a.beta1) * g;
    const float v = a.beta2 * a.v[i] + (1.f - a.beta2) * g * g;
    a.m[i] = m;
    a.v[i] = v;
    const float p = a.p[i] - a.lr * (m / a.bias1) / (sqrtf(v / a.bias2) + a.eps);
    a.p[i] = p;
    int wi = -1;
    if (i < kCapOffB1) wi = kCapBfW1 + (i - kCapOffW1);
    else if (i >= kCapOffW2 && i < kCapOffB2) wi = kCapBfW2 + (i - kCapOffW2);
    else if (i >= kCapOffW3 && i < kCapOffB3) wi = kCapBfW3 + (i - kCapOffW3);
    if (wi >= 0) a.w[wi] = __float2bfloat16_rn(p);
    }

// BF16 copies of the FP32 weights.
__global__ void __launch_bounds__(256) k_cap_cast(const float* __restrict__ p, __nv_bfloat16* __restrict__ w)
    {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kCapBfWeights) return;
    int pi;
    if (i < kCapBfW2) pi = kCapOffW1 + i;
    else if (i < kCapBfW3) pi = kCapOffW2 + (i - kCapBfW2);
    else pi = kCapOffW3 + (i - kCapBfW3);
    w[i] = __float2bfloat16_rn(p[pi]);
    }

// Residual target - output of every row (for the capacity margin) and log1p(count) targets.
__global__ void __launch_bounds__(256) k_cap_targets(const unsigned int* __restrict__ counts, unsigned int N,
                                                     float* __restrict__ target)
    {
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) target[i] = log1pf((float)counts[i]);
    }

// ---------------------------------------------------------------------------------------------
// Exclusive scan of 32-bit counts into 64-bit offsets (three phases, deterministic):
// tile sums, a scan of the tile sums by one block, then each tile's local scan plus its base.
// ---------------------------------------------------------------------------------------------
constexpr int kScan64Block = 256;
constexpr int kScan64Items = 16;
constexpr int kScan64Tile = kScan64Block * kScan64Items;

__global__ void __launch_bounds__(kScan64Block) k_scan64_tiles(const unsigned int* __restrict__ in, unsigned int n,
                                                               unsigned long long* __restrict__ tile_sum)
    {
    __shared__ unsigned long long s_red[kScan64Block / 32];
    const unsigned int base = blockIdx.x * kScan64Tile;
    unsigned long long sum = 0;
    for (int k = 0; k < kScan64Items; ++k)
        {
        const unsigned int i = base + k * kScan64Block + threadIdx.x;
        if (i < n) sum += in[i];
        }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x == 0)
        {
        unsigned long long t = 0;
        for (int w = 0; w < kScan64Block / 32; ++w) t += s_red[w];
        tile_sum[blockIdx.x] = t;
        }
    }

// One block: exclusive scan of the tile sums in place; total to *total.
__global__ void __launch_bounds__(1024) k_scan64_sums(unsigned long long* __restrict__ tile_sum, unsigned int n_tiles,
                                                      unsigned long long* __restrict__ total)
    {
    __shared__ unsigned long long s_w[32];
    __shared__ unsigned long long s_carry;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    const unsigned int lane = threadIdx.x & 31u;
    const unsigned int warp = threadIdx.x >> 5;
    for (unsigned int c = 0; c < n_tiles; c += blockDim.x)
        {
        const unsigned int i = c + threadIdx.x;
        const unsigned long long v = i < n_tiles ? tile_sum[i] : 0ull;
        unsigned long long incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
            {
            const unsigned long long x = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (unsigned int)o) incl += x;
            }
        if (lane == 31u) s_w[warp] = incl;
        __syncthreads();
        if (warp == 0)
            {
            const unsigned long long w = s_w[lane];
            unsigned long long wi = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1)
                {
                const unsigned long long x = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= (unsigned int)o) wi += x;
                }
            s_w[lane] = wi - w;
            }
        __syncthreads();
        const unsigned long long carry = s_carry;
        if (i < n_tiles) tile_sum[i] = carry + s_w[warp] + incl - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) s_carry = carry + s_w[warp] + incl;
        __syncthreads();
        }
    if (threadIdx.x == 0) *total = s_carry;
    }

__global__ void __launch_bounds__(kScan64Block) k_scan64_apply(const unsigned int* __restrict__ in, unsigned int n,
                                                               const unsigned long long* __restrict__ tile_base,
                                                               unsigned long long* __restrict__ out)
    {
    __shared__ unsigned long long s_w[kScan64Block / 32 + 1];
    const unsigned int base = blockIdx.x * kScan64Tile + threadIdx.x * kScan64Items;
    unsigned int v[kScan64Items];
    unsigned long long sum = 0;
#pragma unroll
    for (int k = 0; k < kScan64Items; ++k)
        {
        v[k] = (base + k < n) ? in[base + k] : 0u;
        sum += v[k];
        }
    const unsigned int lane = threadIdx.x & 31u;
    const unsigned int warp = threadIdx.x >> 5;
    unsigned long long incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
        {
        const unsigned long long x = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (unsigned int)o) incl += x;
        }
    if (lane == 31u) s_w[warp] = incl;
    __syncthreads();
    if (threadIdx.x == 0)
        {
        unsigned long long r = 0;
        for (int w = 0; w < kScan64Block / 32; ++w)
            {
            const unsigned long long x = s_w[w];
            s_w[w] = r;
            r += x;
            }
        }
    __syncthreads();
    unsigned long long run = tile_base[blockIdx.x] + s_w[warp] + incl - sum;
#pragma unroll
    for (int k = 0; k < kScan64Items; ++k)
        {
        if (base + k < n) out[base + k] = run;
        run += v[k];
        }
    }

} // namespace gpu
} // namespace neighbor

#endif // NEIGHBOR_KERNELS_CAPACITY_CUH_
