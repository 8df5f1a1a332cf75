// Reference harness driver (TEST / MEASUREMENT INFRASTRUCTURE ONLY).
//
// Runs the reference's own CUDA kernels (mphowardlab/neighbor v0.3.2) on the GPU: they are
// compiled from the reference headers into oracle/_ref/ref_kernels.cubin (ref_kernels.cu), loaded
// here with the driver API and found by name.  The launch sequence re-enacts the reference's host
// classes: LBVH::build (include/neighbor/LBVH.h:242-318: gen_codes, CUB DeviceRadixSort::SortPairs
// on bits [0,30), gen_tree, memset of the locks, bubble_aabbs), LBVHTraverser::setup/compress
// (include/neighbor/LBVHTraverser.h:378-390,481-510) and traverse (:414-450).  The sort is CUB's,
// called exactly as the reference calls it (include/neighbor/kernels/LBVH.cuh:421-443).
//
//   ref_driver bench N steps warmup rc               time the plain two-pass step on uniform
//                                                    trajectory frames, every block size 32..1024
//   ref_driver frames in.f32 N F rc L steps warmup   the same step on F given frames (cycled)
//   ref_driver poly s.f32 Ns l.f32 Nl F L steps warmup   two-tree polydisperse step (diameters 1
//                                                    and 10, cutoff (di+dj)/2 + 0.4) on F frames
//   ref_driver dump  in.f32 N lo3 hi3 rc L3 out [exact_only | sphere r]
//                                                    write the reference's outputs for given
//                                                    points (sphere r: a SphereInsertOp tree)
//   ref_driver hash  in.f32 N rc L out               counts and per-row hashes of the exact list
//   ref_driver frames64 in.f64 N F rc L steps warmup the plain two-pass step on F given double
//                                                    frames (the harness's double insert and
//                                                    exact query ops), every block size
//
// Kernel parameters are passed as byte images of the reference's structs; the layouts below are
// asserted here and, against the reference's own definitions, in ref_kernels.cu.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace
{
struct PointInsertOp { const float3* points; unsigned int N; };
struct SphereInsertOp { const float3* points; float r; unsigned int N; };
struct LBVHData { int* parent; int* left; int* right; unsigned int* primitive; float3* lo; float3* hi; int root; };
struct LBVHCompressedData { int root; int4* data; float3* lo; float3* hi; float3* bins; };
struct CountNeighborsOp { unsigned int* nneigh; };
struct NeighborListOp { unsigned int* neigh_list; unsigned int* nneigh; unsigned int max_neigh; };
struct ImageListOp { const float3* images; unsigned int N; };
struct SphereQueryOp { const float4* spheres; unsigned int N; };
struct NullTransformOp {};
struct RefExactQueryOp { const float4* spheres; unsigned int N; const float3* points; float3 box; float pad; };
struct RefPointInsertOpF64 { const double3* points; unsigned int N; };
struct __align__(16) RefSphereF64 { double x, y, z, w; };
struct RefExactQueryOpF64 { const RefSphereF64* spheres; unsigned int N; const double3* points; double3 box; float pad; };

static_assert(sizeof(PointInsertOp) == 16 && offsetof(PointInsertOp, N) == 8, "layout");
static_assert(sizeof(SphereInsertOp) == 16 && offsetof(SphereInsertOp, r) == 8 && offsetof(SphereInsertOp, N) == 12,
              "layout");
static_assert(sizeof(LBVHData) == 56 && offsetof(LBVHData, root) == 48, "layout");
static_assert(sizeof(LBVHCompressedData) == 40 && offsetof(LBVHCompressedData, data) == 8, "layout");
static_assert(sizeof(CountNeighborsOp) == 8, "layout");
static_assert(sizeof(NeighborListOp) == 24 && offsetof(NeighborListOp, max_neigh) == 16, "layout");
static_assert(sizeof(ImageListOp) == 16 && offsetof(ImageListOp, N) == 8, "layout");
static_assert(sizeof(SphereQueryOp) == 16, "layout");
static_assert(sizeof(NullTransformOp) == 1, "layout");
static_assert(sizeof(RefExactQueryOp) == 40 && offsetof(RefExactQueryOp, points) == 16
              && offsetof(RefExactQueryOp, box) == 24 && offsetof(RefExactQueryOp, pad) == 36, "layout");
static_assert(sizeof(RefPointInsertOpF64) == 16 && offsetof(RefPointInsertOpF64, N) == 8, "layout");
static_assert(sizeof(RefExactQueryOpF64) == 56 && offsetof(RefExactQueryOpF64, N) == 8
              && offsetof(RefExactQueryOpF64, points) == 16 && offsetof(RefExactQueryOpF64, box) == 24
              && offsetof(RefExactQueryOpF64, pad) == 48, "layout");

void check(cudaError_t e, const char* what)
    {
    if (e != cudaSuccess) { fprintf(stderr, "CUDA error %s: %s\n", what, cudaGetErrorString(e)); exit(2); }
    }
void checkd(CUresult e, const char* what)
    {
    if (e != CUDA_SUCCESS) { const char* s = nullptr; cuGetErrorString(e, &s); fprintf(stderr, "CUDA driver error %s: %s\n", what, s ? s : "?"); exit(2); }
    }

struct Kernels
    {
    CUfunction gen_codes = nullptr, gen_tree = nullptr, bubble = nullptr, one = nullptr, compress = nullptr;
    CUfunction gen_codes_sph = nullptr, bubble_sph = nullptr, one_sph = nullptr;
    CUfunction count_stock = nullptr, count_exact = nullptr, list_exact = nullptr, list_stock = nullptr;
    CUfunction gen_codes_f64 = nullptr, bubble_f64 = nullptr, one_f64 = nullptr, count_f64 = nullptr, list_f64 = nullptr;
    };

Kernels load_kernels(const char* cubin)
    {
    CUmodule mod;
    checkd(cuModuleLoad(&mod, cubin), "cuModuleLoad");
    unsigned int n = 0;
    checkd(cuModuleGetFunctionCount(&n, mod), "function count");
    std::vector<CUfunction> fs(n);
    checkd(cuModuleEnumerateFunctions(fs.data(), n, mod), "enumerate");
    Kernels k;
    for (CUfunction e : fs)
        {
        const char* name = nullptr;
        checkd(cuFuncGetName(&name, e), "name");
        const std::string s(name);
        // enumerated handles are not loaded under lazy module loading: fetch by name
        CUfunction f;
        checkd(cuModuleGetFunction(&f, mod, name), "get function");
        auto has = [&](const char* x) { return s.find(x) != std::string::npos; };
        const bool sph = has("SphereInsertOp");
        if (has("RefPointInsertOpF64"))
            {
            if (has("lbvh_gen_codes")) k.gen_codes_f64 = f;
            else if (has("lbvh_bubble_aabbs")) k.bubble_f64 = f;
            else if (has("lbvh_one_primitive")) k.one_f64 = f;
            continue;
            }
        if (has("RefExactQueryOpF64"))
            {
            if (has("CountNeighborsOp")) k.count_f64 = f;
            else if (has("NeighborListOp")) k.list_f64 = f;
            continue;
            }
        if (has("lbvh_gen_codes")) (sph ? k.gen_codes_sph : k.gen_codes) = f;
        else if (has("lbvh_gen_tree")) k.gen_tree = f;
        else if (has("lbvh_bubble_aabbs")) (sph ? k.bubble_sph : k.bubble) = f;
        else if (has("lbvh_one_primitive")) (sph ? k.one_sph : k.one) = f;
        else if (has("lbvh_compress_ropes")) k.compress = f;
        else if (has("lbvh_traverse_ropes") && has("CountNeighborsOp") && has("SphereQueryOp")) k.count_stock = f;
        else if (has("lbvh_traverse_ropes") && has("CountNeighborsOp") && has("RefExactQueryOp")) k.count_exact = f;
        else if (has("lbvh_traverse_ropes") && has("NeighborListOp") && has("RefExactQueryOp")) k.list_exact = f;
        else if (has("lbvh_traverse_ropes") && has("NeighborListOp") && has("SphereQueryOp")) k.list_stock = f;
        }
    if (!k.gen_codes || !k.gen_tree || !k.bubble || !k.one || !k.compress || !k.count_stock || !k.count_exact || !k.list_exact
        || !k.list_stock || !k.gen_codes_sph || !k.bubble_sph || !k.one_sph || !k.gen_codes_f64 || !k.bubble_f64
        || !k.one_f64 || !k.count_f64 || !k.list_f64)
        { fprintf(stderr, "reference kernels missing from %s\n", cubin); exit(3); }
    return k;
    }

// The reference clamps each launcher's block size to the kernel's maxThreadsPerBlock.
unsigned int clamp_block(CUfunction f, unsigned int bs)
    {
    int mx = 1024;
    checkd(cuFuncGetAttribute(&mx, CU_FUNC_ATTRIBUTE_MAX_THREADS_PER_BLOCK, f), "attribute");
    return std::min<unsigned int>(bs, (unsigned int)mx);
    }

void launch(CUfunction f, unsigned int n, unsigned int bs, cudaStream_t s, void** args)
    {
    if (n == 0) return;
    bs = clamp_block(f, bs);
    checkd(cuLaunchKernel(f, (n + bs - 1) / bs, 1, 1, bs, 1, 1, 0, (CUstream)s, args, nullptr), "launch");
    }

// Reference-sized arrays of LBVH + LBVHTraverser (shared_array = managed memory).
struct RefTree
    {
    unsigned int N = 0;
    int *parent = nullptr, *left = nullptr, *right = nullptr;
    float3 *lo = nullptr, *hi = nullptr;
    unsigned int *codes[2] = {nullptr, nullptr}, *idx[2] = {nullptr, nullptr};
    unsigned int* locks = nullptr;
    void* tmp = nullptr;
    size_t tmp_bytes = 0;
    int sel_codes = 0, sel_idx = 0;
    int4* data = nullptr;
    float3 *clo = nullptr, *chi = nullptr, *bins = nullptr;

    void allocate(unsigned int n)
        {
        N = n;
        const size_t nodes = 2 * (size_t)n - 1;
        check(cudaMallocManaged(&parent, nodes * 4), "alloc");
        check(cudaMallocManaged(&left, std::max<size_t>(n - 1, 1) * 4), "alloc");
        check(cudaMallocManaged(&right, std::max<size_t>(n - 1, 1) * 4), "alloc");
        check(cudaMallocManaged(&lo, nodes * 12), "alloc");
        check(cudaMallocManaged(&hi, nodes * 12), "alloc");
        for (int b = 0; b < 2; ++b)
            {
            check(cudaMallocManaged(&codes[b], (size_t)n * 4), "alloc");
            check(cudaMallocManaged(&idx[b], (size_t)n * 4), "alloc");
            }
        check(cudaMallocManaged(&locks, std::max<size_t>(n - 1, 1) * 4), "alloc");
        cub::DoubleBuffer<unsigned int> k(codes[0], codes[1]), v(idx[0], idx[1]);
        check(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, k, v, (int)n, 0, 30), "sort size");
        if (tmp_bytes == 0) tmp_bytes = 4;
        check(cudaMallocManaged(&tmp, tmp_bytes), "alloc");
        check(cudaMallocManaged(&data, nodes * 16), "alloc");
        check(cudaMallocManaged(&clo, 12), "alloc");
        check(cudaMallocManaged(&chi, 12), "alloc");
        check(cudaMallocManaged(&bins, 12), "alloc");
        }

    LBVHData tree_data()
        {
        LBVHData t;
        t.parent = parent; t.left = left; t.right = right; t.primitive = idx[sel_idx]; t.lo = lo; t.hi = hi; t.root = 0;
        return t;
        }

    // LBVH::build (include/neighbor/LBVH.h:242-318) with PointInsertOp, or SphereInsertOp of
    // radius r when r >= 0
    void build(const Kernels& K, const float3* pts, float3 slo, float3 shi, unsigned int bs, cudaStream_t s,
               float r = -1.f)
        {
        PointInsertOp ins{pts, N};
        SphereInsertOp sins{pts, r, N};
        if (r >= 0.f)
            build_with(K, K.gen_codes_sph, K.bubble_sph, K.one_sph, &sins, slo, shi, bs, s);
        else
            build_with(K, K.gen_codes, K.bubble, K.one, &ins, slo, shi, bs, s);
        }

    // the same with the harness's double-precision point insert op
    void build_f64(const Kernels& K, const double3* pts, float3 slo, float3 shi, unsigned int bs, cudaStream_t s)
        {
        RefPointInsertOpF64 ins{pts, N};
        build_with(K, K.gen_codes_f64, K.bubble_f64, K.one_f64, &ins, slo, shi, bs, s);
        }

    void build_with(const Kernels& K, CUfunction gen_codes, CUfunction bubble, CUfunction one, void* insp, float3 slo,
                    float3 shi, unsigned int bs, cudaStream_t s)
        {
        sel_codes = sel_idx = 0;
        if (N == 1)
            {
            LBVHData t = tree_data();
            void* a[] = {&t, insp};
            checkd(cuLaunchKernel(one, 1, 1, 1, 1, 1, 1, 0, (CUstream)s, a, nullptr), "launch");
            return;
            }
        unsigned int n = N;
            {
            void* a[] = {&codes[0], &idx[0], insp, &slo, &shi, &n};
            launch(gen_codes, n, bs, s, a);
            }
        cub::DoubleBuffer<unsigned int> k(codes[0], codes[1]), v(idx[0], idx[1]);
        check(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, k, v, (int)n, 0, 30, s), "sort");
        sel_codes = k.selector;
        sel_idx = v.selector;
        LBVHData t = tree_data();
        const unsigned int* sc = codes[sel_codes];
            {
            void* a[] = {&t, &sc, &n};
            launch(K.gen_tree, n - 1, bs, s, a);
            }
        check(cudaMemsetAsync(locks, 0, (size_t)(n - 1) * 4, s), "memset");
            {
            void* a[] = {&t, insp, &locks, &n};
            launch(bubble, n, bs, s, a);
            }
        }

    // LBVHTraverser::compress (include/neighbor/LBVHTraverser.h:481-510)
    LBVHCompressedData compress(const Kernels& K, unsigned int bs, cudaStream_t s)
        {
        LBVHCompressedData c{0, data, clo, chi, bins};
        NullTransformOp tr;
        LBVHData t = tree_data();
        unsigned int ni = N - 1, nn = 2 * N - 1;
        void* a[] = {&c, &tr, &t, &ni, &nn};
        launch(K.compress, nn, bs, s, a);
        return c;
        }
    };

// ---- helpers of the harness itself (not the reference) ----
__device__ __forceinline__ unsigned int hash32(unsigned int x)
    {
    x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
    return x;
    }
__device__ __forceinline__ float u01(unsigned int h) { return (h >> 8) * (1.0f / 16777216.0f); }

__global__ void k_uniform(float3* p, unsigned int n, float L, unsigned int seed)
    {
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned int h = hash32(i * 3u + seed * 0x9e3779b9u);
    p[i] = make_float3(u01(h) * L, u01(hash32(h + 1u)) * L, u01(hash32(h + 2u)) * L);
    }

// Gaussian move (sigma) and wrap into [0, L): the trajectory frames of the measurement.
__global__ void k_move(const float3* in, float3* out, unsigned int n, float L, float sigma, unsigned int seed)
    {
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float v[3] = {in[i].x, in[i].y, in[i].z};
    for (int d = 0; d < 3; ++d)
        {
        const unsigned int h = hash32(i * 6u + 2u * d + seed * 0x85ebca6bu);
        const float u1 = fmaxf(u01(h), 1e-7f), u2 = u01(hash32(h ^ 0x68e31da4u));
        float x = v[d] + sigma * sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
        x -= L * floorf(x / L);
        if (x >= L) x -= L;
        v[d] = x;
        }
    out[i] = make_float3(v[0], v[1], v[2]);
    }

// Query spheres in the tree's sorted order (the reference benchmark's query order,
// benchmark/lbvh_benchmark.cc:177-184), or in input order when prim is null.
__global__ void k_spheres(const float3* p, const unsigned int* prim, float4* sph, unsigned int n, float rc)
    {
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 x = p[prim ? prim[i] : i];
    sph[i] = make_float4(x.x, x.y, x.z, rc);
    }

float exact_pad(float rc, float coord_max)
    {
    const float m = std::fmax(std::fabs(coord_max), 1.0f) * 2.0f + std::fabs(rc);
    int e;
    std::frexp(m, &e);
    return 16.0f * std::ldexp(1.0f, e - 24) + std::fabs(rc) * 1.0e-6f;
    }

void images27(float3 L, std::vector<float3>& img)
    {
    for (int ix = -1; ix <= 1; ++ix)
        for (int iy = -1; iy <= 1; ++iy)
            for (int iz = -1; iz <= 1; ++iz)
                img.push_back(make_float3(L.x * (float)ix, L.y * (float)iy, L.z * (float)iz));
    }

// Block sizes the reference's tunables accept (LBVH.h:225, LBVHTraverser.h:358: 32..1024 by 32).
std::vector<unsigned int> all_blocks()
    {
    std::vector<unsigned int> b;
    for (unsigned int bs = 32; bs <= 1024; bs += 32) b.push_back(bs);
    return b;
    }

// Buffers of one plain two-pass list: query spheres, counts, list, CUB max.
struct TwoPass
    {
    unsigned int n = 0, cap = 0;
    float4* sph = nullptr;
    unsigned int *nn = nullptr, *list = nullptr, *dmax = nullptr;
    void* rtmp = nullptr;
    size_t rtmp_bytes = 0;
    void allocate(unsigned int q, unsigned int list_cap)
        {
        n = q;
        cap = list_cap;
        check(cudaMalloc(&sph, (size_t)std::max(q, 1u) * 16), "alloc");
        check(cudaMalloc(&nn, (size_t)std::max(q, 1u) * 4), "alloc");
        check(cudaMalloc(&dmax, 4), "alloc");
        check(cudaMalloc(&list, (size_t)std::max(q, 1u) * cap * 4), "alloc");
        check(cub::DeviceReduce::Max(nullptr, rtmp_bytes, nn, dmax, (int)std::max(q, 1u)), "reduce size");
        check(cudaMalloc(&rtmp, rtmp_bytes), "alloc");
        }
    };

// The reference's two-pass list for one set of queries (benchmark/lbvh_benchmark.cc's traversal
// with CountNeighborsOp, the host read of the largest count, then NeighborListOp of that stride;
// include/neighbor/OutputOps.h:28-176): count, CUB max, host read, fill.  Returns the largest
// count.
unsigned int two_pass_with(CUfunction count, CUfunction list, const LBVHCompressedData& c, const void* q, unsigned int Q,
                           const ImageListOp& im, TwoPass& b, unsigned int bs, cudaStream_t s, cudaEvent_t after_count);

unsigned int two_pass(const Kernels& K, const LBVHCompressedData& c, const RefExactQueryOp& q, const ImageListOp& im,
                      TwoPass& b, unsigned int bs, cudaStream_t s, cudaEvent_t after_count = nullptr)
    {
    return two_pass_with(K.count_exact, K.list_exact, c, &q, q.N, im, b, bs, s, after_count);
    }

// the same with the harness's double-precision exact query op
unsigned int two_pass_f64(const Kernels& K, const LBVHCompressedData& c, const RefExactQueryOpF64& q,
                          const ImageListOp& im, TwoPass& b, unsigned int bs, cudaStream_t s,
                          cudaEvent_t after_count = nullptr)
    {
    return two_pass_with(K.count_f64, K.list_f64, c, &q, q.N, im, b, bs, s, after_count);
    }

unsigned int two_pass_with(CUfunction count, CUfunction list, const LBVHCompressedData& c, const void* q, unsigned int Q,
                           const ImageListOp& im, TwoPass& b, unsigned int bs, cudaStream_t s, cudaEvent_t after_count)
    {
    if (Q == 0) return 0;
        {
        CountNeighborsOp out{b.nn};
        void* a[] = {&out, (void*)&c, (void*)q, (void*)&im};
        launch(count, Q, bs, s, a);
        }
    if (after_count) check(cudaEventRecord(after_count, s), "rec");
    check(cub::DeviceReduce::Max(b.rtmp, b.rtmp_bytes, b.nn, b.dmax, (int)Q, s), "reduce");
    unsigned int mx = 0;
    check(cudaMemcpyAsync(&mx, b.dmax, 4, cudaMemcpyDeviceToHost, s), "copy");
    check(cudaStreamSynchronize(s), "sync");
    if (mx > b.cap)
        {
        // a longer row than any before: the list buffer grows (in the warm-up steps of a sweep)
        check(cudaFree(b.list), "free");
        b.cap = mx + mx / 4u;
        check(cudaMalloc(&b.list, (size_t)b.n * b.cap * 4), "alloc");
        }
        {
        NeighborListOp out{b.list, b.nn, std::max(mx, 1u)};
        void* a[] = {&out, (void*)&c, (void*)q, (void*)&im};
        launch(list, Q, bs, s, a);
        }
    return mx;
    }

unsigned long long sum_counts(const unsigned int* d, unsigned int n)
    {
    std::vector<unsigned int> h(n);
    check(cudaMemcpy(h.data(), d, (size_t)n * 4, cudaMemcpyDeviceToHost), "copy");
    unsigned long long t = 0;
    for (unsigned int x : h) t += x;
    return t;
    }

float* read_points(const char* path, size_t count)
    {
    std::vector<float> h(count * 3);
    FILE* f = fopen(path, "rb");
    if (!f || fread(h.data(), 12, count, f) != count) { fprintf(stderr, "cannot read %s\n", path); exit(5); }
    fclose(f);
    float* d;
    check(cudaMalloc(&d, std::max<size_t>(count, 1) * 12), "alloc");
    check(cudaMemcpy(d, h.data(), count * 12, cudaMemcpyHostToDevice), "copy");
    return d;
    }

float3* image_list(float L)
    {
    std::vector<float3> himg;
    images27(make_float3(L, L, L), himg);
    float3* img;
    check(cudaMalloc(&img, 27 * 12), "alloc");
    check(cudaMemcpy(img, himg.data(), 27 * 12, cudaMemcpyHostToDevice), "copy");
    return img;
    }

// Plain two-pass step of one point tree queried by its own points in sorted order (the reference
// benchmark's query order, benchmark/lbvh_benchmark.cc:177-184) on frames[it % F], timed per
// block size over `steps` steps after `warmup`.  Prints one JSON object.
int sweep_self(const Kernels& K, const std::vector<const float3*>& frames, unsigned int n, float rc, float L, int steps,
               int warmup, const char* label)
    {
    const float3 box = make_float3(L, L, L);
    cudaStream_t s;
    check(cudaStreamCreate(&s), "stream");
    float3* img = image_list(L);
    RefTree T;
    T.allocate(n);
    TwoPass b;
    b.allocate(n, 96);
    const float pad = exact_pad(rc, 2 * L);
    check(cudaStreamSynchronize(s), "sync");
    printf("{\"impl\": \"reference-cuda\", \"workload\": \"%s\", \"n\": %u, \"rc\": %g, \"steps\": %d, \"warmup\": %d, "
           "\"results\": [", label, n, rc, steps, warmup);
    bool first = true;
    double pairs_sum = 0;
    for (unsigned int bs : all_blocks())
        {
        cudaEvent_t ev[6];
        for (auto& e : ev) check(cudaEventCreate(&e), "event");
        std::vector<double> step_ms;
        double t_build = 0, t_setup = 0, t_count = 0, t_fill = 0;
        for (int it = 0; it < warmup + steps; ++it)
            {
            const bool timed = it >= warmup;
            const float3* P = frames[it % frames.size()];
            check(cudaEventRecord(ev[0], s), "rec");
            T.build(K, P, make_float3(0, 0, 0), box, bs, s);
            k_spheres<<<(n + 255) / 256, 256, 0, s>>>(P, T.idx[T.sel_idx], b.sph, n, rc);
            check(cudaEventRecord(ev[1], s), "rec");
            LBVHCompressedData c = T.compress(K, bs, s);
            check(cudaEventRecord(ev[2], s), "rec");
            RefExactQueryOp q{b.sph, n, P, box, pad};
            ImageListOp im{img, 27};
            two_pass(K, c, q, im, b, bs, s, ev[3]);
            check(cudaEventRecord(ev[5], s), "rec");
            check(cudaStreamSynchronize(s), "sync");
            if (timed)
                {
                float ms;
                cudaEventElapsedTime(&ms, ev[0], ev[1]); t_build += ms;
                cudaEventElapsedTime(&ms, ev[1], ev[2]); t_setup += ms;
                cudaEventElapsedTime(&ms, ev[2], ev[3]); t_count += ms;
                cudaEventElapsedTime(&ms, ev[3], ev[5]); t_fill += ms;
                cudaEventElapsedTime(&ms, ev[0], ev[5]); step_ms.push_back(ms);
                // pairs of every timed frame, counted with the first block size (the same frames
                // for every block size)
                if (first) pairs_sum += (double)sum_counts(b.nn, n);
                }
            }
        double mean = 0;
        for (double v : step_ms) mean += v;
        mean /= step_ms.size();
        std::vector<double> sorted = step_ms;
        std::sort(sorted.begin(), sorted.end());
        printf("%s{\"block\": %u, \"build_ms\": %.4f, \"setup_ms\": %.4f, \"count_ms\": %.4f, \"fill_ms\": %.4f, "
               "\"step_ms\": %.4f, \"step_ms_median\": %.4f}",
               first ? "" : ", ", bs, t_build / steps, t_setup / steps, t_count / steps, t_fill / steps, mean,
               sorted[sorted.size() / 2]);
        first = false;
        for (auto& e : ev) cudaEventDestroy(e);
        }
    printf("], \"pairs_per_step\": %.1f}\n", pairs_sum / steps);
    return 0;
    }

int run_bench(const Kernels& K, unsigned int n, int steps, int warmup, float rc)
    {
    const float L = std::cbrt(n / 0.85f);
    std::vector<const float3*> frames;
    float3* base;
    check(cudaMalloc(&base, (size_t)n * 12), "alloc");
    k_uniform<<<(n + 255) / 256, 256>>>(base, n, L, 1234u);
    const float3* prev = base;
    for (int f = 0; f < steps + warmup; ++f)
        {
        float3* p;
        check(cudaMalloc(&p, (size_t)n * 12), "alloc");
        k_move<<<(n + 255) / 256, 256>>>(prev, p, n, L, 0.05f, 77u + (unsigned)f);
        frames.push_back(p);
        prev = p;
        }
    check(cudaDeviceSynchronize(), "sync");
    return sweep_self(K, frames, n, rc, L, steps, warmup, "uniform trajectory (sigma 0.05)");
    }

int run_frames(const Kernels& K, const char* path, unsigned int n, int F, float rc, float L, int steps, int warmup)
    {
    float* all = read_points(path, (size_t)n * F);
    std::vector<const float3*> frames;
    for (int f = 0; f < F; ++f) frames.push_back(reinterpret_cast<const float3*>(all) + (size_t)f * n);
    return sweep_self(K, frames, n, rc, L, steps, warmup, "given frames");
    }

// Query spheres in double precision, in the tree's sorted order.
__global__ void k_spheres_f64(const double3* p, const unsigned int* prim, RefSphereF64* sph, unsigned int n, double rc)
    {
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double3 x = p[prim[i]];
    RefSphereF64 q;
    q.x = x.x;
    q.y = x.y;
    q.z = x.z;
    q.w = rc;
    sph[i] = q;
    }

double* read_points_f64(const char* path, size_t count)
    {
    std::vector<double> h(count * 3);
    FILE* f = fopen(path, "rb");
    if (!f || fread(h.data(), 24, count, f) != count) { fprintf(stderr, "cannot read %s\n", path); exit(5); }
    fclose(f);
    double* d;
    check(cudaMalloc(&d, std::max<size_t>(count, 1) * 24), "alloc");
    check(cudaMemcpy(d, h.data(), count * 24, cudaMemcpyHostToDevice), "copy");
    return d;
    }

// The plain two-pass step on double-precision frames (cycled): build with the double insert op,
// setup, count, max, fill with the double exact query (queries in sorted order, 27 images of the
// cube of side L), every block size; as sweep_self, plus the pair total of the last timed frame.
int run_frames64(const Kernels& K, const char* path, unsigned int n, int F, double rc, float L, int steps, int warmup)
    {
    double* all = read_points_f64(path, (size_t)n * F);
    const double3 box = make_double3(L, L, L);
    cudaStream_t s;
    check(cudaStreamCreate(&s), "stream");
    float3* img = image_list(L);
    RefTree T;
    T.allocate(n);
    TwoPass b;
    b.allocate(n, 96);
    RefSphereF64* sph;
    check(cudaMalloc(&sph, (size_t)std::max(n, 1u) * sizeof(RefSphereF64)), "alloc");
    const float pad = exact_pad((float)rc, 2 * L);
    check(cudaStreamSynchronize(s), "sync");
    printf("{\"impl\": \"reference-cuda\", \"workload\": \"given double frames\", \"n\": %u, \"rc\": %g, \"steps\": %d, "
           "\"warmup\": %d, \"results\": [", n, rc, steps, warmup);
    bool first = true;
    double pairs_sum = 0, pairs_last = 0;
    for (unsigned int bs : all_blocks())
        {
        cudaEvent_t ev[6];
        for (auto& e : ev) check(cudaEventCreate(&e), "event");
        std::vector<double> step_ms;
        double t_build = 0, t_setup = 0, t_count = 0, t_fill = 0;
        for (int it = 0; it < warmup + steps; ++it)
            {
            const bool timed = it >= warmup;
            const double3* P = reinterpret_cast<const double3*>(all) + (size_t)(it % F) * n;
            check(cudaEventRecord(ev[0], s), "rec");
            T.build_f64(K, P, make_float3(0, 0, 0), make_float3(L, L, L), bs, s);
            k_spheres_f64<<<(n + 255) / 256, 256, 0, s>>>(P, T.idx[T.sel_idx], sph, n, rc);
            check(cudaEventRecord(ev[1], s), "rec");
            LBVHCompressedData c = T.compress(K, bs, s);
            check(cudaEventRecord(ev[2], s), "rec");
            RefExactQueryOpF64 q{sph, n, P, box, pad};
            ImageListOp im{img, 27};
            two_pass_f64(K, c, q, im, b, bs, s, ev[3]);
            check(cudaEventRecord(ev[5], s), "rec");
            check(cudaStreamSynchronize(s), "sync");
            if (timed)
                {
                float ms;
                cudaEventElapsedTime(&ms, ev[0], ev[1]); t_build += ms;
                cudaEventElapsedTime(&ms, ev[1], ev[2]); t_setup += ms;
                cudaEventElapsedTime(&ms, ev[2], ev[3]); t_count += ms;
                cudaEventElapsedTime(&ms, ev[3], ev[5]); t_fill += ms;
                cudaEventElapsedTime(&ms, ev[0], ev[5]); step_ms.push_back(ms);
                if (first)
                    {
                    pairs_last = (double)sum_counts(b.nn, n);
                    pairs_sum += pairs_last;
                    }
                }
            }
        double mean = 0;
        for (double v : step_ms) mean += v;
        mean /= step_ms.size();
        std::vector<double> sorted = step_ms;
        std::sort(sorted.begin(), sorted.end());
        printf("%s{\"block\": %u, \"build_ms\": %.4f, \"setup_ms\": %.4f, \"count_ms\": %.4f, \"fill_ms\": %.4f, "
               "\"step_ms\": %.4f, \"step_ms_median\": %.4f}",
               first ? "" : ", ", bs, t_build / steps, t_setup / steps, t_count / steps, t_fill / steps, mean,
               sorted[sorted.size() / 2]);
        first = false;
        for (auto& e : ev) cudaEventDestroy(e);
        }
    printf("], \"pairs_per_step\": %.1f, \"pairs_last_frame\": %.1f}\n", pairs_sum / steps, pairs_last);
    return 0;
    }

// Polydisperse step: a tree per species (PointInsertOp), every (query species, tree) pair listed
// with cutoff (d_i + d_j)/2 + 0.4: self pairs query the tree's points in sorted order, cross pairs
// the other species' points in input order.
int run_poly(const Kernels& K, const char* spath, unsigned int ns, const char* lpath, unsigned int nl, int F, float L,
             int steps, int warmup)
    {
    float* sp = read_points(spath, (size_t)ns * F);
    float* lp = read_points(lpath, (size_t)nl * F);
    const float3 box = make_float3(L, L, L);
    const float diam[2] = {1.0f, 10.0f};
    const unsigned int cnt[2] = {ns, nl};
    cudaStream_t s;
    check(cudaStreamCreate(&s), "stream");
    float3* img = image_list(L);
    RefTree T[2];
    T[0].allocate(ns);
    T[1].allocate(nl);
    TwoPass b[2][2];
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) b[i][j].allocate(cnt[i], (i == 0 && j == 0) ? 64u : 4096u);
    printf("{\"impl\": \"reference-cuda\", \"workload\": \"polydisperse\", \"n_small\": %u, \"n_large\": %u, "
           "\"steps\": %d, \"warmup\": %d, \"results\": [", ns, nl, steps, warmup);
    bool first = true;
    double pairs = 0;
    for (unsigned int bs : all_blocks())
        {
        cudaEvent_t e0, e1;
        check(cudaEventCreate(&e0), "event");
        check(cudaEventCreate(&e1), "event");
        std::vector<double> step_ms;
        for (int it = 0; it < warmup + steps; ++it)
            {
            const int f = it % F;
            const float3* P[2] = {reinterpret_cast<const float3*>(sp) + (size_t)f * ns,
                                  reinterpret_cast<const float3*>(lp) + (size_t)f * nl};
            check(cudaEventRecord(e0, s), "rec");
            LBVHCompressedData c[2];
            for (int j = 0; j < 2; ++j)
                {
                T[j].build(K, P[j], make_float3(0, 0, 0), box, bs, s);
                c[j] = T[j].compress(K, bs, s);
                }
            double step_pairs = 0;
            for (int i = 0; i < 2; ++i)
                for (int j = 0; j < 2; ++j)
                    {
                    const float R = 0.5f * (diam[i] + diam[j]) + 0.4f;
                    if (i == j)
                        k_spheres<<<(cnt[i] + 255) / 256, 256, 0, s>>>(P[j], T[j].idx[T[j].sel_idx], b[i][j].sph, cnt[i], R);
                    else
                        k_spheres<<<(cnt[i] + 255) / 256, 256, 0, s>>>(P[i], nullptr, b[i][j].sph, cnt[i], R);
                    RefExactQueryOp q{b[i][j].sph, cnt[i], P[j], box, exact_pad(R, 2 * L)};
                    ImageListOp im{img, 27};
                    two_pass(K, c[j], q, im, b[i][j], bs, s);
                    }
            check(cudaEventRecord(e1, s), "rec");
            check(cudaStreamSynchronize(s), "sync");
            if (it >= warmup)
                {
                float ms;
                cudaEventElapsedTime(&ms, e0, e1);
                step_ms.push_back(ms);
                if (first)
                    for (int i = 0; i < 2; ++i)
                        for (int j = 0; j < 2; ++j) step_pairs += (double)sum_counts(b[i][j].nn, cnt[i]);
                pairs += step_pairs;
                }
            }
        double mean = 0;
        for (double v : step_ms) mean += v;
        mean /= step_ms.size();
        std::sort(step_ms.begin(), step_ms.end());
        printf("%s{\"block\": %u, \"step_ms\": %.4f, \"step_ms_median\": %.4f}", first ? "" : ", ", bs, mean,
               step_ms[step_ms.size() / 2]);
        first = false;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        }
    printf("], \"pairs_per_step\": %.1f}\n", pairs / steps);
    return 0;
    }

// Row hash of a neighbor list, sum over k < count of (entry_k + 1) * C_k plus count * C_count, in
// 64-bit integers (no overflow for rows of up to 64 entries): C_k = ((k + 1) * 2654435761 mod 2^32)
// with the top bit cleared and the low bit set; C_count = 0x2545F491.
__global__ void k_row_hash(const unsigned int* list, const unsigned int* nn, unsigned int stride, unsigned int n,
                           unsigned long long* out)
    {
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned int c = nn[i];
    unsigned long long h = (unsigned long long)c * 0x2545F491ull;
    for (unsigned int k = 0; k < c && k < stride; ++k)
        {
        const unsigned long long ck = (((k + 1u) * 2654435761u) & 0x7fffffffu) | 1u;
        h += (unsigned long long)(list[(size_t)i * stride + k] + 1u) * ck;
        }
    out[i] = h;
    }

// Counts and row hashes of the exact neighbor list of the given points (queries in input order,
// 27 images of the cube of side L), for comparing a large list with the library's row by row.
int run_hash(const Kernels& K, const char* path, unsigned int n, float rc, float L, const char* out_prefix)
    {
    float* P = read_points(path, n);
    const float3 box = make_float3(L, L, L);
    RefTree T;
    T.allocate(n);
    T.build(K, reinterpret_cast<const float3*>(P), make_float3(0, 0, 0), box, 128, 0);
    LBVHCompressedData c = T.compress(K, 128, 0);
    float3* img = image_list(L);
    TwoPass b;
    b.allocate(n, 64);
    k_spheres<<<(n + 255) / 256, 256>>>(reinterpret_cast<const float3*>(P), nullptr, b.sph, n, rc);
    RefExactQueryOp q{b.sph, n, reinterpret_cast<const float3*>(P), box, exact_pad(rc, 2 * L)};
    ImageListOp im{img, 27};
    const unsigned int mx = two_pass(K, c, q, im, b, 128, 0);
    unsigned long long* h;
    check(cudaMalloc(&h, (size_t)n * 8), "alloc");
    k_row_hash<<<(n + 255) / 256, 256>>>(b.list, b.nn, std::max(mx, 1u), n, h);
    check(cudaDeviceSynchronize(), "sync");
    auto dump = [&](const char* name, const void* ptr, size_t bytes) {
        std::string fn = std::string(out_prefix) + "." + name;
        std::vector<char> buf(bytes);
        check(cudaMemcpy(buf.data(), ptr, bytes, cudaMemcpyDefault), "copy");
        FILE* o = fopen(fn.c_str(), "wb");
        fwrite(buf.data(), 1, bytes, o);
        fclose(o);
    };
    dump("count", b.nn, (size_t)n * 4);
    dump("hash", h, (size_t)n * 8);
    printf("{\"hashed\": %u, \"max_count\": %u}\n", n, mx);
    return 0;
    }

int run_dump(const Kernels& K, const char* in_path, unsigned int n, float3 slo, float3 shi, float rc, float3 box,
             const char* out_prefix, bool exact_only, float sphere_r)
    {
    std::vector<float3> hp(n);
    FILE* f = fopen(in_path, "rb");
    if (!f || fread(hp.data(), 12, n, f) != n) { fprintf(stderr, "cannot read %s\n", in_path); return 5; }
    fclose(f);
    float3* P;
    check(cudaMalloc(&P, (size_t)n * 12), "alloc");
    check(cudaMemcpy(P, hp.data(), (size_t)n * 12, cudaMemcpyHostToDevice), "copy");
    RefTree T;
    T.allocate(n);
    unsigned int list_stride = 0, stock_stride = 0;
    unsigned int *list_s = nullptr, *c_list_s = nullptr;
    T.build(K, P, slo, shi, 32, 0, sphere_r);
    LBVHCompressedData c = T.compress(K, 32, 0);
    std::vector<float3> himg;
    images27(box, himg);
    float3* img;
    check(cudaMalloc(&img, 27 * 12), "alloc");
    check(cudaMemcpy(img, himg.data(), 27 * 12, cudaMemcpyHostToDevice), "copy");
    float4* sph;
    unsigned int *c_stock, *c_exact, *c_list, *list;
    check(cudaMalloc(&sph, (size_t)n * 16), "alloc");
    check(cudaMalloc(&c_list, (size_t)n * 4), "alloc");
    check(cudaMalloc(&c_stock, (size_t)n * 4), "alloc");
    check(cudaMalloc(&c_exact, (size_t)n * 4), "alloc");
    // queries: the points in input order
    std::vector<float4> hs(n);
    for (unsigned int i = 0; i < n; ++i) hs[i] = make_float4(hp[i].x, hp[i].y, hp[i].z, rc);
    check(cudaMemcpy(sph, hs.data(), (size_t)n * 16, cudaMemcpyHostToDevice), "copy");
    ImageListOp im{img, 27};
    if (!exact_only)
        {
        SphereQueryOp q{sph, n};
        CountNeighborsOp out{c_stock};
        void* a[] = {&out, &c, &q, &im};
        launch(K.count_stock, n, 32, 0, a);
        // the stock query's neighbor list (a superset of the exact one), stride its largest count
        check(cudaDeviceSynchronize(), "sync");
        std::vector<unsigned int> hs_c(n);
        check(cudaMemcpy(hs_c.data(), c_stock, (size_t)n * 4, cudaMemcpyDeviceToHost), "copy");
        unsigned int ms = 1;
        for (unsigned int v : hs_c) ms = std::max(ms, v);
        check(cudaMalloc(&list_s, (size_t)n * ms * 4), "alloc");
        check(cudaMalloc(&c_list_s, (size_t)n * 4), "alloc");
        check(cudaMemset(list_s, 0xff, (size_t)n * ms * 4), "memset");
        NeighborListOp lout{list_s, c_list_s, ms};
        void* b[] = {&lout, &c, &q, &im};
        launch(K.list_stock, n, 32, 0, b);
        stock_stride = ms;
        }
        {
        float cm = std::max(std::max(std::fabs(slo.x), std::fabs(shi.x)), std::max(box.x, std::max(box.y, box.z)));
        RefExactQueryOp q{sph, n, P, box, exact_pad(rc, 2 * cm)};
        CountNeighborsOp out{c_exact};
        void* a[] = {&out, &c, &q, &im};
        launch(K.count_exact, n, 32, 0, a);
        check(cudaDeviceSynchronize(), "sync");
        // the exact neighbor list with the stride of the largest count
        std::vector<unsigned int> hc(n);
        check(cudaMemcpy(hc.data(), c_exact, (size_t)n * 4, cudaMemcpyDeviceToHost), "copy");
        unsigned int mx = 1;
        for (unsigned int v : hc) mx = std::max(mx, v);
        check(cudaMalloc(&list, (size_t)n * mx * 4), "alloc");
        check(cudaMemset(list, 0xff, (size_t)n * mx * 4), "memset");
        NeighborListOp lout{list, c_list, mx};
        void* b[] = {&lout, &c, &q, &im};
        launch(K.list_exact, n, 32, 0, b);
        list_stride = mx;
        }
    check(cudaDeviceSynchronize(), "sync");
    auto dump = [&](const char* name, const void* ptr, size_t bytes) {
        std::string path = std::string(out_prefix) + "." + name;
        std::vector<char> h(bytes);
        check(cudaMemcpy(h.data(), ptr, bytes, cudaMemcpyDefault), "copy");
        FILE* o = fopen(path.c_str(), "wb");
        fwrite(h.data(), 1, bytes, o);
        fclose(o);
    };
    const size_t nodes = 2 * (size_t)n - 1;
    dump("codes", T.codes[T.sel_codes], (size_t)n * 4);
    dump("primitive", T.idx[T.sel_idx], (size_t)n * 4);
    dump("parent", T.parent, nodes * 4);
    if (n > 1)
        {
        dump("left", T.left, (size_t)(n - 1) * 4);
        dump("right", T.right, (size_t)(n - 1) * 4);
        }
    dump("lo", T.lo, nodes * 12);
    dump("hi", T.hi, nodes * 12);
    dump("data", T.data, nodes * 16);
    if (!exact_only) dump("count_stock", c_stock, (size_t)n * 4);
    dump("count_exact", c_exact, (size_t)n * 4);
    dump("count_list", c_list, (size_t)n * 4);
    dump("list_exact", list, (size_t)n * list_stride * 4);
    if (!exact_only) dump("list_stock", list_s, (size_t)n * stock_stride * 4);
    printf("{\"dumped\": %u, \"list_stride\": %u}\n", n, list_stride);
    return 0;
    }
} // namespace

int main(int argc, char** argv)
    {
    if (argc < 2) { fprintf(stderr, "usage: ref_driver bench|dump ...\n"); return 1; }
    check(cudaFree(0), "init");
    std::string cubin = std::string(argv[0]);
    cubin = cubin.substr(0, cubin.find_last_of('/') + 1) + "ref_kernels.cubin";
    const Kernels K = load_kernels(cubin.c_str());
    const std::string mode = argv[1];
    if (mode == "bench" && argc >= 6)
        return run_bench(K, (unsigned int)atol(argv[2]), atoi(argv[3]), atoi(argv[4]), (float)atof(argv[5]));
    if (mode == "frames" && argc >= 9)
        return run_frames(K, argv[2], (unsigned int)atol(argv[3]), atoi(argv[4]), (float)atof(argv[5]),
                          (float)atof(argv[6]), atoi(argv[7]), atoi(argv[8]));
    if (mode == "poly" && argc >= 10)
        return run_poly(K, argv[2], (unsigned int)atol(argv[3]), argv[4], (unsigned int)atol(argv[5]), atoi(argv[6]),
                        (float)atof(argv[7]), atoi(argv[8]), atoi(argv[9]));
    if (mode == "frames64" && argc >= 9)
        return run_frames64(K, argv[2], (unsigned int)atol(argv[3]), atoi(argv[4]), atof(argv[5]), (float)atof(argv[6]),
                            atoi(argv[7]), atoi(argv[8]));
    if (mode == "hash" && argc >= 7)
        return run_hash(K, argv[2], (unsigned int)atol(argv[3]), (float)atof(argv[4]), (float)atof(argv[5]), argv[6]);
    if (mode == "dump" && argc >= 15)
        return run_dump(K, argv[2], (unsigned int)atol(argv[3]),
                        make_float3((float)atof(argv[4]), (float)atof(argv[5]), (float)atof(argv[6])),
                        make_float3((float)atof(argv[7]), (float)atof(argv[8]), (float)atof(argv[9])),
                        (float)atof(argv[10]),
                        make_float3((float)atof(argv[11]), (float)atof(argv[12]), (float)atof(argv[13])), argv[14],
                        argc >= 16 && std::string(argv[15]) == "exact_only",
                        (argc >= 17 && std::string(argv[15]) == "sphere") ? (float)atof(argv[16]) : -1.f);
    fprintf(stderr, "bad arguments\n");
    return 1;
    }
