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
//   ref_driver bench N steps warmup rc          time the plain two-pass step on uniform frames
//   ref_driver dump  in.f32 N lo3 hi3 rc L3 out  write the reference's outputs for given points
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
struct LBVHData { int* parent; int* left; int* right; unsigned int* primitive; float3* lo; float3* hi; int root; };
struct LBVHCompressedData { int root; int4* data; float3* lo; float3* hi; float3* bins; };
struct CountNeighborsOp { unsigned int* nneigh; };
struct NeighborListOp { unsigned int* neigh_list; unsigned int* nneigh; unsigned int max_neigh; };
struct ImageListOp { const float3* images; unsigned int N; };
struct SphereQueryOp { const float4* spheres; unsigned int N; };
struct NullTransformOp {};
struct RefExactQueryOp { const float4* spheres; unsigned int N; const float3* points; float3 box; float pad; };

static_assert(sizeof(PointInsertOp) == 16 && offsetof(PointInsertOp, N) == 8, "layout");
static_assert(sizeof(LBVHData) == 56 && offsetof(LBVHData, root) == 48, "layout");
static_assert(sizeof(LBVHCompressedData) == 40 && offsetof(LBVHCompressedData, data) == 8, "layout");
static_assert(sizeof(CountNeighborsOp) == 8, "layout");
static_assert(sizeof(NeighborListOp) == 24 && offsetof(NeighborListOp, max_neigh) == 16, "layout");
static_assert(sizeof(ImageListOp) == 16 && offsetof(ImageListOp, N) == 8, "layout");
static_assert(sizeof(SphereQueryOp) == 16, "layout");
static_assert(sizeof(NullTransformOp) == 1, "layout");
static_assert(sizeof(RefExactQueryOp) == 40 && offsetof(RefExactQueryOp, points) == 16
              && offsetof(RefExactQueryOp, box) == 24 && offsetof(RefExactQueryOp, pad) == 36, "layout");

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
    CUfunction count_stock = nullptr, count_exact = nullptr, list_exact = nullptr, list_stock = nullptr;
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
        if (has("lbvh_gen_codes")) k.gen_codes = f;
        else if (has("lbvh_gen_tree")) k.gen_tree = f;
        else if (has("lbvh_bubble_aabbs")) k.bubble = f;
        else if (has("lbvh_one_primitive")) k.one = f;
        else if (has("lbvh_compress_ropes")) k.compress = f;
        else if (has("lbvh_traverse_ropes") && has("CountNeighborsOp") && has("SphereQueryOp")) k.count_stock = f;
        else if (has("lbvh_traverse_ropes") && has("CountNeighborsOp") && has("RefExactQueryOp")) k.count_exact = f;
        else if (has("lbvh_traverse_ropes") && has("NeighborListOp") && has("RefExactQueryOp")) k.list_exact = f;
        else if (has("lbvh_traverse_ropes") && has("NeighborListOp") && has("SphereQueryOp")) k.list_stock = f;
        }
    if (!k.gen_codes || !k.gen_tree || !k.bubble || !k.one || !k.compress || !k.count_stock || !k.count_exact || !k.list_exact
        || !k.list_stock)
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

    // LBVH::build (include/neighbor/LBVH.h:242-318)
    void build(const Kernels& K, const float3* pts, float3 slo, float3 shi, unsigned int bs, cudaStream_t s)
        {
        PointInsertOp ins{pts, N};
        sel_codes = sel_idx = 0;
        if (N == 1)
            {
            LBVHData t = tree_data();
            void* a[] = {&t, &ins};
            checkd(cuLaunchKernel(K.one, 1, 1, 1, 1, 1, 1, 0, (CUstream)s, a, nullptr), "launch");
            return;
            }
        unsigned int n = N;
            {
            void* a[] = {&codes[0], &idx[0], &ins, &slo, &shi, &n};
            launch(K.gen_codes, n, bs, s, a);
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
            void* a[] = {&t, &ins, &locks, &n};
            launch(K.bubble, n, bs, s, a);
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
// benchmark/lbvh_benchmark.cc:177-184).
__global__ void k_spheres(const float3* p, const unsigned int* prim, float4* sph, unsigned int n, float rc)
    {
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 x = p[prim[i]];
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

int run_bench(const Kernels& K, unsigned int n, int steps, int warmup, float rc)
    {
    const float L = std::cbrt(n / 0.85f);
    const float3 box = make_float3(L, L, L);
    cudaStream_t s;
    check(cudaStreamCreate(&s), "stream");
    std::vector<float3*> frames(steps + warmup);
    float3* base;
    check(cudaMalloc(&base, (size_t)n * 12), "alloc");
    k_uniform<<<(n + 255) / 256, 256, 0, s>>>(base, n, L, 1234u);
    const float3* prev = base;
    for (size_t f = 0; f < frames.size(); ++f)
        {
        check(cudaMalloc(&frames[f], (size_t)n * 12), "alloc");
        k_move<<<(n + 255) / 256, 256, 0, s>>>(prev, frames[f], n, L, 0.05f, 77u + (unsigned)f);
        prev = frames[f];
        }
    std::vector<float3> himg;
    images27(box, himg);
    float3* img;
    check(cudaMalloc(&img, 27 * 12), "alloc");
    check(cudaMemcpy(img, himg.data(), 27 * 12, cudaMemcpyHostToDevice), "copy");
    RefTree T;
    T.allocate(n);
    float4* sph;
    unsigned int *nn, *list, *dmax;
    check(cudaMalloc(&sph, (size_t)n * 16), "alloc");
    check(cudaMalloc(&nn, (size_t)n * 4), "alloc");
    check(cudaMalloc(&dmax, 4), "alloc");
    const unsigned int cap = 64;
    check(cudaMalloc(&list, (size_t)n * cap * 4), "alloc");
    void* rtmp = nullptr;
    size_t rtmp_bytes = 0;
    check(cub::DeviceReduce::Max(nullptr, rtmp_bytes, nn, dmax, (int)n), "reduce size");
    check(cudaMalloc(&rtmp, rtmp_bytes), "alloc");
    const float pad = exact_pad(rc, 2 * L);
    check(cudaStreamSynchronize(s), "sync");

    printf("{\"impl\": \"reference-cuda\", \"n\": %u, \"rc\": %g, \"steps\": %d, \"results\": [", n, rc, steps);
    const unsigned int blocks[] = {32, 64, 128, 256, 512};
    bool first = true;
    for (unsigned int bs : blocks)
        {
        cudaEvent_t ev[6];
        for (auto& e : ev) check(cudaEventCreate(&e), "event");
        double t_build = 0, t_setup = 0, t_count = 0, t_fill = 0, t_total = 0, pairs = 0;
        for (int it = 0; it < warmup + steps; ++it)
            {
            const bool timed = it >= warmup;
            const float3* P = frames[it];
            check(cudaEventRecord(ev[0], s), "rec");
            T.build(K, P, make_float3(0, 0, 0), box, bs, s);
            k_spheres<<<(n + 255) / 256, 256, 0, s>>>(P, T.idx[T.sel_idx], sph, n, rc);
            check(cudaEventRecord(ev[1], s), "rec");
            LBVHCompressedData c = T.compress(K, bs, s);
            check(cudaEventRecord(ev[2], s), "rec");
            RefExactQueryOp q{sph, n, P, box, pad};
            // the exact op refines against the points indexed by primitive id: the input order
            ImageListOp im{img, 27};
                {
                CountNeighborsOp out{nn};
                void* a[] = {&out, &c, &q, &im};
                launch(K.count_exact, n, bs, s, a);
                }
            check(cudaEventRecord(ev[3], s), "rec");
            check(cub::DeviceReduce::Max(rtmp, rtmp_bytes, nn, dmax, (int)n, s), "reduce");
            unsigned int mx = 0;
            check(cudaMemcpyAsync(&mx, dmax, 4, cudaMemcpyDeviceToHost, s), "copy");
            check(cudaStreamSynchronize(s), "sync");
            if (mx > cap) { fprintf(stderr, "max neighbors %u exceeds %u\n", mx, cap); return 4; }
            check(cudaEventRecord(ev[4], s), "rec");
                {
                NeighborListOp out{list, nn, mx};
                void* a[] = {&out, &c, &q, &im};
                launch(K.list_exact, n, bs, s, a);
                }
            check(cudaEventRecord(ev[5], s), "rec");
            check(cudaStreamSynchronize(s), "sync");
            if (timed)
                {
                float ms;
                cudaEventElapsedTime(&ms, ev[0], ev[1]); t_build += ms;
                cudaEventElapsedTime(&ms, ev[1], ev[2]); t_setup += ms;
                cudaEventElapsedTime(&ms, ev[2], ev[3]); t_count += ms;
                cudaEventElapsedTime(&ms, ev[4], ev[5]); t_fill += ms;
                cudaEventElapsedTime(&ms, ev[0], ev[5]); t_total += ms;
                std::vector<unsigned int> h(n);
                check(cudaMemcpy(h.data(), nn, (size_t)n * 4, cudaMemcpyDeviceToHost), "copy");
                for (unsigned int x : h) pairs += x;
                }
            }
        printf("%s{\"block\": %u, \"build_ms\": %.4f, \"spheres_and_build_ms\": %.4f, \"setup_ms\": %.4f, \"count_ms\": %.4f, "
               "\"fill_ms\": %.4f, \"step_ms\": %.4f, \"pairs_per_step\": %.1f}",
               first ? "" : ", ", bs, t_build / steps, t_build / steps, t_setup / steps, t_count / steps, t_fill / steps,
               t_total / steps, pairs / steps);
        first = false;
        for (auto& e : ev) cudaEventDestroy(e);
        }
    printf("]}\n");
    return 0;
    }

int run_dump(const Kernels& K, const char* in_path, unsigned int n, float3 slo, float3 shi, float rc, float3 box,
             const char* out_prefix, bool exact_only)
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
    T.build(K, P, slo, shi, 32, 0);
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
    if (mode == "dump" && argc >= 15)
        return run_dump(K, argv[2], (unsigned int)atol(argv[3]),
                        make_float3((float)atof(argv[4]), (float)atof(argv[5]), (float)atof(argv[6])),
                        make_float3((float)atof(argv[7]), (float)atof(argv[8]), (float)atof(argv[9])),
                        (float)atof(argv[10]),
                        make_float3((float)atof(argv[11]), (float)atof(argv[12]), (float)atof(argv[13])), argv[14],
                        argc >= 16 && std::string(argv[15]) == "exact_only");
    fprintf(stderr, "bad arguments\n");
    return 1;
    }
