// frame_list.cpp -- neighbor list of one whole frame on the host cores: the CPU baseline of the
// benchmark.  TEST AND MEASUREMENT INFRASTRUCTURE ONLY (bench.py's cpu_baseline leg and its
// reference arm, and the oracle tests); the product never loads it.
//
// The reference has no CPU path (its only implementation is CUDA), so this is a port of its
// two-pass list to the host: the same exact FP32 minimum-image predicate as the library's
// ExactSphereQueryOp (the reference's validation test, test/lbvh_test.cu:469-482: d = pj - pi,
// wrapped once by +-L when |d| >= L/2, accept ((dx*dx + dy*dy) + dz*dz) <= rc*rc, no
// contraction), and the reference's two-pass pattern (a count pass, the counts read back, a list
// pass; benchmark/lbvh_benchmark.cc:205-237 and include/neighbor/OutputOps.h:28-176) -- but over a
// cell grid (cell >= rc + pad, 27 stencil cells) instead of a tree, which is the standard CPU
// method.  Every stage runs on all host threads (OpenMP):
//   grid    cell of every point (atomic counts), exclusive scan, scatter, points of a cell by id
//   count   per point, the candidates of its 27 cells (gathered once per cell) against the
//           predicate
//   scan    exclusive scan of the counts into 64-bit CSR offsets
//   fill    the same loops writing the neighbor ids (original indices) into the CSR rows
// Rows are in grid order (cell by cell, points of a cell by index): the host counterpart of the
// library's rows by sorted position.
//
// Build: g++ -O3 -std=c++17 -fPIC -fopenmp -ffp-contract=off -fno-trapping-math (no -ffast-math:
// the predicate's operations stay in order and round to nearest; -fno-trapping-math only lets the
// compiler evaluate both arms of the wrap's select, so that the predicate loops vectorise).  Host
// code only; no target-specific flags.

#include "oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

inline int cell_of(float p, float lo, float inv_w, int n) {
    int c = (int)std::floor((p - lo) * inv_w);
    return c < 0 ? 0 : (c >= n ? n - 1 : c);
}

// One dimension of the 27-cell stencil: unique cells (n < 3 would repeat a cell).
inline int stencil1(int c, int n, int* out) {
    if (n == 1) { out[0] = 0; return 1; }
    if (n == 2) { out[0] = 0; out[1] = 1; return 2; }
    out[0] = (c + n - 1) % n;
    out[1] = c;
    out[2] = (c + 1) % n;
    return 3;
}

inline float wrap(float d, float h, float L) {
    return d >= h ? d - L : (d < -h ? d + L : d);
}

struct Grid {
    int n[3] = {1, 1, 1};
    float inv_w[3] = {1.f, 1.f, 1.f};
    std::vector<uint32_t> start;            // cells + 1
    std::vector<float> x, y, z;             // points in cell order
    std::vector<uint32_t> id;               // original index of each
};

double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

void build_grid(Grid& g, const float* pts, uint32_t N, const float lo[3], const float L[3], float width) {
    for (int d = 0; d < 3; ++d) {
        g.n[d] = std::max(1, (int)std::floor(L[d] / width));
        g.inv_w[d] = (float)g.n[d] / L[d];
    }
    const size_t nc = (size_t)g.n[0] * g.n[1] * g.n[2];
    g.start.assign(nc + 1, 0u);
    std::vector<uint32_t> cell(N);
    std::vector<uint32_t> counts(nc, 0u);
    uint32_t* cnt = counts.data();
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)N; ++i) {
        const int cx = cell_of(pts[3 * i], lo[0], g.inv_w[0], g.n[0]);
        const int cy = cell_of(pts[3 * i + 1], lo[1], g.inv_w[1], g.n[1]);
        const int cz = cell_of(pts[3 * i + 2], lo[2], g.inv_w[2], g.n[2]);
        const uint32_t c = (uint32_t)(((size_t)cx * g.n[1] + cy) * g.n[2] + cz);
        cell[i] = c;
        __atomic_fetch_add(cnt + c, 1u, __ATOMIC_RELAXED);
    }
    // exclusive scan of the cell counts, in chunks (one per thread) then their offsets
    int T = 1;
#ifdef _OPENMP
    T = omp_get_max_threads();
#endif
    std::vector<uint64_t> part(T + 1, 0);
#pragma omp parallel num_threads(T)
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        const size_t a = nc * t / T, b = nc * (t + 1) / T;
        uint64_t s = 0;
        for (size_t c = a; c < b; ++c) s += cnt[c];
        part[t + 1] = s;
#pragma omp barrier
#pragma omp single
        for (int k = 0; k < T; ++k) part[k + 1] += part[k];
        uint32_t run = (uint32_t)part[t];
        for (size_t c = a; c < b; ++c) {
            g.start[c] = run;
            run += cnt[c];
        }
    }
    g.start[nc] = N;
    std::vector<uint32_t> cursor(g.start.begin(), g.start.end() - 1);
    g.x.resize(N);
    g.y.resize(N);
    g.z.resize(N);
    g.id.resize(N);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)N; ++i) {
        const uint32_t k = __atomic_fetch_add(cursor.data() + cell[i], 1u, __ATOMIC_RELAXED);
        g.id[k] = (uint32_t)i;
    }
    // points of a cell in index order (the scatter's order depends on the threads)
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t c = 0; c < (int64_t)nc; ++c) {
        uint32_t* b = g.id.data() + g.start[c];
        std::sort(b, g.id.data() + g.start[c + 1]);
        for (uint32_t k = g.start[c]; k < g.start[c + 1]; ++k) {
            const uint32_t i = g.id[k];
            g.x[k] = pts[3 * i];
            g.y[k] = pts[3 * i + 1];
            g.z[k] = pts[3 * i + 2];
        }
    }
}

// The candidates of a cell's 27 stencil cells, gathered into contiguous arrays.
struct Candidates {
    std::vector<float> x, y, z;
    std::vector<uint32_t> id;
    std::vector<uint8_t> hit;
    uint32_t n = 0;
    void gather(const Grid& g, int cx, int cy, int cz) {
        int s0[3], s1[3], s2[3];
        const int n0 = stencil1(cx, g.n[0], s0), n1 = stencil1(cy, g.n[1], s1), n2 = stencil1(cz, g.n[2], s2);
        n = 0;
        for (int a = 0; a < n0; ++a)
            for (int b = 0; b < n1; ++b)
                for (int c = 0; c < n2; ++c) {
                    const size_t cell = ((size_t)s0[a] * g.n[1] + s1[b]) * g.n[2] + s2[c];
                    const uint32_t k0 = g.start[cell], k1 = g.start[cell + 1];
                    if (n + (k1 - k0) > x.size()) {
                        const size_t m = std::max<size_t>(2 * x.size(), n + (k1 - k0) + 64);
                        x.resize(m);
                        y.resize(m);
                        z.resize(m);
                        id.resize(m);
                        hit.resize(m);
                    }
                    for (uint32_t k = k0; k < k1; ++k, ++n) {
                        x[n] = g.x[k];
                        y[n] = g.y[k];
                        z[n] = g.z[k];
                        id[n] = g.id[k];
                    }
                }
    }
};

// One pass over all cells: FILL false counts into counts[slot], true writes the rows.
template <bool FILL>
void pass(const Grid& g, float rc2, const float L[3], uint32_t* counts, const uint64_t* offsets, uint32_t* list) {
    const float h[3] = {0.5f * L[0], 0.5f * L[1], 0.5f * L[2]};
    const int64_t nc = (int64_t)g.n[0] * g.n[1] * g.n[2];
#pragma omp parallel
    {
        Candidates cand;
#pragma omp for schedule(dynamic, 256)
        for (int64_t c = 0; c < nc; ++c) {
            const uint32_t k0 = g.start[c], k1 = g.start[c + 1];
            if (k0 == k1) continue;
            const int cz = (int)(c % g.n[2]);
            const int cy = (int)((c / g.n[2]) % g.n[1]);
            const int cx = (int)(c / ((int64_t)g.n[2] * g.n[1]));
            cand.gather(g, cx, cy, cz);
            const float* X = cand.x.data();
            const float* Y = cand.y.data();
            const float* Z = cand.z.data();
            const uint32_t m = cand.n;
            for (uint32_t k = k0; k < k1; ++k) {
                const float px = g.x[k], py = g.y[k], pz = g.z[k];
                if (!FILL) {
                    uint32_t cnt = 0;
                    for (uint32_t j = 0; j < m; ++j) {
                        const float dx = wrap(X[j] - px, h[0], L[0]);
                        const float dy = wrap(Y[j] - py, h[1], L[1]);
                        const float dz = wrap(Z[j] - pz, h[2], L[2]);
                        cnt += ((dx * dx + dy * dy) + dz * dz) <= rc2 ? 1u : 0u;
                    }
                    counts[k] = cnt;
                } else {
                    // the predicate over all candidates (vectorised), then the hits in order
                    uint8_t* hit = cand.hit.data();
                    for (uint32_t j = 0; j < m; ++j) {
                        const float dx = wrap(X[j] - px, h[0], L[0]);
                        const float dy = wrap(Y[j] - py, h[1], L[1]);
                        const float dz = wrap(Z[j] - pz, h[2], L[2]);
                        hit[j] = ((dx * dx + dy * dy) + dz * dz) <= rc2 ? 1u : 0u;
                    }
                    uint32_t* out = list + offsets[k];
                    uint32_t w = 0;
                    for (uint32_t j = 0; j < m; ++j)
                        if (hit[j]) out[w++] = cand.id[j];
                }
            }
        }
    }
}

}  // namespace

extern "C" {

int orc_frame_list(const float* pts, uint32_t N, const float lo[3], const float L[3], float rc, int nthreads,
                   uint32_t* counts, uint64_t* offsets, uint32_t* list, uint64_t list_cap, uint32_t* order,
                   uint64_t* total, double* seconds) {
    int used = 1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
    used = omp_get_max_threads();
#endif
    const double t0 = now();
    Grid g;
    const float cmax = std::fabs(lo[0]) + std::max(L[0], std::max(L[1], L[2]));
    build_grid(g, pts, N, lo, L, rc + orc_exact_pad(rc, cmax));
    const double t1 = now();
    const float rc2 = rc * rc;
    pass<false>(g, rc2, L, counts, nullptr, nullptr);
    const double t2 = now();
    // exclusive scan of the counts (chunks per thread, then their offsets)
    int T = used;
    std::vector<uint64_t> part(T + 1, 0);
#pragma omp parallel num_threads(T)
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        const size_t a = (size_t)N * t / T, b = (size_t)N * (t + 1) / T;
        uint64_t s = 0;
        for (size_t i = a; i < b; ++i) s += counts[i];
        part[t + 1] = s;
#pragma omp barrier
#pragma omp single
        for (int k = 0; k < T; ++k) part[k + 1] += part[k];
        uint64_t run = part[t];
        for (size_t i = a; i < b; ++i) {
            offsets[i] = run;
            run += counts[i];
        }
    }
    offsets[N] = part[T];
    *total = part[T];
    const double t3 = now();
    if (part[T] > list_cap) return -1;
    pass<true>(g, rc2, L, nullptr, offsets, list);
    const double t4 = now();
    if (order) std::copy(g.id.begin(), g.id.end(), order);
    if (seconds) {
        seconds[0] = t1 - t0;
        seconds[1] = t2 - t1;
        seconds[2] = t3 - t2;
        seconds[3] = t4 - t3;
    }
    return used;
}

// Trajectory frames on the host: uniform points in [lo, lo + L) and i.i.d. Gaussian moves with
// wrap, from a counter-based generator (splitmix64 of seed and index; Box-Muller), so that a frame
// does not depend on the number of threads.
static inline uint64_t mix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
static inline double u01(uint64_t h) { return ((h >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

void orc_uniform_points(float* out, uint32_t N, const float lo[3], const float L[3], uint64_t seed) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)N; ++i)
        for (int d = 0; d < 3; ++d) {
            float v = (float)(lo[d] + u01(mix64(seed * 0x632be59bd9b4e019ull + 3 * (uint64_t)i + d)) * L[d]);
            if (v >= lo[d] + L[d]) v = lo[d];
            out[3 * i + d] = v;
        }
}

void orc_gaussian_move(const float* in, float* out, uint32_t N, const float lo[3], const float L[3], float sigma,
                       uint64_t seed) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)N; ++i)
        for (int d = 0; d < 3; ++d) {
            const uint64_t h = mix64(seed * 0x632be59bd9b4e019ull + 3 * (uint64_t)i + d);
            const double g = std::sqrt(-2.0 * std::log(u01(h))) * std::cos(6.283185307179586 * u01(mix64(h)));
            float v = in[3 * i + d] + (float)(sigma * g);
            v -= L[d] * std::floor((v - lo[d]) / L[d]);
            if (v >= lo[d] + L[d]) v -= L[d];
            if (v < lo[d]) v = lo[d];
            out[3 * i + d] = v;
        }
}

}  // extern "C"
