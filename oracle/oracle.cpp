// oracle.cpp -- CPU restatement of the neighbor LBVH path.  TEST INFRASTRUCTURE ONLY:
// it is the checker for the CUDA product in neighbor_gb300/, loaded by tests/, by
// __graft_entry__.smoke() and by the CPU-baseline leg of bench.py, never by the product.
//
// Build: g++ -O2 -std=c++17 -fPIC -shared -fopenmp -frounding-math -ffp-contract=off
// (-ffp-contract=off matters on aarch64, where gcc would otherwise fuse a*b+c).
//
// Every function cites the reference file:line (mphowardlab/neighbor v0.3.2) it restates.

#include "oracle.h"

#include <algorithm>
#include <cfenv>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif


namespace {

// ---------------------------------------------------------------------------------------
// Directed rounding.  The reference wraps CUDA's __f*_rd/_ru intrinsics, which are the
// IEEE-754 operations with a static rounding mode (include/neighbor/ApproximateMath.h:55-345).
// On the host the same IEEE result comes from switching the dynamic rounding mode.
// ---------------------------------------------------------------------------------------
struct RoundGuard {
    int old;
    explicit RoundGuard(int mode) : old(fegetround()) { fesetround(mode); }
    ~RoundGuard() { fesetround(old); }
};

inline float add_mode(float a, float b, int mode) {
    RoundGuard g(mode);
    volatile float va = a, vb = b;
    volatile float r = va + vb;
    return r;
}
inline float sub_mode(float a, float b, int mode) {
    RoundGuard g(mode);
    volatile float va = a, vb = b;
    volatile float r = va - vb;
    return r;
}
inline float mul_mode(float a, float b, int mode) {
    RoundGuard g(mode);
    volatile float va = a, vb = b;
    volatile float r = va * vb;
    return r;
}
inline float div_mode(float a, float b, int mode) {
    RoundGuard g(mode);
    volatile float va = a, vb = b;
    volatile float r = va / vb;
    return r;
}
inline float fma_mode(float a, float b, float c, int mode) {
    RoundGuard g(mode);
    volatile float va = a, vb = b, vc = c;
    volatile float r = std::fmaf(va, vb, vc);
    return r;
}
inline float d2f_mode(double a, int mode) {
    RoundGuard g(mode);
    volatile double va = a;
    volatile float r = (float)va;
    return r;
}

// FP32 round-to-nearest helpers that the compiler may not contract or reorder.
inline float rn_add(float a, float b) { volatile float r = a + b; return r; }
inline float rn_sub(float a, float b) { volatile float r = a - b; return r; }
inline float rn_mul(float a, float b) { volatile float r = a * b; return r; }
inline float rn_div(float a, float b) { volatile float r = a / b; return r; }

struct f3 { float x, y, z; };
inline f3 ld3(const float* p, size_t i) { return f3{p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }
inline void st3(float* p, size_t i, f3 v) { p[3 * i] = v.x; p[3 * i + 1] = v.y; p[3 * i + 2] = v.z; }

// ---------------------------------------------------------------------------------------
// Insert ops (include/neighbor/InsertOps.h:35-41 point, :75-82 sphere).
// ---------------------------------------------------------------------------------------
inline void insert_box(const float* pts, uint32_t idx, int kind, float r, f3& lo, f3& hi) {
    const f3 p = ld3(pts, idx);
    if (kind == ORC_INSERT_SPHERE) {
        lo = f3{rn_sub(p.x, r), rn_sub(p.y, r), rn_sub(p.z, r)};
        hi = f3{rn_add(p.x, r), rn_add(p.y, r), rn_add(p.z, r)};
    } else {
        lo = p;
        hi = p;
    }
}

// BoundingBox::getCenter (include/neighbor/BoundingVolumes.h:64-72): 0.5f*(lo+hi).
inline f3 box_center(f3 lo, f3 hi) {
    return f3{rn_mul(0.5f, rn_add(lo.x, hi.x)), rn_mul(0.5f, rn_add(lo.y, hi.y)),
              rn_mul(0.5f, rn_add(lo.z, hi.z))};
}

// Spread the low 10 bits of v so that bit b lands at bit 3b
// (same result as expandBits, include/neighbor/kernels/LBVH.cuh:28-35).
inline uint32_t spread3(uint32_t v) {
    uint32_t out = 0;
    for (int b = 0; b < 10; ++b) out |= ((v >> b) & 1u) << (3 * b);
    return out;
}

// fractionToBin (include/neighbor/kernels/LBVH.cuh:105-108): clamp(f*1023, 0, 1023), truncated.
inline uint32_t frac_bin(float f) {
    const float s = rn_mul(f, 1023.f);
    return (uint32_t)std::fmin(std::fmax(s, 0.f), 1023.f);
}

// Karras' delta with the index tie-break (include/neighbor/kernels/LBVH.cuh:73-94).
inline int common_prefix(const uint32_t* codes, uint32_t ci, int64_t i, int64_t j, int64_t N) {
    if (j < 0 || j >= N) return -1;
    const uint32_t cj = codes[j];
    if (ci == cj) {
        const uint32_t x = (uint32_t)i ^ (uint32_t)j;
        return 32 + (x ? __builtin_clz(x) : 32);
    }
    return __builtin_clz(ci ^ cj);
}

inline uint32_t clampu(float v, float lo, float hi) {
    return (uint32_t)std::fmin(std::fmax(v, lo), hi);
}

}  // namespace

extern "C" {

float orc_fadd_rd(float a, float b) { return add_mode(a, b, FE_DOWNWARD); }
float orc_fadd_ru(float a, float b) { return add_mode(a, b, FE_UPWARD); }
float orc_fsub_rd(float a, float b) { return sub_mode(a, b, FE_DOWNWARD); }
float orc_fsub_ru(float a, float b) { return sub_mode(a, b, FE_UPWARD); }
float orc_fmul_rd(float a, float b) { return mul_mode(a, b, FE_DOWNWARD); }
float orc_fmul_ru(float a, float b) { return mul_mode(a, b, FE_UPWARD); }
float orc_fdiv_rd(float a, float b) { return div_mode(a, b, FE_DOWNWARD); }
float orc_fdiv_ru(float a, float b) { return div_mode(a, b, FE_UPWARD); }
float orc_frcp_rd(float a) { return div_mode(1.0f, a, FE_DOWNWARD); }
float orc_frcp_ru(float a) { return div_mode(1.0f, a, FE_UPWARD); }
float orc_fmaf_rd(float a, float b, float c) { return fma_mode(a, b, c, FE_DOWNWARD); }
float orc_fmaf_ru(float a, float b, float c) { return fma_mode(a, b, c, FE_UPWARD); }
float orc_double2float_rd(double a) { return d2f_mode(a, FE_DOWNWARD); }
float orc_double2float_ru(double a) { return d2f_mode(a, FE_UPWARD); }

// lbvh_gen_codes (include/neighbor/kernels/LBVH.cuh:127-157): centre of the insert box,
// fractional coordinate (IEEE division), 10-bit bins, interleave 4X+2Y+Z.
void orc_morton_codes(const float* pts, uint32_t N, int insert_kind, float r,
                      const float scene_lo[3], const float scene_hi[3], uint32_t* codes) {
    const float ex = rn_sub(scene_hi[0], scene_lo[0]);
    const float ey = rn_sub(scene_hi[1], scene_lo[1]);
    const float ez = rn_sub(scene_hi[2], scene_lo[2]);
    for (uint32_t i = 0; i < N; ++i) {
        f3 lo, hi;
        insert_box(pts, i, insert_kind, r, lo, hi);
        const f3 c = box_center(lo, hi);
        const uint32_t bx = frac_bin(rn_div(rn_sub(c.x, scene_lo[0]), ex));
        const uint32_t by = frac_bin(rn_div(rn_sub(c.y, scene_lo[1]), ey));
        const uint32_t bz = frac_bin(rn_div(rn_sub(c.z, scene_lo[2]), ez));
        codes[i] = 4u * spread3(bx) + 2u * spread3(by) + spread3(bz);
    }
}

// LBVH::build (include/neighbor/LBVH.h:242-318).
void orc_build(const float* pts, uint32_t N, int insert_kind, float r,
               const float scene_lo[3], const float scene_hi[3], uint32_t* sorted_codes,
               uint32_t* primitive, int32_t* parent, int32_t* left, int32_t* right, float* lo,
               float* hi) {
    if (N == 0) return;
    if (N == 1) {
        // lbvh_one_primitive (include/neighbor/kernels/LBVH.cuh:340-354); the primitive
        // order is the identity.
        f3 blo, bhi;
        insert_box(pts, 0, insert_kind, r, blo, bhi);
        parent[0] = ORC_SENTINEL;
        st3(lo, 0, blo);
        st3(hi, 0, bhi);
        primitive[0] = 0;
        if (sorted_codes) orc_morton_codes(pts, 1, insert_kind, r, scene_lo, scene_hi, sorted_codes);
        return;
    }
    std::vector<uint32_t> codes(N);
    orc_morton_codes(pts, N, insert_kind, r, scene_lo, scene_hi, codes.data());

    // Stable ascending sort of (code, index) over bits [0,30): the order CUB's
    // DeviceRadixSort::SortPairs produces (include/neighbor/kernels/LBVH.cuh:421-443).
    std::vector<uint32_t> order(N);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(),
                     [&](uint32_t a, uint32_t b) { return codes[a] < codes[b]; });
    std::vector<uint32_t> sc(N);
    for (uint32_t i = 0; i < N; ++i) {
        sc[i] = codes[order[i]];
        primitive[i] = order[i];
    }
    if (sorted_codes) std::memcpy(sorted_codes, sc.data(), N * sizeof(uint32_t));

    // Karras hierarchy (include/neighbor/kernels/LBVH.cuh:169-243, after Karras 2012 Fig. 4).
    const int64_t n = N;
    for (int64_t i = 0; i < n - 1; ++i) {
        const uint32_t ci = sc[i];
        const int fwd = common_prefix(sc.data(), ci, i, i + 1, n);
        const int bwd = common_prefix(sc.data(), ci, i, i - 1, n);
        const int d = (fwd >= bwd) ? 1 : -1;
        const int min_prefix = common_prefix(sc.data(), ci, i, i - d, n);
        int64_t lmax = 2;
        while (common_prefix(sc.data(), ci, i, i + d * lmax, n) > min_prefix) lmax <<= 1;
        int64_t l = 0;
        for (int64_t t = lmax >> 1; t >= 1; t >>= 1)
            if (common_prefix(sc.data(), ci, i, i + (l + t) * d, n) > min_prefix) l += t;
        const int64_t j = i + l * d;
        const int node_prefix = common_prefix(sc.data(), ci, i, j, n);
        int64_t s = 0;
        int64_t t = l;
        do {
            t = (t + 1) >> 1;
            if (s + t < l && common_prefix(sc.data(), ci, i, i + (s + t) * d, n) > node_prefix)
                s += t;
        } while (t > 1);
        const int64_t split = i + s * d + std::min<int64_t>(d, 0);
        const int64_t lc = (std::min(i, j) == split) ? split + (n - 1) : split;
        const int64_t rc = (std::max(i, j) == split + 1) ? split + n : split + 1;
        left[i] = (int32_t)lc;
        right[i] = (int32_t)rc;
        parent[lc] = (int32_t)i;
        parent[rc] = (int32_t)i;
    }
    parent[0] = ORC_SENTINEL;

    // Bottom-up boxes (include/neighbor/kernels/LBVH.cuh:270-327).  min/max are exact, so
    // any child-before-parent order gives the reference's boxes.
    for (uint32_t s = 0; s < N; ++s) {
        f3 blo, bhi;
        insert_box(pts, primitive[s], insert_kind, r, blo, bhi);
        st3(lo, N - 1 + s, blo);
        st3(hi, N - 1 + s, bhi);
    }
    // iterative post-order from the root
    std::vector<int64_t> stack;
    std::vector<uint8_t> expanded(N - 1, 0);
    stack.push_back(0);
    while (!stack.empty()) {
        const int64_t v = stack.back();
        if (!expanded[v]) {
            expanded[v] = 1;
            if (left[v] < (int32_t)(N - 1)) stack.push_back(left[v]);
            if (right[v] < (int32_t)(N - 1)) stack.push_back(right[v]);
            continue;
        }
        stack.pop_back();
        const f3 al = ld3(lo, left[v]), ah = ld3(hi, left[v]);
        const f3 bl = ld3(lo, right[v]), bh = ld3(hi, right[v]);
        st3(lo, v, f3{std::min(al.x, bl.x), std::min(al.y, bl.y), std::min(al.z, bl.z)});
        st3(hi, v, f3{std::max(ah.x, bh.x), std::max(ah.y, bh.y), std::max(ah.z, bh.z)});
    }
}

// lbvh_compress_ropes (include/neighbor/kernels/LBVHTraverser.cuh:45-125).
void orc_compress_ref10(uint32_t N, const int32_t* parent, const int32_t* left,
                        const int32_t* right, const uint32_t* primitive, const float* lo,
                        const float* hi, const uint32_t* map, int32_t* data, float* clo,
                        float* chi, float* bins) {
    if (N == 0) return;
    const uint32_t n_internal = N - 1;
    const uint32_t n_nodes = 2 * N - 1;
    const int root = 0;
    const f3 tlo = ld3(lo, root), thi = ld3(hi, root);
    float L[3] = {orc_fsub_ru(thi.x, tlo.x), orc_fsub_ru(thi.y, tlo.y), orc_fsub_ru(thi.z, tlo.z)};
    for (float& v : L)
        if (v <= 0.f) v = 1.0f;
    const float binv[3] = {orc_fdiv_rd(1023.f, L[0]), orc_fdiv_rd(1023.f, L[1]),
                           orc_fdiv_rd(1023.f, L[2])};
    const float tl[3] = {tlo.x, tlo.y, tlo.z};
    const float th[3] = {thi.x, thi.y, thi.z};
    for (uint32_t idx = 0; idx < n_nodes; ++idx) {
        int rope = ORC_SENTINEL;
        int cur = (int)idx;
        while (cur != root && rope == ORC_SENTINEL) {
            const int p = parent[cur];
            if (left[p] == cur)
                rope = right[p];
            else
                cur = p;
        }
        const float nl[3] = {lo[3 * idx], lo[3 * idx + 1], lo[3 * idx + 2]};
        const float nh[3] = {hi[3 * idx], hi[3 * idx + 1], hi[3 * idx + 2]};
        uint32_t lb[3], hb[3];
        for (int d = 0; d < 3; ++d) {
            lb[d] = (uint32_t)std::floor(orc_fmul_rd(orc_fsub_rd(nl[d], tl[d]), binv[d]));
            hb[d] = (uint32_t)std::floor(orc_fmul_rd(orc_fsub_rd(th[d], nh[d]), binv[d]));
        }
        const uint32_t lo3 = (lb[0] << 20) + (lb[1] << 10) + lb[2];
        const uint32_t hi3 = (hb[0] << 20) + (hb[1] << 10) + hb[2];
        int32_t z;
        if (idx < n_internal) {
            z = left[idx];
        } else {
            uint32_t prim = primitive[idx - n_internal];
            if (map) prim = map[prim];
            z = (int32_t)~prim;
        }
        data[4 * idx + 0] = (int32_t)lo3;
        data[4 * idx + 1] = (int32_t)hi3;
        data[4 * idx + 2] = z;
        data[4 * idx + 3] = rope;
    }
    for (int d = 0; d < 3; ++d) {
        clo[d] = tl[d];
        chi[d] = th[d];
        bins[d] = orc_frcp_rd(binv[d]);
    }
}

int orc_exact_pair(const float* pi, const float* pj, float rc, const float box_L[3]) {
    float d[3];
    for (int k = 0; k < 3; ++k) {
        float dk = rn_sub(pj[k], pi[k]);
        const float Lk = box_L ? box_L[k] : 0.f;
        if (Lk > 0.f) {
            const float h = rn_mul(0.5f, Lk);
            if (dk >= h)
                dk = rn_sub(dk, Lk);
            else if (dk < -h)
                dk = rn_add(dk, Lk);
        }
        d[k] = dk;
    }
    const float d2 = rn_add(rn_add(rn_mul(d[0], d[0]), rn_mul(d[1], d[1])), rn_mul(d[2], d[2]));
    return d2 <= rn_mul(rc, rc);
}

float orc_exact_pad(float rc, float coord_max) {
    // 16 ulps of twice the largest coordinate magnitude, plus a relative margin on rc.
    const float m = std::max(std::fabs(coord_max), 1.0f) * 2.0f + std::fabs(rc);
    int e;
    std::frexp(m, &e);  // m in [2^(e-1), 2^e)
    const float ulp = std::ldexp(1.0f, e - 24);
    return 16.0f * ulp + std::fabs(rc) * 1.0e-6f;
}

// lbvh_traverse_ropes (include/neighbor/kernels/LBVHTraverser.cuh:155-252) with the
// SphereQueryOp / BoundingSphere overlap (include/neighbor/QueryOps.h:32-120,
// include/neighbor/BoundingVolumes.h:119-171) and Count/NeighborList output
// (include/neighbor/OutputOps.h:28-176).
void orc_traverse_ref10(uint32_t N_nodes, const int32_t* data, const float* clo,
                        const float* chi, const float* bins, const float* spheres, uint32_t Q,
                        const float* images, uint32_t n_images, int query_kind,
                        const float* points, const float box_L[3], float pad,
                        uint32_t* nneigh, uint32_t* list, uint32_t max_neigh) {
    (void)N_nodes;
    const float self_img[3] = {0.f, 0.f, 0.f};
    const uint32_t nimg = images ? n_images : 1u;
    const float* img = images ? images : self_img;
    const int nbits = nimg <= 32u ? (int)nimg : 32;
    for (uint32_t q = 0; q < Q; ++q) {
        const float* s = spheres + 4 * q;
        // BoundingSphere(t, R): Rsq = fmul_ru(R, R)
        const float R = (query_kind == ORC_QUERY_EXACT) ? orc_fadd_ru(s[3], pad) : s[3];
        const float Rsq = orc_fmul_ru(R, R);
        auto overlap = [&](const float t[3], const float bl[3], const float bh[3]) {
            float dr[3];
            for (int k = 0; k < 3; ++k)
                dr[k] = orc_fsub_rd(std::fmin(std::fmax(t[k], bl[k]), bh[k]), t[k]);
            const float d2 = orc_fmaf_rd(dr[0], dr[0], orc_fmaf_rd(dr[1], dr[1], orc_fmul_rd(dr[2], dr[2])));
            return d2 <= Rsq;
        };
        uint32_t flags = 0;
        for (int i = 0; i < nbits; ++i) {
            const float t[3] = {rn_add(s[0], img[3 * i]), rn_add(s[1], img[3 * i + 1]),
                                rn_add(s[2], img[3 * i + 2])};
            if (overlap(t, clo, chi)) flags |= 1u << i;
        }
        uint32_t count = 0;
        while (flags) {
            const int bit = __builtin_ctz(flags);
            flags &= ~(1u << bit);
            const float t[3] = {rn_add(s[0], img[3 * bit]), rn_add(s[1], img[3 * bit + 1]),
                                rn_add(s[2], img[3 * bit + 2])};
            int node = 0;
            while (node != ORC_SENTINEL) {
                const uint32_t lo3 = (uint32_t)data[4 * node], hi3 = (uint32_t)data[4 * node + 1];
                const int lft = data[4 * node + 2];
                const uint32_t lb[3] = {(lo3 >> 20) & 0x3ffu, (lo3 >> 10) & 0x3ffu, lo3 & 0x3ffu};
                const uint32_t hb[3] = {(hi3 >> 20) & 0x3ffu, (hi3 >> 10) & 0x3ffu, hi3 & 0x3ffu};
                float bl[3], bh[3];
                for (int k = 0; k < 3; ++k) {
                    bl[k] = orc_fadd_rd(clo[k], orc_fmul_rd((float)lb[k], bins[k]));
                    bh[k] = orc_fsub_ru(chi[k], orc_fmul_rd((float)hb[k], bins[k]));
                }
                node = data[4 * node + 3];
                if (overlap(t, bl, bh)) {
                    if (lft < 0) {
                        const uint32_t prim = (uint32_t)~lft;
                        bool keep = true;
                        if (query_kind == ORC_QUERY_EXACT)
                            keep = orc_exact_pair(s, points + 3 * (size_t)prim, s[3], box_L) != 0;
                        if (keep) {
                            if (list && count < max_neigh) list[(size_t)max_neigh * q + count] = prim;
                            ++count;
                        }
                    } else {
                        node = lft;
                    }
                }
            }
        }
        nneigh[q] = count;
    }
}

void orc_brute_count(const float* qpos, const float* qr, uint32_t Q, const float* pts,
                     uint32_t N, const float box_L[3], uint32_t* nneigh) {
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < (int64_t)Q; ++q) {
        uint32_t c = 0;
        for (uint32_t j = 0; j < N; ++j)
            c += (uint32_t)orc_exact_pair(qpos + 3 * q, pts + 3 * (size_t)j, qr[q], box_L);
        nneigh[q] = c;
    }
}

double orc_pair_distance_minus_rc_f64(const float* pi, const float* pj, float rc,
                                      const float box_L[3]) {
    double d2 = 0.0;
    for (int k = 0; k < 3; ++k) {
        double dk = (double)pj[k] - (double)pi[k];
        const double Lk = box_L ? (double)box_L[k] : 0.0;
        if (Lk > 0.0) dk -= Lk * std::nearbyint(dk / Lk);
        d2 += dk * dk;
    }
    return std::sqrt(d2) - (double)rc;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// OpenMP cell list (the CPU baseline; the reference has no CPU path).
// ---------------------------------------------------------------------------------------
namespace {

struct CellGrid {
    int n[3];
    float inv_w[3];
    std::vector<uint32_t> start;  // n0*n1*n2 + 1
    std::vector<float> x, y, z;   // points grouped by cell
    std::vector<uint32_t> id;     // original index
};

inline int cell_coord(float p, float lo, float inv_w, int n) {
    int c = (int)std::floor(rn_mul(rn_sub(p, lo), inv_w));
    if (c < 0) c = 0;
    if (c >= n) c = n - 1;
    return c;
}

void build_grid(CellGrid& g, const float* pts, uint32_t N, const float lo[3], const float L[3],
                float width) {
    for (int d = 0; d < 3; ++d) {
        g.n[d] = std::max(1, (int)std::floor(L[d] / width));
        g.inv_w[d] = (float)g.n[d] / L[d];
    }
    const size_t nc = (size_t)g.n[0] * g.n[1] * g.n[2];
    std::vector<uint32_t> cell(N);
    std::vector<uint32_t> cnt(nc + 1, 0);
    for (uint32_t i = 0; i < N; ++i) {
        const int cx = cell_coord(pts[3 * i], lo[0], g.inv_w[0], g.n[0]);
        const int cy = cell_coord(pts[3 * i + 1], lo[1], g.inv_w[1], g.n[1]);
        const int cz = cell_coord(pts[3 * i + 2], lo[2], g.inv_w[2], g.n[2]);
        cell[i] = (uint32_t)(((size_t)cx * g.n[1] + cy) * g.n[2] + cz);
        cnt[cell[i] + 1]++;
    }
    for (size_t c = 0; c < nc; ++c) cnt[c + 1] += cnt[c];
    g.start = cnt;
    g.x.resize(N);
    g.y.resize(N);
    g.z.resize(N);
    g.id.resize(N);
    std::vector<uint32_t> fill(cnt.begin(), cnt.end() - 1);
    for (uint32_t i = 0; i < N; ++i) {
        const uint32_t k = fill[cell[i]]++;
        g.x[k] = pts[3 * i];
        g.y[k] = pts[3 * i + 1];
        g.z[k] = pts[3 * i + 2];
        g.id[k] = i;
    }
}

// Unique neighbour offsets along one dimension (avoids visiting a cell twice when n < 3).
inline int stencil(int c, int n, int* out) {
    if (n == 1) { out[0] = 0; return 1; }
    if (n == 2) { out[0] = 0; out[1] = 1; return 2; }
    out[0] = (c + n - 1) % n;
    out[1] = c;
    out[2] = (c + 1) % n;
    return 3;
}

template <class Visit>
inline void for_each_candidate(const CellGrid& g, const float* q, const float lo[3], Visit&& visit) {
    const int c0 = cell_coord(q[0], lo[0], g.inv_w[0], g.n[0]);
    const int c1 = cell_coord(q[1], lo[1], g.inv_w[1], g.n[1]);
    const int c2 = cell_coord(q[2], lo[2], g.inv_w[2], g.n[2]);
    int s0[3], s1[3], s2[3];
    const int n0 = stencil(c0, g.n[0], s0), n1 = stencil(c1, g.n[1], s1), n2 = stencil(c2, g.n[2], s2);
    for (int a = 0; a < n0; ++a)
        for (int b = 0; b < n1; ++b)
            for (int c = 0; c < n2; ++c) {
                const size_t cell = ((size_t)s0[a] * g.n[1] + s1[b]) * g.n[2] + s2[c];
                for (uint32_t k = g.start[cell]; k < g.start[cell + 1]; ++k) visit(k);
            }
}

inline bool pair_hit(const CellGrid& g, uint32_t k, const float* q, float rc2, const float L[3],
                     const float h[3]) {
    float d[3] = {rn_sub(g.x[k], q[0]), rn_sub(g.y[k], q[1]), rn_sub(g.z[k], q[2])};
    for (int t = 0; t < 3; ++t) {
        if (d[t] >= h[t])
            d[t] = rn_sub(d[t], L[t]);
        else if (d[t] < -h[t])
            d[t] = rn_add(d[t], L[t]);
    }
    const float d2 = rn_add(rn_add(rn_mul(d[0], d[0]), rn_mul(d[1], d[1])), rn_mul(d[2], d[2]));
    return d2 <= rc2;
}

float max_radius(const float* qr, float rc, uint32_t Q) {
    float m = rc;
    if (qr)
        for (uint32_t i = 0; i < Q; ++i) m = std::max(m, qr[i]);
    return m;
}

}  // namespace

extern "C" {

int orc_celllist(const float* qpos, const float* qr, float rc, uint32_t Q, const float* pts,
                 uint32_t N, const float box_lo[3], const float box_L[3], uint32_t* nneigh,
                 uint32_t* list, uint32_t max_neigh, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    const float rmax = max_radius(qr, rc, Q);
    const float cmax = std::fabs(box_lo[0]) + std::max(box_L[0], std::max(box_L[1], box_L[2]));
    CellGrid g;
    build_grid(g, pts, N, box_lo, box_L, rmax + orc_exact_pad(rmax, cmax));
    const float h[3] = {rn_mul(0.5f, box_L[0]), rn_mul(0.5f, box_L[1]), rn_mul(0.5f, box_L[2])};
    int used = 1;
#pragma omp parallel
    {
#ifdef _OPENMP
#pragma omp single
        used = omp_get_num_threads();
#endif
#pragma omp for schedule(dynamic, 1024)
        for (int64_t i = 0; i < (int64_t)Q; ++i) {
            const float* q = qpos + 3 * i;
            const float r = qr ? qr[i] : rc;
            const float rc2 = rn_mul(r, r);
            uint32_t c = 0;
            for_each_candidate(g, q, box_lo, [&](uint32_t k) {
                if (pair_hit(g, k, q, rc2, box_L, h)) {
                    if (list && c < max_neigh) list[(size_t)max_neigh * i + c] = g.id[k];
                    ++c;
                }
            });
            nneigh[i] = c;
        }
    }
    return used;
}

int orc_celllist_csr(const float* qpos, const float* qr, float rc, uint32_t Q, const float* pts,
                     uint32_t N, const float box_lo[3], const float box_L[3],
                     const uint64_t* offsets, uint32_t* nbrs, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    const float rmax = max_radius(qr, rc, Q);
    const float cmax = std::fabs(box_lo[0]) + std::max(box_L[0], std::max(box_L[1], box_L[2]));
    CellGrid g;
    build_grid(g, pts, N, box_lo, box_L, rmax + orc_exact_pad(rmax, cmax));
    const float h[3] = {rn_mul(0.5f, box_L[0]), rn_mul(0.5f, box_L[1]), rn_mul(0.5f, box_L[2])};
    int used = 1;
#pragma omp parallel
    {
#ifdef _OPENMP
#pragma omp single
        used = omp_get_num_threads();
#endif
#pragma omp for schedule(dynamic, 1024)
        for (int64_t i = 0; i < (int64_t)Q; ++i) {
            const float* q = qpos + 3 * i;
            const float r = qr ? qr[i] : rc;
            const float rc2 = rn_mul(r, r);
            uint64_t w = offsets[i];
            const uint64_t end = offsets[i + 1];
            for_each_candidate(g, q, box_lo, [&](uint32_t k) {
                if (pair_hit(g, k, q, rc2, box_L, h) && w < end) nbrs[w++] = g.id[k];
            });
            std::sort(nbrs + offsets[i], nbrs + w);
        }
    }
    return used;
}

// ---------------------------------------------------------------------------------------
// The project's 16-bit pre-order node format (no counterpart in the reference; the
// reference compresses to 10-bit int4 nodes in Karras order).
// ---------------------------------------------------------------------------------------
// Bins are 15 bits (0..32767) held in 16-bit fields: the top bit of each field is the guard bit
// of the packed compare the traversal uses.
void orc_fast_frame(const float* root_lo, const float* root_hi, float* frame) {
    for (int d = 0; d < 3; ++d) {
        float ext = orc_fsub_ru(root_hi[d], root_lo[d]);
        if (!(ext > 0.f)) ext = 1.0f;
        frame[d] = root_lo[d];
        frame[3 + d] = orc_fdiv_rd(32767.f, ext);
    }
}

void orc_fast_quantize(const float* frame, const float* lo, const float* hi, uint32_t* qlo,
                       uint32_t* qhi) {
    for (int d = 0; d < 3; ++d) {
        const float a = orc_fmul_rd(orc_fsub_rd(lo[d], frame[d]), frame[3 + d]);
        const float b = orc_fmul_ru(orc_fsub_ru(hi[d], frame[d]), frame[3 + d]);
        qlo[d] = clampu(std::floor(a), 0.f, 32767.f);
        qhi[d] = clampu(std::ceil(b), 0.f, 32767.f);
    }
}

uint32_t orc_fast_nodes(uint32_t N, uint32_t leaf_size, const int32_t* parent,
                        const int32_t* left, const int32_t* right, const uint32_t* primitive,
                        const float* lo, const float* hi, uint32_t* nodes, float* frame) {
    (void)parent;
    if (N == 0) return 0;
    orc_fast_frame(lo, hi, frame);  // root box = node 0
    const uint32_t n_int = N - 1;
    const uint32_t n_nodes = 2 * N - 1;
    std::vector<uint32_t> first(n_nodes), last(n_nodes);
    for (uint32_t s = 0; s < N; ++s) first[n_int + s] = last[n_int + s] = s;
    if (N > 1) {
        std::vector<int64_t> stack{0};
        std::vector<uint8_t> done(n_int, 0);
        while (!stack.empty()) {
            const int64_t v = stack.back();
            if (!done[v]) {
                done[v] = 1;
                if ((uint32_t)left[v] < n_int) stack.push_back(left[v]);
                if ((uint32_t)right[v] < n_int) stack.push_back(right[v]);
                continue;
            }
            stack.pop_back();
            first[v] = first[left[v]];
            last[v] = last[right[v]];
        }
    }
    // Depth-first pre-order records.  A node of more than leaf_size primitives is a box record
    // followed by its two subtrees; a node of 2..leaf_size primitives (a bucket) is a box record
    // followed by the point records of its primitives in sorted order; a single primitive is a
    // point record.  Box: {bins, skip = index just past the subtree}; point: {x, y, z as float
    // bits, 0x80000000 | sorted position}.
    uint32_t n_rec = 0;
    auto emit_box = [&](uint32_t v, uint32_t skip) {
        uint32_t qlo[3], qhi[3];
        orc_fast_quantize(frame, lo + 3 * (size_t)v, hi + 3 * (size_t)v, qlo, qhi);
        uint32_t* o = nodes + 4 * (size_t)n_rec++;
        // upper bins complemented (32767 - hi): "box overlaps query" is then "every field of the
        // box <= the query's field", one guarded packed subtraction per word
        o[0] = qlo[0] | (qlo[1] << 16);
        o[1] = qlo[2] | ((32767u - qhi[0]) << 16);
        o[2] = (32767u - qhi[1]) | ((32767u - qhi[2]) << 16);
        o[3] = skip;
    };
    auto emit_point = [&](uint32_t s) {
        const float* p = lo + 3 * (size_t)(n_int + s);
        uint32_t* o = nodes + 4 * (size_t)n_rec++;
        std::memcpy(o, p, 3 * sizeof(float));
        o[3] = 0x80000000u | (uint32_t)s;
    };
    // records in a subtree: 1 for a point, 1 + size for a bucket, 1 + both subtrees otherwise
    std::vector<uint32_t> count(n_nodes, 0);
    for (uint32_t s = 0; s < N; ++s) count[n_int + s] = 1;
    if (N > 1) {
        std::vector<int64_t> order;
        std::vector<int64_t> st{0};
        while (!st.empty()) {
            const int64_t v = st.back();
            st.pop_back();
            order.push_back(v);
            if ((uint32_t)left[v] < n_int) st.push_back(left[v]);
            if ((uint32_t)right[v] < n_int) st.push_back(right[v]);
        }
        for (auto it = order.rbegin(); it != order.rend(); ++it) {
            const uint32_t v = (uint32_t)*it;
            const uint32_t size = last[v] - first[v] + 1;
            count[v] = size <= leaf_size ? 1 + size : 1 + count[left[v]] + count[right[v]];
        }
    }
    std::vector<uint32_t> st{0};
    while (!st.empty()) {
        const uint32_t v = st.back();
        st.pop_back();
        const uint32_t size = last[v] - first[v] + 1;
        if (size == 1) {
            emit_point(first[v]);
        } else if (size <= leaf_size) {
            emit_box(v, n_rec + count[v]);
            for (uint32_t s = first[v]; s <= last[v]; ++s) emit_point(s);
        } else {
            emit_box(v, n_rec + count[v]);
            st.push_back((uint32_t)right[v]);
            st.push_back((uint32_t)left[v]);
        }
    }
    return n_rec;
}

}  // extern "C"

extern "C" {

// Points of the reference's randomized validation test (test/lbvh_test.cu:401-409):
// std::mt19937(seed), std::uniform_real_distribution<float>(-0.5,0.5), scaled by L.  The test
// builds each point with make_float3(L.x*U(mt), L.y*U(mt), L.z*U(mt)); compiled by nvcc with
// gcc as host compiler those arguments are evaluated right to left, so z is drawn first.
void orc_gen_validate_points(uint32_t N, const float L[3], uint32_t seed, float* out) {
    std::mt19937 mt(seed);
    std::uniform_real_distribution<float> U(-0.5f, 0.5f);
    for (uint32_t i = 0; i < N; ++i) {
        const float uz = U(mt);
        const float uy = U(mt);
        const float ux = U(mt);
        out[3 * i + 0] = rn_mul(L[0], ux);
        out[3 * i + 1] = rn_mul(L[1], uy);
        out[3 * i + 2] = rn_mul(L[2], uz);
    }
}

}  // extern "C"


// ---------------------------------------------------------------------------------------------
// Learned capacity network: features and forward/backward, restating
// include/neighbor/kernels/capacity.cuh (cap_features, k_cap_train_step) on the CPU.
// ---------------------------------------------------------------------------------------------
namespace {
uint32_t cap_part1by2(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
uint32_t cap_compact1by2(uint32_t v) {
    v &= 0x09249249u;
    v = (v | (v >> 2)) & 0x030c30c3u;
    v = (v | (v >> 4)) & 0x0300f00fu;
    v = (v | (v >> 8)) & 0x030000ffu;
    v = (v | (v >> 16)) & 0x000003ffu;
    return v;
}
// FP32 -> BF16 -> FP32, round to nearest even (finite inputs).
float bf16_rne(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u += 0x7fffu + ((u >> 16) & 1u);
    u &= 0xffff0000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}
constexpr int kIn = 32, kH = 64;
constexpr int oW1 = 0, oB1 = oW1 + kH * kIn, oW2 = oB1 + kH, oB2 = oW2 + kH * kH, oW3 = oB2 + kH,
              oB3 = oW3 + kH, kP = oB3 + 1;
} // namespace

void orc_cap_occupancy(const uint32_t* codes, uint32_t N, uint32_t shift, uint32_t* occ) {
    const size_t G = 1024u >> shift;
    std::fill(occ, occ + G * G * G, 0u);
    for (uint32_t s = 0; s < N; ++s) occ[codes[s] >> (3 * shift)]++;
}

void orc_cap_features(const uint32_t* codes, const float* points4, uint32_t N, const float lo[3],
                      const float ext[3], uint32_t shift, int periodic, const uint32_t* occ,
                      float* out) {
    const int G = 1024 >> shift;
    for (uint32_t s = 0; s < N; ++s) {
        float* f = out + (size_t)s * kIn;
        const uint32_t c = codes[s] >> (3 * shift);
        const int cx = (int)cap_compact1by2(c >> 2), cy = (int)cap_compact1by2(c >> 1),
                  cz = (int)cap_compact1by2(c);
        float sum = 0.f;
        for (int k = 0; k < 27; ++k) {
            int nx = cx + k / 9 - 1, ny = cy + (k / 3) % 3 - 1, nz = cz + k % 3 - 1;
            uint32_t o = 0;
            bool inside = true;
            if (periodic) {
                nx = (nx + G) % G;
                ny = (ny + G) % G;
                nz = (nz + G) % G;
            } else {
                inside = nx >= 0 && nx < G && ny >= 0 && ny < G && nz >= 0 && nz < G;
            }
            if (inside)
                o = occ[(cap_part1by2((uint32_t)nx) << 2) | (cap_part1by2((uint32_t)ny) << 1) |
                        cap_part1by2((uint32_t)nz)];
            sum += (float)o;
            f[k] = std::log1p((float)o);
        }
        const float inv = 1.0f / (float)(1u << shift);
        const float* p = points4 + 4 * (size_t)s;
        const int cc[3] = {cx, cy, cz};
        for (int d = 0; d < 3; ++d) {
            const float t = std::fmin(std::fmax(rn_mul(rn_div(rn_sub(p[d], lo[d]), ext[d]), 1023.f), 0.f), 1023.f);
            f[27 + d] = std::fmin(std::fmax((t - (float)(cc[d] << shift)) * inv, 0.f), 1.f);
        }
        f[30] = std::log1p(sum);
        f[31] = 1.f;
    }
}

namespace {
template<class T>
T softplus_t(T z) { return std::max(z, (T)0) + std::log1p(std::exp(-std::fabs(z))); }
template<class T>
T sigmoid_t(T z) { return (T)1 / ((T)1 + std::exp(-z)); }

// One sample, template over arithmetic; R rounds to BF16 (or not).
template<class T, class R>
void cap_sample(const float* P, const float* xf, float target, R round, T* g, T& loss, float& yout) {
    T x[kIn], h1[kH], h2[kH], d2[kH], d1[kH];
    T w1[kH * kIn], w2[kH * kH], w3[kH];
    for (int i = 0; i < kH * kIn; ++i) w1[i] = round(P[oW1 + i]);
    for (int i = 0; i < kH * kH; ++i) w2[i] = round(P[oW2 + i]);
    for (int i = 0; i < kH; ++i) w3[i] = round(P[oW3 + i]);
    for (int k = 0; k < kIn; ++k) x[k] = round(xf[k]);
    for (int j = 0; j < kH; ++j) {
        T acc = 0;
        for (int k = 0; k < kIn; ++k) acc = std::fma(w1[j * kIn + k], x[k], acc);
        h1[j] = round(std::max(acc + (T)P[oB1 + j], (T)0));
    }
    for (int j = 0; j < kH; ++j) {
        T acc = 0;
        for (int k = 0; k < kH; ++k) acc = std::fma(w2[j * kH + k], h1[k], acc);
        h2[j] = std::max(acc + (T)P[oB2 + j], (T)0);
    }
    T z = 0;
    for (int k = 0; k < kH; ++k) z = std::fma(w3[k], h2[k], z);
    z += (T)P[oB3];
    const T y = softplus_t(z);
    yout = (float)y;
    const T dy = y - (T)target;
    loss += (T)0.5 * dy * dy;
    const T dz = dy * sigmoid_t(z);
    for (int j = 0; j < kH; ++j) d2[j] = h2[j] > 0 ? dz * w3[j] : (T)0;
    for (int k = 0; k < kH; ++k) {
        T acc = 0;
        for (int j = 0; j < kH; ++j) acc = std::fma(w2[j * kH + k], d2[j], acc);
        d1[k] = h1[k] > 0 ? acc : (T)0;
    }
    for (int j = 0; j < kH; ++j) {
        g[oB1 + j] += d1[j];
        g[oB2 + j] += d2[j];
        g[oW3 + j] += dz * h2[j];
        for (int k = 0; k < kIn; ++k) g[oW1 + j * kIn + k] += d1[j] * x[k];
        for (int k = 0; k < kH; ++k) g[oW2 + j * kH + k] += d2[j] * h1[k];
    }
    g[oB3] += dz;
}
} // namespace

void orc_cap_forward_backward(const float* params, const float* features, const float* targets,
                              uint32_t N, uint32_t batch, uint32_t offset, uint32_t stride, int bf16,
                              double* grad, double* loss, float* y) {
    std::vector<double> gd(kP, 0.0);
    double ld = 0.0;
    std::vector<float> gf(kP, 0.f);
    float lf = 0.f;
    for (uint32_t b = 0; b < batch; ++b) {
        const uint32_t row = (uint32_t)(((uint64_t)offset + (uint64_t)b * stride) % N);
        float yo = 0.f;
        if (bf16 < 0) {
            double l = 0.0;
            cap_sample<double>(params, features + (size_t)row * kIn, targets[row],
                               [](double v) { return v; }, gd.data(), l, yo);
            ld += l;
        } else if (bf16 > 0) {
            cap_sample<float>(params, features + (size_t)row * kIn, targets[row],
                              [](float v) { return bf16_rne(v); }, gf.data(), lf, yo);
        } else {
            cap_sample<float>(params, features + (size_t)row * kIn, targets[row],
                              [](float v) { return v; }, gf.data(), lf, yo);
        }
        if (y) y[b] = yo;
    }
    for (int i = 0; i < kP; ++i) {
        if (grad) grad[i] = bf16 < 0 ? gd[i] : (double)gf[i];
    }
    if (loss) *loss = bf16 < 0 ? ld : (double)lf;
}
