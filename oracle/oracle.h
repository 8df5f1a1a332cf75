/*
 * oracle.h -- CPU restatement of the neighbor LBVH path (TEST INFRASTRUCTURE ONLY).
 *
 * This library is the checker for the CUDA implementation in neighbor_gb300/. Only the
 * tests, the smoke check and the CPU-baseline leg of bench.py load it. No product code
 * path links or calls it.
 *
 * Every function restates one step of the reference (mphowardlab/neighbor v0.3.2) on the
 * host, citing the file:line it follows. The reference has no CPU path of its own: all of
 * its op methods are __device__ only. Directed rounding (the reference's approx:: family,
 * include/neighbor/ApproximateMath.h:55-345) is restated with fesetround(), so the library
 * must be compiled with -frounding-math -ffp-contract=off.
 *
 * Pinning: the restatement is checked against every known-answer value in the reference's
 * own tests (test/lbvh_test.cu:17-582, test/approx_math_test.cu:15-132), stored as
 * fixtures in tests/golden/reference_kats.json.
 *
 * Layout conventions: float3 arrays are passed as float[3*n]; int4 arrays as int[4*n].
 */
#ifndef NEIGHBOR_ORACLE_H_
#define NEIGHBOR_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_INSERT_POINT 0
#define ORC_INSERT_SPHERE 1

#define ORC_QUERY_SPHERE 0 /* stock SphereQueryOp: refine() returns true (superset) */
#define ORC_QUERY_EXACT 1  /* exact FP32 minimum-image distance predicate */

#define ORC_SENTINEL 0x7fffffff

/* ---- directed rounding (include/neighbor/ApproximateMath.h:55-345) ---- */
float orc_fadd_rd(float a, float b);
float orc_fadd_ru(float a, float b);
float orc_fsub_rd(float a, float b);
float orc_fsub_ru(float a, float b);
float orc_fmul_rd(float a, float b);
float orc_fmul_ru(float a, float b);
float orc_fdiv_rd(float a, float b);
float orc_fdiv_ru(float a, float b);
float orc_frcp_rd(float a);
float orc_frcp_ru(float a);
float orc_fmaf_rd(float a, float b, float c);
float orc_fmaf_ru(float a, float b, float c);
float orc_double2float_rd(double a);
float orc_double2float_ru(double a);

/* ---- build (include/neighbor/LBVH.h:242-318) ---- */
/* 30-bit Morton codes (include/neighbor/kernels/LBVH.cuh:28-52,105-157). */
void orc_morton_codes(const float* pts, uint32_t N, int insert_kind, float r,
                      const float scene_lo[3], const float scene_hi[3], uint32_t* codes);

/* Full LBVH build: stable sort by code, Karras hierarchy, bottom-up boxes.
 * Outputs have the reference's sizes: parent[2N-1], left/right[N-1], lo/hi[2N-1].
 * N==1 follows lbvh_one_primitive (include/neighbor/kernels/LBVH.cuh:340-354). */
void orc_build(const float* pts, uint32_t N, int insert_kind, float r,
               const float scene_lo[3], const float scene_hi[3],
               uint32_t* sorted_codes, uint32_t* primitive,
               int32_t* parent, int32_t* left, int32_t* right,
               float* lo, float* hi);

/* ---- reference compression: 10-bit int4 nodes with ropes
 *      (include/neighbor/kernels/LBVHTraverser.cuh:45-125) ---- */
void orc_compress_ref10(uint32_t N, const int32_t* parent, const int32_t* left,
                        const int32_t* right, const uint32_t* primitive,
                        const float* lo, const float* hi, const uint32_t* map,
                        int32_t* data, float* clo, float* chi, float* bins);

/* ---- reference rope traversal over 10-bit nodes
 *      (include/neighbor/kernels/LBVHTraverser.cuh:155-252) ----
 * spheres: float4 (x,y,z,R) per query.  images: float3[n_images] (NULL => self image only).
 * query_kind ORC_QUERY_SPHERE follows include/neighbor/QueryOps.h:32-120; ORC_QUERY_EXACT
 * pads the overlap radius by `pad` and refines with orc_exact_pair() against points[prim]
 * (points indexed by the cached, transformed primitive id).
 * list may be NULL (CountNeighborsOp); else NeighborListOp with stride max_neigh
 * (include/neighbor/OutputOps.h:113-176). */
void orc_traverse_ref10(uint32_t N_nodes, const int32_t* data, const float* clo,
                        const float* chi, const float* bins, const float* spheres,
                        uint32_t Q, const float* images, uint32_t n_images, int query_kind,
                        const float* points, const float box_L[3], float pad,
                        uint32_t* nneigh, uint32_t* list, uint32_t max_neigh);

/* ---- exact predicate (restates test/lbvh_test.cu:469-482, minimum image) ----
 * Returns 1 when |min_image(pj - pi)|^2 <= rc*rc, all in FP32 round-to-nearest with no
 * contraction.  box_L[d] <= 0 means dimension d is not periodic. */
int orc_exact_pair(const float* pi, const float* pj, float rc, const float box_L[3]);

/* Conservative padding of the overlap radius used by the exact query so that traversal
 * never drops a pair that the predicate accepts. coord_max bounds |coordinate| of all
 * query centres and points, including image translations. */
float orc_exact_pad(float rc, float coord_max);

/* O(Q*N) brute force with the exact predicate over a list of images.
 * Counts every (query, point, image) triple that passes the predicate for the translated
 * sphere test used by the reference test (test/lbvh_test.cu:458-490): each pair is
 * counted once per query because the predicate uses the minimum image. */
void orc_brute_count(const float* qpos, const float* qr, uint32_t Q, const float* pts,
                     uint32_t N, const float box_L[3], uint32_t* nneigh);

/* ---- OpenMP cell list with the same predicate (the timed CPU baseline) ----
 * Periodic box [lo, lo+L) in every dimension (L > 0).  Query i has centre qpos[i] and
 * cutoff qr[i] (qr may be NULL => rc for all).  Counts into nneigh[Q]; if list != NULL,
 * also fills a stride-max_neigh list (writes only while < max_neigh, counts all).
 * Returns the number of threads used. */
int orc_celllist(const float* qpos, const float* qr, float rc, uint32_t Q, const float* pts,
                 uint32_t N, const float box_lo[3], const float box_L[3], uint32_t* nneigh,
                 uint32_t* list, uint32_t max_neigh, int nthreads);

/* CSR form of the same cell list: offsets[Q+1] must hold the counts' exclusive scan;
 * fills neighbors sorted ascending per query. */
int orc_celllist_csr(const float* qpos, const float* qr, float rc, uint32_t Q,
                     const float* pts, uint32_t N, const float box_lo[3],
                     const float box_L[3], const uint64_t* offsets, uint32_t* nbrs,
                     int nthreads);

/* ---- Whole-frame host neighbor list (frame_list.cpp; the benchmark's CPU baseline) ----
 * Self list of all N points in the periodic box [lo, lo+L): grid build, count pass, exclusive
 * scan, fill pass, every stage on the host threads.  Rows in grid order: counts[N],
 * offsets[N+1] (uint64), list[total] original indices (list_cap entries available),
 * order[N] (optional) the point of each row.  seconds[4] (optional): grid, count, scan, fill.
 * Returns the number of threads used, or -1 when total > list_cap (counts and offsets valid). */
int orc_frame_list(const float* pts, uint32_t N, const float lo[3], const float L[3], float rc,
                   int nthreads, uint32_t* counts, uint64_t* offsets, uint32_t* list,
                   uint64_t list_cap, uint32_t* order, uint64_t* total, double* seconds);
/* Host trajectory frames: uniform points in [lo, lo+L) and i.i.d. Gaussian moves (sigma) with
 * wrap, from a counter-based generator (independent of the thread count). */
void orc_uniform_points(float* out, uint32_t N, const float lo[3], const float L[3], uint64_t seed);
void orc_gaussian_move(const float* in, float* out, uint32_t N, const float lo[3], const float L[3],
                       float sigma, uint64_t seed);

/* FP64 check of a pair: returns the signed difference |r| - rc in double precision with a
 * minimum image computed in double. */
double orc_pair_distance_minus_rc_f64(const float* pi, const float* pj, float rc,
                                      const float box_L[3]);

/* ---- the project's own traversal records (restated for bit-exact checks of the CUDA build) ----
 * Depth-first pre-order records of 4 uint32 each.  A box record {lo.x|lo.y<<16,
 * lo.z|~hi.x<<16, ~hi.y|~hi.z<<16, skip} (~h = 32767-h; 15-bit bins of the root box, outward
 * rounded, in 16-bit fields) covers a subtree of more than leaf_size primitives (followed by its two subtrees) or a
 * bucket of 2..leaf_size primitives (followed by their point records); a point record
 * {x, y, z as float bits, 0x80000000 | sorted position} is one primitive.  Returns the record count;
 * frame: {root_lo[3], scale[3]}. */
uint32_t orc_fast_nodes(uint32_t N, uint32_t leaf_size, const int32_t* parent,
                        const int32_t* left, const int32_t* right, const uint32_t* primitive,
                        const float* lo, const float* hi, uint32_t* nodes, float* frame);

/* Quantization frame of the records: root_lo and scale = fdiv_rd(32767, fsub_ru(hi,lo)). */
void orc_fast_frame(const float* root_lo, const float* root_hi, float* frame);

/* Box -> conservative 15-bit bins in the frame (lo rounded down, hi rounded up). */
void orc_fast_quantize(const float* frame, const float* lo, const float* hi, uint32_t* qlo,
                       uint32_t* qhi);

/* Points of the reference's randomized validation test (test/lbvh_test.cu:401-409). */
void orc_gen_validate_points(uint32_t N, const float L[3], uint32_t seed, float* out);

/* ---- learned capacity network (this project's addition; test infrastructure only) ----
 * Coarse Morton cells: bins >> shift per axis, G = 1024 >> shift, cell index = code >> 3*shift.
 * occ[G^3] = points per cell of the sorted codes. */
void orc_cap_occupancy(const uint32_t* codes, uint32_t N, uint32_t shift, uint32_t* occ);

/* The 32 features of each sorted point: log1p of the 27 cell occupancies around its own cell
 * (k = 9(dx+1)+3(dy+1)+(dz+1); wrapped when periodic, 0 outside otherwise), its position in its
 * cell along x, y, z, log1p of the sum of the 27, and 1.  points: float4 payload (x,y,z,id). */
void orc_cap_features(const uint32_t* codes, const float* points4, uint32_t N, const float lo[3],
                      const float ext[3], uint32_t shift, int periodic, const uint32_t* occ,
                      float* out);

/* Forward and backward of the network for rows (offset + b*stride) mod N, b < batch:
 * 32 -> 64 ReLU -> 64 ReLU -> 1 softplus; when bf16 != 0 weights, inputs and the first hidden
 * activations are rounded to BF16 (round to nearest even) as on the GPU, products accumulated
 * with fmaf in ascending index order.  grad[6337] = summed dL/dparams, *loss = summed 0.5 (y - t)^2,
 * y[batch] = outputs (either may be NULL).  Double precision when bf16 < 0 (for finite-difference
 * checks of the restated backward). */
void orc_cap_forward_backward(const float* params, const float* features, const float* targets,
                              uint32_t N, uint32_t batch, uint32_t offset, uint32_t stride, int bf16,
                              double* grad, double* loss, float* y);

#ifdef __cplusplus
}
#endif

#endif
