/*
 * neighbor_gb300.h -- C ABI of the GB300 LBVH neighbor-search library.
 *
 * The reference (mphowardlab/neighbor) is a header-only C++ template library with no C ABI of
 * its own; its callers instantiate LBVH::build / LBVHTraverser::traverse with concrete ops.  This
 * header exports those instantiations as plain functions over device pointers, so a host program
 * in any language can bind them (ctypes, cgo, JNI, ...).  Each declaration names the reference
 * interface it stands for.  The C++ template API in include/neighbor/ stays available for custom
 * ops.
 *
 * Conventions
 *   - All array arguments are device (or managed) pointers; float3 arrays are float[3*n], float4
 *     arrays float[4*n].  `stream` is a cudaStream_t (NULL = legacy default stream).
 *   - Work is enqueued asynchronously on `stream`; results are valid after the stream completes.
 *   - Every function returns NBR_OK (0) or an error code; nbr_last_error() gives the message of
 *     the last failure on the calling thread.  No C++ exception crosses this boundary.
 *   - block_size is the reference's tunable launch parameter (32..1024, step 32).
 */
#ifndef NEIGHBOR_GB300_H_
#define NEIGHBOR_GB300_H_

#ifdef __cplusplus
extern "C" {
#endif

#define NBR_OK 0
#define NBR_ERR_INVALID 1     /* bad handle/argument, > 32 images, invalid tunable */
#define NBR_ERR_CUDA 2        /* CUDA runtime error */
#define NBR_ERR_ALLOC 3       /* allocation failed (reference: Memory.h:182-186 throws) */
#define NBR_ERR_DEVICE_WAIT 4 /* a bounded device wait gave up (see nbr_lbvh_check_status) */
#define NBR_ERR_UNSUPPORTED 5

#define NBR_QUERY_SPHERE 0 /* SphereQueryOp, include/neighbor/QueryOps.h:32-120 (superset) */
#define NBR_QUERY_EXACT 1  /* ExactSphereQueryOp: FP32 minimum-image predicate (exact set) */

typedef struct nbr_lbvh_s* nbr_lbvh;
typedef struct nbr_traverser_s* nbr_traverser;

/* Message of the last failed call on this thread ("" if none). */
const char* nbr_last_error(void);

/* Library version (major, minor). */
int nbr_version(int* major, int* minor);

/* ---- LBVH (reference: class LBVH, include/neighbor/LBVH.h:47-219) ---- */

/* LBVH::LBVH() (LBVH.h:224-227) / destructor. */
int nbr_lbvh_create(nbr_lbvh* out);
int nbr_lbvh_destroy(nbr_lbvh h);

/* Additions: leaf bucket size of the traversal tree (1..64) and sort digit width (8 or 10). */
int nbr_lbvh_set_leaf_size(nbr_lbvh h, unsigned int leaf_size);
int nbr_lbvh_set_radix_bits(nbr_lbvh h, unsigned int bits);
/* Addition: sorted leaves per block of the build's agglomerative climb (128, 256 or 512). */
int nbr_lbvh_set_climb_block(nbr_lbvh h, unsigned int leaves);

/* LBVH::build(LaunchParameters, PointInsertOp, lo, hi) (LBVH.h:242-318, InsertOps.h:18-54).
 * points: float3[N]; lo/hi: scene bounds for Morton binning (host float[3]). */
int nbr_lbvh_build_points(nbr_lbvh h, const float* points, unsigned int N, const float lo[3],
                          const float hi[3], unsigned int block_size, void* stream);

/* LBVH::build(LaunchParameters, SphereInsertOp, lo, hi) (InsertOps.h:57-96). */
int nbr_lbvh_build_spheres(nbr_lbvh h, const float* points, float radius, unsigned int N,
                           const float lo[3], const float hi[3], unsigned int block_size,
                           void* stream);

/* getRoot/getN/getNInternal/getNNodes (LBVH.h:111-133). */
int nbr_lbvh_get_sizes(nbr_lbvh h, int* root, unsigned int* N, unsigned int* n_internal,
                       unsigned int* n_nodes);

/* getParents/getLeftChildren/getRightChildren/getPrimitives/getLowerBounds/getUpperBounds
 * (LBVH.h:135-169): managed pointers, host-readable after the build's stream completes.
 * Any output pointer may be NULL. */
int nbr_lbvh_get_arrays(nbr_lbvh h, const int** parent, const int** left, const int** right,
                        const unsigned int** primitive, const float** lo, const float** hi);

/* Addition: sorted Morton codes of the last build (managed pointer). */
int nbr_lbvh_get_codes(nbr_lbvh h, const unsigned int** codes);

/* getPrimitives (LBVH.h:135-169) alone: the sorted primitive order (managed pointer), without
 * forming the reference-layout tree arrays that nbr_lbvh_get_arrays makes current. */
int nbr_lbvh_get_primitives(nbr_lbvh h, const unsigned int** primitive);

/* Addition: the traversal tree (device pointers): records uint32[4*n] in depth-first pre-order
 * (box record {16-bit bins, skip} or point record {x, y, z, 0x80000000 | primitive id}),
 * points float4[N] (sorted x, y, z, primitive id bits), frame float[9] (root lo, root hi,
 * scale). */
int nbr_lbvh_get_fast(nbr_lbvh h, const unsigned int** records, const float** points,
                      const float** frame, unsigned int* leaf_size);

/* Addition: number of traversal records (synchronises `stream`). */
int nbr_lbvh_num_fast_nodes(nbr_lbvh h, unsigned int* n, void* stream);

/* Addition: synchronise `stream` and report NBR_ERR_DEVICE_WAIT if a bounded wait of the last
 * build gave up. */
int nbr_lbvh_check_status(nbr_lbvh h, void* stream);

/* ---- LBVHTraverser (reference: include/neighbor/LBVHTraverser.h:60-355) ---- */

int nbr_traverser_create(nbr_traverser* out);
int nbr_traverser_destroy(nbr_traverser t);

/* LBVHTraverser::setup(params, lbvh[, MapTransformOp]) (LBVHTraverser.h:378-390).
 * map: uint32[N] device array or NULL (NullTransformOp). */
int nbr_traverser_setup(nbr_traverser t, nbr_lbvh h, const unsigned int* map,
                        unsigned int block_size, void* stream);

/* LBVHTraverser::reset() (LBVHTraverser.h:135-138). */
int nbr_traverser_reset(nbr_traverser t);

/* Addition: 0 = always use the reference-layout kernel, 1 = route eligible traversals to the
 * fast kernel (default). */
int nbr_traverser_set_fast_path(nbr_traverser t, int enabled);

/* Addition: fast-path kernel, 0 = one thread per query (default), 1 = one warp per 32
 * consecutive queries. */
int nbr_traverser_set_mode(nbr_traverser t, int mode);

/* Addition: optional device counters (3 x uint64: node visits, point tests, packets walked)
 * that fast-path traversals add to; NULL disables them. */
int nbr_traverser_set_stats(nbr_traverser t, unsigned long long* counters);

/* Addition: self traversals (nbr_traverse_self) with the self image or the 27-image lattice find
 * each unordered pair once and write it to both rows (1, default) or walk the whole tree per
 * query (0).  Counts, neighbor sets and the order of each row are the same either way. */
int nbr_traverser_set_symmetric(nbr_traverser t, int enabled);

/* Addition: a symmetric count records each query's walk length, and a symmetric fill over the same
 * tree and cutoff gives each block's queries to its lanes in order of those lengths (1, default)
 * or in sorted order (0).  Results are the same either way. */
int nbr_traverser_set_work_order(nbr_traverser t, int enabled);

/* Addition: pair exchange -- a symmetric count keeps, per point, the first 16 pairs it found
 * itself and the first 16 pairs other points found with it (128 bytes per point), and a fill over
 * the same tree, cutoff, images and rows assembles the rows from them without walking (1,
 * default; rows with more pairs walk), or every fill walks (0).  Results are the same either
 * way. */
int nbr_traverser_set_pair_cache(nbr_traverser t, int enabled);

/* Addition: summary of the last counting traversal (nbr_traverse or nbr_traverse_self with
 * list == NULL) on this traverser: the largest count, the total of the counts (ordered pairs,
 * self included) and the rows whose pairs did not fit the pair exchange (symmetric self counts).  Synchronises `stream`: it is the host read
 * of the largest count between the count and the list pass (the reference's benchmark reads its
 * counts on the host after the traversal, benchmark/lbvh_benchmark.cc:233-237); any pointer may
 * be NULL. */
int nbr_traverser_count_summary(nbr_traverser t, unsigned int* max_count, unsigned long long* total,
                                unsigned int* past_exchange, void* stream);
/* Addition: device address of the same four 32-bit words ([0] largest count, [1] rows past the
 * exchange, [2..3] the 64-bit total, low word first), written in stream order by each counting
 * self traversal, for callers that copy them without a synchronisation.  NULL before the first
 * count. */
int nbr_traverser_count_summary_device(nbr_traverser t, const unsigned int** words);

/* Addition, routing by size: traversals of at most max_queries queries walk one group of lanes
 * per query, larger ones one thread per query (default 32,768; 0 = never).  Self traversals of
 * more than min_points points take the symmetric walk with the pair exchange whatever the lane
 * limit (default 4,096; 0 = any size).  Results are the same either way. */
int nbr_traverser_set_warp_walk_max(nbr_traverser t, unsigned int max_queries);
int nbr_traverser_set_symmetric_min_points(nbr_traverser t, unsigned int min_points);
/* Addition: lanes per query of those small traversals (4, 8, 16 or 32; 0 = by size). */
int nbr_traverser_set_walk_lanes(nbr_traverser t, unsigned int lanes);
/* Addition: lanes per query of the exchanging symmetric count (LBVHTraverser::setHalfWalkLanes):
 * 1 (one thread per query), 4, 8, 16 or 32; 0 picks by size (lane groups up to 65,536 points).
 * Results do not depend on it; other widths give NBR_ERR_INVALID. */
int nbr_traverser_set_half_walk_lanes(nbr_traverser t, unsigned int lanes);

/* getData() (LBVHTraverser.h:326-329): int4 nodes in the reference's 10-bit layout (managed),
 * plus the compression frame (lo, hi, bins: managed float[3] each). */
int nbr_traverser_get_data(nbr_traverser t, const int** data, const float** lo, const float** hi,
                           const float** bins);

/* LBVHTraverser::traverse(params, lbvh, query, out, images, transform) (LBVHTraverser.h:414-450)
 * with query = SphereQueryOp or ExactSphereQueryOp (query_kind), out = CountNeighborsOp when
 * list == NULL else NeighborListOp(list, nneigh, max_neigh) (OutputOps.h:28-176),
 * images = ImageListOp<float3> (TranslateOps.h:55-91) when images != NULL, the 27 periodic
 * images of `box` (PeriodicImagesOp, the list test/lbvh_test.cu:427-440 builds) when images ==
 * NULL and n_images == 27, else SelfOp (TranslateOps.h:19-46),
 * transform = NullTransformOp when map == NULL else MapTransformOp (TransformOps.h:25-64).
 *   spheres: float4[Q] (x, y, z, radius or cutoff)
 *   points, box, pad: used by the exact query only (positions indexed by the reported id,
 *   periodic box lengths with 0 = open, radius padding -- see nbr_exact_pad). */
int nbr_traverse(nbr_traverser t, nbr_lbvh h, int query_kind, const float* spheres, unsigned int Q,
                 const float* points, const float box[3], float pad, const float* images,
                 unsigned int n_images, const unsigned int* map, unsigned int* nneigh,
                 unsigned int* list, unsigned int max_neigh, unsigned int block_size, void* stream);

/* Addition: every primitive of a point tree queries the tree with cutoff rc (exact predicate).
 * Queries run in the tree's sorted order; rows_sorted = 1 writes row s for sorted slot s (the
 * layout the reference benchmark uses, benchmark/lbvh_benchmark.cc:177-184), 0 writes row
 * primitive[s].  list == NULL => counts only.  Images as in nbr_traverse. */
int nbr_traverse_self(nbr_traverser t, nbr_lbvh h, float rc, const float box[3], float pad,
                      const float* images, unsigned int n_images, const unsigned int* map,
                      unsigned int* nneigh, unsigned int* list, unsigned int max_neigh,
                      int rows_sorted, unsigned int block_size, void* stream);

/* Addition (no counterpart in the reference, whose Tunable only lists valid block sizes,
 * include/neighbor/Tunable.h:28-118): autotune the self neighbor list of `points` -- time the
 * step build + count + host read of the largest count + fill for every leaf size (1, 2, 4, 8),
 * sort digit width (8, 10) and climb block (256, 512), `reps` timed steps each, and apply the
 * fastest to h (nbr_lbvh_set_leaf_size / _radix_bits / _climb_block).  The choice is cached per
 * (N rounded up to a power of two, rc, number density of lo..hi in quarter octaves); a cached
 * class is applied without timing (*ms = 0).  periodic: the 27 images of box, else the self
 * image.  Synchronises `stream`; results never depend on the configuration. */
int nbr_tune_self(nbr_lbvh h, nbr_traverser t, const float* points, unsigned int N, const float lo[3],
                  const float hi[3], float rc, const float box[3], float pad, int periodic, unsigned int reps,
                  void* stream, unsigned int* leaf_size, unsigned int* radix_bits, unsigned int* climb_block,
                  float* ms);
/* Forget every configuration nbr_tune_self has cached (process-wide). */
int nbr_tune_self_clear(void);

/* Test hook for failure detection (no counterpart in the reference): runs the chained scan
 * used by the build with its first tile never published, so the look-back of the next tile must
 * give up after its bounded wait (about a second) instead of hanging.  Writes the resulting
 * device status word (expected: 2, scan look-back gave up) and returns NBR_OK when the wait
 * ended, the kernels finished and the context is still usable. */
int nbr_debug_wait_timeout(unsigned int* status_out, void* stream);

/* Fault injection for tests (no counterpart in the reference): the next `count` device
 * allocations of the library fail as if the CUDA allocator had refused them; the call that hits
 * one returns NBR_ERR_ALLOC, as the reference throws for a failed allocation
 * (include/neighbor/Memory.h:182-186), and leaves its handle usable. */
int nbr_debug_inject_alloc_failures(unsigned int count);

/* No counterpart in the reference.  The Morton-code and stable-sort stage of the LBVH build for
 * callers that cannot allocate device memory (a host framework that owns every allocation, a
 * latency-critical loop that must not touch the allocator, a fully committed memory budget):
 * codes_out[i] / order_out[i] receive the i-th smallest 30-bit Morton code of the points (scene
 * bounds lo/hi, as nbr_lbvh_build_points) and the index of its point, equal stably sorted, the
 * same arrays nbr_lbvh_get_codes / getPrimitives give after a build.  All working memory is one
 * fixed device array (about 10 MB, held on each GPU that loads the library until exit); N above
 * NBR_NOALLOC_MAX_POINTS is rejected with NBR_ERR_INVALID.  The first call on a device looks the
 * array up and should come before any stream capture.  Calls share the array: calls that may
 * overlap on the GPU must be serialised by the caller. */
#define NBR_NOALLOC_MAX_POINTS (1u << 20)
int nbr_morton_sort_noalloc(const float* points, unsigned int N, const float lo[3],
                            const float hi[3], unsigned int* codes_out, unsigned int* order_out,
                            void* stream);

/* No counterpart in the reference.  Status of the last nbr_morton_sort_noalloc call on the current
 * device: copies the fixed array's status word to the host on `stream` (after that call's work)
 * and synchronises `stream`; allocates nothing.  Returns NBR_ERR_DEVICE_WAIT (status_out != 0)
 * when a bounded look-back wait of that call gave up: its outputs are then not valid.  points,
 * codes_out and order_out of a sort must be memory of the current device (NBR_ERR_INVALID
 * otherwise). */
int nbr_morton_sort_noalloc_status(unsigned int* status_out, void* stream);

/* Test hook for the status above (no counterpart in the reference): the same sort with its first
 * tile never run, so that the next tile's look-back gives up after its bounded wait; the status
 * then reports it.  N must exceed one sort tile (4096 points). */
int nbr_debug_noalloc_wait_timeout(const float* points, unsigned int N, const float lo[3],
                                   const float hi[3], unsigned int* codes_out, unsigned int* order_out,
                                   void* stream);

/* Addition (double-precision inputs, e.g. HOOMD-blue built with Scalar = double): LBVH::build
 * with PointInsertOpF64 -- each point's box is the point rounded outward to FP32
 * (BoundingBox(double3, double3), include/neighbor/BoundingVolumes.h:54-58). */
int nbr_lbvh_build_points_f64(nbr_lbvh h, const double* points, unsigned int N, const float lo[3],
                              const float hi[3], unsigned int block_size, void* stream);

/* Addition: LBVHTraverser::traverse with ExactSphereQueryOpF64 over a tree of double points:
 * spheres double[4Q] (x, y, z, cutoff), points double[3N] indexed by the reported id, box double[3]
 * periodic lengths (0 = open), pad as nbr_exact_pad; images, map and outputs as nbr_traverse.
 * Runs the reference-layout rope traversal with the exact double predicate. */
int nbr_traverse_f64(nbr_traverser t, nbr_lbvh h, const double* spheres, unsigned int Q, const double* points,
                     const double box[3], float pad, const float* images, unsigned int n_images,
                     const unsigned int* map, unsigned int* nneigh, unsigned int* list, unsigned int max_neigh,
                     unsigned int block_size, void* stream);

/* Addition: self queries of a tree built by nbr_lbvh_build_points_f64 from `points` (double[3N],
 * indexed by primitive id), exact double predicate: every primitive queries the tree with cutoff
 * rc, in the tree's sorted order -- the counts and rows of nbr_traverse_f64 over the spheres
 * (points[primitive[s]], rc) for s = 0..N-1 (LBVHTraverser::traverse with ExactSphereQueryOpF64,
 * include/neighbor/LBVHTraverser.h:414-450 for the traversal it stands for).  rows_sorted = 1
 * writes row s for sorted slot s, 0 row primitive[s]; box double[3] periodic lengths (0 = open),
 * pad as nbr_exact_pad; images, map and outputs as nbr_traverse_self.  A count with SelfOp or the
 * 27 periodic images finds each pair once and keeps the pairs, so that the next fill over the same
 * tree, points, cutoff, images and rows writes its rows without walking. */
int nbr_traverse_self_f64(nbr_traverser t, nbr_lbvh h, const double* points, double rc, const double box[3],
                          float pad, const float* images, unsigned int n_images, const unsigned int* map,
                          unsigned int* nneigh, unsigned int* list, unsigned int max_neigh, int rows_sorted,
                          unsigned int block_size, void* stream);

/* Radius padding for the exact query: 16 ulps of twice the largest coordinate magnitude
 * (centres, points and image translations) plus 1e-6 * rc. */
float nbr_exact_pad(float rc, float coord_max);

/* ---- Additions with no counterpart in the reference: CSR lists, learned capacities, one-pass
 * lists.  They replace the reference's two-pass pattern (CountNeighborsOp, host max, then
 * NeighborListOp with that stride; benchmark/lbvh_benchmark.cc:177-196). ---- */

typedef struct nbr_capmodel_s* nbr_capmodel;
typedef struct nbr_onepass_s* nbr_onepass;

/* Self traversal (as nbr_traverse_self) into a CSR list: row r occupies
 * list[offsets[r] .. offsets[r] + caps[r]) (offsets: uint64[N]); the full count always goes to
 * nneigh[r], entries past caps[r] are dropped.  max_capacity = an upper bound of caps (0 =
 * unknown) lets the symmetric traversal run.  Images as in nbr_traverse (list images: whole-tree
 * walk). */
int nbr_traverse_self_csr(nbr_traverser t, nbr_lbvh h, float rc, const float box[3], float pad,
                          const float* images, unsigned int n_images, const unsigned int* map,
                          unsigned int* nneigh, unsigned int* list, const unsigned long long* offsets,
                          const unsigned int* caps, unsigned int max_capacity, int rows_sorted,
                          unsigned int block_size, void* stream);

/* Addition: traverseSelfSubset -- the rows of the sorted positions subset[0..count) of a point
 * tree re-run into a CSR list (offsets/caps as nbr_traverse_self_csr; only those rows and their
 * counts are written), one warp per row.  For rows that overflowed a one-pass list, or a few rows
 * whose capacity changed. */
int nbr_traverse_self_subset_csr(nbr_traverser t, nbr_lbvh h, float rc, const float box[3], float pad,
                                 const float* images, unsigned int n_images, const unsigned int* map,
                                 const unsigned int* subset, unsigned int count, unsigned int* nneigh,
                                 unsigned int* list, const unsigned long long* offsets, const unsigned int* caps,
                                 int rows_sorted, void* stream);

/* Capacity network (32 -> 64 -> 64 -> 1, BF16 weights, FP32 accumulation): create with a seed for
 * the initial weights; parameters as FP32[NBR_CAP_PARAMS] on the host (W1[64][32], b1[64],
 * W2[64][64], b2[64], W3[64], b3). */
#define NBR_CAP_PARAMS 6337
#define NBR_CAP_FEATURES 32
int nbr_capmodel_create(nbr_capmodel* out, unsigned long long seed);
int nbr_capmodel_destroy(nbr_capmodel m);
int nbr_capmodel_get_params(nbr_capmodel m, float* host_params);
int nbr_capmodel_set_params(nbr_capmodel m, const float* host_params);
/* Capacity = ceil(expm1(output + margin(output))) clamped to [1, cap_max].  set_margin sets one
 * margin for every output, get_margin returns the largest; set/get_margins the calibration table of
 * NBR_CAP_MARGIN_BINS margins over bins of 0.5 in the output (the last bin open-ended). */
#define NBR_CAP_MARGIN_BINS 16
int nbr_capmodel_set_margin(nbr_capmodel m, float margin);
int nbr_capmodel_get_margin(nbr_capmodel m, float* margin);
int nbr_capmodel_set_margins(nbr_capmodel m, const float* margins);
int nbr_capmodel_get_margins(nbr_capmodel m, float* margins);

/* Inference kernel (no counterpart in the reference): NBR_CAP_INFER_WARP_TILES = warp tiles of
 * mma.sync m16n8k16 (k_cap_infer), NBR_CAP_INFER_TENSOR_MEMORY = 128-query tiles on tcgen05 with
 * Tensor Memory accumulators (k_cap_infer_tc).  Capacities agree up to FP32 summation order.
 * nbr_capmodel_status reads and clears the device status word of the inference (bit 4 = a
 * bounded wait for a tensor-core MMA gave up; that prediction is incomplete); synchronises. */
#define NBR_CAP_INFER_WARP_TILES 0
#define NBR_CAP_INFER_TENSOR_MEMORY 1
int nbr_capmodel_set_infer_kernel(nbr_capmodel m, int kernel);
int nbr_capmodel_get_infer_kernel(nbr_capmodel m, int* kernel);
int nbr_capmodel_status(nbr_capmodel m, unsigned int* status);

/* Weights file of a trained model: "NBRCAPMD", version 1, its shapes, the FP32 parameters and
 * margin table, and an FNV-1a hash; load returns NBR_ERR_INVALID for a file whose magic,
 * version, shapes, size or hash differ. */
int nbr_capmodel_save(nbr_capmodel m, const char* path);
int nbr_capmodel_load(nbr_capmodel m, const char* path);
/* Coarse-cell level the features use for cutoff rc in a scene of extent hi - lo. */
int nbr_capmodel_level(float rc, const float lo[3], const float hi[3], unsigned int* level);
/* Features (float[N][32]) of every sorted point of a built point tree; lo/hi = the build's scene
 * box, periodic = neighbor cells wrap. */
int nbr_capmodel_features(nbr_capmodel m, nbr_lbvh h, const float lo[3], const float hi[3], float rc,
                          int periodic, float* features, void* stream);
/* Capacity per row (rows as nbr_traverse_self) and, if y != NULL, the network output per row. */
int nbr_capmodel_predict(nbr_capmodel m, nbr_lbvh h, const float lo[3], const float hi[3], float rc,
                         int periodic, int rows_sorted, unsigned int cap_max, unsigned int* caps, float* y,
                         void* stream);
/* log1p(count) training targets. */
int nbr_capmodel_targets(const unsigned int* counts, unsigned int N, float* targets, void* stream);
/* Summed gradient (float[NBR_CAP_PARAMS], device) and summed loss 0.5 (y - target)^2 (device
 * float) of rows (offset + b * stride) mod N, b < batch; no update. */
int nbr_capmodel_gradient(nbr_capmodel m, const float* features, const float* targets, unsigned int N,
                          unsigned int batch, unsigned int offset, unsigned int stride, float* grad,
                          float* loss, void* stream);
/* `steps` Adam steps on random batches; *loss = mean loss of the last batch (synchronises). */
int nbr_capmodel_train(nbr_capmodel m, const float* features, const float* targets, unsigned int N,
                       unsigned int steps, unsigned int batch, float lr, unsigned long long seed,
                       float* loss, void* stream);

/* One-pass self neighbor list: nbr_onepass_capacity gives the device array of N row capacities
 * to fill (e.g. nbr_capmodel_predict); nbr_onepass_build runs one traversal into a CSR list sized
 * by them, then re-runs the rows that overflowed with their exact counts (the list is always
 * exact).  cap_max bounds every capacity.  Synchronises the stream. */
int nbr_onepass_create(nbr_onepass* out);
int nbr_onepass_destroy(nbr_onepass op);
int nbr_onepass_capacity(nbr_onepass op, unsigned int N, unsigned int** caps);
int nbr_onepass_build(nbr_onepass op, nbr_traverser t, nbr_lbvh h, float rc, const float box[3], float pad,
                      int periodic, int rows_sorted, unsigned int cap_max, const unsigned int* map,
                      unsigned int block_size, void* stream, unsigned long long* slots,
                      unsigned int* overflow_rows, unsigned long long* overflow_slots);
/* The learned one-pass step in one call: build h from points (as nbr_lbvh_build_points, scene
 * bounds lo/hi), predict every row's capacity with m (features in the frame lo/hi), and fill the
 * list as nbr_onepass_build.  The prediction runs on a second stream as soon as the build's sort
 * is done, alongside the rest of the build.  Synchronises the stream. */
int nbr_onepass_build_learned(nbr_onepass op, nbr_capmodel m, nbr_traverser t, nbr_lbvh h, const float* points,
                              unsigned int N, const float lo[3], const float hi[3], float rc, const float box[3],
                              float pad, int periodic, int rows_sorted, unsigned int cap_max,
                              const unsigned int* map, unsigned int block_size, void* stream,
                              unsigned long long* slots, unsigned int* overflow_rows,
                              unsigned long long* overflow_slots);
/* The list of the last build: entries, row offsets (uint64[N]), capacities, counts, total slots. */
int nbr_onepass_get(nbr_onepass op, const unsigned int** list, const unsigned long long** offsets,
                    const unsigned int** caps, const unsigned int** nneigh, unsigned long long* total);
/* Exclusive scan of n counts into uint64 offsets; *total = their sum (synchronises), or with
 * total == NULL the scan is only enqueued on `stream`. */
int nbr_onepass_scan(nbr_onepass op, const unsigned int* counts, unsigned int n,
                     unsigned long long* offsets, unsigned long long* total, void* stream);

/* ---- Addition with no counterpart in the reference: batched ensembles of small systems. ----
 * Many independent periodic systems (at most NBR_BATCH_MAX_N points each) built and listed in
 * one launch.  start: host uint[S+1] (system s = points [start[s], start[s+1])), box: host
 * float[3S] periodic lengths (system s's scene is [0, box)), rc cutoff, max_neigh list capacity
 * per point.  Outputs per point of the batch: nneigh[T] and list[T * max_neigh] with global
 * point indices; each system's result equals nbr_lbvh_build_points + nbr_traverse_self (27
 * periodic images, rows by primitive) on that system alone. */
#define NBR_BATCH_MAX_N 16384
typedef struct nbr_batch_s* nbr_batch;
int nbr_batch_create(nbr_batch* out);
int nbr_batch_destroy(nbr_batch b);
int nbr_batch_setup(nbr_batch b, const unsigned int* start, const float* box, unsigned int S, float rc,
                    unsigned int max_neigh);
/* Leaf size (1..64) and threads per block (512 or 1024) of the batched kernel. */
int nbr_batch_set_config(nbr_batch b, unsigned int leaf_size, unsigned int block);
int nbr_batch_get_config(nbr_batch b, unsigned int* leaf_size, unsigned int* block);
int nbr_batch_run(nbr_batch b, const float* points, unsigned int* nneigh, unsigned int* list, void* stream);
/* Autotuner: times every configuration on this batch and keeps the fastest (synchronises). */
int nbr_batch_tune(nbr_batch b, const float* points, unsigned int* nneigh, unsigned int* list, void* stream,
                   unsigned int* leaf_size, unsigned int* block);
/* Capture a run (current configuration, these buffers) in a CUDA graph on `stream` (not the
 * legacy default stream); nbr_batch_replay launches the graph. */
int nbr_batch_capture(nbr_batch b, const float* points, unsigned int* nneigh, unsigned int* list, void* stream);
int nbr_batch_replay(nbr_batch b, void* stream);
/* After a run (synchronises): status bits (1 = a system above NBR_BATCH_MAX_N was skipped) and the
 * largest count (rows with more than max_neigh entries keep max_neigh). */
int nbr_batch_status(nbr_batch b, unsigned int* bits, unsigned int* largest, void* stream);
/* The same work as one plain call per system: build, count, host read of the largest count, fill
 * (for comparison with the batched form).  List entries are system-local primitive ids. */
int nbr_batch_sequential_plain(nbr_lbvh h, nbr_traverser t, const float* points, const unsigned int* start,
                               const float* box, unsigned int S, float rc, unsigned int* nneigh, unsigned int* list,
                               unsigned int max_neigh, unsigned int block_size, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* NEIGHBOR_GB300_H_ */
