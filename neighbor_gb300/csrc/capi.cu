// C ABI over concrete instantiations of the neighbor C++ templates (include/neighbor_gb300.h).
#include <cstring>
#include <exception>
#include <new>
#include <stdexcept>
#include <string>

#include <cuda_runtime.h>

#include "capi_internal.h"

namespace
{
thread_local std::string g_last_error;
}

namespace neighbor_capi
{
void set_last_error(const std::string& msg) { g_last_error = msg; }
}

namespace
{
using neighbor_capi::as_stream;
using neighbor_capi::f3;
using neighbor_capi::fail;
using neighbor_capi::guarded;
using neighbor_capi::valid_block;

template<class OutputOpT, class TransformOpT>
void dispatch_images(neighbor::LBVHTraverser& t, const neighbor::LBVH& h,
                     const neighbor::LBVHTraverser::LaunchParameters& p, int query_kind,
                     const float* spheres, unsigned int Q, const float* points, float3 box, float pad,
                     const float* images, unsigned int n_images, const OutputOpT& out,
                     const TransformOpT& transform)
    {
    if (query_kind == NBR_QUERY_SPHERE)
        {
        neighbor::SphereQueryOp q(reinterpret_cast<float4*>(const_cast<float*>(spheres)), Q);
        if (images)
            t.traverse(p, h, q, out, neighbor::ImageListOp<float3>(reinterpret_cast<const float3*>(images), n_images), transform);
        else if (n_images == 27)
            t.traverse(p, h, q, out, neighbor::PeriodicImagesOp(box), transform);
        else
            t.traverse(p, h, q, out, neighbor::SelfOp(), transform);
        }
    else
        {
        neighbor::ExactSphereQueryOp q(reinterpret_cast<const float4*>(spheres), Q,
                                       reinterpret_cast<const float3*>(points), box, pad);
        if (images)
            t.traverse(p, h, q, out, neighbor::ImageListOp<float3>(reinterpret_cast<const float3*>(images), n_images), transform);
        else if (n_images == 27)
            t.traverse(p, h, q, out, neighbor::PeriodicImagesOp(box), transform);
        else
            t.traverse(p, h, q, out, neighbor::SelfOp(), transform);
        }
    }

template<class OutputOpT>
void dispatch_transform(neighbor::LBVHTraverser& t, const neighbor::LBVH& h,
                        const neighbor::LBVHTraverser::LaunchParameters& p, int query_kind,
                        const float* spheres, unsigned int Q, const float* points, float3 box, float pad,
                        const float* images, unsigned int n_images, const unsigned int* map,
                        const OutputOpT& out)
    {
    if (map)
        dispatch_images(t, h, p, query_kind, spheres, Q, points, box, pad, images, n_images, out,
                        neighbor::MapTransformOp(map));
    else
        dispatch_images(t, h, p, query_kind, spheres, Q, points, box, pad, images, n_images, out,
                        neighbor::NullTransformOp());
    }

template<class OutputOpT>
void self_transform(neighbor::LBVHTraverser& t, const neighbor::LBVH& h,
                    const neighbor::LBVHTraverser::LaunchParameters& p, float rc, float3 box, float pad,
                    const float* images, unsigned int n_images, const unsigned int* map,
                    const OutputOpT& out, bool rows_sorted)
    {
    if (images)
        {
        neighbor::ImageListOp<float3> img(reinterpret_cast<const float3*>(images), n_images);
        if (map)
            t.traverseSelf(p, h, rc, box, pad, out, img, neighbor::MapTransformOp(map), rows_sorted);
        else
            t.traverseSelf(p, h, rc, box, pad, out, img, neighbor::NullTransformOp(), rows_sorted);
        }
    else if (n_images == 27)
        {
        neighbor::PeriodicImagesOp img(box);
        if (map)
            t.traverseSelf(p, h, rc, box, pad, out, img, neighbor::MapTransformOp(map), rows_sorted);
        else
            t.traverseSelf(p, h, rc, box, pad, out, img, neighbor::NullTransformOp(), rows_sorted);
        }
    else
        {
        if (map)
            t.traverseSelf(p, h, rc, box, pad, out, neighbor::SelfOp(), neighbor::MapTransformOp(map), rows_sorted);
        else
            t.traverseSelf(p, h, rc, box, pad, out, neighbor::SelfOp(), neighbor::NullTransformOp(), rows_sorted);
        }
    }
} // namespace

extern "C" {

const char* nbr_last_error(void) { return g_last_error.c_str(); }

int nbr_version(int* major, int* minor)
    {
    if (major) *major = 0;
    if (minor) *minor = 1;
    return NBR_OK;
    }

int nbr_lbvh_create(nbr_lbvh* out)
    {
    if (!out) return fail(NBR_ERR_INVALID, "null output handle");
    return guarded([&] { *out = new nbr_lbvh_s(); });
    }

int nbr_lbvh_destroy(nbr_lbvh h)
    {
    return guarded([&] { delete h; });
    }

int nbr_lbvh_set_leaf_size(nbr_lbvh h, unsigned int leaf_size)
    {
    if (!h) return fail(NBR_ERR_INVALID, "null handle");
    return guarded([&] { h->lbvh.setLeafSize(leaf_size); });
    }

int nbr_lbvh_set_radix_bits(nbr_lbvh h, unsigned int bits)
    {
    if (!h) return fail(NBR_ERR_INVALID, "null handle");
    return guarded([&] { h->lbvh.setRadixBits(bits); });
    }

int nbr_lbvh_set_climb_block(nbr_lbvh h, unsigned int leaves)
    {
    if (!h) return fail(NBR_ERR_INVALID, "null handle");
    return guarded([&] { h->lbvh.setClimbBlock(leaves); });
    }

int nbr_lbvh_build_points(nbr_lbvh h, const float* points, unsigned int N, const float lo[3],
                          const float hi[3], unsigned int block_size, void* stream)
    {
    if (!h || !lo || !hi || (N > 0 && !points)) return fail(NBR_ERR_INVALID, "null argument");
    if (!valid_block(block_size)) return fail(NBR_ERR_INVALID, "Invalid tuning parameter.");
    return guarded([&] {
        h->lbvh.build(neighbor::LBVH::LaunchParameters(block_size, as_stream(stream)),
                      neighbor::PointInsertOp(reinterpret_cast<const float3*>(points), N), f3(lo), f3(hi));
    });
    }

int nbr_lbvh_build_spheres(nbr_lbvh h, const float* points, float radius, unsigned int N,
                           const float lo[3], const float hi[3], unsigned int block_size, void* stream)
    {
    if (!h || !lo || !hi || (N > 0 && !points)) return fail(NBR_ERR_INVALID, "null argument");
    if (!valid_block(block_size)) return fail(NBR_ERR_INVALID, "Invalid tuning parameter.");
    return guarded([&] {
        h->lbvh.build(neighbor::LBVH::LaunchParameters(block_size, as_stream(stream)),
                      neighbor::SphereInsertOp(reinterpret_cast<const float3*>(points), radius, N), f3(lo),
                      f3(hi));
    });
    }

int nbr_lbvh_get_sizes(nbr_lbvh h, int* root, unsigned int* N, unsigned int* n_internal,
                       unsigned int* n_nodes)
    {
    if (!h) return fail(NBR_ERR_INVALID, "null handle");
    if (root) *root = h->lbvh.getRoot();
    if (N) *N = h->lbvh.getN();
    if (n_internal) *n_internal = h->lbvh.getNInternal();
    if (n_nodes) *n_nodes = h->lbvh.getNNodes();
    return NBR_OK;
    }

int nbr_lbvh_get_arrays(nbr_lbvh h, const int** parent, const int** left, const int** right,
                        const unsigned int** primitive, const float** lo, const float** hi)
    {
    if (!h) return fail(NBR_ERR_INVALID, "null handle");
    const neighbor::ConstLBVHData d = h->lbvh.data();
    if (parent) *parent = d.parent;
    if (left) *left = d.left;
    if (right) *right = d.right;
    if (primitive) *primitive = d.primitive;
    if (lo) *lo = reinterpret_cast<const float*>(d.lo);
    if (hi) *hi = reinterpret_cast<const float*>(d.hi);
    return NBR_OK;
    }

int nbr_lbvh_get_primitives(nbr_lbvh h, const unsigned int** primitive)
    {
    if (!h || !primitive) return fail(NBR_ERR_INVALID, "null argument");
    *primitive = h->lbvh.getPrimitives().get();
    return NBR_OK;
    }

int nbr_lbvh_get_codes(nbr_lbvh h, const unsigned int** codes)
    {
    if (!h || !codes) return fail(NBR_ERR_INVALID, "null argument");
    *codes = h->lbvh.getCodes().get();
    return NBR_OK;
    }

int nbr_lbvh_get_fast(nbr_lbvh h, const unsigned int** records, const float** points,
                      const float** frame, unsigned int* leaf_size)
    {
    if (!h) return fail(NBR_ERR_INVALID, "null handle");
    const neighbor::FastLBVHData f = h->lbvh.fastData();
    if (records) *records = reinterpret_cast<const unsigned int*>(f.nodes);
    if (points) *points = reinterpret_cast<const float*>(f.points);
    if (frame) *frame = reinterpret_cast<const float*>(f.frame);
    if (leaf_size) *leaf_size = f.leaf_size;
    return NBR_OK;
    }

int nbr_lbvh_num_fast_nodes(nbr_lbvh h, unsigned int* n, void* stream)
    {
    if (!h || !n) return fail(NBR_ERR_INVALID, "null argument");
    return guarded([&] { *n = h->lbvh.getNumFastNodes(as_stream(stream)); });
    }

int nbr_lbvh_check_status(nbr_lbvh h, void* stream)
    {
    if (!h) return fail(NBR_ERR_INVALID, "null handle");
    return guarded([&] { h->lbvh.checkStatus(as_stream(stream)); });
    }

int nbr_traverser_create(nbr_traverser* out)
    {
    if (!out) return fail(NBR_ERR_INVALID, "null output handle");
    return guarded([&] { *out = new nbr_traverser_s(); });
    }

int nbr_traverser_destroy(nbr_traverser t)
    {
    return guarded([&] { delete t; });
    }

int nbr_traverser_setup(nbr_traverser t, nbr_lbvh h, const unsigned int* map, unsigned int block_size,
                        void* stream)
    {
    if (!t || !h) return fail(NBR_ERR_INVALID, "null handle");
    if (!valid_block(block_size)) return fail(NBR_ERR_INVALID, "Invalid tuning parameter.");
    return guarded([&] {
        const neighbor::LBVHTraverser::LaunchParameters p(block_size, as_stream(stream));
        if (map)
            t->trav.setup(p, h->lbvh, neighbor::MapTransformOp(map));
        else
            t->trav.setup(p, h->lbvh, neighbor::NullTransformOp());
    });
    }

int nbr_traverser_reset(nbr_traverser t)
    {
    if (!t) return fail(NBR_ERR_INVALID, "null handle");
    t->trav.reset();
    return NBR_OK;
    }

int nbr_traverser_set_fast_path(nbr_traverser t, int enabled)
    {
    if (!t) return fail(NBR_ERR_INVALID, "null handle");
    t->trav.setFastPath(enabled != 0);
    return NBR_OK;
    }

int nbr_traverser_set_mode(nbr_traverser t, int mode)
    {
    if (!t) return fail(NBR_ERR_INVALID, "null handle");
    return guarded([&] { t->trav.setMode(mode); });
    }

int nbr_traverser_set_stats(nbr_traverser t, unsigned long long* counters)
    {
    if (!t) return fail(NBR_ERR_INVALID, "null handle");
    t->trav.setStats(counters);
    return NBR_OK;
    }

int nbr_traverser_set_symmetric(nbr_traverser t, int enabled)
    {
    if (!t) return fail(NBR_ERR_INVALID, "null handle");
    t->trav.setSymmetric(enabled != 0);
    return NBR_OK;
    }

int nbr_traverser_set_work_order(nbr_traverser t, int enabled)
    {
    if (!t) return fail(NBR_ERR_INVALID, "null handle");
    t->trav.setWorkOrder(enabled != 0);
    return NBR_OK;
    }

int nbr_traverser_set_pair_cache(nbr_traverser t, int enabled)
    {
    if (!t) return fail(NBR_ERR_INVALID, "null handle");
    t->trav.setPairCache(enabled != 0);
    return NBR_OK;
    }

int nbr_traverser_count_summary(nbr_traverser t, unsigned int* max_count, unsigned long long* total,
                                unsigned int* past_exchange, void* stream)
    {
    if (!t) return fail(NBR_ERR_INVALID, "null handle");
    return guarded([&] {
        unsigned int mx = 0, past = 0;
        unsigned long long tot = 0;
        t->trav.readCountSummary(as_stream(stream), mx, tot, past);
        if (max_count) *max_count = mx;
        if (total) *total = tot;
        if (past_exchange) *past_exchange = past;
    });
    }

int nbr_traverser_count_summary_device(nbr_traverser t, const unsigned int** words)
    {
    if (!t || !words) return fail(NBR_ERR_INVALID, "null argument");
    *words = t->trav.getCountSummary();
    return NBR_OK;
    }

int nbr_traverser_set_warp_walk_max(nbr_traverser t, unsigned int max_queries)
    {
    if (!t) return fail(NBR_ERR_INVALID, "null handle");
    t->trav.setWarpWalkMaxQueries(max_queries);
    return NBR_OK;
    }

int nbr_traverser_set_symmetric_min_points(nbr_traverser t, unsigned int min_points)
    {
    if (!t) return fail(NBR_ERR_INVALID, "null handle");
    t->trav.setSymmetricMinPoints(min_points);
    return NBR_OK;
    }

int nbr_traverser_set_walk_lanes(nbr_traverser t, unsigned int lanes)
    {
    if (!t) return fail(NBR_ERR_INVALID, "null handle");
    return guarded([&] { t->trav.setWalkLanes(lanes); });
    }

int nbr_traverser_set_half_walk_lanes(nbr_traverser t, unsigned int lanes)
    {
    if (!t) return fail(NBR_ERR_INVALID, "null handle");
    return guarded([&] { t->trav.setHalfWalkLanes(lanes); });
    }

int nbr_traverser_get_data(nbr_traverser t, const int** data, const float** lo, const float** hi,
                           const float** bins)
    {
    if (!t) return fail(NBR_ERR_INVALID, "null handle");
    if (data) *data = reinterpret_cast<const int*>(t->trav.getData().get());
    if (lo) *lo = t->trav.getFrameLo();
    if (hi) *hi = t->trav.getFrameHi();
    if (bins) *bins = t->trav.getFrameBins();
    return NBR_OK;
    }

int nbr_traverse(nbr_traverser t, nbr_lbvh h, int query_kind, const float* spheres, unsigned int Q,
                 const float* points, const float box[3], float pad, const float* images,
                 unsigned int n_images, const unsigned int* map, unsigned int* nneigh, unsigned int* list,
                 unsigned int max_neigh, unsigned int block_size, void* stream)
    {
    if (!t || !h) return fail(NBR_ERR_INVALID, "null handle");
    if (query_kind != NBR_QUERY_SPHERE && query_kind != NBR_QUERY_EXACT)
        return fail(NBR_ERR_INVALID, "unknown query kind");
    if (Q > 0 && (!spheres || !nneigh)) return fail(NBR_ERR_INVALID, "null argument");
    if (query_kind == NBR_QUERY_EXACT && (!points || !box)) return fail(NBR_ERR_INVALID, "exact query needs points and box");
    if (!images && n_images == 27 && !box) return fail(NBR_ERR_INVALID, "periodic images need the box");
    if (list && max_neigh == 0) return fail(NBR_ERR_INVALID, "max_neigh must be positive with a list");
    if (images && n_images > 32) return fail(NBR_ERR_INVALID, "A maximum of 32 image vectors are supported by LBVH traversers.");
    if (!valid_block(block_size)) return fail(NBR_ERR_INVALID, "Invalid tuning parameter.");
    const float3 b = box ? f3(box) : make_float3(0.f, 0.f, 0.f);
    return guarded([&] {
        const neighbor::LBVHTraverser::LaunchParameters p(block_size, as_stream(stream));
        if (list)
            dispatch_transform(t->trav, h->lbvh, p, query_kind, spheres, Q, points, b, pad, images, n_images,
                               map, neighbor::NeighborListOp(list, nneigh, max_neigh));
        else
            dispatch_transform(t->trav, h->lbvh, p, query_kind, spheres, Q, points, b, pad, images, n_images,
                               map, neighbor::CountNeighborsOp(nneigh));
    });
    }

int nbr_traverse_self(nbr_traverser t, nbr_lbvh h, float rc, const float box[3], float pad, const float* images,
                      unsigned int n_images, const unsigned int* map, unsigned int* nneigh, unsigned int* list,
                      unsigned int max_neigh, int rows_sorted, unsigned int block_size, void* stream)
    {
    if (!t || !h || !box) return fail(NBR_ERR_INVALID, "null argument");
    if (h->lbvh.getN() > 0 && !nneigh) return fail(NBR_ERR_INVALID, "null output");
    if (list && max_neigh == 0) return fail(NBR_ERR_INVALID, "max_neigh must be positive with a list");
    if (images && n_images > 32) return fail(NBR_ERR_INVALID, "A maximum of 32 image vectors are supported by LBVH traversers.");
    if (!valid_block(block_size)) return fail(NBR_ERR_INVALID, "Invalid tuning parameter.");
    return guarded([&] {
        const neighbor::LBVHTraverser::LaunchParameters p(block_size, as_stream(stream));
        if (list)
            self_transform(t->trav, h->lbvh, p, rc, f3(box), pad, images, n_images, map,
                           neighbor::NeighborListOp(list, nneigh, max_neigh), rows_sorted != 0);
        else
            self_transform(t->trav, h->lbvh, p, rc, f3(box), pad, images, n_images, map,
                           neighbor::CountNeighborsOp(nneigh), rows_sorted != 0);
    });
    }

float nbr_exact_pad(float rc, float coord_max) { return neighbor::exact_query_pad(rc, coord_max); }

int nbr_lbvh_build_points_f64(nbr_lbvh h, const double* points, unsigned int N, const float lo[3],
                              const float hi[3], unsigned int block_size, void* stream)
    {
    if (!h || !lo || !hi || (N > 0 && !points)) return fail(NBR_ERR_INVALID, "null argument");
    if (!valid_block(block_size)) return fail(NBR_ERR_INVALID, "Invalid tuning parameter.");
    return guarded([&] {
        h->lbvh.build(neighbor::LBVH::LaunchParameters(block_size, as_stream(stream)),
                      neighbor::PointInsertOpF64(reinterpret_cast<const double3*>(points), N), f3(lo), f3(hi));
    });
    }

int nbr_traverse_f64(nbr_traverser t, nbr_lbvh h, const double* spheres, unsigned int Q, const double* points,
                     const double box[3], float pad, const float* images, unsigned int n_images,
                     const unsigned int* map, unsigned int* nneigh, unsigned int* list, unsigned int max_neigh,
                     unsigned int block_size, void* stream)
    {
    if (!t || !h || !box) return fail(NBR_ERR_INVALID, "null argument");
    if (Q > 0 && (!spheres || !points || !nneigh)) return fail(NBR_ERR_INVALID, "null argument");
    if (list && max_neigh == 0) return fail(NBR_ERR_INVALID, "max_neigh must be positive with a list");
    if (images && n_images > 32) return fail(NBR_ERR_INVALID, "A maximum of 32 image vectors are supported by LBVH traversers.");
    if (!valid_block(block_size)) return fail(NBR_ERR_INVALID, "Invalid tuning parameter.");
    return guarded([&] {
        const neighbor::LBVHTraverser::LaunchParameters p(block_size, as_stream(stream));
        const double3 b = make_double3(box[0], box[1], box[2]);
        const neighbor::ExactSphereQueryOpF64 q(reinterpret_cast<const double4_16a*>(spheres), Q,
                                                reinterpret_cast<const double3*>(points), b, pad);
        const float3 bf = make_float3((float)box[0], (float)box[1], (float)box[2]);
        auto go = [&](const auto& out) {
            auto with_images = [&](const auto& transform) {
                if (images)
                    t->trav.traverse(p, h->lbvh, q, out,
                                     neighbor::ImageListOp<float3>(reinterpret_cast<const float3*>(images), n_images),
                                     transform);
                else if (n_images == 27)
                    t->trav.traverse(p, h->lbvh, q, out, neighbor::PeriodicImagesOp(bf), transform);
                else
                    t->trav.traverse(p, h->lbvh, q, out, neighbor::SelfOp(), transform);
            };
            if (map)
                with_images(neighbor::MapTransformOp(map));
            else
                with_images(neighbor::NullTransformOp());
        };
        if (list)
            go(neighbor::NeighborListOp(list, nneigh, max_neigh));
        else
            go(neighbor::CountNeighborsOp(nneigh));
    });
    }

int nbr_traverse_self_f64(nbr_traverser t, nbr_lbvh h, const double* points, double rc, const double box[3],
                          float pad, const float* images, unsigned int n_images, const unsigned int* map,
                          unsigned int* nneigh, unsigned int* list, unsigned int max_neigh, int rows_sorted,
                          unsigned int block_size, void* stream)
    {
    if (!t || !h || !box) return fail(NBR_ERR_INVALID, "null argument");
    if (h->lbvh.getN() > 0 && (!points || !nneigh)) return fail(NBR_ERR_INVALID, "null argument");
    if (list && max_neigh == 0) return fail(NBR_ERR_INVALID, "max_neigh must be positive with a list");
    if (images && n_images > 32) return fail(NBR_ERR_INVALID, "A maximum of 32 image vectors are supported by LBVH traversers.");
    if (!valid_block(block_size)) return fail(NBR_ERR_INVALID, "Invalid tuning parameter.");
    return guarded([&] {
        const neighbor::LBVHTraverser::LaunchParameters p(block_size, as_stream(stream));
        const double3* pts = reinterpret_cast<const double3*>(points);
        const double3 b = make_double3(box[0], box[1], box[2]);
        const float3 bf = make_float3((float)box[0], (float)box[1], (float)box[2]);
        auto go = [&](const auto& out) {
            auto with_images = [&](const auto& transform) {
                if (images)
                    t->trav.traverseSelfF64(p, h->lbvh, pts, rc, b, pad, out,
                                            neighbor::ImageListOp<float3>(reinterpret_cast<const float3*>(images),
                                                                          n_images),
                                            transform, rows_sorted != 0);
                else if (n_images == 27)
                    t->trav.traverseSelfF64(p, h->lbvh, pts, rc, b, pad, out, neighbor::PeriodicImagesOp(bf), transform,
                                            rows_sorted != 0);
                else
                    t->trav.traverseSelfF64(p, h->lbvh, pts, rc, b, pad, out, neighbor::SelfOp(), transform,
                                            rows_sorted != 0);
            };
            if (map)
                with_images(neighbor::MapTransformOp(map));
            else
                with_images(neighbor::NullTransformOp());
        };
        if (list)
            go(neighbor::NeighborListOp(list, nneigh, max_neigh));
        else
            go(neighbor::CountNeighborsOp(nneigh));
    });
    }

int nbr_tune_self(nbr_lbvh h, nbr_traverser t, const float* points, unsigned int N, const float lo[3],
                  const float hi[3], float rc, const float box[3], float pad, int periodic, unsigned int reps,
                  void* stream, unsigned int* leaf_size, unsigned int* radix_bits, unsigned int* climb_block,
                  float* ms)
    {
    if (!h || !t || !lo || !hi || !box || (N > 0 && !points)) return fail(NBR_ERR_INVALID, "null argument");
    if (N == 0) return fail(NBR_ERR_INVALID, "nothing to tune: N = 0");
    return guarded([&] {
        neighbor::SelfListTuner tuner;
        const neighbor::SelfListConfig c =
            tuner.tune(h->lbvh, t->trav, reinterpret_cast<const float3*>(points), N, f3(lo), f3(hi), rc, f3(box), pad,
                       periodic != 0, reps, as_stream(stream));
        if (leaf_size) *leaf_size = c.leaf_size;
        if (radix_bits) *radix_bits = c.radix_bits;
        if (climb_block) *climb_block = c.climb_block;
        if (ms) *ms = c.ms;
    });
    }

int nbr_tune_self_clear(void)
    {
    neighbor::SelfListTuner::clearCache();
    return NBR_OK;
    }

int nbr_debug_inject_alloc_failures(unsigned int count)
    {
    neighbor::detail::injected_alloc_failures().store(count);
    return NBR_OK;
    }

int nbr_debug_wait_timeout(unsigned int* status_out, void* stream)
    {
    if (!status_out) return fail(NBR_ERR_INVALID, "null argument");
    return guarded([&] {
        using neighbor::detail::check_cuda;
        cudaStream_t st = as_stream(stream);
        const unsigned int n = 2 * neighbor::gpu::kScanTile;
        const unsigned int tiles = neighbor::detail::ceil_div((size_t)n + 1, neighbor::gpu::kScanTile);
        neighbor::device_array<unsigned int> in, out, words;
        neighbor::device_array<unsigned long long> status;
        in.reserve(n);
        out.reserve((size_t)n + 1);
        status.reserve(tiles + 1);
        words.reserve(2);  // [0] tile ticket, [1] status word
        check_cuda(cudaMemsetAsync(in.get(), 0, n * sizeof(unsigned int), st), "memset");
        check_cuda(cudaMemsetAsync(status.get(), 0, (tiles + 1) * sizeof(unsigned long long), st), "memset");
        const unsigned int init[2] = {1u, 0u};  // tickets start at 1: tile 0 is never taken
        check_cuda(cudaMemcpyAsync(words.get(), init, sizeof(init), cudaMemcpyHostToDevice, st), "copy");
        neighbor::gpu::k_scan_exclusive<<<tiles, neighbor::gpu::kScanBlock, 0, st>>>(
            in.get(), out.get(), n, status.get(), 1u, words.get(), nullptr, words.get() + 1);
        check_cuda(cudaGetLastError(), "launch");
        unsigned int result[2] = {0u, 0u};
        check_cuda(cudaMemcpyAsync(result, words.get(), sizeof(result), cudaMemcpyDeviceToHost, st), "copy");
        check_cuda(cudaStreamSynchronize(st), "sync");
        *status_out = result[1];
    });
    }

} // extern "C"
