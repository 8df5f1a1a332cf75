// C ABI of the additions: CSR self lists, the capacity network and one-pass lists
// (include/neighbor_gb300.h).
#include <string>

#include <cuda_runtime.h>

#include "capi_internal.h"
#include "neighbor/CapacityModel.h"
#include "neighbor/OnePassList.h"

static_assert(NBR_CAP_MARGIN_BINS == neighbor::CapacityModel::kMarginBins, "margin table size");

struct nbr_capmodel_s
    {
    explicit nbr_capmodel_s(unsigned long long seed) : model(seed) {}
    neighbor::CapacityModel model;
    };

struct nbr_onepass_s
    {
    neighbor::OnePassNeighborList list;
    };

namespace
{
using neighbor_capi::as_stream;
using neighbor_capi::f3;
using neighbor_capi::fail;
using neighbor_capi::guarded;
using neighbor_capi::valid_block;

template<class TranslateOpT>
void self_csr(neighbor::LBVHTraverser& t, const neighbor::LBVH& h, const neighbor::LBVHTraverser::LaunchParameters& p,
              float rc, float3 box, float pad, const TranslateOpT& img, const unsigned int* map,
              const neighbor::CSRNeighborListOp& out, bool rows_sorted)
    {
    if (map)
        t.traverseSelf(p, h, rc, box, pad, out, img, neighbor::MapTransformOp(map), rows_sorted);
    else
        t.traverseSelf(p, h, rc, box, pad, out, img, neighbor::NullTransformOp(), rows_sorted);
    }

template<class TranslateOpT>
void self_subset_csr(neighbor::LBVHTraverser& t, const neighbor::LBVH& h,
                     const neighbor::LBVHTraverser::LaunchParameters& p, float rc, float3 box, float pad,
                     const TranslateOpT& img, const unsigned int* map, const neighbor::CSRNeighborListOp& out,
                     bool rows_sorted, const unsigned int* subset, unsigned int count)
    {
    if (map)
        t.traverseSelfSubset(p, h, rc, box, pad, out, img, neighbor::MapTransformOp(map), rows_sorted, subset, count);
    else
        t.traverseSelfSubset(p, h, rc, box, pad, out, img, neighbor::NullTransformOp(), rows_sorted, subset, count);
    }
} // namespace

extern "C" {

int nbr_traverse_self_csr(nbr_traverser t, nbr_lbvh h, float rc, const float box[3], float pad,
                          const float* images, unsigned int n_images, const unsigned int* map,
                          unsigned int* nneigh, unsigned int* list, const unsigned long long* offsets,
                          const unsigned int* caps, unsigned int max_capacity, int rows_sorted,
                          unsigned int block_size, void* stream)
    {
    if (!t || !h || !box) return fail(NBR_ERR_INVALID, "null argument");
    if (h->lbvh.getN() > 0 && (!nneigh || !list || !offsets || !caps)) return fail(NBR_ERR_INVALID, "null output");
    if (images && n_images > 32) return fail(NBR_ERR_INVALID, "A maximum of 32 image vectors are supported by LBVH traversers.");
    if (!valid_block(block_size)) return fail(NBR_ERR_INVALID, "Invalid tuning parameter.");
    return guarded([&] {
        const neighbor::LBVHTraverser::LaunchParameters p(block_size, as_stream(stream));
        const neighbor::CSRNeighborListOp out(list, nneigh, offsets, caps, max_capacity);
        const float3 b = f3(box);
        if (images)
            self_csr(t->trav, h->lbvh, p, rc, b, pad,
                     neighbor::ImageListOp<float3>(reinterpret_cast<const float3*>(images), n_images), map, out,
                     rows_sorted != 0);
        else if (n_images == 27)
            self_csr(t->trav, h->lbvh, p, rc, b, pad, neighbor::PeriodicImagesOp(b), map, out, rows_sorted != 0);
        else
            self_csr(t->trav, h->lbvh, p, rc, b, pad, neighbor::SelfOp(), map, out, rows_sorted != 0);
    });
    }

int nbr_traverse_self_subset_csr(nbr_traverser t, nbr_lbvh h, float rc, const float box[3], float pad,
                                 const float* images, unsigned int n_images, const unsigned int* map,
                                 const unsigned int* subset, unsigned int count, unsigned int* nneigh,
                                 unsigned int* list, const unsigned long long* offsets, const unsigned int* caps,
                                 int rows_sorted, void* stream)
    {
    if (!t || !h || !box) return fail(NBR_ERR_INVALID, "null argument");
    if (count > 0 && (!subset || !nneigh || !list || !offsets || !caps)) return fail(NBR_ERR_INVALID, "null argument");
    if (count > h->lbvh.getN()) return fail(NBR_ERR_INVALID, "subset larger than the tree");
    if (images && n_images > 32) return fail(NBR_ERR_INVALID, "A maximum of 32 image vectors are supported by LBVH traversers.");
    return guarded([&] {
        const neighbor::LBVHTraverser::LaunchParameters p(256, as_stream(stream));
        const neighbor::CSRNeighborListOp out(list, nneigh, offsets, caps, 0u);
        const float3 b = f3(box);
        if (images)
            self_subset_csr(t->trav, h->lbvh, p, rc, b, pad,
                            neighbor::ImageListOp<float3>(reinterpret_cast<const float3*>(images), n_images), map,
                            out, rows_sorted != 0, subset, count);
        else if (n_images == 27)
            self_subset_csr(t->trav, h->lbvh, p, rc, b, pad, neighbor::PeriodicImagesOp(b), map, out,
                            rows_sorted != 0, subset, count);
        else
            self_subset_csr(t->trav, h->lbvh, p, rc, b, pad, neighbor::SelfOp(), map, out, rows_sorted != 0,
                            subset, count);
    });
    }

int nbr_capmodel_create(nbr_capmodel* out, unsigned long long seed)
    {
    if (!out) return fail(NBR_ERR_INVALID, "null output handle");
    return guarded([&] { *out = new nbr_capmodel_s(seed); });
    }

int nbr_capmodel_destroy(nbr_capmodel m)
    {
    return guarded([&] { delete m; });
    }

int nbr_capmodel_get_params(nbr_capmodel m, float* host_params)
    {
    if (!m || !host_params) return fail(NBR_ERR_INVALID, "null argument");
    return guarded([&] { m->model.getParams(host_params); });
    }

int nbr_capmodel_set_params(nbr_capmodel m, const float* host_params)
    {
    if (!m || !host_params) return fail(NBR_ERR_INVALID, "null argument");
    return guarded([&] { m->model.setParams(host_params); });
    }

int nbr_capmodel_set_margin(nbr_capmodel m, float margin)
    {
    if (!m) return fail(NBR_ERR_INVALID, "null handle");
    m->model.setMargin(margin);
    return NBR_OK;
    }

int nbr_capmodel_get_margin(nbr_capmodel m, float* margin)
    {
    if (!m || !margin) return fail(NBR_ERR_INVALID, "null argument");
    *margin = m->model.getMargin();
    return NBR_OK;
    }

int nbr_capmodel_set_margins(nbr_capmodel m, const float* margins)
    {
    if (!m || !margins) return fail(NBR_ERR_INVALID, "null argument");
    m->model.setMargins(margins);
    return NBR_OK;
    }

int nbr_capmodel_get_margins(nbr_capmodel m, float* margins)
    {
    if (!m || !margins) return fail(NBR_ERR_INVALID, "null argument");
    m->model.getMargins(margins);
    return NBR_OK;
    }

int nbr_capmodel_set_infer_kernel(nbr_capmodel m, int kernel)
    {
    if (!m) return fail(NBR_ERR_INVALID, "null handle");
    if (kernel != NBR_CAP_INFER_WARP_TILES && kernel != NBR_CAP_INFER_TENSOR_MEMORY)
        return fail(NBR_ERR_INVALID, "unknown inference kernel");
    m->model.setInferKernel(static_cast<neighbor::CapacityModel::InferKernel>(kernel));
    return NBR_OK;
    }

int nbr_capmodel_get_infer_kernel(nbr_capmodel m, int* kernel)
    {
    if (!m || !kernel) return fail(NBR_ERR_INVALID, "null argument");
    *kernel = static_cast<int>(m->model.getInferKernel());
    return NBR_OK;
    }

int nbr_capmodel_status(nbr_capmodel m, unsigned int* status)
    {
    if (!m || !status) return fail(NBR_ERR_INVALID, "null argument");
    return guarded([&] { *status = m->model.takeStatus(); });
    }

int nbr_capmodel_save(nbr_capmodel m, const char* path)
    {
    if (!m || !path) return fail(NBR_ERR_INVALID, "null argument");
    return guarded([&] { m->model.save(path); });
    }

int nbr_capmodel_load(nbr_capmodel m, const char* path)
    {
    if (!m || !path) return fail(NBR_ERR_INVALID, "null argument");
    return guarded([&] { m->model.load(path); });
    }

int nbr_capmodel_level(float rc, const float lo[3], const float hi[3], unsigned int* level)
    {
    if (!lo || !hi || !level) return fail(NBR_ERR_INVALID, "null argument");
    *level = neighbor::CapacityModel::levelFor(rc, make_float3(hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]));
    return NBR_OK;
    }

int nbr_capmodel_features(nbr_capmodel m, nbr_lbvh h, const float lo[3], const float hi[3], float rc,
                          int periodic, float* features, void* stream)
    {
    if (!m || !h || !lo || !hi || !features) return fail(NBR_ERR_INVALID, "null argument");
    if (!h->lbvh.hasFastData()) return fail(NBR_ERR_INVALID, "features need a tree built from points");
    return guarded([&] {
        m->model.features(h->lbvh, neighbor::CapacityModel::frame(f3(lo), f3(hi), rc, periodic != 0), features,
                          as_stream(stream));
    });
    }

int nbr_capmodel_predict(nbr_capmodel m, nbr_lbvh h, const float lo[3], const float hi[3], float rc,
                         int periodic, int rows_sorted, unsigned int cap_max, unsigned int* caps, float* y,
                         void* stream)
    {
    if (!m || !h || !lo || !hi || !caps) return fail(NBR_ERR_INVALID, "null argument");
    if (!h->lbvh.hasFastData()) return fail(NBR_ERR_INVALID, "prediction needs a tree built from points");
    if (cap_max == 0) return fail(NBR_ERR_INVALID, "cap_max must be positive");
    return guarded([&] {
        m->model.predict(h->lbvh, neighbor::CapacityModel::frame(f3(lo), f3(hi), rc, periodic != 0),
                         rows_sorted != 0, cap_max, caps, y, as_stream(stream));
    });
    }

int nbr_capmodel_targets(const unsigned int* counts, unsigned int N, float* targets, void* stream)
    {
    if ((N > 0) && (!counts || !targets)) return fail(NBR_ERR_INVALID, "null argument");
    if (N == 0) return NBR_OK;
    return guarded([&] { neighbor::CapacityModel::targets(counts, N, targets, as_stream(stream)); });
    }

int nbr_capmodel_gradient(nbr_capmodel m, const float* features, const float* targets, unsigned int N,
                          unsigned int batch, unsigned int offset, unsigned int stride, float* grad,
                          float* loss, void* stream)
    {
    if (!m || !features || !targets || !grad || !loss) return fail(NBR_ERR_INVALID, "null argument");
    if (N == 0 || batch == 0) return fail(NBR_ERR_INVALID, "N and batch must be positive");
    return guarded([&] { m->model.gradient(features, targets, N, batch, offset, stride, grad, loss, as_stream(stream)); });
    }

int nbr_capmodel_train(nbr_capmodel m, const float* features, const float* targets, unsigned int N,
                       unsigned int steps, unsigned int batch, float lr, unsigned long long seed,
                       float* loss, void* stream)
    {
    if (!m || !features || !targets) return fail(NBR_ERR_INVALID, "null argument");
    if (N == 0 || batch == 0) return fail(NBR_ERR_INVALID, "N and batch must be positive");
    return guarded([&] {
        const float l = m->model.train(features, targets, N, steps, batch, lr, seed, as_stream(stream));
        if (loss) *loss = l;
    });
    }

int nbr_onepass_create(nbr_onepass* out)
    {
    if (!out) return fail(NBR_ERR_INVALID, "null output handle");
    return guarded([&] { *out = new nbr_onepass_s(); });
    }

int nbr_onepass_destroy(nbr_onepass op)
    {
    return guarded([&] { delete op; });
    }

int nbr_onepass_capacity(nbr_onepass op, unsigned int N, unsigned int** caps)
    {
    if (!op || !caps) return fail(NBR_ERR_INVALID, "null argument");
    return guarded([&] { *caps = op->list.capacity(N); });
    }

int nbr_onepass_build(nbr_onepass op, nbr_traverser t, nbr_lbvh h, float rc, const float box[3], float pad,
                      int periodic, int rows_sorted, unsigned int cap_max, const unsigned int* map,
                      unsigned int block_size, void* stream, unsigned long long* slots,
                      unsigned int* overflow_rows, unsigned long long* overflow_slots)
    {
    if (!op || !t || !h || !box) return fail(NBR_ERR_INVALID, "null argument");
    if (!valid_block(block_size)) return fail(NBR_ERR_INVALID, "Invalid tuning parameter.");
    if (h->lbvh.getN() > 0 && !h->lbvh.hasFastData()) return fail(NBR_ERR_INVALID, "one-pass lists need a tree built from points");
    return guarded([&] {
        const neighbor::LBVHTraverser::LaunchParameters p(block_size, as_stream(stream));
        neighbor::OnePassNeighborList::Stats st;
        if (map)
            st = op->list.build(p, h->lbvh, t->trav, rc, f3(box), pad, periodic != 0, rows_sorted != 0, cap_max,
                                neighbor::MapTransformOp(map));
        else
            st = op->list.build(p, h->lbvh, t->trav, rc, f3(box), pad, periodic != 0, rows_sorted != 0, cap_max,
                                neighbor::NullTransformOp());
        if (slots) *slots = st.slots;
        if (overflow_rows) *overflow_rows = st.overflow_rows;
        if (overflow_slots) *overflow_slots = st.overflow_slots;
    });
    }

int nbr_onepass_build_learned(nbr_onepass op, nbr_capmodel m, nbr_traverser t, nbr_lbvh h, const float* points,
                              unsigned int N, const float lo[3], const float hi[3], float rc, const float box[3],
                              float pad, int periodic, int rows_sorted, unsigned int cap_max,
                              const unsigned int* map, unsigned int block_size, void* stream,
                              unsigned long long* slots, unsigned int* overflow_rows,
                              unsigned long long* overflow_slots)
    {
    if (!op || !m || !t || !h || !lo || !hi || !box || (N > 0 && !points)) return fail(NBR_ERR_INVALID, "null argument");
    if (!valid_block(block_size)) return fail(NBR_ERR_INVALID, "Invalid tuning parameter.");
    if (cap_max == 0) return fail(NBR_ERR_INVALID, "cap_max must be positive");
    return guarded([&] {
        const neighbor::LBVHTraverser::LaunchParameters p(block_size, as_stream(stream));
        const float3* pts = reinterpret_cast<const float3*>(points);
        neighbor::OnePassNeighborList::Stats st;
        if (map)
            st = op->list.buildLearned(p, h->lbvh, t->trav, m->model, pts, N, f3(lo), f3(hi), rc, f3(box), pad,
                                       periodic != 0, rows_sorted != 0, cap_max, neighbor::MapTransformOp(map));
        else
            st = op->list.buildLearned(p, h->lbvh, t->trav, m->model, pts, N, f3(lo), f3(hi), rc, f3(box), pad,
                                       periodic != 0, rows_sorted != 0, cap_max, neighbor::NullTransformOp());
        if (slots) *slots = st.slots;
        if (overflow_rows) *overflow_rows = st.overflow_rows;
        if (overflow_slots) *overflow_slots = st.overflow_slots;
    });
    }

int nbr_onepass_get(nbr_onepass op, const unsigned int** list, const unsigned long long** offsets,
                    const unsigned int** caps, const unsigned int** nneigh, unsigned long long* total)
    {
    if (!op) return fail(NBR_ERR_INVALID, "null handle");
    if (list) *list = op->list.list();
    if (offsets) *offsets = op->list.offsets();
    if (caps) *caps = op->list.capacities();
    if (nneigh) *nneigh = op->list.nneigh();
    if (total) *total = op->list.totalSlots();
    return NBR_OK;
    }

int nbr_onepass_scan(nbr_onepass op, const unsigned int* counts, unsigned int n, unsigned long long* offsets,
                     unsigned long long* total, void* stream)
    {
    if (!op || (n > 0 && (!counts || !offsets))) return fail(NBR_ERR_INVALID, "null argument");
    return guarded([&] {
        // without a total to return, the scan is only enqueued (no synchronisation)
        const unsigned long long t = n ? op->list.scan(counts, n, offsets, as_stream(stream), total != nullptr) : 0ull;
        if (total) *total = t;
    });
    }

} // extern "C"
