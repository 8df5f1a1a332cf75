// User-written ops through the C++ template API (include/neighbor/neighbor.h), not the C ABI.
//
// The reference's callers instantiate LBVH::build and LBVHTraverser::traverse with ops of their
// own.  This program does the same with:
//   - the double-precision particle ops of the reference's benchmark
//     (benchmark/lbvh_benchmark.cuh:25-92): ParticleInsertOp over Scalar4 particles (a point box
//     rounded outward to FP32) and ParticleQueryOp over Scalar4 spheres (refine() == true);
//   - a user exact query (ExactParticleQueryOp: double minimum-image distance in refine()) and a
//     user output op (NearestOp: count, sum of ids and the nearest other particle of each query);
//   - 27 double3 image vectors through ImageListOp<double3>;
//   - the three-point sequence of the reference's test (test/lbvh_test.cu:17-315: two streams,
//     the tree getters, getData(), CountNeighborsOp, NeighborListOp with max_neigh 2 and a
//     MapTransformOp) driven through the same class templates.
//
//   user_ops kat OUT.json                      the three-point sequence's results
//   user_ops ops IN.f64 N L r OUT_PREFIX       the particle ops on N Scalar4 particles in a
//                                              periodic cube of side L, cutoff r
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "neighbor/neighbor.h"

namespace
{
// HOOMD-blue's Scalar4 with Scalar = double (CUDA 13 names the 16-byte aligned double4 so)
typedef double4_16a Scalar4;

inline Scalar4 make_scalar4(double x, double y, double z, double w)
    {
    Scalar4 v;
    v.x = x;
    v.y = y;
    v.z = z;
    v.w = w;
    return v;
    }

void check(cudaError_t e, const char* what)
    {
    if (e != cudaSuccess)
        {
        fprintf(stderr, "CUDA error %s: %s\n", what, cudaGetErrorString(e));
        exit(2);
        }
    }

// benchmark/lbvh_benchmark.cuh:25-49 with Scalar = double
struct ParticleInsertOp
    {
    ParticleInsertOp(const Scalar4* particles_, unsigned int N_) : particles(particles_), N(N_) {}
    __device__ __forceinline__ neighbor::BoundingBox get(const unsigned int idx) const
        {
        const Scalar4 particle = particles[idx];
        const double3 p = make_double3(particle.x, particle.y, particle.z);
        return neighbor::BoundingBox(p, p);
        }
    __host__ __device__ __forceinline__ unsigned int size() const { return N; }
    const Scalar4* particles;
    const unsigned int N;
    };

// benchmark/lbvh_benchmark.cuh:51-92 with Scalar = double
struct ParticleQueryOp
    {
    ParticleQueryOp(const Scalar4* spheres_, unsigned int N_) : spheres(spheres_), N(N_) {}
    typedef Scalar4 ThreadData;
    typedef neighbor::BoundingSphere Volume;
    __device__ __forceinline__ ThreadData setup(const unsigned int idx) const { return spheres[idx]; }
    __device__ __forceinline__ Volume get(const ThreadData& q, const double3 image) const
        {
        const double3 t = make_double3(q.x + image.x, q.y + image.y, q.z + image.z);
        return neighbor::BoundingSphere(t, q.w);
        }
    __device__ __forceinline__ bool overlap(const Volume& v, const neighbor::BoundingBox& box) const
        {
        return v.overlap(box);
        }
    __device__ __forceinline__ bool refine(const ThreadData&, const int) const { return true; }
    __host__ __device__ __forceinline__ unsigned int size() const { return N; }
    const Scalar4* spheres;
    const unsigned int N;
    };

// Minimum image of one component in double (wrap once by L when |d| reaches L/2).
__device__ __forceinline__ double wrap(double d, double L)
    {
    const double h = __dmul_rn(0.5, L);
    if (d >= h) return __dsub_rn(d, L);
    if (d < -h) return __dadd_rn(d, L);
    return d;
    }

__device__ __forceinline__ double dist2(const Scalar4& a, const Scalar4& b, double L)
    {
    const double dx = wrap(__dsub_rn(b.x, a.x), L);
    const double dy = wrap(__dsub_rn(b.y, a.y), L);
    const double dz = wrap(__dsub_rn(b.z, a.z), L);
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    }

// A user query: the particle query with an exact refine() (double minimum-image distance).
struct ExactParticleQueryOp : ParticleQueryOp
    {
    ExactParticleQueryOp(const Scalar4* spheres_, unsigned int N_, const Scalar4* particles_, double L_)
        : ParticleQueryOp(spheres_, N_), particles(particles_), L(L_)
        {}
    __device__ __forceinline__ bool refine(const ThreadData& q, const int primitive) const
        {
        return dist2(q, particles[primitive], L) <= __dmul_rn(q.w, q.w);
        }
    const Scalar4* particles;
    double L;
    };

// A user output op: per query the number of accepted particles, the sum of their ids and the
// nearest one other than the query itself (ties to the smaller id).
struct NearestOp
    {
    NearestOp(unsigned int* count_, unsigned long long* idsum_, int* nearest_, const Scalar4* particles_, double L_)
        : count(count_), idsum(idsum_), nearest(nearest_), particles(particles_), L(L_)
        {}
    struct ThreadData
        {
        unsigned int idx;
        Scalar4 q;
        unsigned int n;
        unsigned long long sum;
        int best;
        double best_d2;
        };
    __device__ __forceinline__ ThreadData setup(const unsigned int idx, const Scalar4& q) const
        {
        ThreadData t;
        t.idx = idx;
        t.q = q;
        t.n = 0;
        t.sum = 0;
        t.best = -1;
        t.best_d2 = 0.0;
        return t;
        }
    __device__ __forceinline__ void process(ThreadData& t, const int primitive) const
        {
        ++t.n;
        t.sum += (unsigned long long)primitive;
        if ((unsigned int)primitive == t.idx) return;
        const double d2 = dist2(t.q, particles[primitive], L);
        if (t.best < 0 || d2 < t.best_d2 || (d2 == t.best_d2 && primitive < t.best))
            {
            t.best = primitive;
            t.best_d2 = d2;
            }
        }
    __device__ __forceinline__ void finalize(const ThreadData& t) const
        {
        count[t.idx] = t.n;
        idsum[t.idx] = t.sum;
        nearest[t.idx] = t.best;
        }
    unsigned int* count;
    unsigned long long* idsum;
    int* nearest;
    const Scalar4* particles;
    double L;
    };

template<class T>
void write_json_array(FILE* f, const char* name, const T* v, size_t n, bool last = false)
    {
    fprintf(f, "\"%s\": [", name);
    for (size_t i = 0; i < n; ++i) fprintf(f, "%s%lld", i ? ", " : "", (long long)v[i]);
    fprintf(f, "]%s\n", last ? "" : ",");
    }

int run_kat(const char* out_path)
    {
    // test/lbvh_test.cu:26-51
    neighbor::shared_array<float3> points(3);
    points[0] = make_float3(2.5f, 0.f, 0.f);
    points[1] = make_float3(1.5f, 0.f, 0.f);
    points[2] = make_float3(0.5f, 0.f, 0.f);
    neighbor::shared_array<float4> spheres(7);
    spheres[0] = make_float4(0.5f, 0.f, 0.f, 0.5f);
    spheres[1] = make_float4(1.5f, 0.f, 0.f, 0.5f);
    spheres[2] = make_float4(2.5f, 0.f, 0.f, 0.5f);
    spheres[3] = make_float4(1.0f, 0.f, 0.f, 1.0f);
    spheres[4] = make_float4(2.0f, 0.f, 0.f, 1.0f);
    spheres[5] = make_float4(1.5f, 0.f, 0.f, 1.5f);
    spheres[6] = make_float4(-0.5f, 0.f, 0.f, 0.5f);
    cudaStream_t streams[2];
    check(cudaStreamCreate(&streams[0]), "stream");
    streams[1] = 0;
    FILE* f = fopen(out_path, "w");
    if (!f) return 3;
    fprintf(f, "{\n\"builds\": [\n");
    std::vector<neighbor::LBVH*> trees;
    for (int s = 0; s < 2; ++s)
        {
        neighbor::LBVH* lbvh = new neighbor::LBVH();
        lbvh->build(streams[s], neighbor::PointInsertOp(points.get(), 3), make_float3(0, 0, 0),
                    make_float3(1024, 1024, 1024));
        check(cudaStreamSynchronize(streams[s]), "sync");
        const auto& par = lbvh->getParents();
        const auto& lft = lbvh->getLeftChildren();
        const auto& rgt = lbvh->getRightChildren();
        const auto& prim = lbvh->getPrimitives();
        const auto& lo = lbvh->getLowerBounds();
        const auto& hi = lbvh->getUpperBounds();
        check(cudaDeviceSynchronize(), "sync");
        fprintf(f, "{\"N\": %u, \"root\": %d,\n", lbvh->getN(), lbvh->getRoot());
        write_json_array(f, "parents", par.get(), par.size());
        write_json_array(f, "left", lft.get(), lft.size());
        write_json_array(f, "right", rgt.get(), rgt.size());
        write_json_array(f, "primitives", prim.get(), prim.size());
        fprintf(f, "\"lo_x\": [");
        for (size_t i = 0; i < lo.size(); ++i) fprintf(f, "%s%.9g", i ? ", " : "", lo[i].x);
        fprintf(f, "], \"hi_x\": [");
        for (size_t i = 0; i < hi.size(); ++i) fprintf(f, "%s%.9g", i ? ", " : "", hi[i].x);
        fprintf(f, "]}%s\n", s == 0 ? "," : "");
        trees.push_back(lbvh);
        }
    fprintf(f, "],\n");
    neighbor::LBVH& lbvh = *trees[1];

    // counts and the compressed nodes (test/lbvh_test.cu:121-199)
        {
        neighbor::LBVHTraverser traverser;
        neighbor::shared_array<unsigned int> hits(7);
        traverser.traverse(lbvh, neighbor::SphereQueryOp(spheres.get(), 7), neighbor::CountNeighborsOp(hits.get()));
        check(cudaDeviceSynchronize(), "sync");
        const auto& data = traverser.getData();
        std::vector<int> lox, hix, z, w;
        for (int i = 0; i < 5; ++i)
            {
            const int4 nd = data[i];
            lox.push_back((int)(((unsigned int)nd.x >> 20) & 0x3ffu));
            hix.push_back((int)(((unsigned int)nd.y >> 20) & 0x3ffu));
            z.push_back(nd.z);
            w.push_back(nd.w);
            }
        write_json_array(f, "hits", hits.get(), 7);
        write_json_array(f, "lo_x_bin", lox.data(), 5);
        write_json_array(f, "hi_x_bin", hix.data(), 5);
        write_json_array(f, "node_z", z.data(), 5);
        write_json_array(f, "node_w", w.data(), 5);
        }

    // neighbor lists with max_neigh 2 on both streams (test/lbvh_test.cu:202-251)
    fprintf(f, "\"nlists\": [\n");
    for (int s = 0; s < 2; ++s)
        {
        neighbor::LBVHTraverser traverser;
        const unsigned int max_neigh = 2;
        neighbor::shared_array<unsigned int> list(max_neigh * 7), nneigh(7);
        for (size_t i = 0; i < list.size(); ++i) list[i] = 0xffffffffu;
        traverser.traverse(streams[s], lbvh, neighbor::SphereQueryOp(spheres.get(), 7),
                           neighbor::NeighborListOp(list.get(), nneigh.get(), max_neigh));
        check(cudaStreamSynchronize(streams[s]), "sync");
        fprintf(f, "{");
        write_json_array(f, "nneigh", nneigh.get(), 7);
        write_json_array(f, "list", list.get(), list.size(), true);
        fprintf(f, "}%s\n", s == 0 ? "," : "");
        }
    fprintf(f, "],\n");

    // the map transform (test/lbvh_test.cu:253-312)
        {
        neighbor::LBVHTraverser traverser;
        neighbor::shared_array<unsigned int> map(7);
        map[0] = 2;
        map[1] = 1;
        map[2] = 0;
        const unsigned int max_neigh = 2;
        neighbor::shared_array<unsigned int> list(max_neigh * 7), nneigh(7);
        for (size_t i = 0; i < list.size(); ++i) list[i] = 0xffffffffu;
        traverser.traverse(lbvh, neighbor::SphereQueryOp(spheres.get(), 7),
                           neighbor::NeighborListOp(list.get(), nneigh.get(), max_neigh), neighbor::SelfOp(),
                           neighbor::MapTransformOp(map.get()));
        check(cudaDeviceSynchronize(), "sync");
        fprintf(f, "\"mapped\": {");
        write_json_array(f, "nneigh", nneigh.get(), 7);
        write_json_array(f, "list", list.get(), list.size(), true);
        fprintf(f, "}\n}\n");
        }
    fclose(f);
    for (auto* t : trees) delete t;
    check(cudaStreamDestroy(streams[0]), "stream");
    return 0;
    }

int run_ops(const char* in_path, unsigned int N, double L, double r, const char* prefix)
    {
    std::vector<Scalar4> hp(N);
    FILE* f = fopen(in_path, "rb");
    if (!f || fread(hp.data(), sizeof(Scalar4), N, f) != N) return 5;
    fclose(f);
    neighbor::shared_array<Scalar4> particles(N), spheres(N);
    for (unsigned int i = 0; i < N; ++i)
        {
        particles[i] = hp[i];
        spheres[i] = make_scalar4(hp[i].x, hp[i].y, hp[i].z, r);
        }
    neighbor::shared_array<double3> images(27);
    unsigned int k = 0;
    for (int ix = -1; ix <= 1; ++ix)
        for (int iy = -1; iy <= 1; ++iy)
            for (int iz = -1; iz <= 1; ++iz) images[k++] = make_double3(L * ix, L * iy, L * iz);
    const float Lf = (float)L;

    neighbor::LBVH lbvh;
    cudaStream_t st;
    check(cudaStreamCreate(&st), "stream");
    lbvh.build(neighbor::LBVH::LaunchParameters(128, st), ParticleInsertOp(particles.get(), N),
               make_float3(0.f, 0.f, 0.f), make_float3(Lf, Lf, Lf));
    neighbor::LBVHTraverser traverser;
    neighbor::shared_array<unsigned int> superset(N), count(N);
    neighbor::shared_array<unsigned long long> idsum(N);
    neighbor::shared_array<int> nearest(N);
    const neighbor::ImageListOp<double3> img(images.get(), 27);
    traverser.traverse(neighbor::LBVHTraverser::LaunchParameters(256, st), lbvh, ParticleQueryOp(spheres.get(), N),
                       neighbor::CountNeighborsOp(superset.get()), img);
    traverser.traverse(neighbor::LBVHTraverser::LaunchParameters(64, st), lbvh,
                       ExactParticleQueryOp(spheres.get(), N, particles.get(), L),
                       NearestOp(count.get(), idsum.get(), nearest.get(), particles.get(), L), img);
    // the same particles as double self queries with the library's exact double op: a tree of
    // PointInsertOpF64 and the two-pass list of traverseSelfF64 (count, largest count on the host,
    // fill), rows by particle index
    neighbor::shared_array<double3> pos(N);
    for (unsigned int i = 0; i < N; ++i) pos[i] = make_double3(hp[i].x, hp[i].y, hp[i].z);
    neighbor::LBVH lbvh64;
    lbvh64.build(neighbor::LBVH::LaunchParameters(256, st), neighbor::PointInsertOpF64(pos.get(), N),
                 make_float3(0.f, 0.f, 0.f), make_float3(Lf, Lf, Lf));
    neighbor::LBVHTraverser self_traverser;
    const neighbor::LBVHTraverser::LaunchParameters lp(256, st);
    const float pad = neighbor::exact_query_pad((float)r, 2.f * Lf);
    const double3 box64 = make_double3(L, L, L);
    neighbor::shared_array<unsigned int> self_count(N);
    self_traverser.traverseSelfF64(lp, lbvh64, pos.get(), r, box64, pad, neighbor::CountNeighborsOp(self_count.get()),
                                   neighbor::PeriodicImagesOp(make_float3(Lf, Lf, Lf)), neighbor::NullTransformOp(),
                                   false);
    unsigned int max_count = 0, past = 0;
    unsigned long long total = 0;
    self_traverser.readCountSummary(st, max_count, total, past);
    const unsigned int stride = max_count > 0 ? max_count : 1u;
    neighbor::shared_array<unsigned int> self_list((size_t)N * stride), self_rows(N);
    self_traverser.traverseSelfF64(lp, lbvh64, pos.get(), r, box64, pad,
                                   neighbor::NeighborListOp(self_list.get(), self_rows.get(), stride),
                                   neighbor::PeriodicImagesOp(make_float3(Lf, Lf, Lf)), neighbor::NullTransformOp(),
                                   false);
    check(cudaStreamSynchronize(st), "sync");
    check(cudaStreamDestroy(st), "stream");
    std::vector<unsigned long long> self_idsum(N, 0ull);
    for (unsigned int i = 0; i < N; ++i)
        for (unsigned int k = 0; k < self_rows[i] && k < stride; ++k) self_idsum[i] += self_list[(size_t)i * stride + k];
    auto dump = [&](const char* name, const void* p, size_t bytes) {
        const std::string path = std::string(prefix) + "." + name;
        FILE* o = fopen(path.c_str(), "wb");
        fwrite(p, 1, bytes, o);
        fclose(o);
    };
    dump("superset", superset.get(), (size_t)N * 4);
    dump("count", count.get(), (size_t)N * 4);
    dump("idsum", idsum.get(), (size_t)N * 8);
    dump("nearest", nearest.get(), (size_t)N * 4);
    dump("self_count", self_rows.get(), (size_t)N * 4);
    dump("self_idsum", self_idsum.data(), (size_t)N * 8);
    printf("{\"ops\": %u}\n", N);
    return 0;
    }
} // namespace

int main(int argc, char** argv)
    {
    if (argc >= 3 && std::string(argv[1]) == "kat") return run_kat(argv[2]);
    if (argc >= 7 && std::string(argv[1]) == "ops")
        return run_ops(argv[2], (unsigned int)atol(argv[3]), atof(argv[4]), atof(argv[5]), argv[6]);
    fprintf(stderr, "usage: user_ops kat OUT.json | user_ops ops IN.f64 N L r OUT_PREFIX\n");
    return 1;
    }
