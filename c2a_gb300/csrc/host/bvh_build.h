/*
 * bvh_build.h -- host build of C2A's RSS bounding-volume hierarchy and the
 * node/triangle records the kernels read from HBM.
 */
#ifndef C2A_BVH_BUILD_H
#define C2A_BVH_BUILD_H

#include <atomic>
#include <cstdint>
#include <memory>
#include <new>
#include <utility>
#include <vector>

namespace c2a {

/*
 * One BVH node as the CUDA kernels load it: 256 bytes, 16-byte aligned so a
 * node is thirteen 128-bit loads, two 128-byte lines.  Fields are those the CA
 * path reads from C2A_BV (C2A/C2A_BV.h:33-77, PQP BV): parent-relative R and
 * Tr, rectangle lengths l, radius r, angularRadius, build-time R_loc, plus
 * the split measure GetSize() = |l| + 2r precomputed with the same
 * arithmetic.
 */
struct alignas(16) NodeRec {
    double R[9];
    double Tr[3];
    double l[2];
    double r;
    double angR;
    double Rloc[9];
    double size;
    int32_t first_child; /* >= 0: first of two children; < 0: -(triangle) - 1 */
    int32_t depth;       /* depth below the root */
    double pad[5];
};
static_assert(sizeof(NodeRec) == 256, "node record must stay 256 bytes");

/* One triangle, post-build order: vertices, caller id, caller vertex indices. */
struct alignas(16) TriRec {
    double v[9];
    int32_t id;
    int32_t idx[3];
    double pad;
};
static_assert(sizeof(TriRec) == 96, "triangle record must stay 96 bytes");

/* FP32 shadows of the same records, rounded to nearest, for the kernels'
 * certified FP32 filter (112 and 48 bytes). */
struct alignas(16) NodeShadow {
    float R[9];
    float Tr[3];
    float l[2];
    float r;
    float angR;
    float Rloc[9];
    float pad[3];
};
static_assert(sizeof(NodeShadow) == 112, "node shadow must stay 112 bytes");
struct alignas(16) TriShadow {
    float v[9];
    float pad[3];
};
static_assert(sizeof(TriShadow) == 48, "triangle shadow must stay 48 bytes");

/* The node's OBB (the static collide query's bounding volume, fitted in the
 * RSS frame, C2A/src/C2A_BV.cpp:144-170): centre To relative to the parent
 * (as make_parent_relative stores it) and half extents d. */
struct alignas(16) ObbRec {
    double To[3];
    double d[3];
};
static_assert(sizeof(ObbRec) == 48, "OBB record must stay 48 bytes");

/* std::allocator whose value-less construct leaves a record unset, so that
 * resize() does not clear memory the build then writes in full on parallel
 * threads (each page is first touched by the thread that fills it) */
template <class T> struct RecordAlloc : std::allocator<T> {
    template <class U> struct rebind {
        using other = RecordAlloc<U>;
    };
    RecordAlloc() = default;
    template <class U> RecordAlloc(const RecordAlloc<U> &) noexcept {}
    template <class U> void construct(U *p) noexcept { ::new ((void *)p) U; }
    template <class U, class... A> void construct(U *p, A &&...a) { ::new ((void *)p) U(std::forward<A>(a)...); }
};
template <class T> using RecordVec = std::vector<T, RecordAlloc<T>>;

struct BuiltModel {
    RecordVec<ObbRec> obbs;
    RecordVec<NodeRec> nodes;
    RecordVec<TriRec> tris;
    RecordVec<NodeShadow> snodes;
    RecordVec<TriShadow> stris;
    bool shadow_ok = true; /* every shadowed value lies in FP32's normal range (or is 0) */
    int32_t depth = 0;     /* maximum node depth (root = 0) */
};

/* Host threads a build may start for its subtrees, beyond the calling one;
 * one budget can be shared by builds running at the same time. */
class BuildThreads {
  public:
    explicit BuildThreads(int extra) : free_(extra > 0 ? extra : 0) {}
    bool take(); /* one thread, if any is left */
    void give(); /* a thread taken before, or one the caller lends */

  private:
    std::atomic<int> free_;
};

/* C2A_Model::EndModel + C2A_BuildModel: returns 0 or a C2A_ERR_* code.
 * threads: the budget for subtree threads (nullptr: this thread only); the
 * tree is the same either way. */
int build_rss_model(int32_t num_tris, const double *tri_verts, const int32_t *ids, const int32_t *vidx,
                    BuiltModel &out, BuildThreads *threads = nullptr);

/* Symmetric 3x3 eigen-decomposition (columns of v are eigenvectors). */
void jacobi_eigen3(double v[3][3], double d[3], const double a[3][3]);

} // namespace c2a
#endif
