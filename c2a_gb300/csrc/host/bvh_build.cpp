/*
 * bvh_build.cpp -- host build of C2A's RSS hierarchy, one triangle per leaf.
 *
 * Same result, bit for bit, as the reference's C2A_Model::EndModel
 * (C2A/src/C2A_PQP.cpp:332-417) -> C2A_BuildModel (C2A/src/C2A_Build.cpp:
 * 546-574): per node the vertex covariance (C2A_Build.cpp:279-335), its
 * eigenvectors ordered by eigenvalue (394-432), the RSS fit of
 * C2A_BV::FitToTris_Corner (C2A/src/C2A_BV.cpp:354-635) with angularRadius =
 * farthest vertex from the model origin (C2A_BV.cpp:71-111), a split at the
 * mean centroid along the major axis (C2A_Build.cpp:344-385, 456-483), and
 * finally parent-relative R/Tr (C2A_Build.cpp:493-544).  Nodes are numbered in
 * the reference's order (a node's two children are allocated when the node is
 * fitted, the left subtree is built before the right one), so node and
 * triangle indices match the reference's.
 *
 * Subtrees build on parallel host threads when a BuildThreads budget is
 * given.  Every node's fit, sums and partition still run in the reference's
 * order on one thread, and a subtree of k triangles always holds 2k - 1
 * nodes, so each node's number follows from its parent's number and the
 * left part's size alone: the tree is the same bits whatever the threads.
 *
 * PQP's eigen-solver is not part of the reference; the Jacobi sweep below is
 * the one the CPU oracle uses, so both build the same tree.  Compile with
 * -ffp-contract=off.
 */
#include "bvh_build.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <mutex>
#include <new>
#include <stdexcept>
#include <thread>

#include "../../../include/c2a_gb300.h"

namespace c2a {

namespace {

inline double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// v = R^T p (MTxV)
inline void rt_mul(double *v, const double R[3][3], const double *p)
{
    v[0] = R[0][0] * p[0] + R[1][0] * p[1] + R[2][0] * p[2];
    v[1] = R[0][1] * p[0] + R[1][1] * p[1] + R[2][1] * p[2];
    v[2] = R[0][2] * p[0] + R[1][2] * p[1] + R[2][2] * p[2];
}

// v = R p (MxV)
inline void r_mul(double *v, const double R[3][3], const double *p)
{
    v[0] = R[0][0] * p[0] + R[0][1] * p[1] + R[0][2] * p[2];
    v[1] = R[1][0] * p[0] + R[1][1] * p[1] + R[1][2] * p[2];
    v[2] = R[2][0] * p[0] + R[2][1] * p[1] + R[2][2] * p[2];
}

inline double cap_sqrt(double radsqr, double t) { return std::sqrt(radsqr - t > 0 ? radsqr - t : 0); }

struct Tri {
    double p[3][3];
    int32_t id;
    int32_t idx[3];
};

struct AbsNode {
    double R[3][3];
    double Tr[3];
    double To[3]; /* OBB centre, model frame */
    double d[3];  /* OBB half extents */
    double l[2];
    double r;
    double angR;
    int32_t first_child;
    int32_t parent;
    int32_t depth;
};

/* one node still to fit: its triangles tris[first, first+count), and base,
 * the number its first child gets (the reference's allocation counter when
 * this node is fitted) */
struct BuildTask {
    int32_t node, first, count, parent, depth, base;
};

/* subtrees smaller than this stay on the thread that split them */
constexpr int32_t kSpawnGrain = 4096;

class Builder {
  public:
    Builder(RecordVec<Tri> &tris, RecordVec<AbsNode> &nodes, BuildThreads *threads)
        : tris_(tris), nodes_(nodes), threads_(threads)
    {
    }

    void run()
    {
        const BuildTask root{0, 0, (int32_t)tris_.size(), -1, 0, 1};
        if (!threads_ || root.count < 2 * kSpawnGrain) {
            std::vector<double> proj;
            guarded_subtree(root, proj, nullptr);
            return;
        }
        Pool pool;
        pool.queue.push_back(root);
        pool.pending = 1;
        work(pool); // returns once every task is done
        std::vector<std::thread> workers;
        {
            std::lock_guard<std::mutex> lock(pool.mu);
            workers.swap(pool.workers);
        }
        for (std::thread &th : workers) th.join();
    }

  private:
    /* the subtrees waiting for a thread, shared by the build's threads: at
     * most the calling thread plus those taken from the budget, each giving
     * its thread back when the whole tree is done */
    struct Pool {
        std::mutex mu;
        std::condition_variable cv;
        std::vector<BuildTask> queue;
        int pending = 0; /* tasks queued or running */
        int idle = 0;    /* threads waiting for a task */
        std::vector<std::thread> workers;
    };

    void work(Pool &pool)
    {
        std::vector<double> proj;
        for (;;) {
            BuildTask t;
            {
                std::unique_lock<std::mutex> lock(pool.mu);
                while (pool.queue.empty() && pool.pending > 0) {
                    pool.idle++;
                    pool.cv.wait(lock);
                    pool.idle--;
                }
                if (pool.queue.empty()) return; // nothing queued, nothing running: done
                t = pool.queue.back();
                pool.queue.pop_back();
            }
            guarded_subtree(t, proj, &pool);
            std::lock_guard<std::mutex> lock(pool.mu);
            if (--pool.pending == 0) pool.cv.notify_all();
        }
    }

    /* queues subtree t for another thread when one waits for work or can be
     * taken from the budget; false: the caller builds it */
    bool share(Pool &pool, const BuildTask &t)
    {
        std::lock_guard<std::mutex> lock(pool.mu);
        const bool start = pool.idle <= (int)pool.queue.size();
        if (start && !threads_->take()) return false;
        try {
            pool.queue.push_back(t);
        } catch (const std::bad_alloc &) {
            if (start) threads_->give();
            return false;
        }
        pool.pending++;
        if (start) {
            try {
                pool.workers.emplace_back([this, &pool] {
                    work(pool);
                    threads_->give();
                });
            } catch (const std::exception &) { // no thread (system_error) or no room to keep it
                threads_->give();          // the task waits for a thread already running
            }
        }
        pool.cv.notify_one();
        return true;
    }

    void guarded_subtree(const BuildTask &t, std::vector<double> &proj, Pool *pool)
    {
        try {
            build_subtree(t, proj, pool);
        } catch (const std::bad_alloc &) {
            failed_ = true;
        }
    }

    /* builds the subtree of task t0 depth first, left before right; with a
     * pool, a right subtree of at least kSpawnGrain triangles may go to
     * another thread */
    void build_subtree(const BuildTask &t0, std::vector<double> &proj, Pool *pool)
    {
        std::vector<BuildTask> stack;
        stack.push_back(t0);
        while (!stack.empty()) {
            const BuildTask t = stack.back();
            stack.pop_back();
            const int32_t nleft = fit_and_split(t, proj);
            if (t.count == 1) continue;
            // a subtree of k triangles allocates 2k - 2 nodes below its root
            const BuildTask left{t.base, t.first, nleft, t.node, t.depth + 1, t.base + 2};
            const BuildTask right{t.base + 1, t.first + nleft, t.count - nleft, t.node, t.depth + 1,
                                  t.base + 2 * nleft};
            if (!(pool && right.count >= kSpawnGrain && share(*pool, right))) stack.push_back(right);
            stack.push_back(left);
        }
    }

  public:
    bool failed() const { return failed_; }

  private:
    // covariance of the vertices of tris[first, first+n)
    void covariance(double M[3][3], int32_t first, int32_t n) const
    {
        double s1[3] = {0.0, 0.0, 0.0};
        double s00 = 0.0, s11 = 0.0, s22 = 0.0, s01 = 0.0, s02 = 0.0, s12 = 0.0;
        for (int32_t i = first; i < first + n; i++) {
            const double *a = tris_[i].p[0], *b = tris_[i].p[1], *c = tris_[i].p[2];
            s1[0] += a[0] + b[0] + c[0];
            s1[1] += a[1] + b[1] + c[1];
            s1[2] += a[2] + b[2] + c[2];
            s00 += (a[0] * a[0] + b[0] * b[0] + c[0] * c[0]);
            s11 += (a[1] * a[1] + b[1] * b[1] + c[1] * c[1]);
            s22 += (a[2] * a[2] + b[2] * b[2] + c[2] * c[2]);
            s01 += (a[0] * a[1] + b[0] * b[1] + c[0] * c[1]);
            s02 += (a[0] * a[2] + b[0] * b[2] + c[0] * c[2]);
            s12 += (a[1] * a[2] + b[1] * b[2] + c[1] * c[2]);
        }
        const double k = (double)(3 * n);
        M[0][0] = s00 - s1[0] * s1[0] / k;
        M[1][1] = s11 - s1[1] * s1[1] / k;
        M[2][2] = s22 - s1[2] * s1[2] / k;
        M[0][1] = M[1][0] = s01 - s1[0] * s1[1] / k;
        M[1][2] = M[2][1] = s12 - s1[1] * s1[2] / k;
        M[0][2] = M[2][0] = s02 - s1[0] * s1[2] / k;
    }

    // RSS fit of tris[first, first+n) in frame R (FitToTris_Corner, RSS part)
    void fit(AbsNode &b, const double R[3][3], int32_t first, int32_t n, std::vector<double> &proj)
    {
        b.angR = 0.0;
        for (int32_t i = first; i < first + n; i++)
            for (int k = 0; k < 3; k++) {
                const double *p = tris_[i].p[k];
                double d = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
                if (d > b.angR) b.angR = d;
            }
        std::memcpy(b.R, R, sizeof(b.R));
        const int32_t np = 3 * n;
        if (proj.size() < 9 * (size_t)n) proj.resize(9 * (size_t)n);
        double *P = proj.data();
        for (int32_t i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) rt_mul(P + 9 * i + 3 * k, b.R, tris_[first + i].p[k]);
        auto X = [P](int32_t k) { return P[3 * k]; };
        auto Y = [P](int32_t k) { return P[3 * k + 1]; };
        auto Z = [P](int32_t k) { return P[3 * k + 2]; };

        // the OBB in the same frame: projected extents, centre back in the model frame
        {
            double lox = X(0), hix = X(0), loy = Y(0), hiy = Y(0), loz = Z(0), hiz = Z(0);
            for (int32_t i = 1; i < np; i++) {
                if (X(i) < lox) lox = X(i);
                else if (X(i) > hix) hix = X(i);
                if (Y(i) < loy) loy = Y(i);
                else if (Y(i) > hiy) hiy = Y(i);
                if (Z(i) < loz) loz = Z(i);
                else if (Z(i) > hiz) hiz = Z(i);
            }
            const double c[3] = {0.5 * (hix + lox), 0.5 * (hiy + loy), 0.5 * (hiz + loz)};
            r_mul(b.To, b.R, c);
            b.d[0] = 0.5 * (hix - lox);
            b.d[1] = 0.5 * (hiy - loy);
            b.d[2] = 0.5 * (hiz - loz);
        }

        double minz = Z(0), maxz = Z(0);
        for (int32_t i = 1; i < np; i++) {
            if (Z(i) < minz) minz = Z(i);
            else if (Z(i) > maxz) maxz = Z(i);
        }
        b.r = 0.5 * (maxz - minz);
        const double radsqr = b.r * b.r;
        const double cz = 0.5 * (maxz + minz);

        // one in-plane axis: start from the extreme points less their sphere
        // cap, then grow to cover every point's cap
        auto extent = [&](auto coord, double &lo, double &hi) {
            int32_t imin = 0, imax = 0;
            for (int32_t i = 1; i < np; i++) {
                if (coord(i) < coord(imin)) imin = i;
                else if (coord(i) > coord(imax)) imax = i;
            }
            double dz = Z(imin) - cz;
            lo = coord(imin) + cap_sqrt(radsqr, dz * dz);
            dz = Z(imax) - cz;
            hi = coord(imax) - cap_sqrt(radsqr, dz * dz);
            for (int32_t i = 0; i < np; i++)
                if (coord(i) < lo) {
                    dz = Z(i) - cz;
                    double x = coord(i) + cap_sqrt(radsqr, dz * dz);
                    if (x < lo) lo = x;
                }
            for (int32_t i = 0; i < np; i++)
                if (coord(i) > hi) {
                    dz = Z(i) - cz;
                    double x = coord(i) - cap_sqrt(radsqr, dz * dz);
                    if (x > hi) hi = x;
                }
        };
        double minx, maxx, miny, maxy;
        extent(X, minx, maxx);
        extent(Y, miny, maxy);

        // corners: grow diagonally where a point's sphere is not yet covered
        const double a = std::sqrt(0.5);
        for (int32_t i = 0; i < np; i++) {
            const double px = X(i), py = Y(i), dzz = (cz - Z(i)) * (cz - Z(i));
            if (px > maxx) {
                if (py > maxy) {
                    double dx = px - maxx, dy = py - maxy;
                    double u = dx * a + dy * a;
                    double t = (a * u - dx) * (a * u - dx) + (a * u - dy) * (a * u - dy) + dzz;
                    u = u - cap_sqrt(radsqr, t);
                    if (u > 0) {
                        maxx += u * a;
                        maxy += u * a;
                    }
                } else if (py < miny) {
                    double dx = px - maxx, dy = py - miny;
                    double u = dx * a - dy * a;
                    double t = (a * u - dx) * (a * u - dx) + (-a * u - dy) * (-a * u - dy) + dzz;
                    u = u - cap_sqrt(radsqr, t);
                    if (u > 0) {
                        maxx += u * a;
                        miny -= u * a;
                    }
                }
            } else if (px < minx) {
                if (py > maxy) {
                    double dx = px - minx, dy = py - maxy;
                    double u = dy * a - dx * a;
                    double t = (-a * u - dx) * (-a * u - dx) + (a * u - dy) * (a * u - dy) + dzz;
                    u = u - cap_sqrt(radsqr, t);
                    if (u > 0) {
                        minx -= u * a;
                        maxy += u * a;
                    }
                } else if (py < miny) {
                    double dx = px - minx, dy = py - miny;
                    double u = -dx * a - dy * a;
                    double t = (-a * u - dx) * (-a * u - dx) + (-a * u - dy) * (-a * u - dy) + dzz;
                    u = u - cap_sqrt(radsqr, t);
                    if (u > 0) {
                        minx -= u * a;
                        miny -= u * a;
                    }
                }
            }
        }
        const double c[3] = {minx, miny, cz};
        r_mul(b.Tr, b.R, c);
        b.l[0] = maxx - minx;
        if (b.l[0] < 0) b.l[0] = 0;
        b.l[1] = maxy - miny;
        if (b.l[1] < 0) b.l[1] = 0;
    }

    // fits node t.node to its triangles; for more than one numbers its
    // children t.base, t.base + 1 and partitions the range; returns the size
    // of the left part
    int32_t fit_and_split(const BuildTask &t, std::vector<double> &proj)
    {
        const int32_t first = t.first, n = t.count;
        double C[3][3], E[3][3], s[3], R[3][3];
        covariance(C, first, n);
        jacobi_eigen3(E, s, C);
        int mn, mid, mx;
        if (s[0] > s[1]) {
            mx = 0;
            mn = 1;
        } else {
            mn = 0;
            mx = 1;
        }
        if (s[2] < s[mn]) {
            mid = mn;
            mn = 2;
        } else if (s[2] > s[mx]) {
            mid = mx;
            mx = 2;
        } else {
            mid = 2;
        }
        for (int i = 0; i < 3; i++) {
            R[i][0] = E[i][mx];
            R[i][1] = E[i][mid];
        }
        R[0][2] = E[1][mx] * E[2][mid] - E[1][mid] * E[2][mx];
        R[1][2] = E[0][mid] * E[2][mx] - E[0][mx] * E[2][mid];
        R[2][2] = E[0][mx] * E[1][mid] - E[0][mid] * E[1][mx];

        AbsNode &b = nodes_[t.node];
        b.parent = t.parent;
        b.depth = t.depth;
        fit(b, R, first, n, proj);
        if (n == 1) {
            b.first_child = -(first + 1);
            return 1;
        }
        b.first_child = t.base;

        // split at the mean vertex along the major axis; centroids <= mean go left
        const double axis[3] = {R[0][0], R[1][0], R[2][0]};
        double m[3] = {0.0, 0.0, 0.0};
        for (int32_t i = first; i < first + n; i++)
            for (int k = 0; k < 3; k++) m[k] += tris_[i].p[0][k] + tris_[i].p[1][k] + tris_[i].p[2][k];
        const double cnt = (double)(3 * n);
        m[0] /= cnt;
        m[1] /= cnt;
        m[2] /= cnt;
        const double coord = dot3(axis, m);
        int32_t left = 0;
        for (int32_t i = first; i < first + n; i++) {
            double c[3];
            for (int k = 0; k < 3; k++) c[k] = tris_[i].p[0][k];
            for (int k = 0; k < 3; k++) c[k] = c[k] + tris_[i].p[1][k];
            for (int k = 0; k < 3; k++) c[k] = c[k] + tris_[i].p[2][k];
            double x = dot3(c, axis);
            x /= 3.0;
            if (x <= coord) {
                std::swap(tris_[i], tris_[first + left]);
                left++;
            }
        }
        if (left == 0 || left == n) left = n / 2;
        return left;
    }

    RecordVec<Tri> &tris_;
    RecordVec<AbsNode> &nodes_;
    BuildThreads *threads_;
    std::atomic<bool> failed_{false}; /* a thread ran out of memory */
};

} // namespace

void jacobi_eigen3(double v[3][3], double d[3], const double a_in[3][3])
{
    double a[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            a[i][j] = a_in[i][j];
            v[i][j] = (i == j) ? 1.0 : 0.0;
        }
    for (int sweep = 0; sweep < 50; sweep++) {
        if (std::fabs(a[0][1]) + std::fabs(a[0][2]) + std::fabs(a[1][2]) == 0.0) break;
        for (int p = 0; p < 2; p++)
            for (int q = p + 1; q < 3; q++) {
                const double apq = a[p][q], app = a[p][p], aqq = a[q][q];
                if (apq == 0.0) continue;
                if (sweep > 3 && std::fabs(app) + 100.0 * std::fabs(apq) == std::fabs(app) &&
                    std::fabs(aqq) + 100.0 * std::fabs(apq) == std::fabs(aqq)) {
                    a[p][q] = a[q][p] = 0.0;
                    continue;
                }
                // rotation zeroing a[p][q]: t = tan of the smaller root angle
                const double theta = (aqq - app) / (2.0 * apq);
                double t = 1.0 / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                if (theta < 0.0) t = -t;
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                a[p][p] = app - t * apq;
                a[q][q] = aqq + t * apq;
                a[p][q] = a[q][p] = 0.0;
                const int r = 3 - p - q;
                const double arp = a[r][p], arq = a[r][q];
                a[r][p] = a[p][r] = c * arp - s * arq;
                a[r][q] = a[q][r] = s * arp + c * arq;
                for (int k = 0; k < 3; k++) {
                    const double vkp = v[k][p], vkq = v[k][q];
                    v[k][p] = c * vkp - s * vkq;
                    v[k][q] = s * vkp + c * vkq;
                }
            }
    }
    d[0] = a[0][0];
    d[1] = a[1][1];
    d[2] = a[2][2];
}

namespace {
/* FP32 rounding of an FP64 value; flags values outside FP32's normal range */
float shadow_of(double x, bool &ok)
{
    const double a = std::fabs(x);
    if (a != 0.0 && (a < (double)FLT_MIN || a > (double)FLT_MAX)) ok = false;
    return (float)x;
}
} // namespace

bool BuildThreads::take()
{
    int f = free_.load(std::memory_order_relaxed);
    while (f > 0)
        if (free_.compare_exchange_weak(f, f - 1, std::memory_order_acq_rel)) return true;
    return false;
}

void BuildThreads::give() { free_.fetch_add(1, std::memory_order_acq_rel); }

namespace {

constexpr int kMaxParts = 64;           /* at most this many threads per record pass */
constexpr int64_t kPartMin = 16384;     /* records a thread of such a pass handles at least */

/* body(part, lo, hi) over [0, n) in contiguous parts: part 0 on the calling
 * thread, the others on threads taken from the budget (given back after) */
template <class Body> void parallel_parts(int64_t n, BuildThreads *threads, Body body)
{
    std::vector<std::thread> pool;
    std::vector<int> here; // parts no thread could be started for
    pool.reserve(kMaxParts);
    here.reserve(kMaxParts);
    int extra = 0;
    while (threads && extra + 1 < kMaxParts && (int64_t)(extra + 2) * kPartMin <= n && threads->take()) extra++;
    const int parts = extra + 1;
    for (int p = 1; p < parts; p++) {
        const int64_t lo = n * p / parts, hi = n * (p + 1) / parts;
        try {
            pool.emplace_back([&body, p, lo, hi] { body(p, lo, hi); });
        } catch (const std::exception &) {
            here.push_back(p);
        }
    }
    body(0, 0, n / parts);
    for (int p : here) body(p, n * p / parts, n * (p + 1) / parts);
    for (std::thread &th : pool) th.join();
    for (int p = 0; p < extra; p++) threads->give();
}

int build_unchecked(int32_t num_tris, const double *tv, const int32_t *ids, const int32_t *vidx, BuiltModel &out,
                    BuildThreads *threads)
{
    RecordVec<Tri> tris((size_t)num_tris);
    parallel_parts(num_tris, threads, [&](int, int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; i++) {
            std::memcpy(tris[i].p, tv + 9 * (size_t)i, sizeof(tris[i].p));
            tris[i].id = ids ? ids[i] : (int32_t)i;
            for (int k = 0; k < 3; k++) tris[i].idx[k] = vidx ? vidx[3 * (size_t)i + k] : -1;
        }
    });
    const int32_t num_nodes = 2 * num_tris - 1;
    RecordVec<AbsNode> nodes((size_t)num_nodes); // every field set by the build
    {
        Builder b(tris, nodes, threads);
        b.run();
        if (b.failed()) return C2A_ERR_OUT_OF_MEMORY;
    }

    // resized without clearing: the passes below write every byte
    out.nodes.resize((size_t)num_nodes);
    out.obbs.resize((size_t)num_nodes);
    out.tris.resize((size_t)num_tris);
    out.snodes.resize((size_t)num_nodes);
    out.stris.resize((size_t)num_tris);
    // every node and triangle record depends on its own node (and parent) only
    std::vector<int32_t> part_depth(kMaxParts, 0);
    std::vector<char> part_ok(kMaxParts, 1);
    parallel_parts(num_nodes, threads, [&](int part, int64_t lo, int64_t hi) {
        bool ok = true;
        int32_t depth = 0;
        for (int64_t i = lo; i < hi; i++) {
            const AbsNode &b = nodes[i];
            NodeRec &o = out.nodes[i];
            // parent-relative frame: R = Rp^T R, Tr = Rp^T (Tr - Trp); the root is
            // taken relative to the identity exactly as the reference does
            static const double I[3][3] = {{1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 1.0}};
            static const double Z[3] = {0.0, 0.0, 0.0};
            const double(*PR)[3] = b.parent >= 0 ? nodes[b.parent].R : I;
            const double *PT = b.parent >= 0 ? nodes[b.parent].Tr : Z;
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) {
                    o.R[3 * r + c] = PR[0][r] * b.R[0][c] + PR[1][r] * b.R[1][c] + PR[2][r] * b.R[2][c];
                    o.Rloc[3 * r + c] = b.R[r][c];
                }
            const double d[3] = {b.Tr[0] - PT[0], b.Tr[1] - PT[1], b.Tr[2] - PT[2]};
            rt_mul(o.Tr, PR, d);
            const double *PTo = b.parent >= 0 ? nodes[b.parent].To : Z;
            const double dO[3] = {b.To[0] - PTo[0], b.To[1] - PTo[1], b.To[2] - PTo[2]};
            rt_mul(out.obbs[i].To, PR, dO);
            for (int k = 0; k < 3; k++) out.obbs[i].d[k] = b.d[k];
            o.l[0] = b.l[0];
            o.l[1] = b.l[1];
            o.r = b.r;
            o.angR = b.angR;
            o.size = std::sqrt(b.l[0] * b.l[0] + b.l[1] * b.l[1]) + 2 * b.r;
            o.first_child = b.first_child;
            o.depth = b.depth;
            std::memset(o.pad, 0, sizeof(o.pad));
            if (b.depth > depth) depth = b.depth;
            NodeShadow &sh = out.snodes[i];
            for (int k = 0; k < 9; k++) {
                sh.R[k] = shadow_of(o.R[k], ok);
                sh.Rloc[k] = shadow_of(o.Rloc[k], ok);
            }
            for (int k = 0; k < 3; k++) sh.Tr[k] = shadow_of(o.Tr[k], ok);
            sh.l[0] = shadow_of(o.l[0], ok);
            sh.l[1] = shadow_of(o.l[1], ok);
            sh.r = shadow_of(o.r, ok);
            sh.angR = shadow_of(o.angR, ok);
            std::memset(sh.pad, 0, sizeof(sh.pad));
        }
        part_depth[part] = depth;
        part_ok[part] = ok;
    });
    out.depth = 0;
    bool ok = true;
    for (int p = 0; p < kMaxParts; p++) {
        if (part_depth[p] > out.depth) out.depth = part_depth[p];
        ok = ok && part_ok[p];
    }
    std::fill(part_ok.begin(), part_ok.end(), 1);
    parallel_parts(num_tris, threads, [&](int part, int64_t lo, int64_t hi) {
        bool tok = true;
        for (int64_t i = lo; i < hi; i++) {
            TriRec &t = out.tris[i];
            std::memcpy(t.v, tris[i].p, sizeof(t.v));
            t.id = tris[i].id;
            for (int k = 0; k < 3; k++) t.idx[k] = tris[i].idx[k];
            t.pad = 0.0;
            for (int k = 0; k < 9; k++) out.stris[i].v[k] = shadow_of(t.v[k], tok);
            std::memset(out.stris[i].pad, 0, sizeof(out.stris[i].pad));
        }
        part_ok[part] = tok;
    });
    for (int p = 0; p < kMaxParts; p++) ok = ok && part_ok[p];
    out.shadow_ok = ok;
    return 0;
}

} // namespace

int build_rss_model(int32_t num_tris, const double *tv, const int32_t *ids, const int32_t *vidx, BuiltModel &out,
                    BuildThreads *threads)
{
    if (num_tris <= 0 || !tv) return C2A_ERR_EMPTY_MODEL;
    try {
        return build_unchecked(num_tris, tv, ids, vidx, out, threads);
    } catch (const std::bad_alloc &) {
        out = BuiltModel{};
        return C2A_ERR_OUT_OF_MEMORY;
    }
}

} // namespace c2a
