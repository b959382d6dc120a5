/*
 * k_static.cu -- the static proximity queries beside the CA path, one thread
 * per pair of placed models, FP64 in the reference's depth-first order:
 *
 *   C2A_Tolerance with qsize 2 (C2A/src/C2A_PQP.cpp:1762-1845 and its
 *   C2AToleranceRecurse, 1498-1603): the root RSS distance as a trivial
 *   reject, then the node pairs with the closer child first, stopping at the
 *   first triangle pair within the tolerance;
 *   C2A_Collide (C2A_PQP.cpp:910-968 and CollideRecurse, 798-909): the
 *   overlapping OBB pairs, first child before second, every triangle pair at
 *   distance zero recorded in visiting order (or the first only).
 *
 * Node tests, transforms and triangle distances are the ones the CA kernels
 * use (geom.cuh), so the results are the reference's bit for bit.
 */
#include "device/ca_kernel.cuh"
#include "kernels.h"

using namespace c2a;

namespace {

/* a node pair waiting on the stack with its exact transform */
struct StaticFrame {
    int32_t b1, b2;
    M3 R;
    V3 T;
};

/* C2A_BV_Distance: the rectangle distance minus both radii, clamped at 0 (C2A_BV.cpp:666-675) */
__device__ double static_bv_distance(const DevModel &A, const DevModel &B, const M3 &R, V3 T, int b1, int b2)
{
    ExactCtx xc{false};
    const NodeRec *n1 = A.nodes + b1, *n2 = B.nodes + b2;
    const double l1[2] = {__ldg(&n1->l[0]), __ldg(&n1->l[1])}, l2[2] = {__ldg(&n2->l[0]), __ldg(&n2->l[1])};
    V3 S = v3(0, 0, 0);
    double z = rect_dist(R, T, l1, l2, S, xc);
    z -= (__ldg(&n1->r) + __ldg(&n2->r));
    return z < 0.0 ? 0.0 : z;
}

/* TriDistance of leaf triangles ia (A) and ib (B) with B placed by (Rm, Tm) */
__device__ double static_tri_distance(const DevModel &A, const DevModel &B, const M3 &Rm, V3 Tm, int ia, int ib, V3 &p,
                                      V3 &q)
{
    V3 S[3], T[3], t[3];
    load_tri(S, A.tris + ia);
    load_tri(t, B.tris + ib);
    T[0] = mul_add(Rm, t[0], Tm);
    T[1] = mul_add(Rm, t[1], Tm);
    T[2] = mul_add(Rm, t[2], Tm);
    ExactCtx xc{false};
    TriFeat f;
    bool col = false;
    return tri_dist(p, q, S, T, f, col, xc);
}

/* the model-level transform of B in A and the root pair's transform with the
 * root nodes' frames given by (Ra, ta) and (Rb, tb) (C2A_PQP.cpp: MTxM, VmV,
 * MTxV, then the root RSS or OBB frames) */
__device__ void static_root(const double *P, const M3 &Ra, V3 ta, const M3 &Rb, V3 tb, M3 &Rm, V3 &Tm, M3 &Rr, V3 &Tr)
{
    const M3 R1 = pose_R(P), R2 = pose_R(P + 24);
    const V3 T1 = pose_T(P), T2 = pose_T(P + 24);
    Rm = tmmul(R1, R2);
    Tm = tmul(R1, T2 - T1);
    const M3 Rtemp = mmul(Rm, Rb);
    Rr = tmmul(Ra, Rtemp);
    V3 tt = mul_add(Rm, tb, Tm);
    tt = tt - ta;
    Tr = tmul(Ra, tt);
}

/* obb_disjoint of the PQP interface (boxes a and b, b placed by (B, T)):
 * the 15 separating axes, |B| inflated by 1e-6; 0 when none separates */
__device__ int static_obb_disjoint(const M3 &B, V3 Tv, const double *a, const double *b)
{
    const double T[3] = {Tv.x, Tv.y, Tv.z};
    double Bf[9];
#pragma unroll
    for (int k = 0; k < 9; k++) Bf[k] = fabs(B.m[k]) + 1e-6;
    for (int i = 0; i < 3; i++) {
        const double s = b[0] * Bf[3 * i] + b[1] * Bf[3 * i + 1] + b[2] * Bf[3 * i + 2];
        if (fabs(T[i]) > a[i] + s) return 1;
    }
    for (int j = 0; j < 3; j++) {
        const double tproj = T[0] * B.m[j] + T[1] * B.m[3 + j] + T[2] * B.m[6 + j];
        const double s = a[0] * Bf[j] + a[1] * Bf[3 + j] + a[2] * Bf[6 + j];
        if (fabs(tproj) > b[j] + s) return 1;
    }
    for (int i = 0; i < 3; i++) {
        const int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
        for (int j = 0; j < 3; j++) {
            const int j1 = (j + 1) % 3, j2 = (j + 2) % 3;
            const double tproj = T[i2] * B.m[3 * i1 + j] - T[i1] * B.m[3 * i2 + j];
            const double ra = a[i1] * Bf[3 * i2 + j] + a[i2] * Bf[3 * i1 + j];
            const double rb = b[j1] * Bf[3 * i + j2] + b[j2] * Bf[3 * i + j1];
            if (fabs(tproj) > ra + rb) return 2;
        }
    }
    return 0;
}

/* the pair a thread owns: lane l of global warp w takes pair w * ppw + l when
 * l < ppw (ppw 1: a pair per warp, for batches small enough to give every
 * pair a warp; 32: a pair per lane), -1 otherwise */
__device__ int static_pair_index(int ppw)
{
    const int lane = threadIdx.x & 31;
    if (lane >= ppw) return -1;
    const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    return warp * ppw + lane;
}

__device__ bool static_query_ok(const c2a_query &in, const DevModel *models, int num_models)
{
    return in.model_a >= 0 && in.model_a < num_models && in.model_b >= 0 && in.model_b < num_models &&
           (models[in.model_a].flags & C2A_MODEL_LIVE) && (models[in.model_b].flags & C2A_MODEL_LIVE);
}

} // namespace

__global__ void __launch_bounds__(kBlockThreads) c2a_tolerance_kernel(const c2a_query *__restrict__ queries, int n,
                                                                 const double *__restrict__ tolerance,
                                                                 const DevModel *__restrict__ models, int num_models,
                                                                 c2a_tolerance_result *__restrict__ results,
                                                                 int pairs_per_warp)
{
    const int i = static_pair_index(pairs_per_warp);
    if (i < 0 || i >= n) return;
    const c2a_query &in = queries[i];
    c2a_tolerance_result out;
    memset(&out, 0, sizeof(out));
    if (!static_query_ok(in, models, num_models)) {
        out.status = C2A_QUERY_BAD_INPUT;
        results[i] = out;
        return;
    }
    const DevModel &A = models[in.model_a], &B = models[in.model_b];
    double tol = tolerance[i];
    if (tol < 0.0) tol = 0.0;
    M3 Rm, R;
    V3 Tm, T;
    static_root(in.pose, load_R(A.nodes), load_Tr(A.nodes), load_R(B.nodes), load_Tr(B.nodes), Rm, Tm, R, T);
    StaticFrame stack[C2A_STACK_DEPTH];
    int sp = 0;
    int b1 = 0, b2 = 0;
    bool go = static_bv_distance(A, B, R, T, 0, 0) <= tol;
    long long nbv = 0, ntri = 0;
    while (go) {
        const int fc1 = __ldg(&A.nodes[b1].first_child), fc2 = __ldg(&B.nodes[b2].first_child);
        go = false;
        if (fc1 < 0 && fc2 < 0) {
            V3 p, q;
            ntri++;
            const double d = static_tri_distance(A, B, Rm, Tm, -fc1 - 1, -fc2 - 1, p, q);
            if (d <= tol) { /* the first pair within the tolerance ends the query */
                out.closer = 1;
                out.distance = d;
                const V3 u = tmul(Rm, q - Tm); /* back into model B's frame */
                out.p1[0] = p.x; out.p1[1] = p.y; out.p1[2] = p.z;
                out.p2[0] = u.x; out.p2[1] = u.y; out.p2[2] = u.z;
                break;
            }
        } else {
            int side, a1, a2, c1, c2;
            if (fc2 < 0 || (fc1 >= 0 && (__ldg(&A.nodes[b1].size) > __ldg(&B.nodes[b2].size)))) {
                side = 0; a1 = fc1; c1 = fc1 + 1; a2 = c2 = b2;
            } else {
                side = 1; a1 = c1 = b1; a2 = fc2; c2 = fc2 + 1;
            }
            M3 RA, RC;
            V3 TA, TC;
            const NodeRec *na = side == 0 ? A.nodes + a1 : B.nodes + a2, *nc = side == 0 ? A.nodes + c1 : B.nodes + c2;
            const M3 Ra = load_R(na), Rc = load_R(nc);
            if (side == 0) {
                RA = tmmul(Ra, R); TA = tmul(Ra, T - load_Tr(na));
                RC = tmmul(Rc, R); TC = tmul(Rc, T - load_Tr(nc));
            } else {
                RA = mmul(R, Ra); TA = mul_add(R, load_Tr(na), T);
                RC = mmul(R, Rc); TC = mul_add(R, load_Tr(nc), T);
            }
            nbv += 2;
            const double d1 = static_bv_distance(A, B, RA, TA, a1, a2);
            const double d2 = static_bv_distance(A, B, RC, TC, c1, c2);
            const bool c_first = d2 < d1;
            const bool go_first = (c_first ? d2 : d1) <= tol, go_second = (c_first ? d1 : d2) <= tol;
            if (go_second) {
                if (sp >= C2A_STACK_DEPTH) {
                    out.status |= C2A_QUERY_STACK_OVERFLOW;
                    break;
                }
                StaticFrame &f = stack[sp++];
                f.b1 = c_first ? a1 : c1; f.b2 = c_first ? a2 : c2;
                f.R = c_first ? RA : RC; f.T = c_first ? TA : TC;
            }
            if (go_first) {
                b1 = c_first ? c1 : a1; b2 = c_first ? c2 : a2;
                R = c_first ? RC : RA; T = c_first ? TC : TA;
                go = true;
                continue;
            }
        }
        if (sp > 0) {
            const StaticFrame &f = stack[--sp];
            b1 = f.b1; b2 = f.b2; R = f.R; T = f.T;
            go = true;
        }
    }
    out.num_bv_tests = nbv;
    out.num_tri_tests = ntri;
    results[i] = out;
}

__global__ void __launch_bounds__(kBlockThreads) c2a_collide_kernel(const c2a_query *__restrict__ queries, int n, int flag,
                                                               const DevModel *__restrict__ models, int num_models,
                                                               int slots, c2a_collide_result *__restrict__ results,
                                                               int32_t *__restrict__ pairs, int pairs_per_warp)
{
    const int i = static_pair_index(pairs_per_warp);
    if (i < 0 || i >= n) return;
    const c2a_query &in = queries[i];
    c2a_collide_result out;
    memset(&out, 0, sizeof(out));
    if (!static_query_ok(in, models, num_models)) {
        out.status = C2A_QUERY_BAD_INPUT;
        results[i] = out;
        return;
    }
    const DevModel &A = models[in.model_a], &B = models[in.model_b];
    const V3 toa = v3(A.obbs[0].To[0], A.obbs[0].To[1], A.obbs[0].To[2]);
    const V3 tob = v3(B.obbs[0].To[0], B.obbs[0].To[1], B.obbs[0].To[2]);
    M3 Rm, R;
    V3 Tm, T;
    static_root(in.pose, load_R(A.nodes), toa, load_R(B.nodes), tob, Rm, Tm, R, T);
    StaticFrame stack[C2A_STACK_DEPTH];
    int sp = 0, b1 = 0, b2 = 0, found = 0;
    long long nbv = 0, ntri = 0;
    int32_t *mine = pairs ? pairs + 2 * (size_t)i * (size_t)slots : nullptr;
    for (;;) {
        bool go = false;
        nbv++;
        if (static_obb_disjoint(R, T, A.obbs[b1].d, B.obbs[b2].d) == 0) {
            const int fc1 = __ldg(&A.nodes[b1].first_child), fc2 = __ldg(&B.nodes[b2].first_child);
            if (fc1 < 0 && fc2 < 0) {
                V3 p, q;
                ntri++;
                if (static_tri_distance(A, B, Rm, Tm, -fc1 - 1, -fc2 - 1, p, q) == 0.0) {
                    if (mine && found < slots) {
                        mine[2 * found] = __ldg(&A.tris[-fc1 - 1].id);
                        mine[2 * found + 1] = __ldg(&B.tris[-fc2 - 1].id);
                    }
                    found++;
                    if (flag == 2) break; /* first contact only */
                }
            } else {
                /* first child now, second on the stack (CollideRecurse visits them in order) */
                int side, x1a, x2a, x1c, x2c;
                if (fc2 < 0 || (fc1 >= 0 && (__ldg(&A.nodes[b1].size) > __ldg(&B.nodes[b2].size)))) {
                    side = 0; x1a = fc1; x1c = fc1 + 1; x2a = x2c = b2;
                } else {
                    side = 1; x1a = x1c = b1; x2a = fc2; x2c = fc2 + 1;
                }
                const int ka = side == 0 ? x1a : x2a, kc = side == 0 ? x1c : x2c;
                const DevModel &M = side == 0 ? A : B;
                const M3 Ra = load_R(M.nodes + ka), Rc = load_R(M.nodes + kc);
                const V3 oa = v3(M.obbs[ka].To[0], M.obbs[ka].To[1], M.obbs[ka].To[2]);
                const V3 oc = v3(M.obbs[kc].To[0], M.obbs[kc].To[1], M.obbs[kc].To[2]);
                M3 RA, RC;
                V3 TA, TC;
                if (side == 0) {
                    RA = tmmul(Ra, R); TA = tmul(Ra, T - oa);
                    RC = tmmul(Rc, R); TC = tmul(Rc, T - oc);
                } else {
                    RA = mmul(R, Ra); TA = mul_add(R, oa, T);
                    RC = mmul(R, Rc); TC = mul_add(R, oc, T);
                }
                if (sp >= C2A_STACK_DEPTH) {
                    out.status |= C2A_QUERY_STACK_OVERFLOW;
                    break;
                }
                StaticFrame &f = stack[sp++];
                f.b1 = x1c; f.b2 = x2c; f.R = RC; f.T = TC;
                b1 = x1a; b2 = x2a; R = RA; T = TA;
                go = true;
            }
        }
        if (go) continue;
        if (sp == 0) break;
        const StaticFrame &f = stack[--sp];
        b1 = f.b1; b2 = f.b2; R = f.R; T = f.T;
    }
    out.num_pairs = found;
    if (found > slots) out.status |= C2A_QUERY_CONTACT_OVERFLOW;
    out.num_bv_tests = nbv;
    out.num_tri_tests = ntri;
    results[i] = out;
}
