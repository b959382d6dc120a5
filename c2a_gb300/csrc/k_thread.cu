/*
 * k_thread.cu -- the thread-per-query REFERENCE kernels: C2A_Solve, one CA step,
 * contacts at fixed poses.
 */
#include "device/ca_kernel.cuh"
#include "kernels.h"

using namespace c2a;

namespace {
constexpr int kThreads = kBlockThreads;
} // namespace

__global__ void __launch_bounds__(kThreads) c2a_solve_kernel(const c2a_query *__restrict__ queries, int n,
                                                             const DevModel *__restrict__ models, int num_models,
                                                             c2a_params prm, c2a_result *__restrict__ results,
                                                             c2a_contact *__restrict__ contacts,
                                                             unsigned int *__restrict__ counter)
{
    Pending stack[C2A_STACK_DEPTH];
    for (;;) {
        const unsigned int q = atomicAdd(counter, 1u);
        if (q >= (unsigned int)n) break;
        c2a_contact *cq = contacts ? contacts + (size_t)q * (size_t)prm.contacts_per_query : nullptr;
        solve_query(queries[q], models, num_models, prm, results[q], cq, stack, (int)q);
    }
}

__global__ void __launch_bounds__(kThreads) c2a_step_kernel(const c2a_query *__restrict__ queries, int n,
                                                            const double *__restrict__ lambda,
                                                            const int32_t *__restrict__ num_ca,
                                                            const double *__restrict__ prev_mint,
                                                            const DevModel *__restrict__ models, int num_models,
                                                            c2a_params prm, c2a_result *__restrict__ results)
{
    Pending stack[C2A_STACK_DEPTH];
    const int qi = blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= n) return;
    const c2a_query &in = queries[qi];
    c2a_result &out = results[qi];
    out.status = 0;
    if (in.model_a < 0 || in.model_a >= num_models || in.model_b < 0 || in.model_b >= num_models ||
        !(models[in.model_a].flags & C2A_MODEL_LIVE) || !(models[in.model_b].flags & C2A_MODEL_LIVE)) {
        out.status = C2A_QUERY_BAD_INPUT;
        return;
    }
    Query q;
    q.A = models + in.model_a;
    q.B = models + in.model_b;
    q.want_mint = true;
    if (in.seed_a < 0 || in.seed_a >= q.A->num_tris || in.seed_b < 0 || in.seed_b >= q.B->num_tris) {
        out.status = C2A_QUERY_BAD_INPUT;
        return;
    }
    q.status = 0;
    const double *P = in.pose;
    set_motions(q, P);
    q.toc_delta = prm.toc_delta;
    const bool translation = (q.m1.angVel < 1e-8 && q.m2.angVel < 1e-8);
    const double lam = lambda[qi];
    M3 R1, R2;
    V3 T1, T2;
    if (lam == 0.0) {
        R1 = pose_R(P);
        T1 = pose_T(P);
        R2 = pose_R(P + 24);
        T2 = pose_T(P + 24);
    } else {
        double orn[4];
        motion_integrate(q.m1, lam, R1.m, &T1.x, orn);
        motion_integrate(q.m2, lam, R2.m, &T2.x, orn);
    }
    set_pose1(q, R1, T1);
    q.seed_a = in.seed_a;
    q.seed_b = in.seed_b;
    q.nbv = q.ntri = 0;
    q.numCA = num_ca[qi];
    q.mint = prev_mint[qi];
    q.upbound = 1.0 - lam;
    q.distance = 0;
    q.abs_err = q.rel_err = 0;
    toc_step(q, R1, T1, R2, T2, translation, stack);
    out.collisionfree = 0;
    out.numCA = q.numCA;
    out.translation = translation ? 1 : 0;
    out.num_contact = 0;
    out.toc = lam;
    out.distance = q.distance;
    out.mint = q.mint;
    out.num_bv_tests = q.nbv;
    out.num_tri_tests = q.ntri;
    out.seed_a = q.seed_a;
    out.seed_b = q.seed_b;
    out.status = q.status;
}

__global__ void __launch_bounds__(kThreads) c2a_contact_kernel(const c2a_query *__restrict__ queries, int n,
                                                               const double *__restrict__ threshold,
                                                               const DevModel *__restrict__ models, int num_models,
                                                               int slots, c2a_result *__restrict__ results,
                                                               c2a_contact *__restrict__ contacts)
{
    Pending stack[C2A_STACK_DEPTH];
    const int qi = blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= n) return;
    const c2a_query &in = queries[qi];
    c2a_result &out = results[qi];
    out.status = 0;
    out.num_contact = 0;
    if (in.model_a < 0 || in.model_a >= num_models || in.model_b < 0 || in.model_b >= num_models ||
        !(models[in.model_a].flags & C2A_MODEL_LIVE) || !(models[in.model_b].flags & C2A_MODEL_LIVE)) {
        out.status = C2A_QUERY_BAD_INPUT;
        return;
    }
    Query q;
    q.A = models + in.model_a;
    q.B = models + in.model_b;
    q.status = 0;
    q.want_mint = false; /* the contact recursion reads distances only */
    q.e_ok = true;
    q.nbv = q.ntri = 0;
    const double *P = in.pose;
    M3 R;
    V3 T;
    relative_transforms(q, pose_R(P), pose_T(P), pose_R(P + 24), pose_T(P + 24), R, T);
    q.shadows_ok = q.e_ok && ((q.A->flags & q.B->flags) & C2A_MODEL_SHADOW_OK);
    const int cnt = contact_dfs(q, R, T, threshold[qi], stack,
                                contacts ? contacts + (size_t)qi * (size_t)slots : nullptr, slots, qi);
    out.num_contact = cnt;
    out.contact_offset = qi * slots;
    out.status = q.status | (cnt > slots ? C2A_QUERY_CONTACT_OVERFLOW : 0);
}

