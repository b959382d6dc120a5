/*
 * k_front.cu -- the CANONICAL warp kernel and the batch distance query.
 */
#include "device/ca_front.cuh"
#include "kernels.h"

using namespace c2a;

namespace {
constexpr int kThreads = kBlockThreads;
} // namespace

/* CANONICAL mode: one warp per query (persistent; warps take queries from
 * the work counter), each with its own slice of the front buffer */
__global__ void __launch_bounds__(kThreads) c2a_canonical_kernel(const c2a_query *__restrict__ queries, int n,
                                                                 const DevModel *__restrict__ models,
                                                                 int num_models, c2a_params prm,
                                                                 c2a_result *__restrict__ results,
                                                                 c2a_contact *__restrict__ contacts,
                                                                 unsigned int *__restrict__ counter,
                                                                 Pending *__restrict__ fronts,
                                                                 const uint32_t *__restrict__ hints, int nh)
{
    const int lane = threadIdx.x & 31;
    const size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    Pending *stack = fronts + warp * (size_t)C2A_FRONT_CAP;
    for (;;) {
        unsigned int q = 0;
        if (lane == 0) q = atomicAdd(counter, 1u);
        q = __shfl_sync(kFullMask, q, 0);
        if (q >= (unsigned int)n) break;
        c2a_contact *cq = contacts ? contacts + (size_t)q * (size_t)prm.contacts_per_query : nullptr;
        solve_query_canonical(queries[q], models, num_models, prm, results[q], cq, stack, C2A_FRONT_CAP, lane,
                              (int)q, hints ? hints + (size_t)q * nh * 2 : nullptr, nh);
    }
}

/* C2A_Distance for a batch: one warp per pair (persistent), each with its own
 * slice of the front buffer */
__global__ void __launch_bounds__(kThreads) c2a_distance_kernel(const c2a_query *__restrict__ queries, int n,
                                                                const DevModel *__restrict__ models, int num_models,
                                                                c2a_distance_result *__restrict__ results,
                                                                unsigned int *__restrict__ counter,
                                                                Pending *__restrict__ fronts)
{
    const int lane = threadIdx.x & 31;
    const size_t warp = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    Pending *stack = fronts + warp * (size_t)C2A_FRONT_CAP;
    for (;;) {
        unsigned int q = 0;
        if (lane == 0) q = atomicAdd(counter, 1u);
        q = __shfl_sync(kFullMask, q, 0);
        if (q >= (unsigned int)n) break;
        distance_query_warp(queries[q], models, num_models, results[q], stack, C2A_FRONT_CAP, lane);
    }
}

/* dense contact output: exclusive scan of min(num_contact, slots), then a
 * gather of the used slots (one block per 1024 queries, block-local scan
 * followed by a scan of the block totals) */

