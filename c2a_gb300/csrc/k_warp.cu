/*
 * k_warp.cu -- the warp-per-query REFERENCE kernel (the reference's order, each
 * node-pair test split across the lanes) and the geometric work order.
 */
#include "device/ca_warp.cuh"
#include "kernels.h"

using namespace c2a;

namespace {
constexpr int kThreads = kBlockThreads;
} // namespace

/* The order warps take queries in: queries whose bounding spheres close in on
 * each other over the motion go first (they run many CA iterations), the
 * rest after, so the longest queries do not start last.  Results are written
 * by query index; the order changes nothing else. */
__global__ void c2a_schedule_kernel(const c2a_query *__restrict__ queries, int n,
                                    const DevModel *__restrict__ models, int num_models,
                                    int32_t *__restrict__ order, unsigned int *__restrict__ ends)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const c2a_query &q = queries[i];
    bool early = false;
    if (q.model_a >= 0 && q.model_a < num_models && q.model_b >= 0 && q.model_b < num_models &&
        (models[q.model_a].flags & C2A_MODEL_LIVE) && (models[q.model_b].flags & C2A_MODEL_LIVE)) {
        const NodeRec *ra = models[q.model_a].nodes, *rb = models[q.model_b].nodes;
        /* root rectangle centres and bounding radii in each model's frame */
        const V3 ca = mul(load_R(ra), v3(0.5 * ra->l[0], 0.5 * ra->l[1], 0.0)) + load_Tr(ra);
        const V3 cb = mul(load_R(rb), v3(0.5 * rb->l[0], 0.5 * rb->l[1], 0.0)) + load_Tr(rb);
        const double rad = 0.5 * (ra->size + rb->size);
        const double *P = q.pose;
        const V3 pa0 = mul(pose_R(P), ca) + pose_T(P), pb0 = mul(pose_R(P + 24), cb) + pose_T(P + 24);
        const V3 pa1 = mul(pose_R(P + 12), ca) + pose_T(P + 12), pb1 = mul(pose_R(P + 36), cb) + pose_T(P + 36);
        const V3 g0 = pb0 - pa0, g1 = pb1 - pa1;
        /* the segment between the centres' relative start and end positions comes within reach */
        const V3 dg = g1 - g0;
        const double L2 = dot(dg, dg);
        double t = L2 > 0 ? -dot(g0, dg) / L2 : 0.0;
        t = t < 0 ? 0 : (t > 1 ? 1 : t);
        const V3 gm = g0 + mul_s(dg, t);
        early = dot(gm, gm) < rad * rad;
    }
    const unsigned int k = atomicAdd(ends + (early ? 0 : 1), 1u);
    if (early) order[k] = i;
    else order[n - 1 - (int)k] = i;
}

/* REFERENCE mode on one warp per query (persistent): the reference's order,
 * each node-pair test split across the lanes */
#ifndef C2A_WARP_MINB
#define C2A_WARP_MINB 1
#endif
#ifdef C2A_QTIME
/* profiling builds only: each query's start and end on the global timer (ns) */
constexpr unsigned int kQtimeCap = 1u << 17;
__device__ unsigned long long g_qtime[2 * kQtimeCap];
extern "C" int c2a_warp_qtime_read(unsigned long long *out, int n)
{
    if (!out || n < 0 || (unsigned int)n > kQtimeCap) return C2A_ERR_INVALID_ARGUMENT;
    if (cudaDeviceSynchronize() != cudaSuccess) return C2A_ERR_CUDA;
    if (cudaMemcpyFromSymbol(out, g_qtime, sizeof(unsigned long long) * 2 * (size_t)n) != cudaSuccess)
        return C2A_ERR_CUDA;
    return C2A_OK;
}
#endif
__global__ void __launch_bounds__(kThreads, C2A_WARP_MINB) c2a_solve_warp_kernel(const c2a_query *__restrict__ queries, int n,
                                                                  const DevModel *__restrict__ models,
                                                                  int num_models, c2a_params prm,
                                                                  c2a_result *__restrict__ results,
                                                                  c2a_contact *__restrict__ contacts,
                                                                  unsigned int *__restrict__ counter,
                                                                  const int32_t *__restrict__ order, int stack_cap)
{
    extern __shared__ __align__(16) unsigned char c2a_warp_smem[];
    Pending tstack[C2A_STACK_DEPTH]; /* the translation-only step's sequential stack */
    const int lane = threadIdx.x & 31;
    WarpShared &mine = *reinterpret_cast<WarpShared *>(c2a_warp_smem + (threadIdx.x >> 5) *
                                                       warp_shared_bytes(stack_cap));
    mine.cap = stack_cap;
    for (;;) {
        unsigned int q = 0;
        if (lane == 0) q = atomicAdd(counter, 1u);
        q = __shfl_sync(kWFull, q, 0);
        if (q >= (unsigned int)n) break;
        if (order) {
            const int32_t o = order[q];
            if (o < 0 || o >= n) continue; /* not a valid query index: skipped */
            q = (unsigned int)o;
        }
        c2a_contact *cq = contacts ? contacts + (size_t)q * (size_t)prm.contacts_per_query : nullptr;
#ifdef C2A_QTIME
        unsigned long long t0;
        asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t0));
#endif
        solve_query_warp(queries[q], models, num_models, prm, results[q], cq, mine, tstack, (int)q, lane,
                         WarpDfs{mine});
#ifdef C2A_QTIME
        unsigned long long t1;
        asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t1));
        if (lane == 0 && q < kQtimeCap) {
            g_qtime[2 * q] = t0;
            g_qtime[2 * q + 1] = t1;
        }
#endif
    }
}


/* The same traversal for an ordered batch whose head holds its costliest
 * queries.  One block of eight warps per SM (the register file holds one),
 * warp w and warp w + 4 sharing an SM sub-partition.  In the first
 * heavy_blocks blocks, warps 0..3 take the head's queries (order[0 ..
 * n_heavy)) while their sub-partition mates wait, so a heavy query has its
 * sub-partition's FP64 pipe to itself; a mate joins once the head is handed
 * out and its partner is done.  Every other warp takes the rest of the order
 * at full occupancy from the start.  The wait polls with a back-off and is
 * bounded (it only affects speed). */
__global__ void __launch_bounds__(kSplitThreads, 1) c2a_solve_warp_split_kernel(
    const c2a_query *__restrict__ queries, int n, int n_heavy, int heavy_blocks, const DevModel *__restrict__ models,
    int num_models, c2a_params prm, c2a_result *__restrict__ results, c2a_contact *__restrict__ contacts,
    unsigned int *__restrict__ counter, unsigned int *__restrict__ heavy_counter, const int32_t *__restrict__ order,
    int stack_cap)
{
    extern __shared__ __align__(16) unsigned char c2a_warp_smem[];
    __shared__ volatile int busy[4];
    Pending tstack[C2A_STACK_DEPTH];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    WarpShared &mine = *reinterpret_cast<WarpShared *>(c2a_warp_smem + warp * warp_shared_bytes(stack_cap));
    mine.cap = stack_cap;
    if (threadIdx.x < 4) busy[threadIdx.x] = 0;
    __syncthreads();
    const bool heavy_block = (int)blockIdx.x < heavy_blocks;
    if (heavy_block && warp < 4) {
        for (;;) {
            unsigned int q = 0;
            if (lane == 0) q = atomicAdd(heavy_counter, 1u);
            q = __shfl_sync(kWFull, q, 0);
            if (q >= (unsigned int)n_heavy) break;
            const int32_t o = order[q];
            if (o < 0 || o >= n) continue;
            if (lane == 0) busy[warp] = 1;
            __syncwarp();
            c2a_contact *cq = contacts ? contacts + (size_t)o * (size_t)prm.contacts_per_query : nullptr;
            solve_query_warp(queries[o], models, num_models, prm, results[o], cq, mine, tstack, o, lane,
                             WarpDfs{mine});
            __syncwarp();
            if (lane == 0) busy[warp] = 0;
        }
    } else if (heavy_block) {
        /* wait until the head is handed out and the partner's heavy query is done */
        for (int it = 0; it < (1 << 24); it++) {
            int done = 0;
            if (lane == 0)
                done = *reinterpret_cast<volatile unsigned int *>(heavy_counter) >= (unsigned int)n_heavy &&
                       busy[warp - 4] == 0;
            done = __shfl_sync(kWFull, done, 0);
            if (done) break;
            __nanosleep(2000);
        }
    }
    for (;;) { /* the rest of the order */
        unsigned int q = 0;
        if (lane == 0) q = atomicAdd(counter, 1u);
        q = __shfl_sync(kWFull, q, 0);
        if (q >= (unsigned int)(n - n_heavy)) break;
        const int32_t o = order[n_heavy + q];
        if (o < 0 || o >= n) continue;
        c2a_contact *cq = contacts ? contacts + (size_t)o * (size_t)prm.contacts_per_query : nullptr;
        solve_query_warp(queries[o], models, num_models, prm, results[o], cq, mine, tstack, o, lane,
                         WarpDfs{mine});
    }
}

#ifdef C2A_STATS
/* profiling builds only: this translation unit's event counters, copied out and cleared */
extern "C" int c2a_warp_stats_read(unsigned long long *out, int count)
{
    if (!out || count < ST_COUNT) return C2A_ERR_INVALID_ARGUMENT;
    if (cudaDeviceSynchronize() != cudaSuccess) return C2A_ERR_CUDA;
    if (cudaMemcpyFromSymbol(out, g_c2a_stats, sizeof(unsigned long long) * ST_COUNT) != cudaSuccess)
        return C2A_ERR_CUDA;
    unsigned long long zero[ST_COUNT] = {};
    if (cudaMemcpyToSymbol(g_c2a_stats, zero, sizeof(zero)) != cudaSuccess) return C2A_ERR_CUDA;
    return C2A_OK;
}
#endif
