/*
 * k_spec.cu -- the speculative warp-per-query REFERENCE kernel.
 */
#include "device/ca_spec.cuh"
#include "kernels.h"

using namespace c2a;

namespace {
constexpr int kThreads = kBlockThreads;
} // namespace

/* REFERENCE mode by speculative expansion and ordered replay, one warp per
 * query (persistent): each warp's dynamic shared memory holds its query
 * state and contact stack (stack_cap entries) and then its speculation state
 * (nrec records); gscratch holds every warp's FP64 record part */
__global__ void __launch_bounds__(kThreads, 1) c2a_solve_spec_kernel(const c2a_query *__restrict__ queries, int n,
                                                                  const DevModel *__restrict__ models,
                                                                  int num_models, c2a_params prm,
                                                                  c2a_result *__restrict__ results,
                                                                  c2a_contact *__restrict__ contacts,
                                                                  unsigned int *__restrict__ counter,
                                                                  const int32_t *__restrict__ order, int stack_cap,
                                                                  int nrec, unsigned char *__restrict__ gscratch)
{
    extern __shared__ __align__(16) unsigned char c2a_spec_smem[];
    Pending tstack[C2A_STACK_DEPTH]; /* the translation-only step's sequential stack */
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const size_t wb = warp_shared_bytes(stack_cap), per = wb + spec_shared_bytes(nrec);
    unsigned char *base = c2a_spec_smem + (size_t)warp * per;
    WarpShared &mine = *reinterpret_cast<WarpShared *>(base);
    SpecCtx sc;
    spec_layout(sc, base + wb,
                gscratch + ((size_t)blockIdx.x * (kThreads / 32) + (size_t)warp) * spec_global_bytes(nrec), nrec);
    for (int i = lane; i < nrec; i += 32) sc.rec[i].gen = 0;
    mine.cap = stack_cap;
    __syncwarp();
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
        solve_query_warp(queries[q], models, num_models, prm, results[q], cq, mine, tstack, (int)q, lane,
                         SpecDfs{mine, sc});
    }
}


#ifdef C2A_STATS
/* profiling builds only: this translation unit's event counters, copied out and cleared */
extern "C" int c2a_spec_stats_read(unsigned long long *out, int count)
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
