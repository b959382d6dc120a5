/*
 * wave_engine.h -- the batched engine of the CANONICAL mode (c2a_wave.cu).
 *
 * All queries of a batch advance through their CA iterations in lockstep.
 * Inside an iteration, each phase (closest-pair search, fixed-bound step,
 * contacts) is a sequence of waves: one thread per (query, node pair) item,
 * every item of every active query in one launch, children appended to the
 * next wave's list.  Exact FP64 work that the FP32 filter cannot rule out is
 * deferred to separate lists and evaluated once the phase's bounds are final.
 * Results equal the warp-per-query CANONICAL kernel's bit for bit.
 */
#ifndef C2A_WAVE_ENGINE_H
#define C2A_WAVE_ENGINE_H

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/c2a_gb300.h"

namespace c2a {

struct DevModel;
struct WaveBuffers;

/* solves d_queries[0, n) into d_results (contacts in fixed slots of
 * prm.contacts_per_query); synchronises the stream between waves.  bufs is
 * created on first use and reused; *launches counts kernel launches.
 * hints (device, nh pairs of hinted nodes per query, may be NULL) seed the
 * first step's search bound. */
c2a_status wave_solve(WaveBuffers **bufs, int sm_count, cudaStream_t s, const c2a_query *d_queries, int n,
                      const DevModel *d_models, int num_models, const c2a_params &prm, c2a_result *d_results,
                      c2a_contact *d_contacts, int64_t *launches, const uint32_t *hints = nullptr, int nh = 0);

void wave_free(WaveBuffers *bufs);

} // namespace c2a
#endif
