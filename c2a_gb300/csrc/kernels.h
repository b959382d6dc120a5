/*
 * kernels.h -- the CA kernels, defined one family per translation unit
 * (k_thread.cu, k_warp.cu, k_spec.cu, k_front.cu, k_static.cu) so they compile in
 * parallel; c2a_abi.cu launches them.
 */
#ifndef C2A_KERNELS_H
#define C2A_KERNELS_H

#include <cuda_runtime.h>

#include "../../include/c2a_gb300.h"
#include "device/ca_kernel.cuh"

namespace c2a {
constexpr int kBlockThreads = 128; /* threads per block of the persistent solve kernels */
constexpr int kSplitThreads = 256; /* the split warp kernel: eight warps, one block per SM */
} // namespace c2a

__global__ void c2a_solve_kernel(const c2a_query *__restrict__ queries, int n, const c2a::DevModel *__restrict__
    models, int num_models, c2a_params prm, c2a_result *__restrict__ results, c2a_contact *__restrict__ contacts,
    unsigned int *__restrict__ counter);
__global__ void c2a_step_kernel(const c2a_query *__restrict__ queries, int n, const double *__restrict__ lambda, const
    int32_t *__restrict__ num_ca, const double *__restrict__ prev_mint, const c2a::DevModel *__restrict__ models, int
    num_models, c2a_params prm, c2a_result *__restrict__ results);
__global__ void c2a_contact_kernel(const c2a_query *__restrict__ queries, int n, const double *__restrict__ threshold,
    const c2a::DevModel *__restrict__ models, int num_models, int slots, c2a_result *__restrict__ results, c2a_contact
    *__restrict__ contacts);
__global__ void c2a_schedule_kernel(const c2a_query *__restrict__ queries, int n, const c2a::DevModel *__restrict__
    models, int num_models, int32_t *__restrict__ order, unsigned int *__restrict__ ends);
__global__ void c2a_solve_warp_kernel(const c2a_query *__restrict__ queries, int n, const c2a::DevModel *__restrict__
    models, int num_models, c2a_params prm, c2a_result *__restrict__ results, c2a_contact *__restrict__ contacts,
    unsigned int *__restrict__ counter, const int32_t *__restrict__ order, int stack_cap);
__global__ void c2a_solve_spec_kernel(const c2a_query *__restrict__ queries, int n, const c2a::DevModel *__restrict__
    models, int num_models, c2a_params prm, c2a_result *__restrict__ results, c2a_contact *__restrict__ contacts,
    unsigned int *__restrict__ counter, const int32_t *__restrict__ order, int stack_cap, int nrec, unsigned char
    *__restrict__ gscratch);
__global__ void c2a_canonical_kernel(const c2a_query *__restrict__ queries, int n, const c2a::DevModel *__restrict__
    models, int num_models, c2a_params prm, c2a_result *__restrict__ results, c2a_contact *__restrict__ contacts,
    unsigned int *__restrict__ counter, c2a::Pending *__restrict__ fronts, const uint32_t *__restrict__ hints, int
    nh);
__global__ void c2a_distance_kernel(const c2a_query *__restrict__ queries, int n, const c2a::DevModel *__restrict__
    models, int num_models, c2a_distance_result *__restrict__ results, unsigned int *__restrict__ counter,
    c2a::Pending *__restrict__ fronts);

__global__ void c2a_solve_warp_split_kernel(const c2a_query *__restrict__ queries, int n, int n_heavy,
    int heavy_blocks, const c2a::DevModel *__restrict__ models, int num_models, c2a_params prm,
    c2a_result *__restrict__ results, c2a_contact *__restrict__ contacts, unsigned int *__restrict__ counter,
    unsigned int *__restrict__ heavy_counter, const int32_t *__restrict__ order, int stack_cap);
__global__ void c2a_tolerance_kernel(const c2a_query *__restrict__ queries, int n, const double *__restrict__ tolerance,
    const c2a::DevModel *__restrict__ models, int num_models, c2a_tolerance_result *__restrict__ results,
    int pairs_per_warp);
__global__ void c2a_collide_kernel(const c2a_query *__restrict__ queries, int n, int flag,
    const c2a::DevModel *__restrict__ models, int num_models, int slots, c2a_collide_result *__restrict__ results,
    int32_t *__restrict__ pairs, int pairs_per_warp);

#endif
