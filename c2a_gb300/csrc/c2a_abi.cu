/*
 * c2a_abi.cu -- the C ABI of include/c2a_gb300.h: contexts, model upload and
 * the CA kernels' launches.  Everything the reference computes per query runs
 * on the GPU; the host only builds the BVH (as the reference's EndModel
 * does), moves buffers and launches.
 */
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <mutex>
#include <new>
#include <system_error>
#include <thread>
#include <vector>

#include "../../include/c2a_gb300.h"
#include "device/ca_front.cuh"
#include "device/ca_spec.cuh"
#include "device/ca_warp.cuh"
#include "kernels.h"
#include "host/bvh_build.h"
#include "wave_engine.h"

using namespace c2a;

/* records of the speculative engine beyond the replay's path */
#ifndef C2A_SPEC_EXTRA
#define C2A_SPEC_EXTRA 64
#endif

namespace {

/* an NVTX range over an entry point, for profilers (nvtxRangePushA/Pop cost
 * a few nanoseconds and do nothing unless a tool is attached) */
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};
#define C2A_RANGE(name) NvtxRange c2a_range_(name)

} // namespace

namespace {

constexpr int kThreads = kBlockThreads;

struct ModelSlot {
    BuiltModel host;
    NodeRec *d_nodes = nullptr;
    TriRec *d_tris = nullptr;
    NodeShadow *d_snodes = nullptr;
    TriShadow *d_stris = nullptr;
    ObbRec *d_obbs = nullptr;
    bool live = false;
};

/* the kernels' view of one model slot */
DevModel dev_model_of(const ModelSlot &s)
{
    DevModel m;
    m.nodes = s.d_nodes;
    m.tris = s.d_tris;
    m.snodes = s.d_snodes;
    m.stris = s.d_stris;
    m.obbs = s.d_obbs;
    m.num_tris = s.live ? (int32_t)s.host.tris.size() : 0;
    m.num_nodes = s.live ? (int32_t)s.host.nodes.size() : 0;
    m.depth = s.host.depth;
    m.flags = (s.live ? C2A_MODEL_LIVE : 0) | (s.live && s.host.shadow_ok ? C2A_MODEL_SHADOW_OK : 0);
    return m;
}

void free_slot(ModelSlot &s)
{
    if (s.d_nodes) cudaFree(s.d_nodes);
    if (s.d_tris) cudaFree(s.d_tris);
    if (s.d_snodes) cudaFree(s.d_snodes);
    if (s.d_stris) cudaFree(s.d_stris);
    if (s.d_obbs) cudaFree(s.d_obbs);
    s.d_obbs = nullptr;
    s.d_nodes = nullptr;
    s.d_tris = nullptr;
    s.d_snodes = nullptr;
    s.d_stris = nullptr;
}

} // namespace

struct c2a_context {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    std::vector<ModelSlot> models;
    DevModel *d_models = nullptr;
    int d_models_cap = 0;
    bool models_dirty = true;
    unsigned int *d_counter = nullptr; /* work counter of the persistent kernels */
    int64_t launches = 0;
    /* device staging for the host-buffer entry points */
    void *d_buf = nullptr;
    size_t d_buf_size = 0;
    int32_t last_contacts = 0; /* contacts copied back by the last c2a_solve_batch */
    /* per-warp front slices of the canonical kernel (C2A_FRONT_CAP entries each) */
    Pending *d_fronts = nullptr;
    size_t fronts_warps = 0;
    WaveBuffers *wave = nullptr; /* the batched canonical engine's lists */
    int32_t *d_order = nullptr;  /* the order the warp kernel takes queries in */
    size_t order_cap = 0;
    int canonical_blocks_per_sm = 0;
    int warp_blocks_per_sm = 0;
    int split_smem_attr = 0;     /* the split warp kernel's dynamic shared-memory limit set so far */
    int warp_cap = 0;            /* the warp kernel's stack entries the occupancy above was computed for */
    bool warp_smem_attr = false;
    int distance_blocks_per_sm = 0;
    /* the speculative engine: occupancy for (stack cap, records), FP64 record scratch */
    int spec_blocks_per_sm = 0;
    int spec_cap = 0, spec_nrec = 0;
    bool spec_smem_attr = false;
    unsigned char *d_spec = nullptr;
    size_t spec_bytes = 0;
    uint64_t models_gen = 0;     /* changes whenever a model is built or freed (unique across contexts) */
    std::mutex mu;
};

namespace {

c2a_status cuda_status(cudaError_t e)
{
    if (e == cudaSuccess) return C2A_OK;
    if (e == cudaErrorMemoryAllocation) return C2A_ERR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return C2A_ERR_NO_DEVICE;
    return C2A_ERR_CUDA;
}

#define C2A_CUDA(call)                                                                                             \
    do {                                                                                                           \
        cudaError_t e_ = (call);                                                                                   \
        if (e_ != cudaSuccess) {                                                                                   \
            fprintf(stderr, "c2a_gb300: %s failed: %s\n", #call, cudaGetErrorString(e_));                          \
            return cuda_status(e_);                                                                                \
        }                                                                                                          \
    } while (0)

/* uploads the model table when models were added or freed */
c2a_status sync_models(c2a_context *ctx)
{
    if (!ctx->models_dirty) return C2A_OK;
    std::vector<DevModel> table(ctx->models.size());
    for (size_t i = 0; i < ctx->models.size(); i++) table[i] = dev_model_of(ctx->models[i]);
    if ((int)table.size() > ctx->d_models_cap) {
        if (ctx->d_models) cudaFree(ctx->d_models);
        ctx->d_models = nullptr;
        int cap = (int)table.size() * 2 + 4;
        C2A_CUDA(cudaMalloc(&ctx->d_models, sizeof(DevModel) * cap));
        ctx->d_models_cap = cap;
    }
    if (!table.empty())
        C2A_CUDA(cudaMemcpyAsync(ctx->d_models, table.data(), sizeof(DevModel) * table.size(),
                                 cudaMemcpyHostToDevice, ctx->stream));
    C2A_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->models_dirty = false;
    return C2A_OK;
}

c2a_status ensure_buf(c2a_context *ctx, size_t bytes)
{
    if (bytes <= ctx->d_buf_size) return C2A_OK;
    if (ctx->d_buf) cudaFree(ctx->d_buf);
    ctx->d_buf = nullptr;
    ctx->d_buf_size = 0;
    size_t sz = bytes + bytes / 4 + 4096;
    C2A_CUDA(cudaMalloc(&ctx->d_buf, sz));
    ctx->d_buf_size = sz;
    return C2A_OK;
}

/* front slices for `warps` warps (allocates `want` >= warps when it grows) */
c2a_status ensure_fronts(c2a_context *ctx, size_t warps, size_t want)
{
    if (warps <= ctx->fronts_warps) return C2A_OK;
    /* a stream may still read the old slices: wait before freeing */
    C2A_CUDA(cudaDeviceSynchronize());
    if (ctx->d_fronts) cudaFree(ctx->d_fronts);
    ctx->d_fronts = nullptr;
    ctx->fronts_warps = 0;
    if (want < warps) want = warps;
    C2A_CUDA(cudaMalloc(&ctx->d_fronts, want * (size_t)C2A_FRONT_CAP * sizeof(Pending)));
    ctx->fronts_warps = want;
    return C2A_OK;
}

bool params_ok(const c2a_params *p)
{
    return p && p->max_iters >= 0 && p->contacts_per_query >= 0 && p->warps_per_sm >= 0 && p->heavy_prefix >= 0 &&
           (p->mode == C2A_MODE_REFERENCE || p->mode == C2A_MODE_CANONICAL) && p->engine >= C2A_ENGINE_AUTO &&
           p->engine <= C2A_ENGINE_SPEC && !(p->mode == C2A_MODE_REFERENCE && p->engine == C2A_ENGINE_BATCHED) &&
           !(p->mode == C2A_MODE_CANONICAL && (p->engine == C2A_ENGINE_THREAD || p->engine == C2A_ENGINE_SPEC));
}

/* queries must not pair models deeper than the traversal stack */
c2a_status check_depths(c2a_context *ctx, int *deepest_out = nullptr)
{
    int deepest = 0;
    for (const ModelSlot &s : ctx->models)
        if (s.live && s.host.depth > deepest) deepest = s.host.depth;
    if (deepest_out) *deepest_out = deepest;
    if (2 * deepest + 2 > C2A_STACK_DEPTH) return C2A_ERR_TREE_TOO_DEEP;
    return C2A_OK;
}

/* launch shape of the persistent solve kernel: 128-thread blocks, or
 * 32-thread blocks when the batch is too small to give every SM two full
 * blocks (one query per thread, so small batches still reach all SMs) */
struct Shape {
    int blocks, threads;
};
/* resident blocks per SM: what fits (occ), capped by the caller's warps per SM */
int blocks_per_sm(int occ, int warps_per_sm, int threads)
{
    if (warps_per_sm <= 0) return occ;
    const int want = warps_per_sm / (threads / 32);
    return want < 1 ? 1 : (want < occ ? want : occ);
}

Shape shape_for(c2a_context *ctx, int n, int warps_per_sm)
{
    int threads = kThreads;
    if ((n + kThreads - 1) / kThreads < 2 * ctx->sm_count) threads = 32;
    const int most = ctx->sm_count * blocks_per_sm(8 * (kThreads / threads), warps_per_sm, threads);
    int need = (n + threads - 1) / threads;
    if (need < 1) need = 1;
    return Shape{need < most ? need : most, threads};
}

} // namespace

/* ------------------------------------------------------------- kernels */

constexpr int kScanBlock = 1024;

__global__ void __launch_bounds__(kScanBlock) c2a_scan_blocks(c2a_result *__restrict__ results, int n, int slots,
                                                               int32_t *__restrict__ block_sums)
{
    __shared__ int32_t s[kScanBlock];
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    int32_t v = 0;
    if (i < n) {
        const int32_t c = results[i].num_contact;
        v = c < slots ? c : slots;
    }
    s[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < kScanBlock; off <<= 1) {
        int32_t t = threadIdx.x >= off ? s[threadIdx.x - off] : 0;
        __syncthreads();
        s[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) results[i].contact_offset = s[threadIdx.x] - v; /* block-local exclusive */
    if (threadIdx.x == kScanBlock - 1) block_sums[blockIdx.x] = s[threadIdx.x];
}

__global__ void c2a_scan_totals(int32_t *__restrict__ block_sums, int nblocks, int32_t *__restrict__ total)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    int32_t run = 0;
    for (int b = 0; b < nblocks; b++) {
        const int32_t t = block_sums[b];
        block_sums[b] = run;
        run += t;
    }
    *total = run;
}

__global__ void c2a_gather_contacts(c2a_result *__restrict__ results, int n, int slots,
                                    const int32_t *__restrict__ block_sums, const c2a_contact *__restrict__ src,
                                    c2a_contact *__restrict__ dst)
{
    const int q = blockIdx.x;
    if (q >= n) return;
    const int off = results[q].contact_offset + block_sums[q / kScanBlock];
    const int c = results[q].num_contact < slots ? results[q].num_contact : slots;
    for (int k = threadIdx.x; k < c; k += blockDim.x) dst[off + k] = src[(size_t)q * slots + k];
    __syncthreads();
    if (threadIdx.x == 0) results[q].contact_offset = off;
}

/* ------------------------------------------- scratch of the no-alloc entry */

/* The solve kernel's scratch for c2a_solve_batch_noalloc: bytes [0, 4) hold
 * the work counter, bytes [256, 256 + 48 * C2A_NOALLOC_MAX_MODELS) the model
 * table.  Host code only ever sees the symbol's host-side stand-in; the
 * device address comes from cudaGetSymbolAddress (noalloc_scratch below). */
constexpr size_t kNoallocTableOffset = 256;
constexpr size_t kNoallocBytes = 8192;
static_assert(kNoallocTableOffset + sizeof(DevModel) * C2A_NOALLOC_MAX_MODELS <= kNoallocBytes,
              "the no-alloc model table must fit its 8 KiB scratch array");
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned char *g_noalloc_ptr[kMaxDevices] = {};
uint64_t g_noalloc_table_gen[kMaxDevices] = {}; /* models_gen of the table last uploaded on each device */
std::atomic<uint64_t> g_models_gen{0};

uint64_t next_models_gen() { return ++g_models_gen; }

/* device address of the scratch array on `device` (current), looked up once
 * per device; c2a_create calls it, so the first query call finds it set */
c2a_status noalloc_scratch(int device, unsigned char **out)
{
    if (device < 0 || device >= kMaxDevices) return C2A_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[device]) {
        unsigned char *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            fprintf(stderr, "c2a_gb300: cudaGetSymbolAddress(no-alloc scratch) failed: %s\n", cudaGetErrorString(e));
            return cuda_status(e == cudaSuccess ? cudaErrorInvalidSymbol : e);
        }
        g_noalloc_ptr[device] = p;
    }
    *out = g_noalloc_ptr[device];
    return C2A_OK;
}
} // namespace

/* --------------------------------------------------------------- ABI */

extern "C" {

const char *c2a_status_str(c2a_status s)
{
    switch (s) {
    case C2A_OK: return "ok";
    case C2A_ERR_INVALID_ARGUMENT: return "invalid argument";
    case C2A_ERR_NO_DEVICE: return "no CUDA device";
    case C2A_ERR_CUDA: return "CUDA error";
    case C2A_ERR_OUT_OF_MEMORY: return "out of device memory";
    case C2A_ERR_EMPTY_MODEL: return "model has no triangles";
    case C2A_ERR_BAD_MODEL: return "unknown model id";
    case C2A_ERR_TREE_TOO_DEEP: return "hierarchy deeper than the traversal stack";
    case C2A_ERR_QUERY_FAILED: return "a query reported a non-zero status";
    case C2A_ERR_NOALLOC_CAPACITY: return "more models than the no-alloc entry point's fixed table holds";
    default: return "unknown status";
    }
}

c2a_status c2a_create(int device, c2a_context **out)
{
    if (!out) return C2A_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (device == -1) { /* host-only: builds and downloads models, runs no query */
        c2a_context *ctx = new (std::nothrow) c2a_context();
        if (!ctx) return C2A_ERR_OUT_OF_MEMORY;
        ctx->device = -1;
        *out = ctx;
        return C2A_OK;
    }
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return C2A_ERR_NO_DEVICE;
    if (device < 0 || device >= count) return C2A_ERR_INVALID_ARGUMENT;
    C2A_CUDA(cudaSetDevice(device));
    c2a_context *ctx = new (std::nothrow) c2a_context();
    if (!ctx) return C2A_ERR_OUT_OF_MEMORY;
    ctx->device = device;
    cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    ctx->models_gen = next_models_gen();
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&ctx->d_counter, sizeof(unsigned int) * 4) != cudaSuccess) {
        c2a_destroy(ctx);
        return C2A_ERR_CUDA;
    }
    /* set-up of c2a_solve_batch_noalloc, done here because this call may
     * allocate: the scratch array's device address on this device, and the
     * module of its kernel loaded (lazy loading would otherwise load it, and
     * reserve its local memory, on the first no-alloc call) */
    unsigned char *scratch = nullptr;
    cudaFuncAttributes fa;
    if (noalloc_scratch(device, &scratch) != C2A_OK || cudaFuncGetAttributes(&fa, c2a_solve_kernel) != cudaSuccess) {
        c2a_destroy(ctx);
        return C2A_ERR_CUDA;
    }
    *out = ctx;
    return C2A_OK;
}

c2a_status c2a_destroy(c2a_context *ctx)
{
    if (!ctx) return C2A_OK;
    if (ctx->device < 0) {
        delete ctx;
        return C2A_OK;
    }
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (ModelSlot &s : ctx->models) free_slot(s);
    if (ctx->d_models) cudaFree(ctx->d_models);
    if (ctx->d_fronts) cudaFree(ctx->d_fronts);
    if (ctx->d_order) cudaFree(ctx->d_order);
    if (ctx->d_spec) cudaFree(ctx->d_spec);
    wave_free(ctx->wave);
    if (ctx->d_counter) cudaFree(ctx->d_counter);
    if (ctx->d_buf) cudaFree(ctx->d_buf);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return C2A_OK;
}

c2a_status c2a_launch_count(c2a_context *ctx, int64_t *count)
{
    if (!ctx || !count) return C2A_ERR_INVALID_ARGUMENT;
    *count = ctx->launches;
    return C2A_OK;
}

namespace {

constexpr int kMaxBuildThreads = 256;

/* host threads a build may use: the caller's count, else C2A_BUILD_THREADS
 * when set (>= 1), else every hardware thread; at most kMaxBuildThreads */
int build_thread_count(int32_t requested)
{
    int n = requested;
    if (n <= 0)
        if (const char *e = getenv("C2A_BUILD_THREADS")) n = atoi(e);
    if (n <= 0) {
        const unsigned h = std::thread::hardware_concurrency();
        n = h ? (int)h : 1;
    }
    return std::min(n, kMaxBuildThreads);
}

/* uploads a built model and adds it to the context's table (ctx->mu held) */
c2a_status register_model(c2a_context *ctx, ModelSlot &slot, int32_t *model_id)
{
    if (ctx->device < 0) {
        slot.live = true;
        ctx->models.push_back(std::move(slot));
        *model_id = (int32_t)ctx->models.size() - 1;
        return C2A_OK;
    }
    C2A_CUDA(cudaSetDevice(ctx->device));
    const size_t nn = slot.host.nodes.size(), nt = slot.host.tris.size();
    cudaError_t e = cudaMalloc(&slot.d_nodes, sizeof(NodeRec) * nn);
    if (e == cudaSuccess) e = cudaMalloc(&slot.d_tris, sizeof(TriRec) * nt);
    if (e == cudaSuccess) e = cudaMalloc(&slot.d_snodes, sizeof(NodeShadow) * nn);
    if (e == cudaSuccess) e = cudaMalloc(&slot.d_stris, sizeof(TriShadow) * nt);
    if (e == cudaSuccess) e = cudaMalloc(&slot.d_obbs, sizeof(ObbRec) * nn);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(slot.d_obbs, slot.host.obbs.data(), sizeof(ObbRec) * nn, cudaMemcpyHostToDevice,
                            ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(slot.d_nodes, slot.host.nodes.data(), sizeof(NodeRec) * nn, cudaMemcpyHostToDevice,
                            ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(slot.d_tris, slot.host.tris.data(), sizeof(TriRec) * nt, cudaMemcpyHostToDevice,
                            ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(slot.d_snodes, slot.host.snodes.data(), sizeof(NodeShadow) * nn,
                            cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(slot.d_stris, slot.host.stris.data(), sizeof(TriShadow) * nt, cudaMemcpyHostToDevice,
                            ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        fprintf(stderr, "c2a_gb300: model upload failed: %s\n", cudaGetErrorString(e));
        cudaStreamSynchronize(ctx->stream);
        free_slot(slot);
        return cuda_status(e);
    }
    slot.live = true;
    ctx->models.push_back(std::move(slot));
    ctx->models_dirty = true;
    ctx->models_gen = next_models_gen();
    *model_id = (int32_t)ctx->models.size() - 1;
    return C2A_OK;
}

} // namespace

c2a_status c2a_model_build(c2a_context *ctx, int32_t num_tris, const double *tri_verts, const int32_t *ids,
                           const int32_t *vidx, int32_t *model_id)
{
    C2A_RANGE("c2a_model_build");
    if (!ctx || !model_id) return C2A_ERR_INVALID_ARGUMENT;
    ModelSlot slot;
    BuildThreads threads(build_thread_count(0) - 1);
    int rc = build_rss_model(num_tris, tri_verts, ids, vidx, slot.host, &threads);
    if (rc) return rc;
    std::lock_guard<std::mutex> lock(ctx->mu);
    return register_model(ctx, slot, model_id);
}

struct c2a_build_handle {
    c2a_context *ctx = nullptr;
    std::vector<double> verts; /* copies of the caller's arrays */
    std::vector<int32_t> ids, vidx;
    ModelSlot slot;
    int rc = 0;
    std::thread worker;
};

c2a_status c2a_model_build_async(c2a_context *ctx, int32_t num_tris, const double *tri_verts, const int32_t *ids,
                                 const int32_t *vidx, c2a_build_handle **handle)
{
    C2A_RANGE("c2a_model_build_async");
    if (!ctx || !handle) return C2A_ERR_INVALID_ARGUMENT;
    *handle = nullptr;
    if (num_tris <= 0 || !tri_verts) return C2A_ERR_EMPTY_MODEL;
    c2a_build_handle *h = new (std::nothrow) c2a_build_handle;
    if (!h) return C2A_ERR_OUT_OF_MEMORY;
    try {
        h->ctx = ctx;
        h->verts.assign(tri_verts, tri_verts + 9 * (size_t)num_tris);
        if (ids) h->ids.assign(ids, ids + num_tris);
        if (vidx) h->vidx.assign(vidx, vidx + 3 * (size_t)num_tris);
        h->worker = std::thread([h, num_tris] {
            BuildThreads threads(build_thread_count(0) - 1);
            h->rc = build_rss_model(num_tris, h->verts.data(), h->ids.empty() ? nullptr : h->ids.data(),
                                    h->vidx.empty() ? nullptr : h->vidx.data(), h->slot.host, &threads);
        });
    } catch (const std::exception &) { // no memory for the copies, or no thread
        delete h;
        return C2A_ERR_OUT_OF_MEMORY;
    }
    *handle = h;
    return C2A_OK;
}

c2a_status c2a_model_wait(c2a_build_handle *handle, int32_t *model_id)
{
    C2A_RANGE("c2a_model_wait");
    if (!handle) return C2A_ERR_INVALID_ARGUMENT;
    handle->worker.join();
    c2a_status s = handle->rc;
    if (s == C2A_OK) {
        int32_t id = -1;
        {
            std::lock_guard<std::mutex> lock(handle->ctx->mu);
            s = register_model(handle->ctx, handle->slot, &id);
        }
        if (model_id) *model_id = s == C2A_OK ? id : -1;
    } else if (model_id) {
        *model_id = -1;
    }
    delete handle;
    return s;
}

c2a_status c2a_model_build_many(c2a_context *ctx, int32_t count, const int32_t *num_tris,
                                const double *const *tri_verts, const int32_t *const *ids,
                                const int32_t *const *vidx, int32_t threads, int32_t *model_ids)
{
    C2A_RANGE("c2a_model_build_many");
    if (!ctx || count < 0 || (count > 0 && (!num_tris || !tri_verts || !model_ids)) || threads < 0)
        return C2A_ERR_INVALID_ARGUMENT;
    for (int32_t i = 0; i < count; i++)
        if (num_tris[i] <= 0 || !tri_verts[i]) return C2A_ERR_EMPTY_MODEL;
    if (count == 0) return C2A_OK;
    // largest models first; one worker per model at a time, and a worker
    // with no model left lends its thread to the builds still running
    std::vector<int32_t> order((size_t)count);
    for (int32_t i = 0; i < count; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return num_tris[a] > num_tris[b]; });
    std::vector<ModelSlot> slots((size_t)count);
    std::vector<int> rcs((size_t)count, 0);
    const int total = build_thread_count(threads);
    const int workers = std::min(total, (int)count);
    BuildThreads budget(total - workers);
    std::atomic<int32_t> next{0};
    auto work = [&] {
        for (int32_t k; (k = next.fetch_add(1)) < count;) {
            const int32_t i = order[k];
            rcs[i] = build_rss_model(num_tris[i], tri_verts[i], ids ? ids[i] : nullptr, vidx ? vidx[i] : nullptr,
                                     slots[i].host, &budget);
        }
        budget.give();
    };
    std::vector<std::thread> pool;
    for (int w = 1; w < workers; w++) {
        try {
            pool.emplace_back(work);
        } catch (const std::exception &) { // no thread (system_error) or no room to keep it
            break;                          // fewer workers; the ones running take the rest
        }
    }
    work();
    for (std::thread &th : pool) th.join();
    for (int32_t i = 0; i < count; i++)
        if (rcs[i]) return rcs[i];
    std::lock_guard<std::mutex> lock(ctx->mu);
    for (int32_t i = 0; i < count; i++) {
        const c2a_status s = register_model(ctx, slots[i], &model_ids[i]);
        if (s != C2A_OK) {
            for (int32_t j = 0; j < i; j++) {
                ModelSlot &done = ctx->models[model_ids[j]];
                if (ctx->device >= 0) free_slot(done);
                done.live = false;
                done.host = BuiltModel{};
                model_ids[j] = -1;
            }
            model_ids[i] = -1;
            ctx->models_dirty = true;
            ctx->models_gen = next_models_gen();
            return s;
        }
    }
    return C2A_OK;
}

c2a_status c2a_model_info(c2a_context *ctx, int32_t id, int32_t *num_tris, int32_t *num_nodes, int32_t *depth)
{
    if (!ctx) return C2A_ERR_INVALID_ARGUMENT;
    if (id < 0 || id >= (int32_t)ctx->models.size() || !ctx->models[id].live) return C2A_ERR_BAD_MODEL;
    const BuiltModel &m = ctx->models[id].host;
    if (num_tris) *num_tris = (int32_t)m.tris.size();
    if (num_nodes) *num_nodes = (int32_t)m.nodes.size();
    if (depth) *depth = m.depth;
    return C2A_OK;
}

c2a_status c2a_model_download(c2a_context *ctx, int32_t id, double *node_f, int32_t *first_child, double *tri_verts,
                              int32_t *tri_ids, int32_t *tri_vidx)
{
    if (!ctx) return C2A_ERR_INVALID_ARGUMENT;
    if (id < 0 || id >= (int32_t)ctx->models.size() || !ctx->models[id].live) return C2A_ERR_BAD_MODEL;
    const BuiltModel &m = ctx->models[id].host;
    for (size_t i = 0; i < m.nodes.size(); i++) {
        const NodeRec &n = m.nodes[i];
        if (node_f) {
            double *o = node_f + 25 * i;
            std::memcpy(o, n.R, sizeof(n.R));
            std::memcpy(o + 9, n.Tr, sizeof(n.Tr));
            o[12] = n.l[0];
            o[13] = n.l[1];
            o[14] = n.r;
            o[15] = n.angR;
            std::memcpy(o + 16, n.Rloc, sizeof(n.Rloc));
        }
        if (first_child) first_child[i] = n.first_child;
    }
    for (size_t i = 0; i < m.tris.size(); i++) {
        const TriRec &t = m.tris[i];
        if (tri_verts) std::memcpy(tri_verts + 9 * i, t.v, sizeof(t.v));
        if (tri_ids) tri_ids[i] = t.id;
        if (tri_vidx)
            for (int k = 0; k < 3; k++) tri_vidx[3 * i + k] = t.idx[k];
    }
    return C2A_OK;
}

c2a_status c2a_model_download_obb(c2a_context *ctx, int32_t id, double *obb)
{
    if (!ctx || !obb) return C2A_ERR_INVALID_ARGUMENT;
    if (id < 0 || id >= (int32_t)ctx->models.size() || !ctx->models[id].live) return C2A_ERR_BAD_MODEL;
    const BuiltModel &m = ctx->models[id].host;
    for (size_t i = 0; i < m.obbs.size(); i++) {
        std::memcpy(obb + 6 * i, m.obbs[i].To, sizeof(m.obbs[i].To));
        std::memcpy(obb + 6 * i + 3, m.obbs[i].d, sizeof(m.obbs[i].d));
    }
    return C2A_OK;
}

c2a_status c2a_model_free(c2a_context *ctx, int32_t id)
{
    if (!ctx) return C2A_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    if (id < 0 || id >= (int32_t)ctx->models.size() || !ctx->models[id].live) return C2A_ERR_BAD_MODEL;
    ModelSlot &s = ctx->models[id];
    if (ctx->device >= 0) {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        free_slot(s);
    }
    s.live = false;
    s.host = BuiltModel();
    ctx->models_dirty = true;
    ctx->models_gen = next_models_gen();
    return C2A_OK;
}

namespace {
c2a_status solve_device(c2a_context *ctx, const c2a_query *d_queries, int32_t n, const c2a_params *params,
                        c2a_result *d_results, c2a_contact *d_contacts, void *stream, const uint32_t *hints, int nh,
                        const int32_t *user_order = nullptr);
}

c2a_status c2a_solve_batch_device(c2a_context *ctx, const c2a_query *d_queries, int32_t n, const c2a_params *params,
                                  c2a_result *d_results, c2a_contact *d_contacts, void *stream)
{
    C2A_RANGE("c2a_solve_batch_device");
    return solve_device(ctx, d_queries, n, params, d_results, d_contacts, stream, nullptr, 0);
}

c2a_status c2a_solve_batch_ordered(c2a_context *ctx, const c2a_query *d_queries, int32_t n,
                                   const c2a_params *params, const int32_t *d_order, c2a_result *d_results,
                                   c2a_contact *d_contacts, void *stream)
{
    C2A_RANGE("c2a_solve_batch_ordered");
    if (!params || params->mode != C2A_MODE_REFERENCE ||
        (params->engine != C2A_ENGINE_AUTO && params->engine != C2A_ENGINE_WARP &&
         params->engine != C2A_ENGINE_SPEC) ||
        (n > 0 && !d_order))
        return C2A_ERR_INVALID_ARGUMENT;
    return solve_device(ctx, d_queries, n, params, d_results, d_contacts, stream, nullptr, 0, d_order);
}

c2a_status c2a_solve_batch_hinted(c2a_context *ctx, const c2a_query *d_queries, int32_t n, const c2a_params *params,
                                  const uint32_t *d_hints, int32_t hints_per_query, c2a_result *d_results,
                                  c2a_contact *d_contacts, void *stream)
{
    C2A_RANGE("c2a_solve_batch_hinted");
    if (!params || params->mode != C2A_MODE_CANONICAL || hints_per_query < 0 || hints_per_query > 16 ||
        (hints_per_query > 0 && !d_hints))
        return C2A_ERR_INVALID_ARGUMENT;
    return solve_device(ctx, d_queries, n, params, d_results, d_contacts, stream, d_hints, hints_per_query);
}

namespace {
c2a_status solve_device(c2a_context *ctx, const c2a_query *d_queries, int32_t n, const c2a_params *params,
                        c2a_result *d_results, c2a_contact *d_contacts, void *stream, const uint32_t *hints, int nh,
                        const int32_t *user_order)
{
    if (ctx && ctx->device < 0) return C2A_ERR_NO_DEVICE;
    if (!ctx || n < 0 || !params_ok(params) || (n > 0 && (!d_queries || !d_results))) return C2A_ERR_INVALID_ARGUMENT;
    if (n == 0) return C2A_OK;
    C2A_CUDA(cudaSetDevice(ctx->device));
    int deepest = 0;
    c2a_status st = check_depths(ctx, &deepest);
    if (st) return st;
    st = sync_models(ctx);
    if (st) return st;
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    c2a_params prm = *params;
    if (!d_contacts) prm.contacts_per_query = 0;
    if (prm.mode == C2A_MODE_CANONICAL && prm.engine == C2A_ENGINE_BATCHED)
        return wave_solve(&ctx->wave, ctx->sm_count, s, d_queries, n, ctx->d_models, (int)ctx->models.size(), prm,
                          d_results, d_contacts, &ctx->launches, hints, nh);
    if (prm.mode == C2A_MODE_CANONICAL) {
        if (!ctx->canonical_blocks_per_sm) {
            int occ = 0;
            C2A_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, c2a_canonical_kernel, kThreads, 0));
            ctx->canonical_blocks_per_sm = occ > 0 ? occ : 1;
        }
        const int most = ctx->sm_count * blocks_per_sm(ctx->canonical_blocks_per_sm, prm.warps_per_sm, kThreads);
        const int need = (int)(((int64_t)n * 32 + kThreads - 1) / kThreads);
        const int blocks = need < most ? need : most;
        st = ensure_fronts(ctx, (size_t)blocks * (kThreads / 32), (size_t)most * (kThreads / 32));
        if (st) return st;
        C2A_CUDA(cudaMemsetAsync(ctx->d_counter, 0, sizeof(unsigned int), s));
        c2a_canonical_kernel<<<blocks, kThreads, 0, s>>>(d_queries, n, ctx->d_models, (int)ctx->models.size(), prm,
                                                        d_results, d_contacts, ctx->d_counter, ctx->d_fronts, hints,
                                                        nh);
        ctx->launches++;
        C2A_CUDA(cudaGetLastError());
        return C2A_OK;
    }
    C2A_CUDA(cudaMemsetAsync(ctx->d_counter, 0, sizeof(unsigned int), s));
    if (prm.engine != C2A_ENGINE_THREAD && (size_t)n > ctx->order_cap) {
        C2A_CUDA(cudaStreamSynchronize(s));
        if (ctx->d_order) cudaFree(ctx->d_order);
        ctx->d_order = nullptr;
        ctx->order_cap = 0;
        C2A_CUDA(cudaMalloc(&ctx->d_order, sizeof(int32_t) * (size_t)n));
        ctx->order_cap = (size_t)n;
    }
    if (prm.engine == C2A_ENGINE_SPEC) {
        /* the stack holds one pending pair per BVTT level: 2 depth + 2 entries;
         * records: the replay's path (one per BVTT level) plus 64 for speculation */
        const int cap = 2 * deepest + 2 > 4 ? 2 * deepest + 2 : 4;
        const int nrec = 2 * deepest + 2 + C2A_SPEC_EXTRA;
        const size_t per = warp_shared_bytes(cap) + spec_shared_bytes(nrec);
        const size_t smem = per * (kThreads / 32);
        if (!ctx->spec_smem_attr) {
            int optin = 0;
            C2A_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
            C2A_CUDA(cudaFuncSetAttribute(c2a_solve_spec_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
            ctx->spec_smem_attr = true;
        }
        if (ctx->spec_cap != cap || ctx->spec_nrec != nrec) {
            int occ = 0;
            C2A_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, c2a_solve_spec_kernel, kThreads, smem));
            if (occ < 1) return C2A_ERR_TREE_TOO_DEEP; /* the per-warp state does not fit shared memory */
            ctx->spec_blocks_per_sm = occ;
            ctx->spec_cap = cap;
            ctx->spec_nrec = nrec;
        }
        const int most = ctx->sm_count * blocks_per_sm(ctx->spec_blocks_per_sm, prm.warps_per_sm, kThreads);
        const int need = (int)(((int64_t)n * 32 + kThreads - 1) / kThreads);
        const int blocks = need < most ? need : most;
        const size_t gbytes = spec_global_bytes(nrec) * (size_t)blocks * (kThreads / 32);
        if (gbytes > ctx->spec_bytes) {
            C2A_CUDA(cudaStreamSynchronize(s));
            if (ctx->d_spec) cudaFree(ctx->d_spec);
            ctx->d_spec = nullptr;
            ctx->spec_bytes = 0;
            const size_t want = spec_global_bytes(nrec) * (size_t)most * (kThreads / 32);
            C2A_CUDA(cudaMalloc(&ctx->d_spec, want > gbytes ? want : gbytes));
            ctx->spec_bytes = want > gbytes ? want : gbytes;
        }
        if (!user_order) { /* queries whose bounding spheres approach go first */
            C2A_CUDA(cudaMemsetAsync(ctx->d_counter + 1, 0, 2 * sizeof(unsigned int), s));
            c2a_schedule_kernel<<<(n + 255) / 256, 256, 0, s>>>(d_queries, n, ctx->d_models,
                                                                 (int)ctx->models.size(), ctx->d_order,
                                                                 ctx->d_counter + 1);
            ctx->launches++;
        }
        c2a_solve_spec_kernel<<<blocks, kThreads, smem, s>>>(d_queries, n, ctx->d_models, (int)ctx->models.size(), prm,
                                                             d_results, d_contacts, ctx->d_counter,
                                                             user_order ? user_order : ctx->d_order, cap, nrec,
                                                             ctx->d_spec);
        ctx->launches++;
        C2A_CUDA(cudaGetLastError());
        return C2A_OK;
    }
    if (prm.engine != C2A_ENGINE_THREAD) {
        /* the stack holds one pending pair per BVTT level: 2 depth + 2 entries */
        const int cap = 2 * deepest + 2 > 4 ? 2 * deepest + 2 : 4;
        const size_t smem = warp_shared_bytes(cap) * (kThreads / 32);
        if (!ctx->warp_smem_attr) {
            C2A_CUDA(cudaFuncSetAttribute(c2a_solve_warp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)(warp_shared_bytes(C2A_STACK_DEPTH) * (kThreads / 32))));
            ctx->warp_smem_attr = true;
        }
        if (ctx->warp_cap != cap) {
            int occ = 0;
            C2A_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, c2a_solve_warp_kernel, kThreads, smem));
            ctx->warp_blocks_per_sm = occ > 0 ? occ : 1;
            ctx->warp_cap = cap;
        }
        const int heavy = prm.heavy_prefix < n ? prm.heavy_prefix : n;
        if (user_order && heavy > 0) {
            /* the head of the order on SM sub-partitions of its own (c2a_solve_warp_split_kernel) */
            const size_t smem8 = warp_shared_bytes(cap) * (kSplitThreads / 32);
            if ((int)smem8 > ctx->split_smem_attr) {
                C2A_CUDA(cudaFuncSetAttribute(c2a_solve_warp_split_kernel,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem8));
                ctx->split_smem_attr = (int)smem8;
            }
            int hb = (heavy + 3) / 4; /* four heavy warps per block */
            if (hb > ctx->sm_count / 2) hb = ctx->sm_count / 2; /* at least half the SMs at full occupancy */
            C2A_CUDA(cudaMemsetAsync(ctx->d_counter + 3, 0, sizeof(unsigned int), s));
            c2a_solve_warp_split_kernel<<<ctx->sm_count, kSplitThreads, smem8, s>>>(
                d_queries, n, heavy, hb, ctx->d_models, (int)ctx->models.size(), prm, d_results, d_contacts,
                ctx->d_counter, ctx->d_counter + 3, user_order, cap);
            ctx->launches++;
            C2A_CUDA(cudaGetLastError());
            return C2A_OK;
        }
        const int most = ctx->sm_count * blocks_per_sm(ctx->warp_blocks_per_sm, prm.warps_per_sm, kThreads);
        const int need = (int)(((int64_t)n * 32 + kThreads - 1) / kThreads);
        if (!user_order) { /* queries whose bounding spheres approach go first */
            C2A_CUDA(cudaMemsetAsync(ctx->d_counter + 1, 0, 2 * sizeof(unsigned int), s));
            c2a_schedule_kernel<<<(n + 255) / 256, 256, 0, s>>>(d_queries, n, ctx->d_models,
                                                                 (int)ctx->models.size(), ctx->d_order,
                                                                 ctx->d_counter + 1);
            ctx->launches++;
        }
        c2a_solve_warp_kernel<<<need < most ? need : most, kThreads, smem, s>>>(
            d_queries, n, ctx->d_models, (int)ctx->models.size(), prm, d_results, d_contacts, ctx->d_counter,
            user_order ? user_order : ctx->d_order, cap);
        ctx->launches++;
        C2A_CUDA(cudaGetLastError());
        return C2A_OK;
    }
    const Shape sh = shape_for(ctx, n, prm.warps_per_sm);
    c2a_solve_kernel<<<sh.blocks, sh.threads, 0, s>>>(d_queries, n, ctx->d_models, (int)ctx->models.size(), prm,
                                                       d_results, d_contacts, ctx->d_counter);
    ctx->launches++;
    C2A_CUDA(cudaGetLastError());
    return C2A_OK;
}
} // namespace

c2a_status c2a_distance_batch(c2a_context *ctx, const c2a_query *queries, int32_t n, c2a_distance_result *results)
{
    C2A_RANGE("c2a_distance_batch");
    if (ctx && ctx->device < 0) return C2A_ERR_NO_DEVICE;
    if (!ctx || n < 0 || (n > 0 && (!queries || !results))) return C2A_ERR_INVALID_ARGUMENT;
    if (n == 0) return C2A_OK;
    std::lock_guard<std::mutex> lock(ctx->mu);
    C2A_CUDA(cudaSetDevice(ctx->device));
    c2a_status st = sync_models(ctx);
    if (st) return st;
    const size_t nq = (size_t)n;
    auto up = [](size_t b) { return ((b + 255) / 256) * 256; };
    const size_t qbytes = up(sizeof(c2a_query) * nq), rbytes = up(sizeof(c2a_distance_result) * nq);
    st = ensure_buf(ctx, qbytes + rbytes);
    if (st) return st;
    c2a_query *dq = (c2a_query *)ctx->d_buf;
    c2a_distance_result *dr = (c2a_distance_result *)((char *)ctx->d_buf + qbytes);
    C2A_CUDA(cudaMemcpyAsync(dq, queries, sizeof(c2a_query) * nq, cudaMemcpyHostToDevice, ctx->stream));
    if (!ctx->distance_blocks_per_sm) {
        int occ = 0;
        C2A_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, c2a_distance_kernel, kThreads, 0));
        ctx->distance_blocks_per_sm = occ > 0 ? occ : 1;
    }
    const int most = ctx->sm_count * ctx->distance_blocks_per_sm;
    const int need = (int)(((int64_t)n * 32 + kThreads - 1) / kThreads);
    const int blocks = need < most ? need : most;
    st = ensure_fronts(ctx, (size_t)blocks * (kThreads / 32), (size_t)most * (kThreads / 32));
    if (st) return st;
    C2A_CUDA(cudaMemsetAsync(ctx->d_counter, 0, sizeof(unsigned int), ctx->stream));
    c2a_distance_kernel<<<blocks, kThreads, 0, ctx->stream>>>(dq, n, ctx->d_models, (int)ctx->models.size(), dr,
                                                               ctx->d_counter, ctx->d_fronts);
    ctx->launches++;
    C2A_CUDA(cudaGetLastError());
    C2A_CUDA(cudaMemcpyAsync(results, dr, sizeof(c2a_distance_result) * nq, cudaMemcpyDeviceToHost, ctx->stream));
    C2A_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int32_t i = 0; i < n; i++)
        if (results[i].status) return C2A_ERR_QUERY_FAILED;
    return C2A_OK;
}

namespace {
/* the host-buffer entry points: queries in, the batch (in the caller's device
 * order when d_order is given), results and dense contacts out */
c2a_status solve_host(c2a_context *ctx, const c2a_query *queries, int32_t n, const c2a_params *params,
                      c2a_result *results, c2a_contact *contacts, const int32_t *d_order)
{
    if (ctx && ctx->device < 0) return C2A_ERR_NO_DEVICE;
    if (!ctx || n < 0 || !params_ok(params) || (n > 0 && (!queries || !results))) return C2A_ERR_INVALID_ARGUMENT;
    if (n == 0) return C2A_OK;
    std::lock_guard<std::mutex> lock(ctx->mu);
    C2A_CUDA(cudaSetDevice(ctx->device));
    const size_t nq = (size_t)n;
    const size_t cpq = contacts ? (size_t)params->contacts_per_query : 0;
    const size_t nblocks = (nq + kScanBlock - 1) / kScanBlock;
    auto up = [](size_t b) { return ((b + 255) / 256) * 256; };
    const size_t qbytes = up(sizeof(c2a_query) * nq), rbytes = up(sizeof(c2a_result) * nq);
    const size_t cbytes = up(sizeof(c2a_contact) * nq * cpq), sbytes = up(sizeof(int32_t) * (nblocks + 1));
    c2a_status st = ensure_buf(ctx, qbytes + rbytes + 2 * cbytes + sbytes);
    if (st) return st;
    char *base = (char *)ctx->d_buf;
    c2a_query *dq = (c2a_query *)base;
    c2a_result *dr = (c2a_result *)(base + qbytes);
    c2a_contact *dc = cpq ? (c2a_contact *)(base + qbytes + rbytes) : nullptr;
    c2a_contact *dense = cpq ? (c2a_contact *)(base + qbytes + rbytes + cbytes) : nullptr;
    int32_t *sums = (int32_t *)(base + qbytes + rbytes + 2 * cbytes);
    C2A_CUDA(cudaMemcpyAsync(dq, queries, sizeof(c2a_query) * nq, cudaMemcpyHostToDevice, ctx->stream));
    c2a_params prm = *params;
    if (!cpq) prm.contacts_per_query = 0;
    st = d_order ? c2a_solve_batch_ordered(ctx, dq, n, &prm, d_order, dr, dc, ctx->stream)
                 : c2a_solve_batch_device(ctx, dq, n, &prm, dr, dc, ctx->stream);
    if (st) return st;
    int32_t total = 0;
    if (cpq) {
        c2a_scan_blocks<<<(unsigned)nblocks, kScanBlock, 0, ctx->stream>>>(dr, n, (int)cpq, sums);
        c2a_scan_totals<<<1, 1, 0, ctx->stream>>>(sums, (int)nblocks, sums + nblocks);
        c2a_gather_contacts<<<(unsigned)nq, 32, 0, ctx->stream>>>(dr, n, (int)cpq, sums, dc, dense);
        ctx->launches += 3;
        C2A_CUDA(cudaGetLastError());
        C2A_CUDA(cudaMemcpyAsync(&total, sums + nblocks, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    }
    C2A_CUDA(cudaMemcpyAsync(results, dr, sizeof(c2a_result) * nq, cudaMemcpyDeviceToHost, ctx->stream));
    C2A_CUDA(cudaStreamSynchronize(ctx->stream));
    if (cpq && total > 0) {
        C2A_CUDA(cudaMemcpyAsync(contacts, dense, sizeof(c2a_contact) * (size_t)total, cudaMemcpyDeviceToHost,
                                 ctx->stream));
        C2A_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    ctx->last_contacts = total;
    for (int32_t i = 0; i < n; i++)
        if (results[i].status & ~(C2A_QUERY_ITER_CAP | C2A_QUERY_CONTACT_OVERFLOW)) return C2A_ERR_QUERY_FAILED;
    return C2A_OK;
}
} // namespace

c2a_status c2a_solve_batch(c2a_context *ctx, const c2a_query *queries, int32_t n, const c2a_params *params,
                           c2a_result *results, c2a_contact *contacts)
{
    C2A_RANGE("c2a_solve_batch");
    return solve_host(ctx, queries, n, params, results, contacts, nullptr);
}

c2a_status c2a_solve_batch_ordered_host(c2a_context *ctx, const c2a_query *queries, int32_t n,
                                        const c2a_params *params, const int32_t *d_order, c2a_result *results,
                                        c2a_contact *contacts)
{
    C2A_RANGE("c2a_solve_batch_ordered_host");
    if (n > 0 && !d_order) return C2A_ERR_INVALID_ARGUMENT;
    return solve_host(ctx, queries, n, params, results, contacts, d_order);
}

c2a_status c2a_solve_batch_noalloc(c2a_context *ctx, const c2a_query *d_queries, int32_t n,
                                   const c2a_params *params, c2a_result *d_results, c2a_contact *d_contacts,
                                   void *stream)
{
    C2A_RANGE("c2a_solve_batch_noalloc");
    if (ctx && ctx->device < 0) return C2A_ERR_NO_DEVICE;
    if (!ctx || n < 0 || !params_ok(params) || (n > 0 && (!d_queries || !d_results))) return C2A_ERR_INVALID_ARGUMENT;
    if (n == 0) return C2A_OK;
    if (params->mode != C2A_MODE_REFERENCE) {
        fprintf(stderr, "c2a_solve_batch_noalloc: only C2A_MODE_REFERENCE runs without allocations\n");
        return C2A_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lock(ctx->mu);
    const size_t num_models = ctx->models.size();
    if (num_models > C2A_NOALLOC_MAX_MODELS) {
        fprintf(stderr,
                "c2a_solve_batch_noalloc: the context holds %zu models; the fixed table of this entry point holds "
                "at most %d\n",
                num_models, C2A_NOALLOC_MAX_MODELS);
        return C2A_ERR_NOALLOC_CAPACITY;
    }
    C2A_CUDA(cudaSetDevice(ctx->device));
    c2a_status st = check_depths(ctx);
    if (st) return st;
    unsigned char *scratch = nullptr;
    st = noalloc_scratch(ctx->device, &scratch); /* looked up by c2a_create; no CUDA call here */
    if (st) return st;
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    DevModel *d_table = reinterpret_cast<DevModel *>(scratch + kNoallocTableOffset);
    unsigned int *d_counter = reinterpret_cast<unsigned int *>(scratch);
    {
        /* the model table is uploaded only when the array holds another
         * context's table or this context's models changed since; the copy
         * is from the stack, so wait for it before the frame goes away */
        std::lock_guard<std::mutex> glock(g_noalloc_mu);
        if (g_noalloc_table_gen[ctx->device] != ctx->models_gen) {
            DevModel table[C2A_NOALLOC_MAX_MODELS];
            for (size_t i = 0; i < num_models; i++) table[i] = dev_model_of(ctx->models[i]);
            if (num_models)
                C2A_CUDA(cudaMemcpyAsync(d_table, table, sizeof(DevModel) * num_models, cudaMemcpyHostToDevice, s));
            C2A_CUDA(cudaStreamSynchronize(s));
            g_noalloc_table_gen[ctx->device] = ctx->models_gen;
        }
    }
    C2A_CUDA(cudaMemsetAsync(d_counter, 0, sizeof(unsigned int), s)); /* the last call left its count here */
    c2a_params prm = *params;
    if (!d_contacts) prm.contacts_per_query = 0;
    const Shape sh = shape_for(ctx, n, prm.warps_per_sm);
    c2a_solve_kernel<<<sh.blocks, sh.threads, 0, s>>>(d_queries, n, d_table, (int)num_models, prm, d_results,
                                                       d_contacts, d_counter);
    ctx->launches++;
    C2A_CUDA(cudaGetLastError());
    return C2A_OK;
}

static_assert(sizeof(c2a_tolerance_result) == 80 && sizeof(c2a_collide_result) == 24, "record layouts");

namespace {
/* a pair per warp while the batch leaves every pair a warp slot (16 per SM),
 * else a pair per lane: the lanes of a warp walk different trees, so packing
 * pairs into a warp serialises their paths */
int static_pairs_per_warp(const c2a_context *ctx, int n) { return n <= ctx->sm_count * 16 ? 1 : 32; }

/* the host-buffer static queries: queries (and the per-query doubles) in,
 * one launch, results (and the pairs) out */
c2a_status static_prepare(c2a_context *ctx, const c2a_query *queries, int32_t n)
{
    if (ctx && ctx->device < 0) return C2A_ERR_NO_DEVICE;
    if (!ctx || n < 0 || (n > 0 && !queries)) return C2A_ERR_INVALID_ARGUMENT;
    C2A_CUDA(cudaSetDevice(ctx->device));
    c2a_status st = check_depths(ctx);
    if (st) return st;
    return sync_models(ctx);
}
} // namespace

c2a_status c2a_tolerance_batch(c2a_context *ctx, const c2a_query *queries, int32_t n, const double *tolerance,
                               c2a_tolerance_result *results)
{
    C2A_RANGE("c2a_tolerance_batch");
    if (n > 0 && (!tolerance || !results)) return C2A_ERR_INVALID_ARGUMENT;
    if (ctx) {
        std::lock_guard<std::mutex> lock(ctx->mu);
        c2a_status st = static_prepare(ctx, queries, n);
        if (st || n == 0) return st;
        const size_t nq = (size_t)n;
        const size_t a = ((sizeof(c2a_query) * nq + 255) / 256) * 256, b = ((sizeof(double) * nq + 255) / 256) * 256;
        st = ensure_buf(ctx, a + b + sizeof(c2a_tolerance_result) * nq);
        if (st) return st;
        char *base = (char *)ctx->d_buf;
        c2a_query *dq = (c2a_query *)base;
        double *dt = (double *)(base + a);
        c2a_tolerance_result *dr = (c2a_tolerance_result *)(base + a + b);
        C2A_CUDA(cudaMemcpyAsync(dq, queries, sizeof(c2a_query) * nq, cudaMemcpyHostToDevice, ctx->stream));
        C2A_CUDA(cudaMemcpyAsync(dt, tolerance, sizeof(double) * nq, cudaMemcpyHostToDevice, ctx->stream));
        const int ppw = static_pairs_per_warp(ctx, n);
        const int warps = (n + ppw - 1) / ppw;
        c2a_tolerance_kernel<<<(warps * 32 + kThreads - 1) / kThreads, kThreads, 0, ctx->stream>>>(
            dq, n, dt, ctx->d_models, (int)ctx->models.size(), dr, ppw);
        ctx->launches++;
        C2A_CUDA(cudaGetLastError());
        C2A_CUDA(cudaMemcpyAsync(results, dr, sizeof(c2a_tolerance_result) * nq, cudaMemcpyDeviceToHost, ctx->stream));
        C2A_CUDA(cudaStreamSynchronize(ctx->stream));
        for (int32_t i = 0; i < n; i++)
            if (results[i].status) return C2A_ERR_QUERY_FAILED;
        return C2A_OK;
    }
    return C2A_ERR_INVALID_ARGUMENT;
}

c2a_status c2a_collide_batch(c2a_context *ctx, const c2a_query *queries, int32_t n, int32_t flag,
                             int32_t pairs_per_query, c2a_collide_result *results, int32_t *pairs)
{
    C2A_RANGE("c2a_collide_batch");
    if (n > 0 && !results) return C2A_ERR_INVALID_ARGUMENT;
    if (pairs_per_query < 0 || (flag != 1 && flag != 2)) return C2A_ERR_INVALID_ARGUMENT;
    if (!ctx) return C2A_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(ctx->mu);
    c2a_status st = static_prepare(ctx, queries, n);
    if (st || n == 0) return st;
    const size_t nq = (size_t)n, slots = pairs ? (size_t)pairs_per_query : 0;
    const size_t a = ((sizeof(c2a_query) * nq + 255) / 256) * 256;
    const size_t r = ((sizeof(c2a_collide_result) * nq + 255) / 256) * 256;
    st = ensure_buf(ctx, a + r + 2 * sizeof(int32_t) * nq * slots);
    if (st) return st;
    char *base = (char *)ctx->d_buf;
    c2a_query *dq = (c2a_query *)base;
    c2a_collide_result *dr = (c2a_collide_result *)(base + a);
    int32_t *dp = slots ? (int32_t *)(base + a + r) : nullptr;
    C2A_CUDA(cudaMemcpyAsync(dq, queries, sizeof(c2a_query) * nq, cudaMemcpyHostToDevice, ctx->stream));
    const int ppw = static_pairs_per_warp(ctx, n);
    const int warps = (n + ppw - 1) / ppw;
    c2a_collide_kernel<<<(warps * 32 + kThreads - 1) / kThreads, kThreads, 0, ctx->stream>>>(
        dq, n, flag, ctx->d_models, (int)ctx->models.size(), (int)slots, dr, dp, ppw);
    ctx->launches++;
    C2A_CUDA(cudaGetLastError());
    C2A_CUDA(cudaMemcpyAsync(results, dr, sizeof(c2a_collide_result) * nq, cudaMemcpyDeviceToHost, ctx->stream));
    if (slots)
        C2A_CUDA(cudaMemcpyAsync(pairs, dp, 2 * sizeof(int32_t) * nq * slots, cudaMemcpyDeviceToHost, ctx->stream));
    C2A_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int32_t i = 0; i < n; i++)
        if (results[i].status & ~C2A_QUERY_CONTACT_OVERFLOW) return C2A_ERR_QUERY_FAILED;
    return C2A_OK;
}

c2a_status c2a_toc_step_batch(c2a_context *ctx, const c2a_query *queries, int32_t n, const double *lambda,
                              const int32_t *num_ca, const double *prev_mint, const c2a_params *params,
                              c2a_result *results)
{
    C2A_RANGE("c2a_toc_step_batch");
    if (ctx && ctx->device < 0) return C2A_ERR_NO_DEVICE;
    if (!ctx || n < 0 || !params_ok(params) || params->mode != C2A_MODE_REFERENCE ||
        (n > 0 && (!queries || !lambda || !num_ca || !prev_mint || !results)))
        return C2A_ERR_INVALID_ARGUMENT;
    if (n == 0) return C2A_OK;
    std::lock_guard<std::mutex> lock(ctx->mu);
    C2A_CUDA(cudaSetDevice(ctx->device));
    c2a_status st = check_depths(ctx);
    if (st) return st;
    st = sync_models(ctx);
    if (st) return st;
    const size_t nq = (size_t)n;
    const size_t a = ((sizeof(c2a_query) * nq + 255) / 256) * 256, b = ((sizeof(double) * nq + 255) / 256) * 256;
    const size_t c = ((sizeof(int32_t) * nq + 255) / 256) * 256, r = sizeof(c2a_result) * nq;
    st = ensure_buf(ctx, a + 2 * b + c + r);
    if (st) return st;
    char *base = (char *)ctx->d_buf;
    c2a_query *dq = (c2a_query *)base;
    double *dl = (double *)(base + a);
    double *dm = (double *)(base + a + b);
    int32_t *dn = (int32_t *)(base + a + 2 * b);
    c2a_result *dr = (c2a_result *)(base + a + 2 * b + c);
    C2A_CUDA(cudaMemcpyAsync(dq, queries, sizeof(c2a_query) * nq, cudaMemcpyHostToDevice, ctx->stream));
    C2A_CUDA(cudaMemcpyAsync(dl, lambda, sizeof(double) * nq, cudaMemcpyHostToDevice, ctx->stream));
    C2A_CUDA(cudaMemcpyAsync(dm, prev_mint, sizeof(double) * nq, cudaMemcpyHostToDevice, ctx->stream));
    C2A_CUDA(cudaMemcpyAsync(dn, num_ca, sizeof(int32_t) * nq, cudaMemcpyHostToDevice, ctx->stream));
    c2a_step_kernel<<<(n + kThreads - 1) / kThreads, kThreads, 0, ctx->stream>>>(
        dq, n, dl, dn, dm, ctx->d_models, (int)ctx->models.size(), *params, dr);
    ctx->launches++;
    C2A_CUDA(cudaGetLastError());
    C2A_CUDA(cudaMemcpyAsync(results, dr, r, cudaMemcpyDeviceToHost, ctx->stream));
    C2A_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int32_t i = 0; i < n; i++)
        if (results[i].status) return C2A_ERR_QUERY_FAILED;
    return C2A_OK;
}

c2a_status c2a_contact_only_batch(c2a_context *ctx, const c2a_query *queries, int32_t n, const double *threshold,
                                  int32_t contacts_per_query, c2a_result *results, c2a_contact *contacts)
{
    C2A_RANGE("c2a_contact_only_batch");
    if (ctx && ctx->device < 0) return C2A_ERR_NO_DEVICE;
    if (!ctx || n < 0 || contacts_per_query < 0 || (n > 0 && (!queries || !threshold || !results)))
        return C2A_ERR_INVALID_ARGUMENT;
    if (n == 0) return C2A_OK;
    std::lock_guard<std::mutex> lock(ctx->mu);
    C2A_CUDA(cudaSetDevice(ctx->device));
    c2a_status st = check_depths(ctx);
    if (st) return st;
    st = sync_models(ctx);
    if (st) return st;
    const size_t nq = (size_t)n, cpq = contacts ? (size_t)contacts_per_query : 0;
    const size_t a = ((sizeof(c2a_query) * nq + 255) / 256) * 256, b = ((sizeof(double) * nq + 255) / 256) * 256;
    const size_t r = ((sizeof(c2a_result) * nq + 255) / 256) * 256, cb = sizeof(c2a_contact) * nq * cpq;
    st = ensure_buf(ctx, a + b + r + cb);
    if (st) return st;
    char *base = (char *)ctx->d_buf;
    c2a_query *dq = (c2a_query *)base;
    double *dt = (double *)(base + a);
    c2a_result *dr = (c2a_result *)(base + a + b);
    c2a_contact *dc = cpq ? (c2a_contact *)(base + a + b + r) : nullptr;
    C2A_CUDA(cudaMemcpyAsync(dq, queries, sizeof(c2a_query) * nq, cudaMemcpyHostToDevice, ctx->stream));
    C2A_CUDA(cudaMemcpyAsync(dt, threshold, sizeof(double) * nq, cudaMemcpyHostToDevice, ctx->stream));
    c2a_contact_kernel<<<(n + kThreads - 1) / kThreads, kThreads, 0, ctx->stream>>>(
        dq, n, dt, ctx->d_models, (int)ctx->models.size(), (int)cpq, dr, dc);
    ctx->launches++;
    C2A_CUDA(cudaGetLastError());
    C2A_CUDA(cudaMemcpyAsync(results, dr, sizeof(c2a_result) * nq, cudaMemcpyDeviceToHost, ctx->stream));
    if (cpq) C2A_CUDA(cudaMemcpyAsync(contacts, dc, cb, cudaMemcpyDeviceToHost, ctx->stream));
    C2A_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int32_t i = 0; i < n; i++)
        if (results[i].status & ~C2A_QUERY_CONTACT_OVERFLOW) return C2A_ERR_QUERY_FAILED;
    return C2A_OK;
}

#ifdef C2A_STATS
/* profiling builds only: copies the event counters out and clears them */
c2a_status c2a_stats_read(unsigned long long *out, int count)
{
    if (!out || count < ST_COUNT) return C2A_ERR_INVALID_ARGUMENT;
    C2A_CUDA(cudaDeviceSynchronize());
    C2A_CUDA(cudaMemcpyFromSymbol(out, g_c2a_stats, sizeof(unsigned long long) * ST_COUNT));
    unsigned long long zero[ST_COUNT] = {};
    C2A_CUDA(cudaMemcpyToSymbol(g_c2a_stats, zero, sizeof(zero)));
    return C2A_OK;
}
#endif

c2a_status c2a_motion_setup(const double *R0, const double *T0, const double *R1, const double *T1, double *out)
{
    if (!R0 || !T0 || !R1 || !T1 || !out) return C2A_ERR_INVALID_ARGUMENT;
    Motion m;
    motion_setup(m, R0, T0, R1, T1);
    for (int i = 0; i < 3; i++) {
        out[i] = m.axis[i];
        out[4 + i] = m.cv[i];
    }
    out[3] = m.angVel;
    for (int i = 0; i < 4; i++) out[7 + i] = m.q0[i];
    return C2A_OK;
}

c2a_status c2a_motion_integrate(const double *R0, const double *T0, const double *R1, const double *T1, double t,
                                double *R, double *T, double *qua)
{
    if (!R0 || !T0 || !R1 || !T1) return C2A_ERR_INVALID_ARGUMENT;
    Motion m;
    motion_setup(m, R0, T0, R1, T1);
    double Rr[9], Tt[3], orn[4];
    motion_integrate(m, t, Rr, Tt, orn);
    if (R) std::memcpy(R, Rr, sizeof(Rr));
    if (T) std::memcpy(T, Tt, sizeof(Tt));
    if (qua) {
        qua[0] = orn[3];
        qua[1] = orn[0];
        qua[2] = orn[1];
        qua[3] = orn[2];
        qua[4] = Tt[0];
        qua[5] = Tt[1];
        qua[6] = Tt[2];
    }
    return C2A_OK;
}

} // extern "C"
