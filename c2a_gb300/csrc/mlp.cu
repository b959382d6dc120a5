/*
 * mlp.cu -- the learned seeding's network kernels (include/c2a_mlp.h).
 *
 * GEMM: out = A B^T on tcgen05 with the accumulator in tensor memory, the
 * operands brought in by TMA (k_gemm_tma; the layout and the pipeline are
 * described above the kernel).  The epilogue adds the bias and applies GELU
 * (erff, called) in registers and writes FP32 and/or bf16.
 *
 * Everything else (transposes, GELU backward, softmax cross-entropy, column
 * sums, Adam, the input assembly and its embedding scatter, top-k) is
 * bandwidth-bound elementwise or row-wise work.
 */
#include <cuda.h> /* CUtensorMap and its enums; the encoder is reached through the runtime's entry-point query */
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/c2a_mlp.h"

namespace {

c2a_status launch_status()
{
    const cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) return C2A_OK;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return C2A_ERR_NO_DEVICE;
    return C2A_ERR_CUDA;
}

__device__ __forceinline__ float bf2f(uint16_t h) { return __uint_as_float((uint32_t)h << 16); }
__device__ __forceinline__ uint16_t f2bf(float f) { return __bfloat16_as_ushort(__float2bfloat16_rn(f)); }

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x)
{
    const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
    return cdf + x * pdf;
}

/* ------------------------------------------------------------------ GEMM */

/* out = A B^T with A (M x K) and B (N x K) bf16, K contiguous, on the
 * fifth-generation tensor cores.  A CTA of four warps owns a 128 x 128 output
 * tile; its FP32 accumulator lives in 128 columns of tensor memory
 * (tcgen05.alloc).  The A and B tiles arrive by TMA (cp.async.bulk.tensor
 * with 128-byte swizzle; K past the end is filled with zeros) in steps of 64
 * into three shared-memory stages; one thread issues the TMA copies, another
 * the tcgen05.mma (M 128, N 128, K 16, bf16 x bf16 -> FP32; SWIZZLE_128B
 * K-major descriptors: 8-row groups 1 KiB apart, the K = 16 sub-steps 32 bytes
 * apart inside the 128-byte swizzle atom), with a full and an empty mbarrier
 * per stage between them (tcgen05.commit arms the empty one).  After the last
 * commit all four warps read the accumulator with tcgen05.ld (warp w: rows
 * 32 w .. 32 w + 31, one row per thread), add the bias, apply GELU and write
 * FP32 and/or bf16 in 16-byte stores.  Two CTAs fit an SM (100 KiB of shared
 * memory, 128 TMEM columns each).  Every mbarrier wait is bounded by the
 * global timer: a wait that runs out records an error (c2a_mlp_check) and the
 * CTA still releases its tensor memory. */
constexpr int kTcM = 128, kTcN = 128, kTcK = 64, kTcThreads = 128;
__device__ int g_tc_err; /* set when a bounded mbarrier wait of k_gemm_tma ran out */

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

/* instruction descriptor of kind::f16: FP32 accumulator, bf16 A and B, both K-major, N 128, M 128 */
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTcN >> 3) << 17) |
                              ((uint32_t)(kTcM >> 4) << 24);

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;\n" : "=l"(t));
    return t;
}

/* true once the barrier's phase with this parity completed; false after two
 * seconds (non-blocking tests with a growing back-off) */
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity)
{
    const uint64_t t0 = global_ns();
    for (unsigned back = 0;; back = back < 256 ? back + 32 : 256) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(done)
                     : "r"(bar), "r"(parity)
                     : "memory");
        if (done) return true;
        if (global_ns() - t0 > 2000000000ull) return false;
        __nanosleep(back);
    }
}

__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.u32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
                 ::"r"(tmem), "l"(adesc), "l"(bdesc), "r"(kTcIdesc), "r"(accumulate));
}

constexpr int kTmStages = 3;
constexpr int kTmStageA = kTcM * kTcK * 2, kTmStageB = kTcN * kTcK * 2; /* 16 KiB each */
constexpr int kTmSmem = kTmStages * (kTmStageA + kTmStageB) + 2048;     /* + barriers and 1 KiB alignment */

__device__ __forceinline__ uint64_t tm_desc(uint32_t saddr)
{
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | (1ull << 16) | ((uint64_t)(1024u >> 4) << 32) | (1ull << 46) |
           (2ull << 61);
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
                 "[%4];\n" ::"r"(dst),
                 "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar)
                 : "memory");
}

__global__ void __launch_bounds__(kTcThreads) k_gemm_tma(const __grid_constant__ CUtensorMap tmA,
                                                         const __grid_constant__ CUtensorMap tmB,
                                                         const float *__restrict__ bias, int M, int N, int K,
                                                         int flags, float *__restrict__ out_f32,
                                                         uint16_t *__restrict__ out_bf16, int *__restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char tm_raw[];
    const uint32_t raw = smem_u32(tm_raw);
    unsigned char *base = tm_raw + ((1024u - (raw & 1023u)) & 1023u); /* swizzle atoms need 1 KiB alignment */
    const uint32_t sA = smem_u32(base), sB = sA + kTmStages * kTmStageA;
    uint64_t *bars = reinterpret_cast<uint64_t *>(base + kTmStages * (kTmStageA + kTmStageB));
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * kTmStages + 1);
    const uint32_t full0 = smem_u32(bars), empty0 = full0 + 8 * kTmStages, done = full0 + 16 * kTmStages;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * kTcM, n0 = blockIdx.x * kTcN;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kTmStages; s++) {
            mbar_init(full0 + 8 * s, 1);
            mbar_init(empty0 + 8 * s, 1);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"((uint64_t)&tmA) : "memory");
        asm volatile("prefetch.tensormap [%0];\n" ::"l"((uint64_t)&tmB) : "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tmem_slot)),
                     "r"((uint32_t)kTcN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    const int steps = (K + kTcK - 1) / kTcK;
    bool ok = true;
    if (warp == 0 && lane == 0) { /* producer: TMA copies into a stage once its last MMAs are done */
        for (int kt = 0; kt < steps; kt++) {
            const int s = kt % kTmStages, use = kt / kTmStages;
            if (use >= 1) ok = mbar_wait(empty0 + 8 * s, (uint32_t)((use - 1) & 1)) && ok;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(full0 + 8 * s),
                         "r"((uint32_t)(kTmStageA + kTmStageB))
                         : "memory");
            tma_load_2d(sA + s * kTmStageA, &tmA, kt * kTcK, m0, full0 + 8 * s);
            tma_load_2d(sB + s * kTmStageB, &tmB, kt * kTcK, n0, full0 + 8 * s);
        }
    } else if (warp == 1 && lane == 0) { /* MMA issuer */
        for (int kt = 0; kt < steps; kt++) {
            const int s = kt % kTmStages, use = kt / kTmStages;
            ok = mbar_wait(full0 + 8 * s, (uint32_t)(use & 1)) && ok;
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t a0 = sA + s * kTmStageA, b0 = sB + s * kTmStageB;
#pragma unroll
            for (int kk = 0; kk < kTcK / 16; kk++)
                tc_mma(tmem, tm_desc(a0 + 32 * kk), tm_desc(b0 + 32 * kk), (kt > 0 || kk > 0) ? 1u : 0u);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                             empty0 + 8 * s)
                         : "memory");
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(done)
                     : "memory");
    }
    __syncwarp();
    ok = mbar_wait(done, 0u) && ok;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");

    const int row = m0 + 32 * warp + lane;
#pragma unroll 1
    for (int c0 = 0; c0 < kTcN; c0 += 32) {
        uint32_t v[32];
        const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0;
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                     "%13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, "
                     "[%32];\n"
                     : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                       "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                       "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                       "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                       "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                     : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        if (row < M) { /* this row's 32 columns in 16-byte stores */
#pragma unroll
            for (int g = 0; g < 32; g += 8) {
                const int col = n0 + c0 + g;
                float x[8];
#pragma unroll
                for (int e = 0; e < 8; e++) {
                    x[e] = __uint_as_float(v[g + e]);
                    if (flags & C2A_MLP_BIAS) x[e] += bias[col + e];
                }
                const size_t o = (size_t)row * N + col;
                if (out_f32) {
                    reinterpret_cast<float4 *>(out_f32 + o)[0] = make_float4(x[0], x[1], x[2], x[3]);
                    reinterpret_cast<float4 *>(out_f32 + o)[1] = make_float4(x[4], x[5], x[6], x[7]);
                }
                if (out_bf16) {
                    uint32_t w[4];
#pragma unroll
                    for (int e = 0; e < 8; e += 2) {
                        float a = x[e], b = x[e + 1];
                        if (flags & C2A_MLP_GELU) {
                            a = gelu(a);
                            b = gelu(b);
                        }
                        w[e / 2] = (uint32_t)f2bf(a) | ((uint32_t)f2bf(b) << 16);
                    }
                    *reinterpret_cast<uint4 *>(out_bf16 + o) = make_uint4(w[0], w[1], w[2], w[3]);
                }
            }
        }
    }
    if (!ok) atomicExch(err, 1);
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"((uint32_t)kTcN));
    }
}

/* ------------------------------------------------------ elementwise/rows */

__global__ void k_transpose(const uint16_t *__restrict__ in, int rows, int cols, uint16_t *__restrict__ out)
{
    __shared__ uint16_t tile[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += 8) tile[i][threadIdx.x] = in[(size_t)(r0 + i) * cols + c0 + threadIdx.x];
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += 8) out[(size_t)(c0 + i) * rows + r0 + threadIdx.x] = tile[threadIdx.x][i];
}

__global__ void k_gelu_backward(const float *__restrict__ d_act, const float *__restrict__ pre, int64_t count,
                                uint16_t *__restrict__ d_pre)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        d_pre[i] = f2bf(d_act[i] * gelu_grad(pre[i]));
}

__device__ __forceinline__ float block_reduce(float v, float *sh, bool is_max)
{
    for (int o = 16; o > 0; o >>= 1) {
        const float w = __shfl_xor_sync(0xffffffffu, v, o);
        v = is_max ? fmaxf(v, w) : v + w;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    v = lane < nw ? sh[lane] : (is_max ? -INFINITY : 0.0f);
    for (int o = 16; o > 0; o >>= 1) {
        const float w = __shfl_xor_sync(0xffffffffu, v, o);
        v = is_max ? fmaxf(v, w) : v + w;
    }
    return v;
}

__global__ void __launch_bounds__(256) k_softmax_xent(const float *__restrict__ logits, const int32_t *__restrict__ labels,
                                                      int N, float scale, float *__restrict__ loss,
                                                      uint16_t *__restrict__ d_logits)
{
    __shared__ float sh[32];
    const int m = blockIdx.x;
    const float *x = logits + (size_t)m * N;
    uint16_t *d = d_logits + (size_t)m * N;
    const int lab = labels[m];
    if (lab < 0 || lab >= N) {
        for (int n = threadIdx.x; n < N; n += blockDim.x) d[n] = 0;
        if (threadIdx.x == 0) loss[m] = 0.0f;
        return;
    }
    float mx = -INFINITY;
    for (int n = threadIdx.x; n < N; n += blockDim.x) mx = fmaxf(mx, x[n]);
    mx = block_reduce(mx, sh, true);
    float s = 0.0f;
    for (int n = threadIdx.x; n < N; n += blockDim.x) s += expf(x[n] - mx);
    s = block_reduce(s, sh, false);
    const float inv = 1.0f / s;
    for (int n = threadIdx.x; n < N; n += blockDim.x) {
        const float p = expf(x[n] - mx) * inv;
        d[n] = f2bf((p - (n == lab ? 1.0f : 0.0f)) * scale);
    }
    if (threadIdx.x == 0) loss[m] = logf(s) + mx - x[lab];
}

/* the expected class index of a row under its softmax */
__global__ void __launch_bounds__(256) k_expect(const float *__restrict__ logits, int N, float *__restrict__ out)
{
    __shared__ float sh[32];
    const float *x = logits + (size_t)blockIdx.x * N;
    float mx = -INFINITY;
    for (int n = threadIdx.x; n < N; n += blockDim.x) mx = fmaxf(mx, x[n]);
    mx = block_reduce(mx, sh, true);
    float s0 = 0.0f, s1 = 0.0f;
    for (int n = threadIdx.x; n < N; n += blockDim.x) {
        const float e = expf(x[n] - mx);
        s0 += e;
        s1 += e * (float)n;
    }
    s0 = block_reduce(s0, sh, false);
    s1 = block_reduce(s1, sh, false);
    if (threadIdx.x == 0) out[blockIdx.x] = s1 / s0;
}

/* column sums: block = 32 columns x 8 row groups */
__global__ void k_colsum(const uint16_t *__restrict__ in, int M, int N, float *__restrict__ out)
{
    __shared__ float sh[8][33];
    const int col = blockIdx.x * 32 + threadIdx.x;
    float s = 0.0f;
    if (col < N)
        for (int m = threadIdx.y; m < M; m += 8) s += bf2f(in[(size_t)m * N + col]);
    sh[threadIdx.y][threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.y == 0 && col < N) {
        float t = 0.0f;
        for (int i = 0; i < 8; i++) t += sh[i][threadIdx.x];
        out[col] = t;
    }
}

__global__ void k_adam(float *__restrict__ w, float *__restrict__ m, float *__restrict__ v, const float *__restrict__ g,
                       int64_t count, float lr, float b1, float b2, float eps, float c1, float c2,
                       uint16_t *__restrict__ wb, uint16_t *__restrict__ wbt, int rows, int cols)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        w[i] = wi;
        const uint16_t h = f2bf(wi);
        if (wb) wb[i] = h;
        if (wbt) {
            const int64_t r = i / cols, c = i - r * cols;
            wbt[c * rows + r] = h;
        }
    }
}

__global__ void k_assemble(const float *__restrict__ feat, const int32_t *__restrict__ ia,
                           const int32_t *__restrict__ ib, const float *__restrict__ emb, int n_valid, int M, int K,
                           uint16_t *__restrict__ x)
{
    const int64_t total = (int64_t)M * K;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int m = (int)(i / K), k = (int)(i - (int64_t)m * K);
        float v = 0.0f;
        if (m < n_valid) {
            if (k < 18) v = feat[(size_t)m * 18 + k];
            else if (k < 34) v = emb[(size_t)ia[m] * 16 + (k - 18)];
            else if (k < 50) v = emb[(size_t)ib[m] * 16 + (k - 34)];
        }
        x[i] = f2bf(v);
    }
}

__global__ void k_embed_backward(const float *__restrict__ dx, const int32_t *__restrict__ ia,
                                 const int32_t *__restrict__ ib, int n_valid, int K, float *__restrict__ g_emb)
{
    const int64_t total = (int64_t)n_valid * 32;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int m = (int)(i >> 5), k = (int)(i & 31);
        const float d = dx[(size_t)m * K + 18 + k];
        if (k < 16) atomicAdd(g_emb + (size_t)ia[m] * 16 + k, d);
        else atomicAdd(g_emb + (size_t)ib[m] * 16 + (k - 16), d);
    }
}

/* top-k of a row on one warp: each lane keeps its k best (value desc, index
 * asc), then k rounds of a warp arg-max over the lanes' heads */
__global__ void k_topk(const float *__restrict__ logits, int M, int N, int k, int32_t *__restrict__ index)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= M) return;
    const float *x = logits + (size_t)warp * N;
    float bv[16];
    int bi[16];
    for (int i = 0; i < 16; i++) {
        bv[i] = -INFINITY;
        bi[i] = 0x7fffffff;
    }
    for (int n = lane; n < N; n += 32) {
        float v = x[n];
        int id = n;
        for (int i = 0; i < k; i++) { /* insertion into the descending list */
            const bool better = v > bv[i] || (v == bv[i] && id < bi[i]);
            if (better) {
                const float tv = bv[i];
                const int ti = bi[i];
                bv[i] = v;
                bi[i] = id;
                v = tv;
                id = ti;
            }
        }
    }
    int head = 0;
    for (int r = 0; r < k; r++) {
        float v = head < k ? bv[head] : -INFINITY;
        int id = head < k ? bi[head] : 0x7fffffff;
        for (int o = 16; o > 0; o >>= 1) {
            const float v2 = __shfl_xor_sync(0xffffffffu, v, o);
            const int i2 = __shfl_xor_sync(0xffffffffu, id, o);
            if (v2 > v || (v2 == v && i2 < id)) {
                v = v2;
                id = i2;
            }
        }
        if (lane == 0) index[(size_t)warp * k + r] = id;
        if (head < k && bi[head] == id) head++;
    }
}

int grid_for(int64_t count, int threads)
{
    int64_t b = (count + threads - 1) / threads;
    return (int)(b < 152 * 32 ? (b > 0 ? b : 1) : 152 * 32);
}

} // namespace

extern "C" {

typedef CUresult (*PFN_encode_tiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                     const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                     CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

c2a_status c2a_mlp_gemm(const uint16_t *A, const uint16_t *B, const float *bias, int32_t M, int32_t N, int32_t K,
                        int32_t flags, float *out_f32, uint16_t *out_bf16, void *stream)
{
    if (!A || !B || M <= 0 || N <= 0 || K <= 0 || M % kTcM || N % kTcN || K % 32 ||
        ((flags & C2A_MLP_BIAS) && !bias) || ((uintptr_t)A & 15) || ((uintptr_t)B & 15))
        return C2A_ERR_INVALID_ARGUMENT;
    static PFN_encode_tiled encode = nullptr;
    static bool attr[128] = {}; /* the shared-memory opt-in is a per-device attribute */
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 128) return C2A_ERR_CUDA;
    if (!encode) { /* the CUDA driver API's tensor-map encoder, reached through the runtime */
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn)
            return C2A_ERR_CUDA;
        encode = (PFN_encode_tiled)fn;
    }
    if (!attr[dev]) {
        if (cudaFuncSetAttribute(k_gemm_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, kTmSmem) != cudaSuccess)
            return C2A_ERR_CUDA;
        attr[dev] = true;
    }
    CUtensorMap ta, tb;
    const cuuint64_t da[2] = {(cuuint64_t)K, (cuuint64_t)M}, db[2] = {(cuuint64_t)K, (cuuint64_t)N};
    const cuuint64_t stride[1] = {(cuuint64_t)K * 2};
    const cuuint32_t box[2] = {(cuuint32_t)kTcK, (cuuint32_t)kTcM}, es[2] = {1, 1};
    if (encode(&ta, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void *)A, da, stride, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
            CUDA_SUCCESS ||
        encode(&tb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void *)B, db, stride, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) !=
            CUDA_SUCCESS)
        return C2A_ERR_INVALID_ARGUMENT;
    int *err = nullptr;
    if (cudaGetSymbolAddress((void **)&err, g_tc_err) != cudaSuccess) return C2A_ERR_CUDA;
    const dim3 grid(N / kTcN, M / kTcM);
    k_gemm_tma<<<grid, kTcThreads, kTmSmem, (cudaStream_t)stream>>>(ta, tb, bias, M, N, K, flags, out_f32, out_bf16,
                                                                     err);
    return launch_status();
}

c2a_status c2a_mlp_check(void *stream)
{
    int v = 0;
    const int zero = 0;
    if (cudaMemcpyFromSymbolAsync(&v, g_tc_err, sizeof(int), 0, cudaMemcpyDeviceToHost, (cudaStream_t)stream) !=
            cudaSuccess ||
        cudaMemcpyToSymbolAsync(g_tc_err, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, (cudaStream_t)stream) !=
            cudaSuccess ||
        cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess)
        return C2A_ERR_CUDA;
    return v ? C2A_ERR_CUDA : C2A_OK;
}

c2a_status c2a_mlp_transpose(const uint16_t *in, int32_t rows, int32_t cols, uint16_t *out, void *stream)
{
    if (!in || !out || rows <= 0 || cols <= 0 || rows % 32 || cols % 32) return C2A_ERR_INVALID_ARGUMENT;
    k_transpose<<<dim3(cols / 32, rows / 32), dim3(32, 8), 0, (cudaStream_t)stream>>>(in, rows, cols, out);
    return launch_status();
}

c2a_status c2a_mlp_gelu_backward(const float *d_act, const float *pre, int64_t count, uint16_t *d_pre, void *stream)
{
    if (!d_act || !pre || !d_pre || count <= 0) return C2A_ERR_INVALID_ARGUMENT;
    k_gelu_backward<<<grid_for(count, 256), 256, 0, (cudaStream_t)stream>>>(d_act, pre, count, d_pre);
    return launch_status();
}

c2a_status c2a_mlp_softmax_xent(const float *logits, const int32_t *labels, int32_t M, int32_t N, float scale,
                                float *loss, uint16_t *d_logits, void *stream)
{
    if (!logits || !labels || !loss || !d_logits || M <= 0 || N <= 0) return C2A_ERR_INVALID_ARGUMENT;
    k_softmax_xent<<<M, 256, 0, (cudaStream_t)stream>>>(logits, labels, N, scale, loss, d_logits);
    return launch_status();
}

c2a_status c2a_mlp_expect(const float *logits, int32_t M, int32_t N, float *out, void *stream)
{
    if (!logits || !out || M <= 0 || N <= 0) return C2A_ERR_INVALID_ARGUMENT;
    k_expect<<<M, 256, 0, (cudaStream_t)stream>>>(logits, N, out);
    return launch_status();
}

namespace {
constexpr int kOrderChunk = 1024; /* keys per block of the ordering kernels */

__device__ __forceinline__ int order_bin(float key, float key_max)
{
    float t = key_max > 0.f ? __fdiv_rn(key, key_max) : 0.f;
    t = t < 0.f ? 0.f : (t > 1.f ? 1.f : t);
    if (t != t) t = 0.f; /* NaN: last */
    int level = (int)__fadd_rn(__fmul_rn(t, (float)(C2A_ORDER_BINS - 1)), 0.5f); /* no contraction */
    return (C2A_ORDER_BINS - 1) - level; /* bin 0 holds the largest keys */
}

/* per-chunk histograms, bin-major: hist[bin * chunks + chunk] */
__global__ void __launch_bounds__(kOrderChunk) k_order_hist(const float *__restrict__ key, int n, float key_max,
                                                            int32_t *__restrict__ hist, int chunks)
{
    __shared__ int32_t h[C2A_ORDER_BINS];
    for (int b = threadIdx.x; b < C2A_ORDER_BINS; b += blockDim.x) h[b] = 0;
    __syncthreads();
    const int i = blockIdx.x * kOrderChunk + threadIdx.x;
    if (i < n) atomicAdd(&h[order_bin(key[i], key_max)], 1);
    __syncthreads();
    for (int b = threadIdx.x; b < C2A_ORDER_BINS; b += blockDim.x) hist[(size_t)b * chunks + blockIdx.x] = h[b];
}

/* exclusive scan of the bin-major histogram in place (one block) */
__global__ void __launch_bounds__(kOrderChunk) k_order_scan(int32_t *__restrict__ hist, int total)
{
    __shared__ int32_t part[kOrderChunk];
    const int per = (total + kOrderChunk - 1) / kOrderChunk;
    const int lo = threadIdx.x * per, hi = min(lo + per, total);
    int32_t s = 0;
    for (int k = lo; k < hi; k++) s += hist[k];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < kOrderChunk; off <<= 1) { /* inclusive Hillis-Steele scan of the partial sums */
        const int32_t v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    int32_t run = threadIdx.x ? part[threadIdx.x - 1] : 0;
    for (int k = lo; k < hi; k++) {
        const int32_t c = hist[k];
        hist[k] = run;
        run += c;
    }
}

/* scatter: a key's place is its (bin, chunk) offset plus the number of keys
 * of the same bin before it in its chunk (warps in order, lanes by match) */
__global__ void __launch_bounds__(kOrderChunk) k_order_scatter(const float *__restrict__ key, int n, float key_max,
                                                               const int32_t *__restrict__ offs, int chunks,
                                                               int32_t *__restrict__ order)
{
    __shared__ int32_t seen[C2A_ORDER_BINS];
    for (int b = threadIdx.x; b < C2A_ORDER_BINS; b += blockDim.x) seen[b] = 0;
    __syncthreads();
    const int i = blockIdx.x * kOrderChunk + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int bin = i < n ? order_bin(key[i], key_max) : -1 - lane; /* out-of-range lanes match nobody */
    const unsigned same = __match_any_sync(0xffffffffu, bin);
    const int before = __popc(same & ((1u << lane) - 1u));
    for (int w = 0; w < kOrderChunk / 32; w++) {
        if (warp == w && i < n) {
            order[offs[(size_t)bin * chunks + blockIdx.x] + seen[bin] + before] = i;
        }
        __syncthreads();
        if (warp == w && i < n && before == 0) seen[bin] += __popc(same);
        __syncthreads();
    }
}
} // namespace

c2a_status c2a_mlp_order_desc(const float *key, int32_t n, float key_max, int32_t *order, int32_t *scratch,
                              void *stream)
{
    if (n < 0 || (n > 0 && (!key || !order || !scratch))) return C2A_ERR_INVALID_ARGUMENT;
    if (n == 0) return C2A_OK;
    const int chunks = (n + kOrderChunk - 1) / kOrderChunk;
    cudaStream_t s = (cudaStream_t)stream;
    k_order_hist<<<chunks, kOrderChunk, 0, s>>>(key, n, key_max, scratch, chunks);
    k_order_scan<<<1, kOrderChunk, 0, s>>>(scratch, chunks * C2A_ORDER_BINS);
    k_order_scatter<<<chunks, kOrderChunk, 0, s>>>(key, n, key_max, scratch, chunks, order);
    return launch_status();
}

c2a_status c2a_mlp_colsum(const uint16_t *in, int32_t M, int32_t N, float *out, void *stream)
{
    if (!in || !out || M <= 0 || N <= 0) return C2A_ERR_INVALID_ARGUMENT;
    k_colsum<<<(N + 31) / 32, dim3(32, 8), 0, (cudaStream_t)stream>>>(in, M, N, out);
    return launch_status();
}

c2a_status c2a_mlp_adam(float *w, float *m, float *v, const float *g, int64_t count, float lr, float beta1,
                        float beta2, float eps, int32_t t, uint16_t *w_bf16, uint16_t *w_bf16_t, int32_t rows,
                        int32_t cols, void *stream)
{
    if (!w || !m || !v || !g || count <= 0 || t < 1 || (w_bf16_t && (int64_t)rows * cols != count))
        return C2A_ERR_INVALID_ARGUMENT;
    const float c1 = 1.0f - powf(beta1, (float)t), c2 = 1.0f - powf(beta2, (float)t);
    k_adam<<<grid_for(count, 256), 256, 0, (cudaStream_t)stream>>>(w, m, v, g, count, lr, beta1, beta2, eps, c1, c2,
                                                                    w_bf16, w_bf16_t, rows, cols);
    return launch_status();
}

c2a_status c2a_mlp_assemble(const float *feat, const int32_t *ia, const int32_t *ib, const float *emb,
                            int32_t n_valid, int32_t M, int32_t K, uint16_t *x, void *stream)
{
    if (!feat || !ia || !ib || !emb || !x || K < 50 || K % 32 || n_valid < 0 || n_valid > M || M <= 0)
        return C2A_ERR_INVALID_ARGUMENT;
    k_assemble<<<grid_for((int64_t)M * K, 256), 256, 0, (cudaStream_t)stream>>>(feat, ia, ib, emb, n_valid, M, K, x);
    return launch_status();
}

c2a_status c2a_mlp_embed_backward(const float *dx, const int32_t *ia, const int32_t *ib, int32_t n_valid, int32_t K,
                                  float *g_emb, void *stream)
{
    if (!dx || !ia || !ib || !g_emb || K < 50 || n_valid < 0) return C2A_ERR_INVALID_ARGUMENT;
    if (n_valid == 0) return C2A_OK;
    k_embed_backward<<<grid_for((int64_t)n_valid * 32, 256), 256, 0, (cudaStream_t)stream>>>(dx, ia, ib, n_valid, K,
                                                                                             g_emb);
    return launch_status();
}

c2a_status c2a_mlp_topk(const float *logits, int32_t M, int32_t N, int32_t k, int32_t *index, void *stream)
{
    if (!logits || !index || M <= 0 || N <= 0 || k < 1 || k > 16 || k > N) return C2A_ERR_INVALID_ARGUMENT;
    k_topk<<<(M * 32 + 255) / 256, 256, 0, (cudaStream_t)stream>>>(logits, M, N, k, index);
    return launch_status();
}

} // extern "C"
