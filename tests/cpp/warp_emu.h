/*
 * warp_emu.h -- a host emulation of one CUDA warp, for running the kernels'
 * warp-level device code on the CPU in tests.
 *
 * 32 host threads play the 32 lanes of one warp.  The warp intrinsics the
 * CA code uses (__shfl_sync, __shfl_xor_sync, __ballot_sync, __all_sync,
 * __syncwarp) are collective: every lane writes its value, all 32 meet at a
 * barrier, then read.  A lane that never arrives -- warp-divergent code
 * reaching a full-mask collective on some lanes only, which is undefined on
 * the GPU -- makes the barrier time out, and the emulation aborts naming
 * the lane.  Memory the kernel would keep in shared memory is a buffer all
 * 32 threads see; __ldg is a plain load.
 *
 * Include this before the device headers; it defines __CUDACC__ so they take
 * their CUDA spellings, and maps the CUDA qualifiers to host C++.
 */
#ifndef C2A_WARP_EMU_H
#define C2A_WARP_EMU_H

#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>

#define __CUDACC__ 1
#define __host__
#define __device__
#define __global__
#define __forceinline__ inline
#define __noinline__ __attribute__((noinline))
#define __align__(n) alignas(n)

struct alignas(16) double2 {
    double x, y;
};
struct alignas(16) float4 {
    float x, y, z, w;
};

namespace warp_emu {

struct Warp {
    std::atomic<int> arrived{0};
    std::atomic<unsigned> generation{0};
    uint64_t slot[32];
    std::atomic<unsigned> ballot{0};
    double timeout_s = 60.0;
};

inline Warp *&current()
{
    static Warp *w = nullptr;
    return w;
}
inline int &lane_id()
{
    thread_local int lane = 0;
    return lane;
}

/* all 32 lanes meet; a lane left waiting longer than the timeout aborts */
inline void barrier()
{
    Warp &w = *current();
    const unsigned gen = w.generation.load(std::memory_order_acquire);
    if (w.arrived.fetch_add(1, std::memory_order_acq_rel) == 31) {
        w.arrived.store(0, std::memory_order_relaxed);
        w.generation.fetch_add(1, std::memory_order_acq_rel);
        return;
    }
    const auto t0 = std::chrono::steady_clock::now();
    unsigned spins = 0;
    while (w.generation.load(std::memory_order_acquire) == gen) {
        std::this_thread::yield();
        if (++spins % 4096 == 0 &&
            std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() > w.timeout_s) {
            fprintf(stderr, "warp_emu: lane %d waited %.0f s at a warp collective that not every lane reached\n",
                    lane_id(), w.timeout_s);
            std::abort();
        }
    }
}

template <class T> inline T shfl(T v, int src)
{
    static_assert(sizeof(T) <= 8, "one lane value per slot");
    Warp &w = *current();
    uint64_t u = 0;
    std::memcpy(&u, &v, sizeof(T));
    w.slot[lane_id()] = u;
    barrier();
    const uint64_t r = w.slot[src & 31];
    barrier();
    T out;
    std::memcpy(&out, &r, sizeof(T));
    return out;
}

} // namespace warp_emu

template <class T> inline T __ldg(const T *p) { return *p; }
inline float __int_as_float(int i)
{
    float f;
    std::memcpy(&f, &i, 4);
    return f;
}
inline int __float_as_int(float f)
{
    int i;
    std::memcpy(&i, &f, 4);
    return i;
}
inline int __ffs(int x) { return __builtin_ffs(x); }
inline int __ffs(unsigned x) { return __builtin_ffs((int)x); }
inline int __popc(unsigned x) { return __builtin_popcount(x); }
inline void __syncwarp(unsigned = 0xffffffffu) { warp_emu::barrier(); }
template <class T> inline T __shfl_sync(unsigned, T v, int src) { return warp_emu::shfl(v, src); }
template <class T> inline T __shfl_xor_sync(unsigned, T v, int m) { return warp_emu::shfl(v, warp_emu::lane_id() ^ m); }
inline unsigned __ballot_sync(unsigned, int pred)
{
    warp_emu::Warp &w = *warp_emu::current();
    warp_emu::barrier(); /* the previous ballot's readers are done */
    if (warp_emu::lane_id() == 0) w.ballot.store(0);
    warp_emu::barrier();
    if (pred) w.ballot.fetch_or(1u << warp_emu::lane_id());
    warp_emu::barrier();
    return w.ballot.load();
}
inline int __all_sync(unsigned m, int pred) { return __ballot_sync(m, pred) == 0xffffffffu; }
inline int __any_sync(unsigned m, int pred) { return __ballot_sync(m, pred) != 0u; }
inline unsigned long long atomicAdd(unsigned long long *p, unsigned long long v)
{
    return __atomic_fetch_add(p, v, __ATOMIC_RELAXED);
}
inline long long clock64() { return 0; }

#endif
