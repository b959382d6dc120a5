/*
 * spec_emu.cpp -- the warp-per-query REFERENCE engines (the sequential warp
 * traversal and the speculative one) run on the CPU through warp_emu.h, for
 * the CPU tests (tests/test_spec_emu.py).
 *
 * It builds models with the library's host BVH build and runs the same
 * device functions the kernels run -- solve_query_warp with WarpDfs or
 * SpecDfs -- one query at a time on one emulated warp.  The results must be
 * the oracle's, bit for bit; a warp collective that some lanes skip aborts.
 */
#include "warp_emu.h"

#include <vector>

namespace c2a {
struct Query;
}
/* each emulated lane keeps its own copy of the warp-uniform query state, and
 * uniform writes are fenced by warp barriers (the lanes do not run in lockstep) */
c2a::Query &emu_lane_query();
#define C2A_WARP_QUERY(sh) emu_lane_query()
#define C2A_WSET(dst, v)                                                                                           \
    do {                                                                                                           \
        auto emu_v_ = (v);                                                                                         \
        __syncwarp();                                                                                              \
        (dst) = emu_v_;                                                                                            \
        __syncwarp();                                                                                              \
    } while (0)

#include "../../c2a_gb300/csrc/device/ca_spec.cuh"

using namespace c2a;

c2a::Query &emu_lane_query()
{
    thread_local Query q;
    return q;
}

namespace {

std::vector<BuiltModel> g_models;

DevModel dev_model(const BuiltModel &m)
{
    DevModel d;
    d.nodes = m.nodes.data();
    d.tris = m.tris.data();
    d.snodes = m.snodes.data();
    d.stris = m.stris.data();
    d.num_tris = (int32_t)m.tris.size();
    d.num_nodes = (int32_t)m.nodes.size();
    d.depth = m.depth;
    d.flags = C2A_MODEL_LIVE | (m.shadow_ok ? C2A_MODEL_SHADOW_OK : 0);
    return d;
}

} // namespace

extern "C" {

/* builds a model; returns its id or a negative status */
int spec_emu_model(int num_tris, const double *tri_verts, const int *vidx)
{
    BuiltModel m;
    const int rc = build_rss_model(num_tris, tri_verts, nullptr, vidx, m);
    if (rc) return -rc;
    g_models.push_back(std::move(m));
    return (int)g_models.size() - 1;
}

void spec_emu_reset() { g_models.clear(); }

#ifdef C2A_STATS
/* event counters of a profiling build of the emulation, copied out and cleared */
int spec_emu_stats(unsigned long long *out, int count)
{
    for (int i = 0; i < count && i < ST_COUNT; i++) {
        out[i] = g_c2a_stats[i];
        g_c2a_stats[i] = 0;
    }
    return ST_COUNT;
}
#endif

/* n queries, one emulated warp each in turn; engine C2A_ENGINE_WARP: the
 * sequential warp traversal, C2A_ENGINE_SPEC: the speculative one;
 * contacts: n x contacts_per_query slots */
int spec_emu_solve(const c2a_query *queries, int n, const c2a_params *params, c2a_result *results,
                   c2a_contact *contacts, double timeout_s)
{
    std::vector<DevModel> table;
    int deepest = 0;
    for (const BuiltModel &m : g_models) {
        table.push_back(dev_model(m));
        if (m.depth > deepest) deepest = m.depth;
    }
#ifndef SPEC_EMU_EXTRA_RECORDS
#define SPEC_EMU_EXTRA_RECORDS 64
#endif
    const int cap = 2 * deepest + 2 > 4 ? 2 * deepest + 2 : 4;
    const int nrec = 2 * deepest + 2 + SPEC_EMU_EXTRA_RECORDS;
    std::vector<unsigned char> wsh(warp_shared_bytes(cap) + 16), ssh(spec_shared_bytes(nrec) + 16),
        gsc(spec_global_bytes(nrec) + 16);
    auto al = [](std::vector<unsigned char> &v) {
        return reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(v.data()) + 15) & ~(uintptr_t)15);
    };
    WarpShared &sh = *reinterpret_cast<WarpShared *>(al(wsh));
    sh.cap = cap;
    warp_emu::Warp warp;
    warp.timeout_s = timeout_s;
    warp_emu::current() = &warp;
    const bool spec = params->engine == C2A_ENGINE_SPEC;
    std::vector<std::thread> lanes;
    for (int lane = 0; lane < 32; lane++) {
        lanes.emplace_back([&, lane]() {
            warp_emu::lane_id() = lane;
            std::vector<Pending> tstack(C2A_STACK_DEPTH);
            SpecCtx sc;
            spec_layout(sc, al(ssh), al(gsc), nrec);
            for (int i = lane; i < nrec; i += 32) sc.rec[i].gen = 0;
            __syncwarp();
            for (int q = 0; q < n; q++) {
                c2a_contact *cq = contacts ? contacts + (size_t)q * (size_t)params->contacts_per_query : nullptr;
                if (spec)
                    solve_query_warp(queries[q], table.data(), (int)table.size(), *params, results[q], cq, sh,
                                     tstack.data(), q, lane, SpecDfs{sh, sc});
                else
                    solve_query_warp(queries[q], table.data(), (int)table.size(), *params, results[q], cq, sh,
                                     tstack.data(), q, lane, WarpDfs{sh});
                __syncwarp();
            }
        });
    }
    for (std::thread &t : lanes) t.join();
    warp_emu::current() = nullptr;
    return 0;
}

} // extern "C"
