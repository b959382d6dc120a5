/*
 * rect_table_ef.cuh -- the half-warp RectDist of rect_table.cuh in the
 * certified FP32 filter: the same input slots, stage-1 products, stage-2
 * sums, sort comparisons and per-case operand tables, each value an EF
 * (ef.cuh) computed with the FP64 code's expression tree, so its bound
 * covers the FP64 value of the same slot.  Comparisons are three-valued;
 * a comparison a result depends on that the bounds cannot settle marks the
 * child test uncertain, and the caller recomputes it in FP64.
 */
#ifndef C2A_RECT_TABLE_EF_CUH
#define C2A_RECT_TABLE_EF_CUH

#include "rect_table.cuh"

namespace c2a {

/* every input slot (all lanes of a half write the same values) */
C2A_DEV void rte_inputs(const M3T<EF> &R, V3T<EF> T, const EF a[2], const EF b[2], EF *V)
{
    V[0] = a[0];
    V[1] = a[1];
    V[2] = b[0];
    V[3] = b[1];
    V[4] = R.m[0];
    V[5] = R.m[1];
    V[6] = R.m[3];
    V[7] = R.m[4];
    V[8] = T.x;
    V[9] = T.y;
    V[10] = ef_exact(0.0f);
}

/* lane k's stage-1 slot (k < kRtStage1): a product of two input slots, or Tba.x / Tba.y as tmul evaluates them */
C2A_DEV EF rte_stage1(int k, const M3T<EF> &R, V3T<EF> T, const EF *V)
{
    if (k < 8) {
        const uint32_t w = C2A_RT(rt_s1, k);
        return V[w & 0x7f] * V[(w >> 8) & 0x7f];
    }
    const int c = k - 8;
    return R.m[c] * T.x + R.m[3 + c] * T.y + R.m[6 + c] * T.z;
}

C2A_DEV EF rte_signed(uint32_t b, const EF *V) /* slot | negate << 7; negation is exact */
{
    const EF v = V[b & 0x7f];
    return (b & 0x80) ? EF{-v.v, v.e} : v;
}

/* stage-2 slot i (< kRtStage2) */
C2A_DEV EF rte_stage2(int i, const EF *V)
{
    const uint32_t w = C2A_RT(rt_s2, i);
    const EF s = rte_signed(w & 0xff, V) + rte_signed((w >> 8) & 0xff, V);
    return (w >> 24) ? s + rte_signed((w >> 16) & 0xff, V) : s;
}

/* comparison g (< 8) of the preamble's sorts: 1 true, 0 false, -1 undecided */
C2A_DEV int rte_compare(int g, const EF *V)
{
    const uint32_t w = C2A_RT(rt_cmp, g);
    return ef_lt3(rte_signed(w & 0xff, V), rte_signed((w >> 8) & 0xff, V));
}

C2A_DEV EF rte_operand(uint32_t r, unsigned mask, const EF *V)
{
    const unsigned g = (r >> 16) & 15u;
    const bool f = g != 15u && !((mask >> g) & 1u);
    return rte_signed(f ? (r >> 8) & 0xff : r & 0xff, V);
}

/* the operands of case j (< 16) */
C2A_DEV void rte_case_operands(int j, unsigned mask, const EF *V, EF L[4], EF R[4], EF s1[7], EF s2[7], EF e[5],
                               EF &qb, int &px, int &py, int &qkind, int &cb, int &cu)
{
    const int o = j * kRtRefs;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        L[i] = rte_operand(C2A_RT(rt_case_ref, o + i), mask, V);
        R[i] = rte_operand(C2A_RT(rt_case_ref, o + 4 + i), mask, V);
    }
#pragma unroll
    for (int i = 0; i < 7; i++) {
        s1[i] = rte_operand(C2A_RT(rt_case_ref, o + 8 + i), mask, V);
        s2[i] = rte_operand(C2A_RT(rt_case_ref, o + 15 + i), mask, V);
    }
#pragma unroll
    for (int i = 0; i < 5; i++) e[i] = rte_operand(C2A_RT(rt_case_ref, o + 22 + i), mask, V);
    qb = rte_operand(C2A_RT(rt_case_ref, o + 27), mask, V);
    const uint32_t n = C2A_RT(rt_case_int, j);
    px = n & 15; py = (n >> 4) & 15; qkind = (n >> 8) & 15; cb = (n >> 12) & 15; cu = (n >> 16) & 15;
}

/* case j's condition with the sequential code's short-circuit; ctx.bad when a
 * comparison it took was undecided */
C2A_DEV bool rte_case_holds(const EF L[4], const EF R[4], const EF s1[7], const EF s2[7], EFCtx &ctx)
{
    return LT(L[0], R[0]) && LT(L[1], R[1]) &&
           (LT(L[2], R[2]) || in_slab_inl(s1[0], s1[1], s1[2], s1[3], s1[4], s1[5], s1[6], ctx)) &&
           (LT(L[3], R[3]) || in_slab_inl(s2[0], s2[1], s2[2], s2[3], s2[4], s2[5], s2[6], ctx));
}

/* the edge pair's distance and S once its case holds (rt_case_value's arithmetic) */
C2A_DEV EF rte_case_value(const EF e[5], EF qb, int px, int py, int qkind, int cb, int cu, const M3T<EF> &Rab,
                          V3T<EF> Tab, const EF a[2], V3T<EF> &S, EFCtx &ctx)
{
    EF t, u;
    edge_params_inl(t, u, e[0], e[1], e[2], e[3], e[4], ctx);
    const EF zero = ef_exact(0.0f);
    const EF Px = px == 0 ? a[0] : px == 1 ? a[1] : px == 4 ? t : zero;
    const EF Py = py == 0 ? a[0] : py == 1 ? a[1] : py == 4 ? t : zero;
    const EF rbx = cb ? Rab.m[1] : Rab.m[0], rby = cb ? Rab.m[4] : Rab.m[3], rbz = cb ? Rab.m[7] : Rab.m[6];
    const EF rux = cu ? Rab.m[1] : Rab.m[0], ruy = cu ? Rab.m[4] : Rab.m[3], ruz = cu ? Rab.m[7] : Rab.m[6];
    const bool two = qkind == 2;
    const EF bx = Tab.x + rbx * qb, by = Tab.y + rby * qb, bz = Tab.z + rbz * qb;
    const V3T<EF> Q = v3t((two ? bx : Tab.x) + rux * u, (two ? by : Tab.y) + ruy * u, (two ? bz : Tab.z) + ruz * u);
    S = v3t(Q.x - Px, Q.y - Py, Q.z - zero);
    return ef_sqrt(S.x * S.x + S.y * S.y + S.z * S.z);
}

} // namespace c2a
#endif
