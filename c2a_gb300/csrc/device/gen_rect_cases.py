"""Generates rect_cases.cuh: C2ARectDist's sixteen edge-pair cases as one
lane-parallel code path.

rect_dist in geom.cuh is the sequential form: after a preamble (the
rectangles' projected bounds), sixteen cases are tested in order and the
first whose condition holds returns its edge-pair distance; otherwise the
face-separation tail decides.  Every case has the same shape,

    if (CMP(x1, y1) && CMP(x2, y2) &&
        (CMP(x3, y3) || in_slab(7 args)) && (CMP(x4, y4) || in_slab(7 args))) {
        edge_params(t, u, 5 args);
        C2A_EDGE_HIT(px, py, rect_point1/2(...));
    }

so lane j of a half-warp can evaluate case j with one code path: every
lane computes the preamble and every distinct argument expression (the
same expression trees as the sequential code), a switch on j only picks
operands, and the shared path runs the comparisons, both in_slab tests,
edge_params and the point.  The caller takes the first lane whose case
holds, which is what the sequential order returns.

    python c2a_gb300/csrc/device/gen_rect_cases.py   # rewrites rect_cases.cuh
"""
from __future__ import annotations

import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "geom.cuh")
OUT = os.path.join(HERE, "rect_cases.cuh")


def split_top(s: str, sep: str) -> list[str]:
    """Splits s at top-level occurrences of sep (outside parentheses)."""
    out, depth, cur, i = [], 0, "", 0
    while i < len(s):
        c = s[i]
        if c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
        if depth == 0 and s.startswith(sep, i):
            out.append(cur.strip())
            cur = ""
            i += len(sep)
            continue
        cur += c
        i += 1
    out.append(cur.strip())
    return out


def strip_parens(s: str) -> str:
    s = s.strip()
    while s.startswith("(") and s.endswith(")"):
        depth = 0
        for k, c in enumerate(s):
            depth += c == "("
            depth -= c == ")"
            if depth == 0 and k < len(s) - 1:
                return s
        s = s[1:-1].strip()
    return s


def call_args(s: str, name: str) -> list[str]:
    s = s.strip()
    assert s.startswith(name + "(") and s.endswith(")"), (name, s)
    return split_top(s[len(name) + 1:-1], ",")


def parse_cmp(s: str) -> tuple[str, str]:
    """GT(x, y) -> (y, x); LT(x, y) -> (x, y): the condition is first < second."""
    s = s.strip()
    op = s[:2]
    x, y = call_args(s, op)
    return (y, x) if op == "GT" else (x, y)


def main():
    text = open(SRC).read()
    start = text.index("C2A_NOINL T rect_dist(")
    body_start = text.index("{", start) + 1
    depth, k = 1, body_start
    while depth:
        depth += text[k] == "{"
        depth -= text[k] == "}"
        k += 1
    body = text[body_start:k - 1]
    case_re = re.compile(r"\n    if \((?P<cond>[^;{}]*?)\) \{\n\s*edge_params\((?P<edge>[^;]*)\);\n\s*"
                         r"C2A_EDGE_HIT\((?P<hit>[^;]*)\);\n    \}", re.S)
    cases = list(case_re.finditer(body))
    assert len(cases) == 16, len(cases)
    # preamble: everything but the cases, the hit macro, the early returns and the tail
    tail_at = body.index("/* no edge pair")
    pre = case_re.sub("", body[:tail_at])
    pre = re.sub(r"#define C2A_EDGE_HIT.*?while \(0\)\n", "", pre, flags=re.S)
    pre = pre.replace("#undef C2A_EDGE_HIT\n", "").replace("    if (ctx.bad) return zero;\n", "")
    pre = pre.replace("    T t, u;\n    V3T<T> P, Q;\n", "")
    pre = re.sub(r"\n\s*/\*[^*]*\*/", "", pre)
    exprs: dict[str, str] = {}

    def ref(e: str) -> str:
        e = " ".join(e.split())
        if re.fullmatch(r"[A-Za-z_][A-Za-z0-9_]*(\[\d\])?(\.[xyz])?", e) or e == "zero":
            return e
        if e not in exprs:
            exprs[e] = f"x{len(exprs)}"
        return exprs[e]

    rows = []
    for m in cases:
        conj = split_top(" ".join(m.group("cond").split()), "&&")
        assert len(conj) == 4, conj
        c1, c2 = parse_cmp(conj[0]), parse_cmp(conj[1])
        slabs = []
        for c in conj[2:]:
            alt = split_top(strip_parens(c), "||")
            assert len(alt) == 2, alt
            slabs.append((parse_cmp(alt[0]), [ref(a) for a in call_args(alt[1], "in_slab")[:7]]))
        edge = [ref(a) for a in split_top(" ".join(m.group("edge").split()), ",")[2:7]]
        hit = split_top(" ".join(m.group("hit").split()), ",")
        px, py, q = hit[0], hit[1], ",".join(hit[2:]).strip()
        if q.startswith("rect_point2"):
            qa = call_args(q, "rect_point2")
            qkind, cb, qb, cu = 2, qa[2], ref(qa[3]), qa[4]
        else:
            qa = call_args(q, "rect_point1")
            qkind, cb, qb, cu = 1, "0", "zero", qa[2]
        rows.append(dict(c=[c1, c2, slabs[0][0], slabs[1][0]], s1=slabs[0][1], s2=slabs[1][1], e=edge, px=px, py=py,
                         qkind=qkind, cb=cb, qb=qb, cu=cu))

    def pt(v: str) -> str:
        return "4" if v == "t" else {"a[0]": "0", "a[1]": "1", "zero": "2"}[v]

    lines = []
    w = lines.append
    w("/* generated by gen_rect_cases.py from rect_dist in geom.cuh; do not edit */")
    w("#ifndef C2A_RECT_CASES_CUH")
    w("#define C2A_RECT_CASES_CUH")
    w("")
    w('#include "geom.cuh"')
    w("")
    w("namespace c2a {")
    w("")
    w("/* Kleene AND / OR over {1, 0, -1 (undecided)} */")
    w("C2A_DEV int rc_and3(int a, int b) { return (a == 0 || b == 0) ? 0 : (a == 1 && b == 1) ? 1 : -1; }")
    w("C2A_DEV int rc_or3(int a, int b) { return (a == 1 || b == 1) ? 1 : (a == 0 && b == 0) ? 0 : -1; }")
    w("")
    w("/* case j (0..15) of C2ARectDist.  hit: 1 its condition holds, 0 it does not,")
    w(" * -1 undecided (the FP32 filter only; each part keeps its own context, so a")
    w(" * part the sequential form would not evaluate decides nothing); vbad: the")
    w(" * distance and S are not certified; ctx: the shared preamble's decisions.")
    w(" * The caller takes the first case that holds. */")
    w("template <class T, class C>")
    w("C2A_DEV T rect_case(int j, const M3T<T> &Rab, V3T<T> Tab, const T a[2], const T b[2], V3T<T> &S, int &hit,")
    w("                    bool &vbad, C &ctx)")
    w("{")
    for line in pre.strip("\n").split("\n"):
        w(line)
    for e, name in exprs.items():
        w(f"    const T {name} = {e};")
    w("    T L[4], R[4], s1[7], s2[7], e[5], qb = zero;")
    w("    int px = 0, py = 0, qkind = 1, cb = 0, cu = 0;")
    w("    switch (j) {")
    for j, r in enumerate(rows):
        w(f"    case {j}:")
        for i, (l_, r_) in enumerate(r["c"]):
            w(f"        L[{i}] = {l_}; R[{i}] = {r_};")
        w("        " + " ".join(f"s1[{i}] = {v};" for i, v in enumerate(r["s1"])))
        w("        " + " ".join(f"s2[{i}] = {v};" for i, v in enumerate(r["s2"])))
        w("        " + " ".join(f"e[{i}] = {v};" for i, v in enumerate(r["e"])))
        w(f"        px = {pt(r['px'])}; py = {pt(r['py'])}; qkind = {r['qkind']}; cb = {r['cb']}; qb = {r['qb']};"
          f" cu = {r['cu']};")
        w("        break;")
    w("    default:")
    w("        break;")
    w("    }")
    w("    /* every part evaluated on every lane (all are pure), each with its own context */")
    w("    C c0 = ctx, c1 = ctx, c2 = ctx, c3 = ctx, ci1 = ctx, ci2 = ctx, ce = ctx;")
    w("    const bool k0 = cmp_lt(L[0], R[0], c0, 0), k1 = cmp_lt(L[1], R[1], c1, 0);")
    w("    const bool k2 = cmp_lt(L[2], R[2], c2, 0), k3 = cmp_lt(L[3], R[3], c3, 0);")
    w("    const bool i1 = in_slab(s1[0], s1[1], s1[2], s1[3], s1[4], s1[5], s1[6], ci1);")
    w("    const bool i2 = in_slab(s2[0], s2[1], s2[2], s2[3], s2[4], s2[5], s2[6], ci2);")
    w("    const int t0 = c0.bad ? -1 : k0, t1 = c1.bad ? -1 : k1, t2 = c2.bad ? -1 : k2, t3 = c3.bad ? -1 : k3;")
    w("    const int u1 = ci1.bad ? -1 : i1, u2 = ci2.bad ? -1 : i2;")
    w("    hit = (j < 16 && !ctx.bad) ? rc_and3(rc_and3(t0, t1), rc_and3(rc_or3(t2, u1), rc_or3(t3, u2))) : (ctx.bad ? -1 : 0);")
    w("    T t, u;")
    w("    edge_params(t, u, e[0], e[1], e[2], e[3], e[4], ce);")
    w("    const T Px = px == 0 ? a[0] : px == 1 ? a[1] : px == 4 ? t : zero;")
    w("    const T Py = py == 0 ? a[0] : py == 1 ? a[1] : py == 4 ? t : zero;")
    w("    const V3T<T> P = v3t<T>(Px, Py, zero);")
    w("    /* rect_point2 / rect_point1 with the column picks as selects (cb, cu in {0, 1}) */")
    w("    const T rbx = cb ? Rab.m[1] : Rab.m[0], rby = cb ? Rab.m[4] : Rab.m[3], rbz = cb ? Rab.m[7] : Rab.m[6];")
    w("    const T rux = cu ? Rab.m[1] : Rab.m[0], ruy = cu ? Rab.m[4] : Rab.m[3], ruz = cu ? Rab.m[7] : Rab.m[6];")
    w("    const V3T<T> Q2 = v3t(Tab.x + rbx * qb + rux * u, Tab.y + rby * qb + ruy * u, Tab.z + rbz * qb + ruz * u);")
    w("    const V3T<T> Q1 = v3t(Tab.x + rux * u, Tab.y + ruy * u, Tab.z + ruz * u);")
    w("    const V3T<T> Q = qkind == 2 ? Q2 : Q1;")
    w("    S = v3t(Q.x - P.x, Q.y - P.y, Q.z - P.z);")
    w("    vbad = ce.bad;")
    w("    return num_sqrt(dot(S, S));")
    w("}")
    w("")
    # the tail as its own function
    tail = body[tail_at:]
    tail_pre = []
    for line in pre.strip("\n").split("\n"):
        if "const T A0B0" in line or "const V3T<T> Tba" in line:
            tail_pre.append(line)
    w("/* the face-separation tail of C2ARectDist (no edge pair holds) */")
    w("template <class T, class C>")
    w("C2A_DEV T rect_tail(const M3T<T> &Rab, V3T<T> Tab, const T a[2], const T b[2], V3T<T> &S, C &ctx)")
    w("{")
    w("    const T zero = K(0.0);")
    w("    const V3T<T> Tba = tmul(Rab, Tab);")
    for line in tail.rstrip().rstrip("}").rstrip().split("\n"):
        w(line)
    w("}")
    w("")
    w("} // namespace c2a")
    w("#endif")
    open(OUT, "w").write("\n".join(lines) + "\n")
    print(f"{OUT}: 16 cases, {len(exprs)} shared expressions")


if __name__ == "__main__":
    main()
