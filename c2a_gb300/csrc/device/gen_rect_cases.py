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

It also writes rect_table.cuh, the same computation with the shared work
spread over the half-warp: the preamble's products, sums and sorts and the
shared argument expressions become numbered slots that lanes compute a few
at a time (each with the sequential code's expression tree), and every case
reads its operands from the slots through a table instead of a switch.

    python c2a_gb300/csrc/device/gen_rect_cases.py   # rewrites rect_cases.cuh and rect_table.cuh
"""
from __future__ import annotations

import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "geom.cuh")
OUT = os.path.join(HERE, "rect_cases.cuh")
OUT_TABLE = os.path.join(HERE, "rect_table.cuh")


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


def parse():
    """rect_dist's preamble lines, shared argument expressions, per-case operands and tail."""
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

    return pre, exprs, rows, body[tail_at:]


def pt(v: str) -> str:
    return "4" if v == "t" else {"a[0]": "0", "a[1]": "1", "zero": "2"}[v]


def main():
    pre, exprs, rows, tail = parse()

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
    lane_lines = []
    lw = lane_lines.append
    # the whole distance on one lane: preamble once, the cases in order with
    # their operands picked per case, the winner's value once
    lw("/* C2ARectDist on one lane without diverging across the cases: the preamble")
    lw(" * once, then the sixteen cases in the reference's order, each through the")
    lw(" * same code path with its operands picked by a switch, until one holds; its")
    lw(" * edge-pair distance, or the face-separation tail when none does.  Same")
    lw(" * expression trees and the same first-hit rule as rect_dist; with the FP32")
    lw(" * filter an undecided case sets ctx.bad (the caller recomputes in FP64). */")
    lw("template <class T, class C>")
    lw("C2A_DEV T rect_dist_lane(const M3T<T> &Rab, V3T<T> Tab, const T a[2], const T b[2], V3T<T> &S, C &ctx)")
    lw("{")
    for line in pre.strip("\n").split("\n"):
        lw(line)
    for e, name in exprs.items():
        lw(f"    const T {name} = {e};")
    lw("    int win = -1;")
    lw("#pragma unroll 1")
    lw("    for (int j = 0; j < 16 && !ctx.bad; j++) {")
    lw("        T L[4], R[4], s1[7], s2[7];")
    lw("        switch (j) {")
    for j, r in enumerate(rows):
        lw(f"        case {j}:")
        for i, (l_, r_) in enumerate(r["c"]):
            lw(f"            L[{i}] = {l_}; R[{i}] = {r_};")
        lw("            " + " ".join(f"s1[{i}] = {v};" for i, v in enumerate(r["s1"])))
        lw("            " + " ".join(f"s2[{i}] = {v};" for i, v in enumerate(r["s2"])))
        lw("            break;")
    lw("        default:")
    lw("            break;")
    lw("        }")
    lw("        C c0 = ctx, c1 = ctx, c2 = ctx, c3 = ctx, ci1 = ctx, ci2 = ctx;")
    lw("        const bool k0 = cmp_lt(L[0], R[0], c0, 0), k1 = cmp_lt(L[1], R[1], c1, 0);")
    lw("        const int t0 = c0.bad ? -1 : k0, t1 = c1.bad ? -1 : k1;")
    lw("        if (rc_and3(t0, t1) == 0) continue; /* the usual outcome: no in_slab needed */")
    lw("        const bool k2 = cmp_lt(L[2], R[2], c2, 0), k3 = cmp_lt(L[3], R[3], c3, 0);")
    lw("        const int t2 = c2.bad ? -1 : k2, t3 = c3.bad ? -1 : k3;")
    lw("        int u1 = 1, u2 = 1;")
    lw("        if (t2 != 1) {")
    lw("            const bool i1 = in_slab_inl(s1[0], s1[1], s1[2], s1[3], s1[4], s1[5], s1[6], ci1);")
    lw("            u1 = ci1.bad ? -1 : i1;")
    lw("        }")
    lw("        if (t3 != 1) {")
    lw("            const bool i2 = in_slab_inl(s2[0], s2[1], s2[2], s2[3], s2[4], s2[5], s2[6], ci2);")
    lw("            u2 = ci2.bad ? -1 : i2;")
    lw("        }")
    lw("        const int hit = rc_and3(rc_and3(t0, t1), rc_and3(rc_or3(t2, u1), rc_or3(t3, u2)));")
    lw("        if (hit < 0) ctx.bad = true;")
    lw("        else if (hit == 1) {")
    lw("            win = j;")
    lw("            break;")
    lw("        }")
    lw("    }")
    lw("    if (ctx.bad) return zero;")
    lw("    if (win < 0) return rect_tail(Rab, Tab, a, b, S, ctx);")
    lw("    T e[5], qb = zero;")
    lw("    int px = 0, py = 0, qkind = 1, cb = 0, cu = 0;")
    lw("    switch (win) {")
    for j, r in enumerate(rows):
        lw(f"    case {j}:")
        lw("        " + " ".join(f"e[{i}] = {v};" for i, v in enumerate(r["e"])))
        lw(f"        px = {pt(r['px'])}; py = {pt(r['py'])}; qkind = {r['qkind']}; cb = {r['cb']}; qb = {r['qb']};"
          f" cu = {r['cu']};")
        lw("        break;")
    lw("    default:")
    lw("        break;")
    lw("    }")
    lw("    T t, u;")
    lw("    edge_params_inl(t, u, e[0], e[1], e[2], e[3], e[4], ctx);")
    lw("    const T Px = px == 0 ? a[0] : px == 1 ? a[1] : px == 4 ? t : zero;")
    lw("    const T Py = py == 0 ? a[0] : py == 1 ? a[1] : py == 4 ? t : zero;")
    lw("    const V3T<T> P = v3t<T>(Px, Py, zero);")
    lw("    const T rbx = cb ? Rab.m[1] : Rab.m[0], rby = cb ? Rab.m[4] : Rab.m[3], rbz = cb ? Rab.m[7] : Rab.m[6];")
    lw("    const T rux = cu ? Rab.m[1] : Rab.m[0], ruy = cu ? Rab.m[4] : Rab.m[3], ruz = cu ? Rab.m[7] : Rab.m[6];")
    lw("    const V3T<T> Q2 = v3t(Tab.x + rbx * qb + rux * u, Tab.y + rby * qb + ruy * u, Tab.z + rbz * qb + ruz * u);")
    lw("    const V3T<T> Q1 = v3t(Tab.x + rux * u, Tab.y + ruy * u, Tab.z + ruz * u);")
    lw("    const V3T<T> Q = qkind == 2 ? Q2 : Q1;")
    lw("    S = v3t(Q.x - P.x, Q.y - P.y, Q.z - P.z);")
    lw("    return num_sqrt(dot(S, S));")
    lw("}")
    lw("")
    lines.extend(lane_lines)
    w("} // namespace c2a")
    w("#endif")
    open(OUT, "w").write("\n".join(lines) + "\n")
    print(f"{OUT}: 16 cases, {len(exprs)} shared expressions")
    write_table(pre, exprs, rows)


# ------------------------------------------------------------ rect_table.cuh

IN_SLOTS = ["a[0]", "a[1]", "b[0]", "b[1]", "A0B0", "A0B1", "A1B0", "A1B1", "Tab.x", "Tab.y", "zero"]
S1_SLOTS = ["aA0B0", "aA0B1", "aA1B0", "aA1B1", "bA0B0", "bA1B0", "bA0B1", "bA1B1", "Tba.x", "Tba.y"]


def chain_of(e: str) -> list[tuple[int, str]]:
    """'-p + q - r' -> [(-1, 'p'), (1, 'q'), (-1, 'r')] (left-associative)."""
    toks = re.findall(r"[+-]|[^+\s-][^+-]*", e.replace(" ", ""))
    out, sign = [], 1
    for t in toks:
        if t in "+-":
            sign = sign * (-1 if t == "-" else 1) if out or t == "-" else sign
            if not out and t == "-":
                sign = -1
            continue
        out.append((sign, t))
        sign = 1
    return out


def write_table(pre: str, exprs: dict, rows: list):
    slot = {n: i for i, n in enumerate(IN_SLOTS)}
    for i, n in enumerate(S1_SLOTS):
        slot[n] = len(IN_SLOTS) + i
    s2_base = len(IN_SLOTS) + len(S1_SLOTS)
    chains: dict[str, list] = {}   # stage-2 name -> signed atom chain
    alias: dict[str, tuple] = {}   # name -> (sign, slot name)
    # the products (check the parsed preamble says what IN/S1 assume)
    prods = dict(re.findall(r"(\w+) = ([ab]\[\d\] \* A\dB\d)", pre))
    assert sorted(prods) == sorted(S1_SLOTS[:8]), prods
    assert "const V3T<T> Tba = tmul(Rab, Tab);" in pre
    for m in re.finditer(r"const T ((?:\w+ = [^,;]+(?:, )?)+);", pre):
        for part in split_top(m.group(1), ","):
            name, e = [x.strip() for x in part.split("=", 1)]
            if name in slot:
                continue
            ch = chain_of(e)
            if name in ("A0B0", "A0B1", "A1B0", "A1B1", "zero"):
                continue
            if len(ch) == 1:
                alias[name] = ch[0]
                continue
            # a stage-2 name on the left expands into its own chain (same tree)
            full = []
            for k, (sg, at) in enumerate(ch):
                if at in chains:
                    assert k == 0 and sg == 1, (name, e)
                    full.extend(chains[at])
                elif at in alias:
                    s0, a0 = alias[at]
                    full.append((sg * s0, a0))
                else:
                    full.append((sg, at))
            chains[name] = full
    for e, x in exprs.items():
        ch = chain_of(e)
        if len(ch) == 1:
            alias[x] = ch[0]
        else:
            chains[x] = ch
    s2 = list(chains)
    for i, n in enumerate(s2):
        slot[n] = s2_base + i
        assert 2 <= len(chains[n]) <= 3, (n, chains[n])
        for _, at in chains[n]:
            assert at in slot and slot[at] < s2_base, (n, at)
    nslots = s2_base + len(s2)
    assert nslots <= 64, nslots

    def sref(name: str) -> tuple[int, int]:
        if name in alias:
            sg, at = alias[name]
            return slot[at], int(sg < 0)
        return slot[name], 0

    groups = []
    sorted_of: dict[str, tuple] = {}
    for m in re.finditer(r"if \(LT\((\w+), (\w+)\)\) \{([^}]*)\}\s*else \{([^}]*)\}", pre):
        g = len(groups)
        groups.append((sref(m.group(1)), sref(m.group(2))))
        tv = dict(re.findall(r"(\w+) = (\w+);", m.group(3)))
        fv = dict(re.findall(r"(\w+) = (\w+);", m.group(4)))
        assert sorted(tv) == sorted(fv)
        for n in tv:
            sorted_of[n] = (g, sref(tv[n]), sref(fv[n]))
    assert len(groups) == 8, len(groups)

    def ref(name: str) -> int:
        if name in sorted_of:
            g, (ts, tn), (fs, fn) = sorted_of[name]
        else:
            (ts, tn), g = sref(name), 15
            fs, fn = ts, tn
        return ts | (tn << 7) | (fs << 8) | (fn << 15) | (g << 16)

    def code(v: str) -> int:
        return int(pt(v))

    case_refs, case_ints = [], []
    for r in rows:
        refs = [x for pair in r["c"] for x in pair]
        refs = [refs[0], refs[2], refs[4], refs[6], refs[1], refs[3], refs[5], refs[7]]  # L[0..3], R[0..3]
        refs += r["s1"] + r["s2"] + r["e"] + [r["qb"]]
        assert len(refs) == 28
        case_refs += [ref(x) for x in refs]
        case_ints.append(code(r["px"]) | (code(r["py"]) << 4) | (r["qkind"] << 8) | (int(r["cb"]) << 12) |
                         (int(r["cu"]) << 16))
    s1_tab = []
    for n in S1_SLOTS[:8]:
        p, q = [x.strip() for x in prods[n].split("*")]
        s1_tab.append(slot[p] | (slot[q] << 8))
    s2_tab = []
    for n in s2:
        ch = chains[n] + [(1, "zero")] * (3 - len(chains[n]))
        w = 0
        for k, (sg, at) in enumerate(ch):
            w |= (slot[at] | (int(sg < 0) << 7)) << (8 * k)
        s2_tab.append(w | (int(len(chains[n]) == 3) << 24))
    cmp_tab = [(l[0] | (l[1] << 7)) | ((r_[0] | (r_[1] << 7)) << 8) for l, r_ in groups]

    L = []
    w = L.append
    w("/* generated by gen_rect_cases.py from rect_dist in geom.cuh; do not edit */")
    w("#ifndef C2A_RECT_TABLE_CUH")
    w("#define C2A_RECT_TABLE_CUH")
    w("")
    w('#include "geom.cuh"')
    w("")
    w("namespace c2a {")
    w("")
    w("/* C2ARectDist with its shared work spread over a half-warp.  Slots (one")
    w(" * double each, per half): the inputs, then the products and Tab in B's frame")
    w(" * (stage 1), then every sum the preamble and the cases share (stage 2, each")
    w(" * a chain p +- q [+- r] with the sequential code's tree).  The eight sorts")
    w(" * of the preamble become eight comparisons whose outcomes (a mask) pick")
    w(" * between two slots.  A reference packs: slot | negate << 7 for the")
    w(" * comparison-true pick, the same << 8 for the false pick, the comparison")
    w(" * << 16 (15: none). */")
    w(f"constexpr int kRtInputs = {len(IN_SLOTS)};")
    w(f"constexpr int kRtStage1 = {len(S1_SLOTS)};")
    w(f"constexpr int kRtStage2 = {len(s2)};")
    w(f"constexpr int kRtSlots = {nslots};")
    w(f"constexpr int kRtStage2Base = {s2_base};")
    w("constexpr int kRtRefs = 28; /* L[4], R[4], s1[7], s2[7], e[5], qb */")
    w("")

    def arr(name, vals, per=8):
        body = []
        for i in range(0, len(vals), per):
            body.append("    " + ", ".join(f"0x{v:08x}u" for v in vals[i:i + per]) + ",")
        return body

    tables = [("rt_s1", s1_tab), ("rt_s2", s2_tab), ("rt_cmp", cmp_tab), ("rt_case_ref", case_refs),
              ("rt_case_int", case_ints)]
    w("#ifdef __CUDACC__")
    for n, v in tables:
        w(f"__device__ const uint32_t {n}_d[{len(v)}] = {{")
        L.extend(arr(n, v))
        w("};")
    w("#endif")
    for n, v in tables:
        w(f"static const uint32_t {n}_h[{len(v)}] = {{")
        L.extend(arr(n, v))
        w("};")
    w("#ifdef __CUDA_ARCH__")
    w("#define C2A_RT(name, i) __ldg(&name##_d[i])")
    w("#else")
    w("#define C2A_RT(name, i) (name##_h[i])")
    w("#endif")
    w("")
    w("/* lane k's input slot (k < kRtInputs) */")
    w("C2A_DEV double rt_input(int k, const M3 &R, V3 T, const double a[2], const double b[2])")
    w("{")
    vals = ["a[0]", "a[1]", "b[0]", "b[1]", "R.m[0]", "R.m[1]", "R.m[3]", "R.m[4]", "T.x", "T.y", "0.0"]
    expr = vals[-1]
    for k in range(len(vals) - 2, -1, -1):
        expr = f"k == {k} ? {vals[k]} : ({expr})"
    w(f"    return {expr};")
    w("}")
    w("")
    w("/* every input slot (all lanes of a half write the same values) */")
    w("C2A_DEV void rt_inputs(const M3 &R, V3 T, const double a[2], const double b[2], double *V)")
    w("{")
    vals2 = ["a[0]", "a[1]", "b[0]", "b[1]", "R.m[0]", "R.m[1]", "R.m[3]", "R.m[4]", "T.x", "T.y", "0.0"]
    for k, v in enumerate(vals2):
        w(f"    V[{k}] = {v};")
    w("}")
    w("")
    w("/* lane k's stage-1 slot (k < kRtStage1): a product of two input slots, or")
    w(" * Tba.x / Tba.y as tmul evaluates them */")
    w("C2A_DEV double rt_stage1(int k, const M3 &R, V3 T, const double *V)")
    w("{")
    w("    if (k < 8) {")
    w("        const uint32_t w = C2A_RT(rt_s1, k);")
    w("        return V[w & 0x7f] * V[(w >> 8) & 0x7f];")
    w("    }")
    w("    const int c = k - 8; /* column c of R: Tba[c] = R[0][c] T.x + R[1][c] T.y + R[2][c] T.z */")
    w("    return R.m[c] * T.x + R.m[3 + c] * T.y + R.m[6 + c] * T.z;")
    w("}")
    w("")
    w("C2A_DEV double rt_signed(uint32_t b, const double *V) /* slot | negate << 7 */")
    w("{")
    w("    const double v = V[b & 0x7f];")
    w("    return (b & 0x80) ? -v : v;")
    w("}")
    w("")
    w("/* stage-2 slot i (< kRtStage2) */")
    w("C2A_DEV double rt_stage2(int i, const double *V)")
    w("{")
    w("    const uint32_t w = C2A_RT(rt_s2, i);")
    w("    const double s = rt_signed(w & 0xff, V) + rt_signed((w >> 8) & 0xff, V);")
    w("    const double s3 = s + rt_signed((w >> 16) & 0xff, V);")
    w("    return (w >> 24) ? s3 : s;")
    w("}")
    w("")
    w("/* comparison g (< 8) of the preamble's sorts */")
    w("C2A_DEV bool rt_compare(int g, const double *V)")
    w("{")
    w("    const uint32_t w = C2A_RT(rt_cmp, g);")
    w("    return rt_signed(w & 0xff, V) < rt_signed((w >> 8) & 0xff, V);")
    w("}")
    w("")
    w("/* a case operand through its reference, given the comparisons' mask */")
    w("C2A_DEV double rt_operand(uint32_t r, unsigned mask, const double *V)")
    w("{")
    w("    const unsigned g = (r >> 16) & 15u;")
    w("    const bool f = g != 15u && !((mask >> g) & 1u);")
    w("    return rt_signed(f ? (r >> 8) & 0xff : r & 0xff, V);")
    w("}")
    w("")
    w("/* the operands of case j (< 16) */")
    w("C2A_DEV void rt_case_operands(int j, unsigned mask, const double *V, double L[4], double R[4], double s1[7],")
    w("                              double s2[7], double e[5], double &qb, int &px, int &py, int &qkind, int &cb,")
    w("                              int &cu)")
    w("{")
    w("    const int o = j * kRtRefs;")
    w("#pragma unroll")
    w("    for (int i = 0; i < 4; i++) {")
    w("        L[i] = rt_operand(C2A_RT(rt_case_ref, o + i), mask, V);")
    w("        R[i] = rt_operand(C2A_RT(rt_case_ref, o + 4 + i), mask, V);")
    w("    }")
    w("#pragma unroll")
    w("    for (int i = 0; i < 7; i++) {")
    w("        s1[i] = rt_operand(C2A_RT(rt_case_ref, o + 8 + i), mask, V);")
    w("        s2[i] = rt_operand(C2A_RT(rt_case_ref, o + 15 + i), mask, V);")
    w("    }")
    w("#pragma unroll")
    w("    for (int i = 0; i < 5; i++) e[i] = rt_operand(C2A_RT(rt_case_ref, o + 22 + i), mask, V);")
    w("    qb = rt_operand(C2A_RT(rt_case_ref, o + 27), mask, V);")
    w("    const uint32_t n = C2A_RT(rt_case_int, j);")
    w("    px = n & 15; py = (n >> 4) & 15; qkind = (n >> 8) & 15; cb = (n >> 12) & 15; cu = (n >> 16) & 15;")
    w("}")
    w("")
    w("/* case j's condition, short-circuit like the sequential code (in_slab only")
    w(" * where the sequential code evaluates it) */")
    w("C2A_DEV bool rt_case_holds(const double L[4], const double R[4], const double s1[7], const double s2[7])")
    w("{")
    w("    ExactCtx xc{false};")
    w("    return L[0] < R[0] && L[1] < R[1] &&")
    w("           (L[2] < R[2] || in_slab(s1[0], s1[1], s1[2], s1[3], s1[4], s1[5], s1[6], xc)) &&")
    w("           (L[3] < R[3] || in_slab(s2[0], s2[1], s2[2], s2[3], s2[4], s2[5], s2[6], xc));")
    w("}")
    w("")
    w("/* the edge pair's distance and S once its case holds (rect_cases.cuh's")
    w(" * arithmetic; Q's two forms share their first sum's tree) */")
    w("C2A_DEV double rt_case_value(const double e[5], double qb, int px, int py, int qkind, int cb, int cu,")
    w("                             const M3 &Rab, V3 Tab, const double a[2], V3 &S)")
    w("{")
    w("    ExactCtx xc{false};")
    w("    double t, u;")
    w("    edge_params(t, u, e[0], e[1], e[2], e[3], e[4], xc);")
    w("    const double Px = px == 0 ? a[0] : px == 1 ? a[1] : px == 4 ? t : 0.0;")
    w("    const double Py = py == 0 ? a[0] : py == 1 ? a[1] : py == 4 ? t : 0.0;")
    w("    const double rbx = cb ? Rab.m[1] : Rab.m[0], rby = cb ? Rab.m[4] : Rab.m[3], rbz = cb ? Rab.m[7] : Rab.m[6];")
    w("    const double rux = cu ? Rab.m[1] : Rab.m[0], ruy = cu ? Rab.m[4] : Rab.m[3], ruz = cu ? Rab.m[7] : Rab.m[6];")
    w("    const bool two = qkind == 2;")
    w("    const double bx = Tab.x + rbx * qb, by = Tab.y + rby * qb, bz = Tab.z + rbz * qb;")
    w("    const V3 Q = v3((two ? bx : Tab.x) + rux * u, (two ? by : Tab.y) + ruy * u, (two ? bz : Tab.z) + ruz * u);")
    w("    S = v3(Q.x - Px, Q.y - Py, Q.z - 0.0);")
    w("    return sqrt(S.x * S.x + S.y * S.y + S.z * S.z);")
    w("}")
    w("")
    w("} // namespace c2a")
    w("#endif")
    open(OUT_TABLE, "w").write("\n".join(L) + "\n")
    print(f"{OUT_TABLE}: {nslots} slots ({len(s2)} stage-2 sums), {len(groups)} comparisons")


if __name__ == "__main__":
    main()
