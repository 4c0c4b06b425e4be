#!/usr/bin/env python3
"""Rewrite the combined bulk distortion form over Q on the 25-point stencil.

For a bulk site whose six neighbours are bulk too, every neighbour derivative
the L1-L4 bulk forms read is a central difference, 0.5 (Q(up) - Q(down)), so
the linear form over (q, neighbour q, neighbour derivatives) is a linear form
over Q at the site, its 6 neighbours, its 12 diagonal neighbours and the 6
sites two steps away.  This script reads the generated bulk tables
(``open-qmin_gb300/csrc/qmin_bulk_forms.h``, from gen_distortion_tables.py)
and writes ``open-qmin_gb300/csrc/qmin_bulk_q25.h``: per-term integer
coefficients (value k * L / 8) and straight-line forms over the accessor
QQ(dx, dy, dz, c).  It needs no reference tree.

Without L4 the form is written with shared sums: where two stencil values
enter several components' sums with coefficients in a fixed ratio (1, -1, 2,
-2, 1/2 or -1/2 for every elastic constant), their combination is formed once
and weighted once per component (greedy pairing, most reuse first).  On
GB300 the FP64 deep-site force is bound by the FP64 pipe, and this takes the
stencil from 121 to 106 FP64 operations per site.  The plain L4-free form
(one term per stencil value) stays beside it: the batched FP32 kernel, bound
by latency rather than by an arithmetic pipe, runs faster with it.  The rewritten form is
checked term by term against the plain one before it is written.

    python3 oracle/ref/gen_q25_form.py           # write the header
    python3 oracle/ref/gen_q25_form.py --check   # exit 1 if the header differs
"""
import collections
import itertools
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SRC = os.path.join(ROOT, "open-qmin_gb300", "csrc", "qmin_bulk_forms.h")
OUT = os.path.join(ROOT, "open-qmin_gb300", "csrc", "qmin_bulk_q25.h")
OFF6 = [(-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1)]
AX = [(1, 0, 0), (0, 1, 0), (0, 0, 1)]


def read_bulk():
    s = open(SRC).read()
    n = [int(x) for x in re.search(r"qmin_bulk_n\[5\] = \{([^}]*)\}", s).group(1).split(",")]
    inp = re.search(r"qmin_bulk_in\[5\]\[QMIN_BULK_W\] = \{(.*?)\};", s, re.S).group(1)
    inp = [[int(x) for x in row.split(",") if x.strip()] for row in re.findall(r"\{([^{}]*)\}", inp)]
    kk = re.search(r"qmin_bulk_k\[4\]\[5\]\[QMIN_BULK_W\] = \{(.*)\};", s, re.S).group(1)
    rows = [[int(x) for x in row.split(",") if x.strip()] for row in re.findall(r"\{([^{}]*)\}", kk)]
    K = [[rows[t * 5 + c] for c in range(5)] for t in range(4)]  # terms L2, L3, L4, L1; value k L / 4
    return n, inp, K


def main():
    n, inp, K = read_bulk()
    forms = []  # per component: [((offset, comp), [k per term])] in units of L / 8
    for c in range(5):
        W = collections.OrderedDict()

        def add(key, vec, scale):
            cur = W.setdefault(key, [0, 0, 0, 0])
            for t in range(4):
                cur[t] += scale * vec[t]

        for m in range(n[c]):
            j = inp[c][m]
            vec = [K[t][c][m] for t in range(4)]
            if j < 5:
                add(((0, 0, 0), j), vec, 2)
            elif j < 35:
                add((OFF6[(j - 5) // 5], (j - 5) % 5), vec, 2)
            else:
                d = j - 35
                o, a, cc = OFF6[d // 15], AX[(d % 15) // 5], d % 5
                up = tuple(o[i] + a[i] for i in range(3))
                dn = tuple(o[i] - a[i] for i in range(3))
                add((up, cc), vec, 1)
                add((dn, cc), vec, -1)
        forms.append([(k, v) for k, v in W.items() if any(v)])
    width = max(len(f) for f in forms)
    inter, cforms = shared_sums(forms)
    assert max(len(f) for f in cforms) <= width
    lines = ["/* Generated by oracle/ref/gen_q25_form.py from qmin_bulk_forms.h.  Do not edit.",
             " * The combined bulk form (L1-L4) of a site whose neighbours are all bulk, over Q on",
             " * the 25-point stencil: s[c] = sum_m cq[c * QMIN_Q25_W + m] * QQ(dx, dy, dz, comp),",
             " * cq = sum_t L_t k_t / 8 with the terms ordered L2, L3, L4, L1 (qmin_q25_k).",
             " * Without L4: the same sums over shared combinations of stencil values,",
             " * cq from qmin_q25c_k (QMIN_BULK_Q25_NO_L4), or term by term (_PLAIN). */", "#pragma once",
             f"#define QMIN_Q25_W {width}"]
    lines.append("static const int qmin_q25_n[5] = {" + ",".join(str(len(f)) for f in forms) + "};")
    lines.append("static const int qmin_q25_k[4][5][QMIN_Q25_W] = " + table(forms, width) + ";")
    lines.append("static const int qmin_q25c_k[4][5][QMIN_Q25_W] = " + table(cforms, width) + ";")
    lines.append("#define QMIN_BULK_Q25(cq, s) \\")
    for c, f in enumerate(forms):
        terms = [f"(cq)[{c * width + m}] * QQ({o[0]},{o[1]},{o[2]},{cc})" for m, ((o, cc), _) in enumerate(f)]
        lines.append(f"    (s)[{c}] = " + " + ".join(terms) + "; \\")
    lines.append("    do {} while (0)")
    lines.append("#define QMIN_BULK_Q25_NO_L4(cq, s) \\")
    for k, (a, b, r) in enumerate(inter):
        lines.append(f"    const auto q25u_{k} = {operand(a)} {'+' if r > 0 else '-'} "
                     + (f"{abs(r)!r} * " if abs(r) != 1 else "") + f"{operand(b)}; \\")
    for c, f in enumerate(cforms):
        terms = [f"(cq)[{c * width + m}] * {operand(key)}" for m, (key, _) in enumerate(f)]
        lines.append(f"    (s)[{c}] = " + " + ".join(terms) + "; \\")
    lines.append("    do {} while (0)")
    # the plain L4-free form, one term per stencil value (qmin_q25_k layout)
    lines.append("#define QMIN_BULK_Q25_NO_L4_PLAIN(cq, s) \\")
    for c, f in enumerate(forms):
        terms = [f"(cq)[{c * width + m}] * QQ({o[0]},{o[1]},{o[2]},{cc})" for m, ((o, cc), v) in enumerate(f)
                 if v[0] or v[1] or v[3]]
        lines.append(f"    (s)[{c}] = " + " + ".join(terms) + "; \\")
    lines.append("    do {} while (0)")
    lines.append("")
    text = "\n".join(lines)
    if "--check" in sys.argv:
        same = os.path.exists(OUT) and open(OUT).read() == text
        print("up to date" if same else "differs: " + OUT)
        sys.exit(0 if same else 1)
    open(OUT, "w").write(text)
    print("terms per component", [len(f) for f in forms], "width", width,
          "without L4", [sum(1 for _, v in f if v[0] or v[1] or v[3]) for f in forms],
          "shared sums", len(inter), "terms", [len(f) for f in cforms])


def table(forms, width):
    ks = []
    for t in range(4):
        comp_rows = []
        for f in forms:
            row = [v[t] for _, v in f] + [0] * (width - len(f))
            comp_rows.append("{" + ",".join(str(x) for x in row) + "}")
        ks.append("{" + ",".join(comp_rows) + "}")
    return "{" + ",".join(ks) + "}"


def operand(key):
    if key[0] == "u":
        return f"q25u_{key[1]}"
    (o, cc) = key[1]
    return f"QQ({o[0]},{o[1]},{o[2]},{cc})"


RATIOS = (1, -1, 2, -2, 0.5, -0.5)


def ratio(a, b):
    """r with b = r a for every elastic constant, else None"""
    for r in RATIOS:
        if all(bb == r * aa for aa, bb in zip(a, b)):
            return r
    return None


def shared_sums(forms):
    """Greedy pairing over the L4-free forms: repeatedly take the pair of
    operands (a, b) whose combination a + r b appears, with the same ratio r,
    in the most components (at least two), form it once and let it replace
    the pair there.  Returns the combinations [(a, b, r)] in evaluation order
    and per component [(operand, k)] with operands ("q", (offset, comp)) or
    ("u", index); k in the (L2, L3, L4, L1) order, L4 = 0."""
    outs = []
    for f in forms:
        d = collections.OrderedDict()
        for key, v in f:
            if v[0] or v[1] or v[3]:
                d[("q", key)] = (v[0], v[1], 0, v[3])
        outs.append(d)
    inter = []
    while True:
        cnt = collections.Counter()
        for d in outs:
            for a, b in itertools.combinations(d.keys(), 2):
                r = ratio(d[a], d[b])
                if r is not None:
                    cnt[(a, b, r)] += 1
        best = None
        for cand, n in cnt.items():  # first of the most reused; ties keep table order
            if n >= 2 and (best is None or n > best[1]):
                best = (cand, n)
        if best is None:
            break
        a, b, r = best[0]
        u = ("u", len(inter))
        inter.append((a, b, r))
        for d in outs:
            if a in d and b in d and ratio(d[a], d[b]) == r:
                k = d[a]
                items = [(key, v) for key, v in d.items() if key not in (a, b)]
                d.clear()
                d[u] = k
                d.update(items)
    check(forms, inter, outs)
    return inter, [list(d.items()) for d in outs]


def check(forms, inter, outs):
    """the rewritten form equals the plain L4-free form term by term"""
    def expand(key):
        if key[0] == "q":
            return {key[1]: 1.0}
        a, b, r = inter[key[1]]
        e = collections.Counter()
        for kk, w in expand(a).items():
            e[kk] += w
        for kk, w in expand(b).items():
            e[kk] += r * w
        return e

    for f, d in zip(forms, outs):
        want = {key: tuple(v[t] for t in (0, 1, 3)) for key, v in f if v[0] or v[1] or v[3]}
        got = collections.defaultdict(lambda: [0.0, 0.0, 0.0])
        for key, k in d.items():
            for kk, w in expand(key).items():
                for i, t in enumerate((0, 1, 3)):
                    got[kk][i] += w * k[t]
        got = {kk: tuple(v) for kk, v in got.items() if any(v)}
        assert set(got) == set(want) and all(
            all(abs(x - y) < 1e-12 for x, y in zip(got[kk], want[kk])) for kk in want), "shared-sum form differs"


if __name__ == "__main__":
    main()
