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

    python3 oracle/ref/gen_q25_form.py
"""
import collections
import os
import re

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
    lines = ["/* Generated by oracle/ref/gen_q25_form.py from qmin_bulk_forms.h.  Do not edit.",
             " * The combined bulk form (L1-L4) of a site whose neighbours are all bulk, over Q on",
             " * the 25-point stencil: s[c] = sum_m cq[c * QMIN_Q25_W + m] * QQ(dx, dy, dz, comp),",
             " * cq = sum_t L_t k_t / 8 with the terms ordered L2, L3, L4, L1. */", "#pragma once",
             f"#define QMIN_Q25_W {width}"]
    lines.append("static const int qmin_q25_n[5] = {" + ",".join(str(len(f)) for f in forms) + "};")
    ks = []
    for t in range(4):
        comp_rows = []
        for f in forms:
            row = [v[t] for _, v in f] + [0] * (width - len(f))
            comp_rows.append("{" + ",".join(str(x) for x in row) + "}")
        ks.append("{" + ",".join(comp_rows) + "}")
    lines.append("static const int qmin_q25_k[4][5][QMIN_Q25_W] = {" + ",".join(ks) + "};")
    for name, skip_l4 in (("QMIN_BULK_Q25", False), ("QMIN_BULK_Q25_NO_L4", True)):
        lines.append(f"#define {name}(cq, s) \\")
        for c, f in enumerate(forms):
            terms = []
            for m, ((o, cc), v) in enumerate(f):
                if skip_l4 and v[0] == 0 and v[1] == 0 and v[3] == 0:
                    continue
                terms.append(f"(cq)[{c * width + m}] * QQ({o[0]},{o[1]},{o[2]},{cc})")
            lines.append(f"    (s)[{c}] = " + " + ".join(terms) + "; \\")
        lines.append("    do {} while (0)")
    lines.append("")
    open(OUT, "w").write("\n".join(lines))
    print("terms per component", [len(f) for f in forms], "width", width,
          "without L4", [sum(1 for _, v in f if v[0] or v[1] or v[3]) for f in forms])


if __name__ == "__main__":
    main()
