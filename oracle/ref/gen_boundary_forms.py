#!/usr/bin/env python3
"""Rewrite the 27-case boundary L2/L3/L4 forms as straight-line code.

The boundary distortion forces (lcForces.h boundaryL2/L3/L4 forms, chosen by
lcForce::getBoundaryCase, lcForces.h:13-25) are linear forms over 125 inputs
(q, the six neighbours' q, the six neighbours' first derivatives) whose
integer coefficients the probe recovered into
``open-qmin_gb300/csrc/qmin_distortion_tables.h`` (one sparse table per term,
case and component).  This script merges the three terms of each case and
component over the union of their inputs and writes
``open-qmin_gb300/csrc/qmin_boundary_forms.h``:

* ``qmin_bnd_slot[64]``: boundary case (xx + 4 yy + 16 zz) -> slot 0..26;
* ``qmin_bnd_k[27][5][QMIN_BND_W][3]``: per-term integer coefficients
  (L2, L3, L4) of each merged input, and ``qmin_bnd_dn[...]`` marking the
  derivative inputs, from which the host builds the per-parameter-set
  coefficients ``cbd = sum_t L_t k_t / 4`` (halved for derivative inputs,
  which the accessors deliver as twice the derivative);
* ``QMIN_BOUNDARY_FORMS(slot, cbd, s)``: a switch over the 27 slots, each a
  straight-line form over the accessors QIN(c), QN(slot, c), DN(slot, d).

It needs no reference tree.

    python3 oracle/ref/gen_boundary_forms.py
"""
import collections
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SRC = os.path.join(ROOT, "open-qmin_gb300", "csrc", "qmin_distortion_tables.h")
OUT = os.path.join(ROOT, "open-qmin_gb300", "csrc", "qmin_boundary_forms.h")


def read_tables():
    s = open(SRC).read()

    def arr(name):
        return [int(x) for x in re.search(r"#define " + name + r" \{([^}]*)\}", s).group(1).split(",") if x.strip()]

    return arr("QMIN_DT_OFFSET_INIT"), arr("QMIN_DT_INPUT_INIT"), arr("QMIN_DT_K_INIT")


def accessor(j):
    if j < 5:
        return f"QIN({j})"
    if j < 35:
        return f"QN({(j - 5) // 5},{(j - 5) % 5})"
    return f"DN({(j - 35) // 15},{(j - 35) % 15})"


def main():
    off, inp, kk = read_tables()
    cases = []  # (bcase, [per component: [(input, [k_L2, k_L3, k_L4])]])
    for zz in range(3):
        for yy in range(3):
            for xx in range(3):
                b = xx + 4 * yy + 16 * zz
                comps = []
                for c in range(5):
                    u = collections.OrderedDict()
                    for t in range(3):
                        for e in range(off[(t * 64 + b) * 5 + c], off[(t * 64 + b) * 5 + c + 1]):
                            u.setdefault(inp[e], [0, 0, 0])[t] += kk[e]
                    comps.append([(j, v) for j, v in u.items() if any(v)])
                cases.append((b, comps))
    width = max(len(f) for _, comps in cases for f in comps)
    slot = [-1] * 64
    for n, (b, _) in enumerate(cases):
        slot[b] = n
    lines = ["/* Generated by oracle/ref/gen_boundary_forms.py from qmin_distortion_tables.h.  Do not edit.",
             " * The boundary L2/L3/L4 forms merged per case and component: for boundary case slot n,",
             " * s[c] = sum_m cbd[(n * 5 + c) * QMIN_BND_W + m] * input_m, cbd = sum_t L_t k_t / 4",
             " * (halved for derivative inputs), terms ordered L2, L3, L4. */", "#pragma once",
             f"#define QMIN_BND_W {width}", f"#define QMIN_BND_CASES {len(cases)}"]
    lines.append("static const signed char qmin_bnd_slot[64] = {" + ",".join(str(x) for x in slot) + "};")
    krows, drows = [], []
    for _, comps in cases:
        kc, dc = [], []
        for f in comps:
            ent = [f"{{{v[0]},{v[1]},{v[2]}}}" for _, v in f] + ["{0,0,0}"] * (width - len(f))
            kc.append("{" + ",".join(ent) + "}")
            dc.append("{" + ",".join(["1" if j >= 35 else "0" for j, _ in f] + ["0"] * (width - len(f))) + "}")
        krows.append("{" + ",".join(kc) + "}")
        drows.append("{" + ",".join(dc) + "}")
    lines.append(f"static const signed char qmin_bnd_k[{len(cases)}][5][QMIN_BND_W][3] = {{" + ",".join(krows) + "};")
    lines.append(f"static const unsigned char qmin_bnd_dn[{len(cases)}][5][QMIN_BND_W] = {{" + ",".join(drows) + "};")
    lines.append("#define QMIN_BOUNDARY_FORMS(slot, cbd, s) \\")
    lines.append("    switch (slot) { \\")
    for n, (_, comps) in enumerate(cases):
        lines.append(f"    case {n}: \\")
        for c, f in enumerate(comps):
            base = (n * 5 + c) * width
            terms = [f"(cbd)[{base + m}] * {accessor(j)}" for m, (j, _) in enumerate(f)]
            lines.append(f"        (s)[{c}] = " + (" + ".join(terms) if terms else "0") + "; \\")
        lines.append("        break; \\")
    lines.append("    default: \\")
    lines.append("        (s)[0] = (s)[1] = (s)[2] = (s)[3] = (s)[4] = 0; \\")
    lines.append("    }")
    lines.append("")
    open(OUT, "w").write("\n".join(lines))
    print("cases", len(cases), "width", width, "terms", sum(len(f) for _, comps in cases for f in comps))


if __name__ == "__main__":
    main()
