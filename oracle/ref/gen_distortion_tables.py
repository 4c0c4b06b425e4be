#!/usr/bin/env python3
"""Regenerate the multi-constant distortion coefficient tables.

The reference's L2, L3 and L4 distortion forces (lcForces.h: bulkL2Force,
boundaryL2Force, bulkL3Force, boundaryL3Force, bulkL4Force, boundaryL4Force)
are linear forms over 125 inputs: the site's q (5), its six neighbours' q
(30) and its six neighbours' first-derivative vectors (90).  Their generated
coefficients contain irregular terms that a re-derivation from the continuum
functional does not reproduce, so parity needs the very same linear forms.
``stencil_probe`` (built by this directory's Makefile from the reference
tree) recovers them by evaluating each form on unit vectors; this script turns
its output into two headers:

* ``oracle/distortion_coeffs.h``: a flat coefficient list for the C restatement;
* ``open-qmin_gb300/csrc/qmin_distortion_tables.h``: packed sparse tables
  for the CUDA kernels.

Case numbering follows lcForces.h:13-25: case = xx + 4*yy + 16*zz with
xx, yy, zz in {0, 1 (up neighbour is an object), 2 (down neighbour is an
object; down wins)}.  The bulk form equals case 0.  Every coefficient is a
multiple of L/4 and is stored as an integer k with value k*L/4.

Run from the repository root (needs the reference tree):
    make -C oracle/ref && python3 oracle/ref/gen_distortion_tables.py
"""
import collections
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PROBE = os.path.join(ROOT, "oracle", "_ref", "stencil_probe")

TERMS = ["L2", "L3", "L4"]
VALID_CASES = [c for c in range(64) if (c & 3) != 3 and ((c >> 2) & 3) != 3 and ((c >> 4) & 3) != 3]


def main():
    out = subprocess.run([PROBE], check=True, capture_output=True, text=True).stdout
    coef = collections.defaultdict(dict)
    for line in out.splitlines():
        t, case, c, i, v = line.split()
        # the probe runs with L = 2, so a printed value v means v * L / 2 = (2v) * L / 4
        k = 2.0 * float(v)
        if k != round(k):
            sys.exit(f"non-quarter coefficient {line}")
        coef[(t, int(case), int(c))][int(i)] = int(round(k))
    for t in TERMS:
        for c in range(5):
            if coef[(t, -1, c)] != coef[(t, 0, c)]:
                sys.exit(f"{t}: bulk form differs from boundary case 0")

    header = ("/* Generated by oracle/ref/gen_distortion_tables.py from the reference's\n"
              " * lcForces.h stencils (black-box probe).  Do not edit.  Value = k * L / 4. */\n")
    # flat (term, case, component, input, k) list for the oracle
    lines = [header, "#ifndef QMIN_ORACLE_DISTORTION_COEFFS_H", "#define QMIN_ORACLE_DISTORTION_COEFFS_H",
             "/* {term 0=L2 1=L3 2=L4, case, component, input, k} */",
             "static const short qo_distortion_entries[][5] = {"]
    n = 0
    for ti, t in enumerate(TERMS):
        for case in VALID_CASES:
            row = []
            for c in range(5):
                for i, k in sorted(coef[(t, case, c)].items()):
                    row.append("{%d,%d,%d,%d,%d}" % (ti, case, c, i, k))
                    n += 1
            lines.append(" " + ",".join(row) + ",")
    lines += ["};", "#define QO_DISTORTION_NENTRIES %d" % n, "#endif", ""]
    with open(os.path.join(ROOT, "oracle", "distortion_coeffs.h"), "w") as f:
        f.write("\n".join(lines))

    # packed sparse tables for the kernels: per (term, case, component) a run of
    # (input, k) pairs; offsets index into the pair arrays.
    inputs, ks, offsets = [], [], []
    for t in TERMS:
        for case in range(64):
            for c in range(5):
                offsets.append(len(inputs))
                if case in VALID_CASES:
                    for i, k in sorted(coef[(t, case, c)].items()):
                        inputs.append(i)
                        ks.append(k)
    offsets.append(len(inputs))
    lines = [header, "#pragma once", "#include <stdint.h>",
             f"#define QMIN_DT_NPAIRS {len(inputs)}",
             "/* offset[(term*64 + case)*5 + component] .. offset[... + 1] */",
             "/* initialiser lists, so that host and device copies can be defined from them */",
             "#define QMIN_DT_OFFSET_INIT {" + ",".join(str(x) for x in offsets) + "}",
             "#define QMIN_DT_INPUT_INIT {" + ",".join(str(x) for x in inputs) + "}",
             "#define QMIN_DT_K_INIT {" + ",".join(str(x) for x in ks) + "}", ""]
    with open(os.path.join(ROOT, "open-qmin_gb300", "csrc", "qmin_distortion_tables.h"), "w") as f:
        f.write("\n".join(lines))
    # straight-line bulk forms: one linear form per component over the union of
    # the L1 (bulk, lcForces.h:26-37), L2, L3 and L4 bulk patterns; the kernels
    # multiply each input by a per-handle coefficient cb[k][n] = sum_t L_t k_t / 4
    # computed on the host.  The L1 bulk form written in the same units
    # (k L1 / 4): S = L1 (6 q - sum of the six neighbours), then S0 += S0 + S3,
    # S3 += S0 + S3, S1, S2, S4 doubled.
    l1 = {c: {} for c in range(5)}
    for c in range(5):
        partners = {0: {0: 2, 3: 1}, 3: {0: 1, 3: 2}}.get(c, {c: 2})
        for comp, m in partners.items():
            l1[c][comp] = l1[c].get(comp, 0) + 4 * 6 * m
            for slot in range(6):
                j = 5 + 5 * slot + comp
                l1[c][j] = l1[c].get(j, 0) - 4 * m
        coef[("L1", 0, c)] = l1[c]
    TERMS4 = ["L2", "L3", "L4", "L1"]
    union = [sorted(set().union(*[coef[(t, 0, c)].keys() for t in TERMS4])) for c in range(5)]
    W = max(len(u) for u in union)
    l4only = [[n for n, j in enumerate(union[c]) if all(coef[(t, 0, c)].get(j, 0) == 0 for t in ("L2", "L3", "L1"))]
              for c in range(5)]
    lines = [header.replace("Do not edit.", "Do not edit.  Bulk (case 0) forms, straight-line."), "#pragma once",
             f"#define QMIN_BULK_W {W}",
             "/* inputs of component k: qmin_bulk_in[k][0 .. qmin_bulk_n[k]) (0..4 q, 5..34 neighbour q,",
             "   35..124 neighbour derivatives); per-term integer coefficients qmin_bulk_k[term][k][n],",
             "   terms L2, L3, L4, L1 */",
             "static const int qmin_bulk_n[5] = {" + ",".join(str(len(u)) for u in union) + "};",
             "static const int qmin_bulk_in[5][QMIN_BULK_W] = {" +
             ",".join("{" + ",".join(str(x) for x in u + [0] * (W - len(u))) + "}" for u in union) + "};",
             "static const int qmin_bulk_k[4][5][QMIN_BULK_W] = {" +
             ",".join("{" + ",".join("{" + ",".join([str(coef[(t, 0, c)].get(x, 0)) for x in union[c]] +
                                                     ["0"] * (W - len(union[c]))) + "}" for c in range(5)) + "}"
                      for t in TERMS4) + "};",
             "",
             "/* s[k] = sum_n cb[k*QMIN_BULK_W + n] * input; QIN(c) = own q component,",
             "   QN(slot, c) = neighbour q, DN(slot, d) = neighbour derivative component.",
             "   QMIN_BULK_FORMS_NO_L4 omits the inputs only the L4 term uses. */"]

    def term(j):
        if j < 5:
            return f"QIN({j})"
        if j < 35:
            return f"QN({(j - 5) // 5},{(j - 5) % 5})"
        return f"DN({(j - 35) // 15},{(j - 35) % 15})"
    for name, skip in (("QMIN_BULK_FORMS", [[] for _ in range(5)]), ("QMIN_BULK_FORMS_NO_L4", l4only)):
        lines.append(f"#define {name}(cb, s) \\")
        for c in range(5):
            body = " + ".join(f"(cb)[{c * W + n}] * {term(j)}" for n, j in enumerate(union[c]) if n not in skip[c])
            lines.append(f"    (s)[{c}] = {body}; \\")
        lines.append("    do {} while (0)")
        lines.append("")
    with open(os.path.join(ROOT, "open-qmin_gb300", "csrc", "qmin_bulk_forms.h"), "w") as f:
        f.write("\n".join(lines))
    print(f"wrote tables: {len(inputs)} nonzero coefficients; bulk union widths {[len(u) for u in union]}, "
          f"L4-only {[len(x) for x in l4only]}")


if __name__ == "__main__":
    main()
