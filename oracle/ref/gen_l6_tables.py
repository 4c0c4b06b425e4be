#!/usr/bin/env python3
"""Regenerate the L6 distortion coefficient tables.

The reference's L6 force (lcForces.h: bulkL6Force, boundaryL6Force) is a
homogeneous quadratic form over the same 125 inputs as the L2-L4 forms (q,
six neighbour q, six neighbour first-derivative vectors):
f_c = (L6 / 2) * sum_{i<=j} B_c[i][j] x_i x_j.  ``stencil_probe_l6`` (built by
this directory's Makefile from the reference tree) recovers B by evaluating
the compiled functions on unit vectors and on pairs of them; every B is a
multiple of 1/2, stored here as the integer k = 2B.  This script writes:

* ``oracle/distortion_coeffs_l6.h``: a flat {case, component, i, j, k} list
  for the C restatement (case -1 = bulk form);
* ``open-qmin_gb300/csrc/qmin_l6_forms.h``: the bulk form as straight-line
  code over the accessors QIN/QN/DN (DN delivers twice the derivative, so
  each derivative factor's 1/2 is folded into the constant) and the 27
  boundary cases as packed sparse tables.

Run from the repository root (needs the reference tree):
    make -C oracle/ref && python3 oracle/ref/gen_l6_tables.py
"""
import collections
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PROBE = os.path.join(ROOT, "oracle", "_ref", "stencil_probe_l6")
VALID_CASES = [c for c in range(64) if (c & 3) != 3 and ((c >> 2) & 3) != 3 and ((c >> 4) & 3) != 3]
HEADER = ("/* Generated by oracle/ref/gen_l6_tables.py from the reference's lcForces.h\n"
          " * L6 stencils (black-box probe).  Do not edit. */\n")


def accessor(n):
    if n < 5:
        return f"QIN({n})"
    if n < 35:
        return f"QN({(n - 5) // 5},{(n - 5) % 5})"
    return f"DN({(n - 35) // 15},{(n - 35) % 15})"


def main():
    out = subprocess.run([PROBE], check=True, capture_output=True, text=True).stdout
    coef = collections.defaultdict(dict)  # (case, comp) -> {(i, j): k}
    for line in out.splitlines():
        _, case, c, i, j, v = line.split()
        k = 2.0 * float(v)
        if k != round(k):
            sys.exit(f"non-half coefficient {line}")
        coef[(int(case), int(c))][(int(i), int(j))] = int(round(k))
    for c in range(5):
        if coef[(-1, c)] != coef[(0, c)]:
            sys.exit("L6: bulk form differs from boundary case 0")
    if max(abs(k) for d in coef.values() for k in d.values()) > 127:
        sys.exit("coefficient outside int8")

    # ---- oracle: flat list
    rows = [HEADER, "#ifndef QMIN_ORACLE_DISTORTION_COEFFS_L6_H", "#define QMIN_ORACLE_DISTORTION_COEFFS_L6_H",
            "/* {case (-1 bulk), component, input i, input j (i <= j), k}: f_c += (L6/2) (k/2) x_i x_j */",
            "static const short qo_l6_entries[][5] = {"]
    n = 0
    for case in [-1] + VALID_CASES:
        for c in range(5):
            for (i, j), k in sorted(coef[(case, c)].items()):
                rows.append(f"    {{{case}, {c}, {i}, {j}, {k}}},")
                n += 1
    rows += ["};", f"#define QO_L6_N {n}", "#endif", ""]
    with open(os.path.join(ROOT, "oracle", "distortion_coeffs_l6.h"), "w") as f:
        f.write("\n".join(rows))

    # ---- CUDA: bulk straight-line form, grouped by the first factor
    lines = [HEADER, "#pragma once",
             "/* s[c] = sum_{i<=j} B_c[i][j] x_i x_j for the bulk (type 0 and -2) sites; the caller adds (L6/2) s.",
             "   QIN(c) own q, QN(slot, c) neighbour q, DN(slot, d) twice the neighbour derivative. */",
             "#define QMIN_L6_BULK(T, s) \\"]
    for c in range(5):
        groups = collections.defaultdict(list)
        for (i, j), k in sorted(coef[(-1, c)].items()):
            groups[i].append((j, k))
        parts = []
        for i, lst in sorted(groups.items()):
            inner = []
            for j, k in lst:
                nd = (i >= 35) + (j >= 35)
                val = (k / 2.0) * (0.5 ** nd)
                inner.append(f"T({val!r}) * {accessor(j)}")
            parts.append(f"{accessor(i)} * (" + " + ".join(inner) + ")")
        lines.append(f"    (s)[{c}] = " + " + ".join(parts) + "; \\")
    lines.append("    do {} while (0)")
    lines.append("")
    # ---- CUDA: boundary cases as sparse tables (offset per (case, component))
    off, ii, jj, kk = [0], [], [], []
    for case in range(64):
        for c in range(5):
            if case in VALID_CASES:
                for (i, j), k in sorted(coef[(case, c)].items()):
                    ii.append(i)
                    jj.append(j)
                    kk.append(k)
            off.append(len(ii))
    lines.append(f"#define QMIN_L6_NPAIRS {len(ii)}")
    lines.append("/* entries of (case, component) = [off[case*5+c], off[case*5+c+1]); value (k/2) x_i x_j with")
    lines.append("   derivative inputs as true derivatives */")
    for name, vals in (("OFFSET", off), ("I", ii), ("J", jj), ("K", kk)):
        lines.append(f"#define QMIN_L6_{name}_INIT {{" + ",".join(str(v) for v in vals) + "}")
    lines.append("")
    with open(os.path.join(ROOT, "open-qmin_gb300", "csrc", "qmin_l6_forms.h"), "w") as f:
        f.write("\n".join(lines))
    print(f"{n} oracle entries, {len(ii)} boundary pairs, bulk terms per component",
          [len(coef[(-1, c)]) for c in range(5)])


if __name__ == "__main__":
    main()
