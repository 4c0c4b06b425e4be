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
    make -C oracle/ref REF=/root/reference && python3 oracle/ref/gen_distortion_tables.py
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
             "static const uint16_t qmin_dt_offset[3 * 64 * 5 + 1] = {" +
             ",".join(str(x) for x in offsets) + "};",
             "static const uint8_t qmin_dt_input[QMIN_DT_NPAIRS] = {" + ",".join(str(x) for x in inputs) + "};",
             "static const int8_t qmin_dt_k[QMIN_DT_NPAIRS] = {" + ",".join(str(x) for x in ks) + "};", ""]
    with open(os.path.join(ROOT, "open-qmin_gb300", "csrc", "qmin_distortion_tables.h"), "w") as f:
        f.write("\n".join(lines))
    print(f"wrote tables: {len(inputs)} nonzero coefficients")


if __name__ == "__main__":
    main()
