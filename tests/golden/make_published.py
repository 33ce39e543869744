"""Extracts the reference's published BP5-variant CG results into
tests/golden/published_bp5_cg.json: the convergence table of
bakeoff_problems_dealii/tests/scaling_bp35_kokkos_kernel/results/1_GPU.out
(FE_Q(4), QGauss(5), identity-preconditioned CG, ReductionControl(1e9, 1e-16,
1e-9), f = 1, cycles 8..20 of the size sweep).

Run: python tests/golden/make_published.py   (needs the reference checkout)
"""
import json
import os
import re

REF = os.environ.get("MFGB_REFERENCE_ROOT", "/root/reference")
LOG = "bakeoff_problems_dealii/tests/scaling_bp35_kokkos_kernel/results/1_GPU.out"


def main():
    lines = open(os.path.join(REF, LOG)).read().splitlines()
    # the table is re-printed after every cycle; the last print is complete
    start = [i for i, l in enumerate(lines) if re.search(r"cells\s+dofs\s+matvec\s+CG_tot_time", l)][-1]
    rows = []
    for k, l in enumerate(lines[start + 1:], start=start + 2):
        parts = l.replace("0:", "", 1).split()
        if len(parts) != 7:
            break
        cells, dofs, mv, cgt, cgit, its, red = parts
        rows.append({"line": k, "cells": int(cells), "dofs": int(dofs), "matvec_s": float(mv),
                     "cg_total_s": float(cgt), "cg_its": int(its), "cg_reduction": float(red)})
    out = {"source": LOG, "degree": 4, "rows": rows}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "published_bp5_cg.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path, len(rows), "rows")


if __name__ == "__main__":
    main()
