"""Generates tests/golden/reference_bk5.json from the reference's own CPU code
(compiled from the reference sources into oracle/_ref by oracle/build_ref.sh).

Contents:
  verification_norms  -- the norm printed by CEED_BK/src/BK5/serial_verification.cc
                         (G = 2, in = 3, dbasis = cos(i*nq+a), nelmt = 1000), p = 1..8
  random_cases        -- BK5::Serial::SumFactorization<double> on seeded random
                         dbasis / in and a random per-point metric g(q) copied into
                         all six G components (the reference serial kernel reads
                         every component at offset 0, CEED_BK/include/kernels/BK5/
                         serial_kernels.hpp:28-33, so only such inputs give the
                         mathematically intended result), nelmt = 2, p = 1..8
  lagrange_D          -- LagrangeBasis<double>::derivative at the GLL points
                         (sum_factorization/include/math/lagrange_basis.hpp:44-65)

Run: python tests/golden/make_golden.py   (needs the reference checkout)
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle  # noqa: E402


def main():
    oracle.build_ref()
    R = oracle.ref_lib()
    assert R is not None, "reference sources are needed to generate the golden file"
    out = {"verification_norms": {}, "random_cases": {}, "lagrange_D": {}}
    for p in range(1, 9):
        out["verification_norms"][str(p)] = R.ref_bk5_serial_verification_norm(p, 1000)
    rng = np.random.default_rng(20251203)
    for p in range(1, 9):
        nq = p + 1
        nt = nq ** 3
        nelmt = 2
        dbasis = rng.uniform(-1, 1, nq * nq)
        g = rng.uniform(0.5, 2.0, nelmt * nt)
        G = np.repeat(g.reshape(nelmt, 1, nt), 6, axis=1).reshape(-1).copy()
        u = rng.uniform(-1, 1, nelmt * nt)
        y = np.zeros(nelmt * nt)
        R.ref_bk5_serial(nq, nelmt, oracle._p(dbasis), oracle._p(G), oracle._p(u), oracle._p(y))
        out["random_cases"][str(p)] = {"dbasis": dbasis.tolist(), "g": g.tolist(),
                                       "in": u.tolist(), "out": y.tolist()}
        x, _ = oracle.gll(nq)
        D = [[R.ref_lagrange_derivative(nq, oracle._p(x), b, float(x[q])) for b in range(nq)]
             for q in range(nq)]
        out["lagrange_D"][str(p)] = {"nodes": x.tolist(), "D": D}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_bk5.json")
    with open(path, "w") as f:
        json.dump(out, f)
    print("wrote", path, os.path.getsize(path), "bytes")
    bk13()


def bk13():
    """tests/golden/reference_bk1_bk3.json from the reference's serial BK1 and BK3
    (CEED_BK/include/kernels/BK{1,3}/serial_kernels.hpp), nq = p + 2, nm = p + 1:
      bk1_norms / bk3_norms -- the serial_verification norms (nelmt = 1000), p = 1..8
      bk1_cases / bk3_cases -- seeded random basis, dbasis, JxW or all six G
                               components, in; nelmt = 1.  G is stored here as
                               [e][6][nq^3] (the CUDA kernel's layout); the serial
                               kernel reads [e][p][q][6][r], so it is reordered for it."""
    R = oracle.ref_lib()
    out = {"bk1_norms": {}, "bk3_norms": {}, "bk1_cases": {}, "bk3_cases": {}}
    for p in range(1, 9):
        out["bk1_norms"][str(p)] = R.ref_bk1_serial_verification_norm(p, 1000)
        out["bk3_norms"][str(p)] = R.ref_bk3_serial_verification_norm(p, 1000)
    rng = np.random.default_rng(20251204)
    for p in range(1, 9):
        nq, nm, nelmt = p + 2, p + 1, 1
        nq3, nm3 = nq ** 3, nm ** 3
        basis = rng.uniform(-1, 1, nq * nm)
        dbasis = rng.uniform(-1, 1, nq * nq)
        jxw = rng.uniform(0.5, 2.0, nelmt * nq3)
        G = rng.uniform(-1, 1, (nelmt, 6, nq3))
        G[:, 0] += 3.0
        G[:, 3] += 3.0
        G[:, 5] += 3.0
        u = rng.uniform(-1, 1, nelmt * nm3)
        y1 = np.zeros(nelmt * nm3)
        R.ref_bk1_serial(nq, nelmt, oracle._p(basis), oracle._p(jxw), oracle._p(u), oracle._p(y1))
        # serial layout [e][p][q][6][r] from [e][6][(p q r)]
        Gs = np.ascontiguousarray(G.reshape(nelmt, 6, nq, nq, nq).transpose(0, 2, 3, 1, 4))
        y3 = np.zeros(nelmt * nm3)
        R.ref_bk3_serial(nq, nelmt, oracle._p(basis), oracle._p(dbasis), oracle._p(Gs),
                         oracle._p(u), oracle._p(y3))
        out["bk1_cases"][str(p)] = {"basis": basis.tolist(), "JxW": jxw.tolist(), "in": u.tolist(),
                                    "out": y1.tolist()}
        out["bk3_cases"][str(p)] = {"basis": basis.tolist(), "dbasis": dbasis.tolist(),
                                    "G": G.reshape(-1).tolist(), "in": u.tolist(), "out": y3.tolist()}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_bk1_bk3.json")
    with open(path, "w") as f:
        json.dump(out, f)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
