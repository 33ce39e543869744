"""CPU oracle (test infrastructure only) for the geometric multigrid
preconditioner: the same hierarchy, transfers, Chebyshev smoother and V-cycle
as the CUDA library, in FP64 numpy over the C oracle's operator.

The reference has no multigrid for this path, so this oracle restates the
standard algorithms the library implements (parity unpinned by the
reference):
  * levels: p -> p//2 -> ... -> 1 on the fine mesh, then Q1 on coarsened
    meshes while the largest cell count exceeds coarse_cells: level l keeps
    the fine nodes min(k 2^l, n) of each axis (ceil(n / 2^l) cells, nested for
    any n; only the last cell of an axis can be narrower); every level keeps
    the fine degree's geometry interpolant
  * p-transfer: cell-wise tensor-product Lagrange interpolation at the fine
    GLL points; restriction = transpose with 1/valence weighting of fine DoFs
  * h-transfer: Q1 interpolation on nested structured grids
  * Chebyshev (Saad, Iterative Methods for Sparse Linear Systems, alg. 12.1)
    around Jacobi on [lmax/range, lmax], lmax = 1.2 x power-iteration estimate
  * coarse: exact solve on the interior DoFs (the library converges a Jacobi-CG
    to 1e-12 relative, which agrees to that tolerance)
"""
from __future__ import annotations

import numpy as np

from . import oracle as orc


def _power_start(n: int) -> np.ndarray:
    """The deterministic start vector the library uses: entry i is 0.5 + the top
    53 bits of SplitMix64 (Steele, Lea, Flood 2014) of the state (i + 1) * golden
    as a fraction of 2^53 (power_start_value, mfgb_mg_kernels.cuh)."""
    z = np.arange(1, n + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = z * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    z = z ^ (z >> np.uint64(31))
    return 0.5 + (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


class Level:
    def __init__(self, nx, ny, nz, degree, amplitude, geometry_degree=0, stride=1,
                 nf=(0, 0, 0)):
        self.box = (nx, ny, nz)
        self.degree = degree
        self.stride, self.nf = stride, nf
        self.prob = orc.BoxProblem(nx, ny, nz, degree, amplitude=amplitude,
                                   geometry_degree=geometry_degree, stride=stride, nf=nf)
        self.n = self.prob.n_dofs
        d = self.prob.diagonal()
        self.dinv = orc.invert_diagonal(d)
        self.constrained = self.prob.constrained
        self.lmax = None
        self.to_coarse = 0

    def apply(self, x):
        return self.prob.apply(x)


class MGOracle:
    def __init__(self, nx, ny, nz, degree, amplitude=0.05, chebyshev_degree=5,
                 smoothing_range=15.0, eig_iterations=20, coarse_cells=4):
        self.k = chebyshev_degree
        self.range = smoothing_range
        nf = (nx, ny, nz)
        boxes, kinds = [(nx, ny, nz, degree, 1)], []
        p = degree
        while p > 1:
            p = max(1, p // 2)
            boxes.append((nx, ny, nz, p, 1))
            kinds.append(1)
        s = 2
        while max(nx, ny, nz) > coarse_cells:
            nx, ny, nz = (-(-f // s) for f in nf)
            boxes.append((nx, ny, nz, 1, s))
            kinds.append(2)
            s *= 2
        kinds.append(0)
        self.nf = nf
        self.levels = []
        for (bx, by, bz, bp, bs), kind in zip(boxes, kinds):
            L = Level(bx, by, bz, bp, amplitude, geometry_degree=degree, stride=bs,
                      nf=nf if bs > 1 else (0, 0, 0))
            L.to_coarse = kind
            self.levels.append(L)
        for L in self.levels[:-1]:
            L.lmax = 1.2 * self._lmax(L, eig_iterations)
        for L, C in zip(self.levels[:-1], self.levels[1:]):
            if L.to_coarse == 1:
                xf, _ = orc.gll(L.degree + 1)
                xc, _ = orc.gll(C.degree + 1)
                L.B = orc.interpolation_matrix(xc, xf)  # [fine pt, coarse basis]
                val = np.zeros(L.n)
                np.add.at(val, L.prob.map[L.prob.map != orc.INVALID_DOF].astype(np.int64), 1.0)
                L.inv_val = np.where(val > 0, 1.0 / np.maximum(val, 1e-300), 0.0)
        C = self.levels[-1]
        free = np.setdiff1d(np.arange(C.n), C.constrained)
        A = np.zeros((free.size, free.size))
        for j, dof in enumerate(free):
            e = np.zeros(C.n)
            e[dof] = 1.0
            A[:, j] = C.apply(e)[free]
        self.coarse_free, self.coarse_A = free, A

    @staticmethod
    def _lmax(L, iters):
        v = _power_start(L.n)
        v[L.constrained] = 0.0
        lam = 0.0
        for _ in range(iters):
            v = v / np.sqrt(v @ v)
            w = L.apply(v)
            w[L.constrained] = 0.0
            w = w * L.dinv
            lam = v @ w
            v = w
        return lam

    # ---- transfers -------------------------------------------------------
    @staticmethod
    def _cells_view(L, vec):
        n = L.degree + 1
        m = L.prob.map.reshape(-1, n, n, n)
        valid = m != orc.INVALID_DOF
        vals = np.where(valid, vec[np.where(valid, m, 0).astype(np.int64)], 0.0)
        return m, valid, vals

    def p_prolongate(self, L, C, xc):
        _, _, cv = self._cells_view(C, xc)
        B = L.B
        fine = np.einsum("ia,jb,kc,eabc->eijk", B, B, B, cv)
        n = L.degree + 1
        m = L.prob.map.reshape(-1, n, n, n)
        t = np.zeros(L.n)
        valid = m != orc.INVALID_DOF
        t[m[valid].astype(np.int64)] = fine[valid]
        return t

    def p_restrict(self, L, C, rf):
        _, _, fv = self._cells_view(L, rf * L.inv_val)
        B = L.B
        coarse = np.einsum("ia,jb,kc,eijk->eabc", B, B, B, fv)
        n = C.degree + 1
        m = C.prob.map.reshape(-1, n, n, n)
        rc = np.zeros(C.n)
        valid = m != orc.INVALID_DOF
        np.add.at(rc, m[valid].astype(np.int64), coarse[valid])
        return rc

    @staticmethod
    def _h_matrix_1d(nf, s):
        """Q1 interpolation on one axis from the level of stride 2s to the level
        of stride s: [fine nodes, coarse nodes]; node k of a level sits at fine
        mesh node min(k stride, nf)."""
        m = -(-nf // s)
        mc = -(-nf // (2 * s))
        P = np.zeros((m + 1, mc + 1))
        for I in range(m + 1):
            if I % 2 == 0:
                P[I, I // 2] = 1.0
            else:
                A, pos, B = (I - 1) * s, min(I * s, nf), min((I + 1) * s, nf)
                w = (pos - A) / (B - A)
                P[I, I // 2] = 1.0 - w
                P[I, I // 2 + 1] = w
        return P

    def _h_mats(self, L):
        return [self._h_matrix_1d(f, L.stride) for f in self.nf]

    def h_prolongate_add(self, L, C, xc, xf):
        cx, cy, cz = C.box
        Px, Py, Pz = self._h_mats(L)
        X = xc.reshape(cz + 1, cy + 1, cx + 1)
        F = np.einsum("Kk,Jj,Ii,kji->KJI", Pz, Py, Px, X).reshape(-1)
        mask = np.ones(L.n, bool)
        mask[L.constrained] = False
        return xf + np.where(mask, F, 0.0)

    def h_restrict(self, L, C, rf):
        fx, fy, fz = L.box
        Px, Py, Pz = self._h_mats(L)
        R = rf.reshape(fz + 1, fy + 1, fx + 1)
        rc = np.einsum("Kk,Jj,Ii,KJI->kji", Pz, Py, Px, R).reshape(-1)
        rc[C.constrained] = 0.0
        return rc

    # ---- smoother / cycle -----------------------------------------------
    def chebyshev(self, L, b, x=None):
        lmax, lmin = L.lmax, L.lmax / self.range
        theta, delta = 0.5 * (lmax + lmin), 0.5 * (lmax - lmin)
        sigma = theta / delta
        rho = 1.0 / sigma
        if x is None:
            r = b.copy()
            d = (1.0 / theta) * L.dinv * r
            x = d.copy()
        else:
            r = b - L.apply(x)
            d = (1.0 / theta) * L.dinv * r
            x = x + d
        for _ in range(1, self.k):
            r = r - L.apply(d)
            rho_new = 1.0 / (2.0 * sigma - rho)
            d = rho_new * rho * d + (2.0 * rho_new / delta) * L.dinv * r
            x = x + d
            rho = rho_new
        return x

    def vcycle(self, b, l=0):
        L = self.levels[l]
        if l + 1 == len(self.levels):
            x = np.zeros(L.n)
            if self.coarse_free.size:
                x[self.coarse_free] = np.linalg.solve(self.coarse_A, b[self.coarse_free])
            return x
        C = self.levels[l + 1]
        x = self.chebyshev(L, b)
        r = b - L.apply(x)
        bc = self.p_restrict(L, C, r) if L.to_coarse == 1 else self.h_restrict(L, C, r)
        xc = self.vcycle(bc, l + 1)
        if L.to_coarse == 1:
            x = x + self.p_prolongate(L, C, xc)
        else:
            x = self.h_prolongate_add(L, C, xc, x)
        return self.chebyshev(L, b, x)

    def pcg(self, b, reduce=1e-10, tol=1e-300, max_steps=1000):
        """FP64 CG preconditioned by the V-cycle (deal.II SolverCG semantics)."""
        L = self.levels[0]
        x = np.zeros(L.n)
        r = b - L.apply(x)
        res0 = np.sqrt(r @ r)
        tol_eff = max(tol, reduce * res0)
        info = {"initial": res0, "steps": 0, "last": res0, "converged": res0 <= tol_eff}
        if info["converged"]:
            return x, info
        z = self.vcycle(r)
        p = z.copy()
        rz = r @ z
        for it in range(1, max_steps + 1):
            v = L.apply(p)
            alpha = rz / (p @ v)
            x += alpha * p
            r -= alpha * v
            res = np.sqrt(r @ r)
            info.update(steps=it, last=res)
            if res <= tol_eff:
                info["converged"] = True
                break
            z = self.vcycle(r)
            rz_new = r @ z
            p = z + (rz_new / rz) * p
            rz = rz_new
        return x, info
