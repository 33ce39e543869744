"""CPU oracle (test infrastructure only): numpy/ctypes front end of mf_oracle.c.

Only tests/, the smoke check and bench.py's CPU-baseline leg import this module,
always as the checker.  The shipped library never routes through it.

Every function forwards to the C restatement in ``mf_oracle.c``; see the header
of that file for the reference files (dealii-X/benchmarks) each step follows.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

INVALID_DOF = 0xFFFFFFFF


def build() -> str:
    """Compile mf_oracle.c into oracle/libmf_oracle.so (gcc, OpenMP)."""
    subprocess.check_call(["sh", os.path.join(_HERE, "build_oracle.sh")])
    return os.path.join(_HERE, "libmf_oracle.so")


def build_ref() -> str | None:
    """Compile the reference's header-only CPU BK5 + Lagrange basis into
    oracle/_ref (only where the reference sources exist)."""
    subprocess.check_call(["sh", os.path.join(_HERE, "build_ref.sh")])
    path = os.path.join(_HERE, "_ref", "libref_bk5.so")
    return path if os.path.exists(path) else None


class _Box(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("degree", ctypes.c_int),
        ("lo", ctypes.c_double * 3), ("hi", ctypes.c_double * 3),
        ("amplitude", ctypes.c_double), ("geometry_degree", ctypes.c_int),
        ("stride", ctypes.c_int), ("nf", ctypes.c_int * 3),
    ]


class _Ctl(ctypes.Structure):
    _fields_ = [("max_steps", ctypes.c_int), ("tol", ctypes.c_double), ("reduce", ctypes.c_double)]


class _Info(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int), ("initial", ctypes.c_double),
                ("last", ctypes.c_double), ("converged", ctypes.c_int)]


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "libmf_oracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        i64 = ctypes.c_int64
        L.orc_gll.argtypes = [ctypes.c_int, P, P]
        L.orc_gauss.argtypes = [ctypes.c_int, P, P]
        L.orc_lagrange_value.argtypes = [ctypes.c_int, P, ctypes.c_int, ctypes.c_double]
        L.orc_lagrange_value.restype = ctypes.c_double
        L.orc_lagrange_derivative.argtypes = [ctypes.c_int, P, ctypes.c_int, ctypes.c_double]
        L.orc_lagrange_derivative.restype = ctypes.c_double
        L.orc_derivative_matrix.argtypes = [ctypes.c_int, P, P]
        L.orc_interpolation_matrix.argtypes = [ctypes.c_int, P, ctypes.c_int, P, P]
        L.orc_box_n_dofs.argtypes = [ctypes.POINTER(_Box)]
        L.orc_box_n_dofs.restype = i64
        L.orc_box_n_cells.argtypes = [ctypes.POINTER(_Box)]
        L.orc_box_n_cells.restype = i64
        L.orc_box_cell_nodes.argtypes = [ctypes.POINTER(_Box), i64, P]
        L.orc_box_dof_map.argtypes = [ctypes.POINTER(_Box), P, P]
        L.orc_box_dof_map.restype = i64
        L.orc_box_geometry.argtypes = [ctypes.POINTER(_Box), P]
        L.orc_box_geometry.restype = i64
        L.orc_cell_geometry.argtypes = [ctypes.c_int, P, P, P, P]
        L.orc_cell_geometry.restype = ctypes.c_int
        L.orc_bk5_evector.argtypes = [ctypes.c_int, i64, P, P, P, P]
        L.orc_bk3_evector.argtypes = [ctypes.c_int, ctypes.c_int, i64, P, P, P, P, P]
        L.orc_bk1_evector.argtypes = [ctypes.c_int, ctypes.c_int, i64, P, P, P, P]
        L.orc_bk5_apply.argtypes = [ctypes.c_int, i64, P, P, P, i64, i64, P, P, P]
        L.orc_bk5_diagonal.argtypes = [ctypes.c_int, i64, P, P, P, i64, i64, P, P]
        L.orc_invert_diagonal.argtypes = [i64, P]
        L.orc_mt19937_64_nth.argtypes = [ctypes.c_uint64, i64]
        L.orc_mt19937_64_nth.restype = ctypes.c_uint64
        L.orc_rhs_uniform.argtypes = [ctypes.c_uint64, i64, i64, P, P]
        L.orc_cg_solve.argtypes = [ctypes.c_int, i64, P, P, P, i64, i64, P, P, P, P, _Ctl]
        L.orc_cg_solve.restype = _Info
        L.orc_num_threads.restype = ctypes.c_int
        _LIB = L
    return _LIB


def ref_lib():
    """The reference's own CPU BK5 + Lagrange basis, or None where the
    reference sources were not available to build it."""
    global _REF
    if _REF is None:
        path = os.path.join(_HERE, "_ref", "libref_bk5.so")
        if not os.path.exists(path):
            return None
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        L.ref_bk5_serial.argtypes = [ctypes.c_uint, ctypes.c_uint, P, P, P, P]
        L.ref_bk5_serial.restype = ctypes.c_double
        L.ref_bk5_serial_verification_norm.argtypes = [ctypes.c_uint, ctypes.c_uint]
        L.ref_bk5_serial_verification_norm.restype = ctypes.c_double
        L.ref_lagrange_value.argtypes = [ctypes.c_uint, P, ctypes.c_uint, ctypes.c_double]
        L.ref_lagrange_value.restype = ctypes.c_double
        L.ref_lagrange_derivative.argtypes = [ctypes.c_uint, P, ctypes.c_uint, ctypes.c_double]
        L.ref_lagrange_derivative.restype = ctypes.c_double
        L.ref_bk1_serial.argtypes = [ctypes.c_uint, ctypes.c_uint, P, P, P, P]
        L.ref_bk1_serial.restype = ctypes.c_double
        L.ref_bk1_serial_verification_norm.argtypes = [ctypes.c_uint, ctypes.c_uint]
        L.ref_bk1_serial_verification_norm.restype = ctypes.c_double
        L.ref_bk3_serial.argtypes = [ctypes.c_uint, ctypes.c_uint, P, P, P, P, P]
        L.ref_bk3_serial.restype = ctypes.c_double
        L.ref_bk3_serial_verification_norm.argtypes = [ctypes.c_uint, ctypes.c_uint]
        L.ref_bk3_serial_verification_norm.restype = ctypes.c_double
        _REF = L
    return _REF


def _p(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def gll(n: int):
    x = np.zeros(n); w = np.zeros(n)
    lib().orc_gll(n, _p(x), _p(w))
    return x, w


def gauss(n: int):
    x = np.zeros(n); w = np.zeros(n)
    lib().orc_gauss(n, _p(x), _p(w))
    return x, w


def derivative_matrix(nodes: np.ndarray) -> np.ndarray:
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    n = nodes.size
    D = np.zeros((n, n))
    lib().orc_derivative_matrix(n, _p(nodes), _p(D))
    return D


def interpolation_matrix(nodes_from: np.ndarray, pts_to: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(nodes_from, dtype=np.float64)
    b = np.ascontiguousarray(pts_to, dtype=np.float64)
    B = np.zeros((b.size, a.size))
    lib().orc_interpolation_matrix(a.size, _p(a), b.size, _p(b), _p(B))
    return B


@dataclass
class BoxProblem:
    """Structured Q_p box mesh with its map, geometry and constraints (oracle side)."""
    nx: int
    ny: int
    nz: int
    degree: int
    amplitude: float = 0.05
    lo: tuple = (0.0, 0.0, 0.0)
    hi: tuple = (1.0, 1.0, 1.0)
    geometry_degree: int = 0
    stride: int = 1            # > 1: coarsened level of a uniform mesh with nf cells
    nf: tuple = (0, 0, 0)      # per axis (nx = ceil(nf / stride))

    def __post_init__(self):
        if self.stride > 1:
            for n, f in zip((self.nx, self.ny, self.nz), self.nf):
                if n != -(-f // self.stride):
                    raise ValueError("cell counts must be ceil(nf / stride)")
        self._box = _Box(self.nx, self.ny, self.nz, self.degree,
                         (ctypes.c_double * 3)(*self.lo), (ctypes.c_double * 3)(*self.hi),
                         self.amplitude, self.geometry_degree, self.stride,
                         (ctypes.c_int * 3)(*self.nf))
        L = lib()
        self.n = self.degree + 1
        self.n_dofs = int(L.orc_box_n_dofs(ctypes.byref(self._box)))
        self.n_cells = int(L.orc_box_n_cells(ctypes.byref(self._box)))
        nq = self.n ** 3
        self.map = np.zeros(self.n_cells * nq, dtype=np.uint32)
        nc = L.orc_box_dof_map(ctypes.byref(self._box), _p(self.map), None)
        self.constrained = np.zeros(nc, dtype=np.int64)
        L.orc_box_dof_map(ctypes.byref(self._box), None, _p(self.constrained))
        self.G = np.zeros(self.n_cells * 6 * nq)
        self.n_bad_cells = int(L.orc_box_geometry(ctypes.byref(self._box), _p(self.G)))
        x, _ = gll(self.n)
        self.D = derivative_matrix(x)

    def cell_nodes(self, cell: int) -> np.ndarray:
        ng = (self.geometry_degree or self.degree) + 1
        xyz = np.zeros(ng ** 3 * 3)
        lib().orc_box_cell_nodes(ctypes.byref(self._box), cell, _p(xyz))
        return xyz.reshape(-1, 3)

    def apply(self, src: np.ndarray) -> np.ndarray:
        return apply(self.n, self.map, self.D, self.G, self.n_dofs, self.constrained, src)

    def diagonal(self) -> np.ndarray:
        return diagonal(self.n, self.map, self.D, self.G, self.n_dofs, self.constrained)

    def rhs(self, seed: int) -> np.ndarray:
        return rhs_uniform(seed, self.n_dofs, self.constrained)

    def cg(self, b, diag_inv=None, max_steps=100000, tol=1e-300, reduce=1e-8, x0=None):
        return cg_solve(self.n, self.map, self.D, self.G, self.n_dofs, self.constrained,
                        diag_inv, b, max_steps=max_steps, tol=tol, reduce=reduce, x0=x0)


def evector(n: int, D: np.ndarray, G: np.ndarray, u: np.ndarray) -> np.ndarray:
    D = np.ascontiguousarray(D, dtype=np.float64)
    G = np.ascontiguousarray(G, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    nelmt = u.size // n ** 3
    out = np.zeros_like(u)
    lib().orc_bk5_evector(n, nelmt, _p(D), _p(G), _p(u), _p(out))
    return out


def bk3_evector(nm, nq, basis, dbasis, G, u):
    """CEED BK3 E-vector: basis [nq, nm], dbasis [nq, nq], G [e][6][nq^3], u [e][nm^3]."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.zeros_like(u)
    lib().orc_bk3_evector(nm, nq, u.size // nm ** 3, _p(np.ascontiguousarray(basis, dtype=np.float64)),
                          _p(np.ascontiguousarray(dbasis, dtype=np.float64)),
                          _p(np.ascontiguousarray(G, dtype=np.float64)), _p(u), _p(out))
    return out


def bk1_evector(nm, nq, basis, JxW, u):
    """CEED BK1 E-vector mass operator: basis [nq, nm], JxW [e][nq^3], u [e][nm^3]."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    out = np.zeros_like(u)
    lib().orc_bk1_evector(nm, nq, u.size // nm ** 3, _p(np.ascontiguousarray(basis, dtype=np.float64)),
                          _p(np.ascontiguousarray(JxW, dtype=np.float64)), _p(u), _p(out))
    return out


def apply(n, dof_map, D, G, n_dofs, constrained, src):
    src = np.ascontiguousarray(src, dtype=np.float64)
    dst = np.zeros(n_dofs)
    n_cells = dof_map.size // n ** 3
    lib().orc_bk5_apply(n, n_cells, _p(dof_map), _p(np.ascontiguousarray(D)), _p(G), n_dofs,
                        constrained.size, _p(constrained), _p(src), _p(dst))
    return dst


def diagonal(n, dof_map, D, G, n_dofs, constrained):
    d = np.zeros(n_dofs)
    n_cells = dof_map.size // n ** 3
    lib().orc_bk5_diagonal(n, n_cells, _p(dof_map), _p(np.ascontiguousarray(D)), _p(G), n_dofs,
                           constrained.size, _p(constrained), _p(d))
    return d


def invert_diagonal(d: np.ndarray) -> np.ndarray:
    d = np.array(d, dtype=np.float64, copy=True)
    lib().orc_invert_diagonal(d.size, _p(d))
    return d


def mt19937_64_nth(seed: int, nth: int) -> int:
    return int(lib().orc_mt19937_64_nth(seed, nth))


def rhs_uniform(seed, n_dofs, constrained):
    b = np.zeros(n_dofs)
    lib().orc_rhs_uniform(seed, n_dofs, constrained.size, _p(constrained), _p(b))
    return b


def cg_solve(n, dof_map, D, G, n_dofs, constrained, diag_inv, b, max_steps=100000,
             tol=1e-300, reduce=1e-8, x0=None):
    x = np.zeros(n_dofs) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
    b = np.ascontiguousarray(b, dtype=np.float64)
    n_cells = dof_map.size // n ** 3
    info = lib().orc_cg_solve(n, n_cells, _p(dof_map), _p(np.ascontiguousarray(D)), _p(G),
                              n_dofs, constrained.size, _p(constrained),
                              _p(diag_inv) if diag_inv is not None else None,
                              _p(b), _p(x), _Ctl(max_steps, tol, reduce))
    return x, {"steps": info.steps, "initial": info.initial, "last": info.last,
               "converged": bool(info.converged)}


def num_threads() -> int:
    return int(lib().orc_num_threads())


# ---- Gauss-quadrature (BP5-variant / BP3) operator --------------------------
def _gauss_sigs():
    L = lib()
    if getattr(L, "_gauss_ready", False):
        return L
    P, i64 = ctypes.c_void_p, ctypes.c_int64
    L.orc_gauss_basis_matrices.argtypes = [ctypes.c_int, ctypes.c_int, P, P]
    L.orc_box_geometry_gauss.argtypes = [ctypes.POINTER(_Box), ctypes.c_int, P]
    L.orc_box_geometry_gauss.restype = i64
    L.orc_box_rhs_unit_gauss.argtypes = [ctypes.POINTER(_Box), ctypes.c_int, i64, P, P]
    L.orc_bk5g_apply.argtypes = [ctypes.c_int, ctypes.c_int, P, P, i64, P, P, i64, i64, P, P, P]
    L.orc_cg_solve_gauss.argtypes = [ctypes.c_int, ctypes.c_int, P, P, i64, P, P, i64, i64, P, P,
                                     P, P, _Ctl]
    L.orc_cg_solve_gauss.restype = _Info
    L.orc_box_geometry_gauss_jxw.argtypes = [ctypes.POINTER(_Box), ctypes.c_int, P, P]
    L.orc_box_geometry_gauss_jxw.restype = i64
    L.orc_helmholtz_apply.argtypes = [ctypes.c_int, ctypes.c_int, P, P, i64, P, P, P, i64, i64, P,
                                      P, P]
    L.orc_gauss_diagonal.argtypes = [ctypes.c_int, ctypes.c_int, P, P, i64, P, P, P, i64, i64, P, P]
    L.orc_cg_solve_helmholtz.argtypes = [ctypes.c_int, ctypes.c_int, P, P, i64, P, P, P, i64, i64,
                                         P, P, P, P, _Ctl]
    L.orc_cg_solve_helmholtz.restype = _Info
    L._gauss_ready = True
    return L


class GaussProblem(BoxProblem):
    """The box problem discretised with nq Gauss points per direction and
    interpolation from the GLL nodal values (the deal.II-kernel form of the
    reference's BP5 variant, nq = p + 1, or BP3, nq = p + 2)."""

    def __init__(self, nx, ny, nz, degree, nq=None, amplitude=0.0, lo=(0.0, 0.0, 0.0),
                 hi=(1.0, 1.0, 1.0), geometry_degree=0):
        super().__init__(nx, ny, nz, degree, amplitude, lo, hi, geometry_degree)
        L = _gauss_sigs()
        self.nq = nq or degree + 1
        n, q = self.n, self.nq
        self.B = np.zeros((q, n))
        self.DG = np.zeros((q, q))
        L.orc_gauss_basis_matrices(self.degree, q, _p(self.B), _p(self.DG))
        self.Gg = np.zeros(self.n_cells * 6 * q ** 3)
        self.n_bad_cells_gauss = int(L.orc_box_geometry_gauss(ctypes.byref(self._box), q,
                                                              _p(self.Gg)))

    def apply(self, src):
        src = np.ascontiguousarray(src, dtype=np.float64)
        dst = np.zeros(self.n_dofs)
        _gauss_sigs().orc_bk5g_apply(self.n, self.nq, _p(self.B), _p(self.DG), self.n_cells,
                                     _p(self.map), _p(self.Gg), self.n_dofs,
                                     self.constrained.size, _p(self.constrained), _p(src),
                                     _p(dst))
        return dst

    def rhs_unit(self):
        b = np.zeros(self.n_dofs)
        _gauss_sigs().orc_box_rhs_unit_gauss(ctypes.byref(self._box), self.nq,
                                             self.constrained.size, _p(self.constrained), _p(b))
        return b

    def cg(self, b, diag_inv=None, max_steps=1000000000, tol=1e-16, reduce=1e-9, x0=None):
        x = np.zeros(self.n_dofs) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
        b = np.ascontiguousarray(b, dtype=np.float64)
        info = _gauss_sigs().orc_cg_solve_gauss(
            self.n, self.nq, _p(self.B), _p(self.DG), self.n_cells, _p(self.map), _p(self.Gg),
            self.n_dofs, self.constrained.size, _p(self.constrained),
            _p(diag_inv) if diag_inv is not None else None, _p(b), _p(x),
            _Ctl(min(max_steps, 2**31 - 1), tol, reduce))
        return x, {"steps": info.steps, "initial": info.initial, "last": info.last,
                   "converged": bool(info.converged)}


def reference_scaling_mesh(cycle: int, degree: int):
    """The mesh of cycle `cycle` of the reference's BP5-variant scaling study
    (bakeoff_problems_dealii/tests/scaling_bp35_kokkos_kernel/program.cc:451-487):
    n_refine = cycle // 3, the first (cycle % 3) directions span [-1, 2.8] with
    two coarse cells, the others [-1, 0.9] with one, refined n_refine times."""
    n_refine, rem = cycle // 3, cycle % 3
    cells, hi = [], []
    for d in range(3):
        sub = 2 if d < rem else 1
        cells.append(sub << n_refine)
        hi.append(2.8 if d < rem else 0.9)
    return cells, (-1.0, -1.0, -1.0), tuple(hi)


class HelmholtzProblem(GaussProblem):
    """bp5_kokkos's Helmholtz operator (Step64::HelmholtzOperator,
    bp5_kokkos/benchmark.cc:51-251): mass + stiffness at nq = p + 1 Gauss points
    on the GLL nodal values, Dirichlet rows as identity."""

    def __init__(self, nx, ny, nz, degree, amplitude=0.0, lo=(0.0, 0.0, 0.0),
                 hi=(1.0, 1.0, 1.0), geometry_degree=0):
        super().__init__(nx, ny, nz, degree, None, amplitude, lo, hi, geometry_degree)
        q = self.nq
        self.JxW = np.zeros(self.n_cells * q ** 3)
        G2 = np.zeros_like(self.Gg)
        _gauss_sigs().orc_box_geometry_gauss_jxw(ctypes.byref(self._box), q, _p(G2), _p(self.JxW))

    def apply(self, src):
        src = np.ascontiguousarray(src, dtype=np.float64)
        dst = np.zeros(self.n_dofs)
        _gauss_sigs().orc_helmholtz_apply(self.n, self.nq, _p(self.B), _p(self.DG), self.n_cells,
                                          _p(self.map), _p(self.Gg), _p(self.JxW), self.n_dofs,
                                          self.constrained.size, _p(self.constrained), _p(src),
                                          _p(dst))
        return dst

    def diagonal(self):
        d = np.zeros(self.n_dofs)
        _gauss_sigs().orc_gauss_diagonal(self.n, self.nq, _p(self.B), _p(self.DG), self.n_cells,
                                         _p(self.map), _p(self.Gg), _p(self.JxW), self.n_dofs,
                                         self.constrained.size, _p(self.constrained), _p(d))
        return d

    def cg(self, b, diag_inv=None, max_steps=100, tol=1e-15, reduce=1e-8, x0=None):
        """SolverCG + ReductionControl (defaults: bp5_kokkos/benchmark.cc:355)."""
        x = np.zeros(self.n_dofs) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
        b = np.ascontiguousarray(b, dtype=np.float64)
        info = _gauss_sigs().orc_cg_solve_helmholtz(
            self.n, self.nq, _p(self.B), _p(self.DG), self.n_cells, _p(self.map), _p(self.Gg),
            _p(self.JxW), self.n_dofs, self.constrained.size, _p(self.constrained),
            _p(diag_inv) if diag_inv is not None else None, _p(b), _p(x),
            _Ctl(min(max_steps, 2**31 - 1), tol, reduce))
        return x, {"steps": info.steps, "initial": info.initial, "last": info.last,
                   "converged": bool(info.converged)}

