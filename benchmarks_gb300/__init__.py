"""GB300-native matrix-free BK5/BP5 Laplacian engine (host side).

Python mirror of the reference's operator/solver interface for this path --
deal.II's ``MatrixType`` concept as used by ``Portable::LaplaceOperatorBK35``
(bakeoff_problems_dealii/include/portable_laplace_operator_bk35.h:16-95) and
``Step64::HelmholtzOperator`` (bp5_kokkos/benchmark.cc:141-175), plus
``SolverCG``/``ReductionControl``/``DiagonalMatrix``/``PreconditionIdentity``
-- over the C ABI of ``libmfgb.so`` (include/mfgb.h).  Vectors are CUDA
``torch.float64`` tensors (PyTorch is only device memory and streams here);
every compute call goes to the CUDA library, and importing the operator
classes without the built library raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

from . import _abi
from ._abi import MfgbError, ARITH_FP64, ARITH_FP64_DF, lib, library_path  # noqa: F401

__all__ = [
    "BoxMesh", "LaplaceOperator", "ReductionControl", "SolverCG", "DiagonalMatrix",
    "PreconditionIdentity", "MGPreconditioner", "MfgbError", "ARITH_FP64", "ARITH_FP64_DF", "lib", "library_path",
    "bk5_evector", "bk5_lvector", "bk1_evector", "bk3_evector", "dot", "HelmholtzOperator",
    "BatchSolver", "batch_workload",
]

_ARITH = {"fp64": ARITH_FP64, "df": ARITH_FP64_DF, "fp64_df": ARITH_FP64_DF,
          "tc": _abi.ARITH_FP64_TC, "fp64_tc": _abi.ARITH_FP64_TC,
          ARITH_FP64: ARITH_FP64, ARITH_FP64_DF: ARITH_FP64_DF,
          _abi.ARITH_FP64_TC: _abi.ARITH_FP64_TC}


def _arith(a) -> int:
    try:
        return _ARITH[a]
    except KeyError:
        raise ValueError(f"unknown arithmetic mode {a!r}") from None


def _torch():
    import torch
    return torch


def _stream_ptr():
    torch = _torch()
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _check_vec(v, n, name):
    torch = _torch()
    if not isinstance(v, torch.Tensor) or v.dtype != torch.float64 or not v.is_cuda:
        raise TypeError(f"{name} must be a CUDA float64 tensor")
    if v.numel() != n or not v.is_contiguous():
        raise ValueError(f"{name} must be contiguous with {n} entries")
    return ctypes.c_void_p(v.data_ptr())


@dataclass(frozen=True)
class BoxMesh:
    """Structured hex mesh of the unit cube (or a box): nx*ny*nz cells of
    degree p, GLL nodes moved by x_d += a sin(2 pi x) sin(2 pi y) sin(2 pi z),
    Dirichlet u = 0 on the boundary."""
    nx: int
    ny: int
    nz: int
    degree: int
    amplitude: float = 0.05
    lo: tuple = (0.0, 0.0, 0.0)
    hi: tuple = (1.0, 1.0, 1.0)
    geometry_degree: int = 0

    @property
    def n_dofs(self) -> int:
        p = self.degree
        return (p * self.nx + 1) * (p * self.ny + 1) * (p * self.nz + 1)

    @property
    def n_cells(self) -> int:
        return self.nx * self.ny * self.nz

    def _desc(self):
        return _abi.BoxDesc(self.nx, self.ny, self.nz, self.degree,
                            (ctypes.c_double * 3)(*self.lo), (ctypes.c_double * 3)(*self.hi),
                            self.amplitude, self.geometry_degree)


class LaplaceOperator:
    """BK5 Laplacian on Q_p hexahedra with GLL collocation (the
    ``LaplaceOperatorBK35`` interface): ``vmult``, ``Tvmult``, ``m``, ``n``,
    ``initialize_dof_vector``, ``compute_diagonal``,
    ``get_matrix_diagonal_inverse``.

    ``arith`` selects the arithmetic inside the kernels: ``"fp64"`` (native
    DFMA) or ``"df"`` (FP64-accurate double-float on the FP32 pipes, the
    default; both meet 1e-12 relative to the FP64 oracle)."""

    def __init__(self, mesh: BoxMesh | None = None, *, degree=None, n_dofs=None, dof_map=None,
                 G=None, constrained=None, arith="df", quadrature="gll"):
        L = lib()
        self._op = ctypes.c_void_p()
        if quadrature not in ("gll", "gauss", "helmholtz", "bp3"):
            raise ValueError("quadrature must be 'gll' (collocation), 'gauss' (BP5 variant, q = p+1), "
                             "'helmholtz' (mass + stiffness at the Gauss points) or 'bp3' (q = p+2)")
        self.quadrature = quadrature
        if mesh is not None:
            desc = mesh._desc()
            create = {"gll": L.mfgb_operator_create_box, "gauss": L.mfgb_operator_create_box_gauss,
                      "helmholtz": L.mfgb_operator_create_box_helmholtz,
                      "bp3": L.mfgb_operator_create_box_bp3}[quadrature]
            _abi.check(create(ctypes.byref(desc), ctypes.byref(self._op)))
            self.mesh = mesh
        else:
            import numpy as np
            dof_map = np.ascontiguousarray(dof_map, dtype=np.uint32)
            G = np.ascontiguousarray(G, dtype=np.float64)
            constrained = np.ascontiguousarray(
                constrained if constrained is not None else np.zeros(0), dtype=np.int64)
            n3 = (degree + 1) ** 3
            n_cells = dof_map.size // n3
            _abi.check(L.mfgb_operator_create(
                int(degree), int(n_dofs), int(n_cells),
                dof_map.ctypes.data_as(ctypes.c_void_p), G.ctypes.data_as(ctypes.c_void_p),
                int(constrained.size), constrained.ctypes.data_as(ctypes.c_void_p),
                ctypes.byref(self._op)))
            self.mesh = None
        nd, nc, dg, ncons = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int(), ctypes.c_int64()
        _abi.check(L.mfgb_operator_info(self._op, ctypes.byref(nd), ctypes.byref(nc),
                                        ctypes.byref(dg), ctypes.byref(ncons)))
        self._n_dofs, self.n_cells, self.degree, self.n_constrained = (
            nd.value, nc.value, dg.value, ncons.value)
        self.arith = _arith(arith)
        self._inv_diag = None

    def __del__(self):
        op = getattr(self, "_op", None)
        if op is not None and op.value:
            try:
                lib().mfgb_operator_destroy(op)
            except Exception:
                pass
            self._op = None

    # deal.II MatrixType concept ------------------------------------------
    def m(self) -> int:
        return self._n_dofs

    def n(self) -> int:
        return self._n_dofs

    def initialize_dof_vector(self, vec=None):
        torch = _torch()
        return torch.zeros(self._n_dofs, dtype=torch.float64, device="cuda")

    def vmult(self, dst, src, arith=None):
        a = self.arith if arith is None else _arith(arith)
        _abi.check(lib().mfgb_vmult(self._op, _check_vec(dst, self._n_dofs, "dst"),
                                    _check_vec(src, self._n_dofs, "src"), a, _stream_ptr()))
        return dst

    def vmult_vector(self, dst, src, arith=None):
        """BK6: the operator on 3 interleaved components (length 3 n)."""
        a = self.arith if arith is None else _arith(arith)
        _abi.check(lib().mfgb_vmult_vector(self._op, _check_vec(dst, 3 * self._n_dofs, "dst"),
                                           _check_vec(src, 3 * self._n_dofs, "src"), 3, a,
                                           _stream_ptr()))
        return dst

    def Tvmult(self, dst, src, arith=None):
        # the operator is symmetric (portable_laplace_operator_bk35.h:386-400)
        return self.vmult(dst, src, arith)

    def compute_diagonal(self):
        d = self.initialize_dof_vector()
        L = lib()
        _abi.check(L.mfgb_compute_diagonal(self._op, _check_vec(d, self._n_dofs, "diag"),
                                           _stream_ptr()))
        inv = d.clone()
        _abi.check(L.mfgb_invert_diagonal(self._n_dofs, _check_vec(inv, self._n_dofs, "diag"),
                                          _stream_ptr()))
        self._diag = d
        self._inv_diag = DiagonalMatrix(inv)
        return d

    def vmult_dummy(self, dst, src, ghost_exchange_on=True, computation_on=True):
        """``vmult_dummy`` of the reference operator (portable_laplace_operator_bk35.h:
        170-225): ``computation_on`` runs dst = 0 and the cell loop,
        ``ghost_exchange_on`` the identity rows (the exchange itself is a no-op on
        one GPU)."""
        n = self._n_dofs
        if computation_on:
            dst.zero_()
            _abi.check(lib().mfgb_vmult_add(self._op, _check_vec(dst, n, "dst"),
                                            _check_vec(src, n, "src"), self.arith, _stream_ptr()))
        if ghost_exchange_on:
            _abi.check(lib().mfgb_copy_constrained(self._op, _check_vec(dst, n, "dst"),
                                                   _check_vec(src, n, "src"), _stream_ptr()))
        return dst

    def vmult_host(self, dst, src, arith=None):
        """dst = A src on host (CPU, ideally pinned) float64 tensors; the copies
        are pipelined with the apply (``mfgb_vmult_host``)."""
        for v, name in ((dst, "dst"), (src, "src")):
            if v.is_cuda or v.dtype != _torch().float64 or not v.is_contiguous() or \
                    v.numel() != self._n_dofs:
                raise ValueError(f"{name}: contiguous float64 host tensor of {self._n_dofs} entries")
        _abi.check(lib().mfgb_vmult_host(self._op, ctypes.c_void_p(dst.data_ptr()),
                                         ctypes.c_void_p(src.data_ptr()),
                                         self.arith if arith is None else _arith(arith),
                                         _stream_ptr()))
        return dst

    def get_matrix_diagonal_inverse(self):
        if self._inv_diag is None:
            self.compute_diagonal()
        return self._inv_diag

    def el(self, row, col):
        if row != col:
            raise NotImplementedError("only diagonal entries are available")
        if self._inv_diag is None:
            self.compute_diagonal()
        return float(self._diag[row])

    # extras --------------------------------------------------------------
    def rhs_uniform(self, seed: int):
        b = self.initialize_dof_vector()
        _abi.check(lib().mfgb_rhs_uniform(self._op, ctypes.c_uint64(seed),
                                          _check_vec(b, self._n_dofs, "b"), _stream_ptr()))
        return b

    def export(self):
        """(dof_map, G, constrained) copied to numpy arrays."""
        import numpy as np
        n3 = (self.degree + 1) ** 3
        dof_map = np.zeros(self.n_cells * n3, dtype=np.uint32)
        G = np.zeros(self.n_cells * 6 * n3)
        cons = np.zeros(self.n_constrained, dtype=np.int64)
        _abi.check(lib().mfgb_operator_export(self._op, dof_map.ctypes.data_as(ctypes.c_void_p),
                                              G.ctypes.data_as(ctypes.c_void_p),
                                              cons.ctypes.data_as(ctypes.c_void_p)))
        return dof_map, G, cons

    @property
    def handle(self):
        return self._op


class HelmholtzOperator(LaplaceOperator):
    """``Step64::HelmholtzOperator`` of bp5_kokkos (benchmark.cc:141-251): mass
    plus stiffness at QGauss(p+1) on the GLL nodal values, with the same
    ``vmult`` / ``initialize_dof_vector`` / ``compute_diagonal`` /
    ``get_matrix_diagonal_inverse`` interface."""

    def __init__(self, mesh: BoxMesh, arith="df"):
        super().__init__(mesh, arith=arith, quadrature="helmholtz")


class DiagonalMatrix:
    """deal.II DiagonalMatrix: holds the vector it multiplies with."""

    def __init__(self, vector):
        self.vector = vector

    def get_vector(self):
        return self.vector

    def vmult(self, dst, src):
        dst.copy_(self.vector * src)
        return dst


class PreconditionIdentity:
    def vmult(self, dst, src):
        dst.copy_(src)
        return dst


class MGPreconditioner:
    """Geometric p-/h-multigrid V-cycle for a box mesh (mfgb_mg_* in the C ABI):
    p_fine -> p_fine/2 -> ... -> 1, then Q1 on coarsened meshes (level l keeps
    the fine nodes min(k 2^l, n) of each axis, nested for any n); Chebyshev
    smoothing around Jacobi; FP64 Jacobi-CG coarse solve.  ``precision`` 32
    runs the V-cycle in FP32 (the mixed-precision preconditioner inside FP64
    CG), 64 in FP64."""

    def __init__(self, mesh: BoxMesh, precision=32, chebyshev_degree=5, smoothing_range=15.0,
                 eig_iterations=20, coarse_cells=4, coarse_tol=1e-12, operator=None):
        """``operator``: the LaplaceOperator of the same mesh; the finest level then
        borrows it (no second geometry set-up) and keeps a reference to it."""
        self.mesh = mesh
        self.precision = precision
        self._mg = ctypes.c_void_p()
        prm = _abi.MgParams(precision, chebyshev_degree, smoothing_range, eig_iterations,
                            coarse_cells, coarse_tol)
        if operator is not None:
            if operator.mesh is None or operator.mesh != mesh or operator.quadrature != "gll":
                raise ValueError("operator must be the GLL LaplaceOperator of the same mesh")
            self._operator = operator  # outlives the hierarchy
            _abi.check(lib().mfgb_mg_setup_shared(operator.handle, ctypes.byref(prm),
                                                  ctypes.byref(self._mg)))
        else:
            desc = mesh._desc()
            _abi.check(lib().mfgb_mg_setup(ctypes.byref(desc), ctypes.byref(prm),
                                           ctypes.byref(self._mg)))
        nl = ctypes.c_int()
        _abi.check(lib().mfgb_mg_info(self._mg, ctypes.byref(nl), None, None, None))
        dofs = (ctypes.c_int64 * nl.value)()
        deg = (ctypes.c_int * nl.value)()
        lmax = (ctypes.c_double * nl.value)()
        _abi.check(lib().mfgb_mg_info(self._mg, None, dofs, deg, lmax))
        self.levels = [{"dofs": dofs[i], "degree": deg[i], "lambda_max": lmax[i]}
                       for i in range(nl.value)]

    def __del__(self):
        mg = getattr(self, "_mg", None)
        if mg is not None and mg.value:
            try:
                lib().mfgb_mg_destroy(mg)
            except Exception:
                pass
            self._mg = None

    def vmult(self, dst, src):
        n = self.levels[0]["dofs"]
        _abi.check(lib().mfgb_mg_vmult(self._mg, _check_vec(dst, n, "dst"),
                                       _check_vec(src, n, "src"), _stream_ptr()))
        return dst

    @property
    def handle(self):
        return self._mg


class ReductionControl:
    """deal.II ReductionControl(max_steps, tol, reduce)."""

    def __init__(self, max_steps=100, tol=1e-10, reduce=1e-2):
        self.max_steps, self.tol, self.reduce = int(max_steps), float(tol), float(reduce)
        self._last_step = 0
        self._initial = self._last = 0.0

    def last_step(self):
        return self._last_step

    def initial_value(self):
        return self._initial

    def last_value(self):
        return self._last


class SolverCG:
    """deal.II SolverCG; ``solve(A, x, b, P)`` runs on the device through
    ``mfgb_cg_solve`` and raises ``MfgbError`` (status NOT_CONVERGED) like
    deal.II's ``SolverControl::NoConvergence`` when max_steps is reached."""

    def __init__(self, control: ReductionControl):
        self.control = control

    def solve(self, A: LaplaceOperator, x, b, preconditioner=None, arith=None):
        ctl = _abi.CgControl(self.control.max_steps, self.control.tol, self.control.reduce,
                             A.arith if arith is None else _arith(arith))
        info = _abi.SolveInfo()
        inv = None
        if isinstance(preconditioner, MGPreconditioner):
            st = lib().mfgb_mg_cg_solve(A.handle, preconditioner.handle,
                                        _check_vec(b, A.n(), "b"), _check_vec(x, A.n(), "x"),
                                        ctypes.byref(ctl), ctypes.byref(info), _stream_ptr())
            self.control._last_step = info.steps
            self.control._initial = info.initial
            self.control._last = info.last
            _abi.check(st)
            return x
        if isinstance(preconditioner, DiagonalMatrix):
            inv = _check_vec(preconditioner.vector, A.n(), "preconditioner")
        elif preconditioner is not None and not isinstance(preconditioner, PreconditionIdentity):
            raise TypeError("preconditioner must be PreconditionIdentity or DiagonalMatrix")
        st = lib().mfgb_cg_solve(A.handle, _check_vec(b, A.n(), "b"), _check_vec(x, A.n(), "x"),
                                 inv, ctypes.byref(ctl), ctypes.byref(info), _stream_ptr())
        self.control._last_step = info.steps
        self.control._initial = info.initial
        self.control._last = info.last
        _abi.check(st)
        return x


def bk5_evector(degree, dbasis, G, u, out, arith="fp64"):
    """E-vector kernel seam (CEED_BK BK5::Parallel::LaplaceOperator)."""
    n3 = (degree + 1) ** 3
    nelmt = u.numel() // n3
    _abi.check(lib().mfgb_bk5_evector(
        int(degree), nelmt, ctypes.c_void_p(dbasis.data_ptr()), ctypes.c_void_p(G.data_ptr()),
        ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(out.data_ptr()), _arith(arith),
        _stream_ptr()))
    return out


def bk1_evector(degree, basis, JxW, u, out, arith="fp64"):
    """E-vector seam of the CEED BK1 mass operator (BK1::Parallel::MassOperator),
    nq = degree + 2 points: basis [nq * nm], JxW [e][nq^3], u/out [e][nm^3].
    arith "fp64", "df", or "tc" (FP64 tensor cores, degree 1..6)."""
    nm3 = (degree + 1) ** 3
    _abi.check(lib().mfgb_bk1_evector(
        int(degree), u.numel() // nm3, ctypes.c_void_p(basis.data_ptr()),
        ctypes.c_void_p(JxW.data_ptr()), ctypes.c_void_p(u.data_ptr()),
        ctypes.c_void_p(out.data_ptr()), _arith(arith), _stream_ptr()))
    return out


def bk3_evector(degree, basis, dbasis, G, u, out, arith="fp64"):
    """E-vector seam of the CEED BK3 Laplacian (BK3::Parallel::LaplaceOperator),
    nq = degree + 2 points: basis [nq * nm], dbasis [nq * nq], G [e][6][nq^3],
    u/out [e][nm^3]."""
    nm3 = (degree + 1) ** 3
    _abi.check(lib().mfgb_bk3_evector(
        int(degree), u.numel() // nm3, ctypes.c_void_p(basis.data_ptr()),
        ctypes.c_void_p(dbasis.data_ptr()), ctypes.c_void_p(G.data_ptr()),
        ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(out.data_ptr()), _arith(arith),
        _stream_ptr()))
    return out


def bk5_lvector(degree, dbasis, G, src, dst, dof_indices, arith="fp64"):
    """L-vector kernel seam (BK3::Parallel::KokkosKernel_1D_Block, GLL form):
    accumulates into dst."""
    n3 = (degree + 1) ** 3
    n_cells = dof_indices.numel() // n3
    _abi.check(lib().mfgb_bk5_lvector(
        int(degree), n_cells, ctypes.c_void_p(dbasis.data_ptr()), ctypes.c_void_p(G.data_ptr()),
        ctypes.c_void_p(src.data_ptr()), ctypes.c_void_p(dst.data_ptr()),
        ctypes.c_void_p(dof_indices.data_ptr()), _arith(arith), _stream_ptr()))
    return dst


def dot(a, b) -> float:
    r = ctypes.c_double()
    _abi.check(lib().mfgb_dot(a.numel(), ctypes.c_void_p(a.data_ptr()),
                              ctypes.c_void_p(b.data_ptr()), ctypes.byref(r), _stream_ptr()))
    return r.value


from .batch import BatchSolver, batch_workload  # noqa: E402


def check_device_errors():
    """Reads and clears the device error word on the current stream
    (mfgb_check_device_errors): raises MfgbError with status TIMEOUT if a kernel
    gave up on a bulk-copy wait since the last check."""
    _abi.check(lib().mfgb_check_device_errors(_stream_ptr()))
