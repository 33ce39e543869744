"""Batched solves (no counterpart in the reference): many independent BP5
problems -- each with its own box mesh, degree, deformation and right-hand
side -- solved together by FP64 CG with per-problem scalars and the FP32
multigrid V-cycle applied to every problem at once (``mfgb_batch_*``).

Vectors are the problems' DoF vectors concatenated in problem order;
``offsets[i]:offsets[i+1]`` is problem i.  ``batch_workload`` draws the
256-problem mix the batched benchmark uses (degree uniform in 2..7, n^3
cells with n uniform in 6..32, amplitude uniform in [0, 0.1], one seed per
problem)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _abi
from ._abi import lib


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def batch_workload(n_problems=256, seed=2024, degrees=(2, 7), cells=(6, 32), amplitude=(0.0, 0.1)):
    """(meshes, rhs seeds) of a seeded random batch."""
    from . import BoxMesh
    g = np.random.default_rng(seed)
    meshes, seeds = [], []
    for _ in range(n_problems):
        p = int(g.integers(degrees[0], degrees[1] + 1))
        n = int(g.integers(cells[0], cells[1] + 1))
        a = float(g.uniform(*amplitude))
        meshes.append(BoxMesh(n, n, n, degree=p, amplitude=a))
        seeds.append(int(g.integers(0, 2**63)))
    return meshes, seeds


class BatchSolver:
    def __init__(self, meshes, chebyshev_degree=5, smoothing_range=15.0, eig_iterations=20,
                 coarse_cells=4):
        self.meshes = list(meshes)
        n = len(self.meshes)
        descs = (_abi.BoxDesc * n)(*[m._desc() for m in self.meshes])
        prm = _abi.MgParams(32, chebyshev_degree, smoothing_range, eig_iterations, coarse_cells,
                            1e-12)
        self._b = ctypes.c_void_p()
        _abi.check(lib().mfgb_batch_create(descs, n, ctypes.byref(prm), ctypes.byref(self._b)))
        nd = ctypes.c_int()
        _abi.check(lib().mfgb_batch_info(self._b, None, None, ctypes.byref(nd), None, None))
        offs = (ctypes.c_int64 * (n + 1))()
        ddofs = (ctypes.c_int64 * nd.value)()
        lev = (ctypes.c_int * n)()
        _abi.check(lib().mfgb_batch_info(self._b, None, offs, None, ddofs, lev))
        self.offsets = np.array(offs[:], dtype=np.int64)
        self.depth_dofs = list(ddofs[:])
        self.levels = list(lev[:])
        self.n_problems = n
        self.n_dofs = int(self.offsets[-1])
        self.infos = []

    def __del__(self):
        b = getattr(self, "_b", None)
        if b is not None and b.value:
            try:
                lib().mfgb_batch_destroy(b)
            except Exception:
                pass
            self._b = None

    def _vec(self, v, name):
        import torch
        if not (isinstance(v, torch.Tensor) and v.is_cuda and v.dtype == torch.float64
                and v.is_contiguous() and v.numel() == self.n_dofs):
            raise ValueError(f"{name}: contiguous float64 CUDA tensor of {self.n_dofs} entries")
        return _ptr(v)

    def initialize_dof_vector(self):
        import torch
        return torch.zeros(self.n_dofs, dtype=torch.float64, device="cuda")

    def split(self, v):
        return [v[self.offsets[i]:self.offsets[i + 1]] for i in range(self.n_problems)]

    def rhs_uniform(self, seeds):
        from . import _stream_ptr
        b = self.initialize_dof_vector()
        s = (ctypes.c_uint64 * self.n_problems)(*[int(x) for x in seeds])
        _abi.check(lib().mfgb_batch_rhs_uniform(self._b, s, _ptr(b), _stream_ptr()))
        return b

    def vmult(self, dst, src):
        from . import _stream_ptr
        _abi.check(lib().mfgb_batch_vmult(self._b, self._vec(dst, "dst"), self._vec(src, "src"),
                                          _stream_ptr()))
        return dst

    def precondition(self, dst, src):
        from . import _stream_ptr
        _abi.check(lib().mfgb_batch_precondition(self._b, self._vec(dst, "dst"),
                                                 self._vec(src, "src"), _stream_ptr()))
        return dst

    def solve(self, x, b, max_steps=200, tol=1e-300, reduce=1e-10):
        """Per-problem SolverCG(ReductionControl(max_steps, tol, reduce)); fills
        ``self.infos`` (steps, initial, last, converged per problem) and raises
        MfgbError (NOT_CONVERGED) if any problem reached max_steps."""
        from . import _stream_ptr
        ctl = _abi.CgControl(int(max_steps), float(tol), float(reduce), 1)
        infos = (_abi.SolveInfo * self.n_problems)()
        st = lib().mfgb_batch_cg_solve(self._b, self._vec(b, "b"), self._vec(x, "x"),
                                       ctypes.byref(ctl), infos, _stream_ptr())
        self.infos = [{"steps": i.steps, "initial": i.initial, "last": i.last,
                       "converged": bool(i.converged)} for i in infos]
        r = ctypes.c_int()
        _abi.check(lib().mfgb_batch_last_solve_stats(self._b, ctypes.byref(r)))
        self.replans = r.value
        _abi.check(lib().mfgb_batch_last_solve_launches(self._b, ctypes.byref(r)))
        self.launches = r.value
        _abi.check(st)
        return x

