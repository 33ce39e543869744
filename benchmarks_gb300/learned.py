"""Learned smoother weights for the multigrid V-cycle (no counterpart in the
reference).

A 73-64-64-1 MLP maps a cell's corner Jacobians and degree to
lambda_e ~ lambda_max(D_e^-1 A_e).  The finest-level Chebyshev smoother then
uses the positive diagonal D~ = sum_e lambda_e^alpha D_e
(``mfgb_mg_set_smoother_weights``), which keeps the preconditioner linear and
SPD, so plain CG stays valid.  Training data come from the FP64 operator itself
(per-cell power iterations, ``mfgb_cell_lambda``); training runs on the GPU with
the library's own forward/backward/Adam kernels; inference uses BF16 tensor
cores.  The exponent alpha is chosen by calibration solves of the multigrid
itself (on strongly deformed meshes alpha = 1/2 saves an iteration where
alpha = 1 does not); if no exponent needs fewer iterations than the plain
smoother, the plain smoother is kept (``LearnedSmoother.attach`` returns which
one is used).
"""
from __future__ import annotations

import ctypes
import struct

import numpy as np

from . import _abi
from ._abi import lib

N_IN = 73
MAGIC = b"MFGBMLP\x00"
VERSION = 1


def _torch():
    import torch
    return torch


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def cell_features(A):
    """float32 [n_cells, 73] on the device."""
    torch = _torch()
    F = torch.empty((A.n_cells, N_IN), dtype=torch.float32, device="cuda")
    _abi.check(lib().mfgb_cell_features(A.handle, _ptr(F), None))
    return F


def cell_lambda(A, iterations=200):
    """lambda_max(D_e^-1 A_e) per cell (FP64 power iteration), float64 on the device."""
    torch = _torch()
    lam = torch.empty(A.n_cells, dtype=torch.float64, device="cuda")
    _abi.check(lib().mfgb_cell_lambda(A.handle, _ptr(lam), int(iterations), None))
    return lam


def cell_error_reduction(A, M, n_vectors=4, seed=11):
    """Per-cell error reduction of one V-cycle of the multigrid M over A's mesh,
    rho_c = |(I - M A) e|_c / |e|_c over n_vectors seeded random errors: the
    training data the FP64 multigrid itself generates (mfgb_cell_error_reduction);
    float64 [n_cells] on the device."""
    torch = _torch()
    from . import _stream_ptr
    r = torch.empty(A.n_cells, dtype=torch.float64, device="cuda")
    _abi.check(lib().mfgb_cell_error_reduction(A.handle, M.handle, int(n_vectors),
                                               ctypes.c_uint64(seed), _ptr(r), _stream_ptr()))
    return r


class LearnedSmoother:
    def __init__(self, params=None, seed=0):
        torch = _torch()
        n = lib().mfgb_mlp_n_params()
        if params is None:
            g = np.random.default_rng(seed)
            w1 = g.normal(0, np.sqrt(2.0 / N_IN), (64, N_IN))
            w2 = g.normal(0, np.sqrt(2.0 / 64), (64, 64))
            w3 = g.normal(0, np.sqrt(1.0 / 64), 64)
            params = np.concatenate([w1.ravel(), np.zeros(64), w2.ravel(), np.zeros(64), w3, [1.0]])
        params = np.asarray(params, dtype=np.float32)
        if params.size != n:
            raise ValueError(f"expected {n} parameters, got {params.size}")
        self.params = torch.from_numpy(np.array(params, dtype=np.float32)).cuda()
        self.loss_history = []

    # ---- data and training -------------------------------------------------
    @staticmethod
    def training_data(meshes, lambda_iterations=200):
        """Features and FP64-operator targets for every cell of the meshes."""
        import benchmarks_gb300 as mf
        torch = _torch()
        Xs, ts = [], []
        for mesh in meshes:
            A = mf.LaplaceOperator(mesh)
            Xs.append(cell_features(A))
            ts.append(cell_lambda(A, lambda_iterations).float())
        return torch.cat(Xs), torch.cat(ts)

    def train(self, X, t, steps=3000, batch=1024, lr=1e-3, seed=1):
        loss = np.zeros(steps, dtype=np.float32)
        _abi.check(lib().mfgb_mlp_train(_ptr(self.params), _ptr(X), _ptr(t), X.shape[0], steps,
                                        batch, ctypes.c_float(lr), ctypes.c_uint64(seed),
                                        loss.ctypes.data_as(ctypes.c_void_p)))
        self.loss_history = loss
        return loss

    def loss_grad(self, X, t):
        g = np.zeros(lib().mfgb_mlp_n_params(), dtype=np.float32)
        L = ctypes.c_float()
        _abi.check(lib().mfgb_mlp_loss_grad(_ptr(self.params), _ptr(X), _ptr(t), X.shape[0],
                                            g.ctypes.data_as(ctypes.c_void_p), ctypes.byref(L)))
        return L.value, g

    # ---- inference -----------------------------------------------------------
    def predict(self, X):
        """BF16 tensor-core inference, float64 [n] on the device."""
        torch = _torch()
        y = torch.empty(X.shape[0], dtype=torch.float64, device="cuda")
        _abi.check(lib().mfgb_mlp_infer(_ptr(self.params), _ptr(X), X.shape[0], _ptr(y), None))
        return y

    def predict_f32(self, X):
        torch = _torch()
        y = torch.empty(X.shape[0], dtype=torch.float32, device="cuda")
        _abi.check(lib().mfgb_mlp_forward_f32(_ptr(self.params), _ptr(X), X.shape[0], _ptr(y)))
        return y

    # ---- use in the multigrid ------------------------------------------------
    def attach(self, mg, A, calibrate=True, reduce=1e-6, seed=7, exponents=(0.25, 0.5, 1.0)):
        """Set the predicted cell weights lambda^alpha on the finest level of `mg`
        (for the operator `A` of the same mesh).  With `calibrate`, one solve
        per exponent and one with the plain smoother on a seeded right-hand side
        decide; the best learned weights are kept only if they need fewer
        iterations than the plain smoother.  Returns (used_learned,
        iterations_plain, iterations_learned, alpha) -- iterations_learned and
        alpha of the best exponent."""
        import benchmarks_gb300 as mf
        lam = self.predict(cell_features(A))
        if not calibrate:
            w = (lam ** exponents[0]).contiguous()
            _abi.check(lib().mfgb_mg_set_smoother_weights(mg.handle, _ptr(w)))
            return True, None, None, exponents[0]

        def its():
            b = A.rhs_uniform(seed)
            x = A.initialize_dof_vector()
            ctl = mf.ReductionControl(1000, 1e-300, reduce)
            mf.SolverCG(ctl).solve(A, x, b, mg)
            return ctl.last_step()

        _abi.check(lib().mfgb_mg_set_smoother_weights(mg.handle, None))
        plain = its()
        best, best_alpha = None, None
        for alpha in exponents:
            w = (lam ** alpha).contiguous()
            _abi.check(lib().mfgb_mg_set_smoother_weights(mg.handle, _ptr(w)))
            k = its()
            if best is None or k < best:
                best, best_alpha = k, alpha
        if best < plain:
            w = (lam ** best_alpha).contiguous()
            _abi.check(lib().mfgb_mg_set_smoother_weights(mg.handle, _ptr(w)))
            return True, plain, best, best_alpha
        _abi.check(lib().mfgb_mg_set_smoother_weights(mg.handle, None))  # fall back
        return False, plain, best, best_alpha

    # ---- persistence: magic, version, count, float32 parameters ----------------
    def save(self, path):
        p = self.params.cpu().numpy().astype(np.float32)
        with open(path, "wb") as f:
            f.write(MAGIC + struct.pack("<II", VERSION, p.size) + p.tobytes())

    @classmethod
    def load(cls, path):
        with open(path, "rb") as f:
            data = f.read()
        if data[:8] != MAGIC:
            raise ValueError("not a learned-smoother weight file")
        ver, n = struct.unpack("<II", data[8:16])
        if ver != VERSION:
            raise ValueError(f"unsupported weight file version {ver}")
        return cls(np.frombuffer(data[16:16 + 4 * n], dtype=np.float32))
