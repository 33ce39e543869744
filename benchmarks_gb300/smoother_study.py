"""Smoother-weight study on strongly deformed meshes: MG-CG iterations to 1e-10
(FP32 V-cycle in FP64 CG) with the plain Jacobi-Chebyshev smoother, with cell
weights from the multigrid's own error-reduction data rho_c (one FP64 V-cycle
on seeded random errors, ``learned.cell_error_reduction``) raised to several
exponents, with the exact cell spectra lambda^(1/2), and with weights iterated
on the reduction data w <- w (rho_w / mean)^g.  One JSON line per mesh.

    python -m benchmarks_gb300.smoother_study
"""
from __future__ import annotations

import ctypes
import json

from . import _abi
from ._abi import lib

MESHES = ((32, 3, 0.10), (24, 4, 0.12), (16, 6, 0.12))


def _iterations(mf, A, M, b, max_steps=300):
    x = A.initialize_dof_vector()
    ctl = mf.ReductionControl(max_steps, 1e-300, 1e-10)
    try:
        mf.SolverCG(ctl).solve(A, x, b, M)
    except mf.MfgbError:
        return None  # not converged within max_steps
    return ctl.last_step()


def _set_weights(M, w):
    if w is None:
        _abi.check(lib().mfgb_mg_set_smoother_weights(M.handle, None))
        return None
    w = w.contiguous()
    _abi.check(lib().mfgb_mg_set_smoother_weights(M.handle, ctypes.c_void_p(w.data_ptr())))
    return w  # keep alive while in use


def study(n, p, a, exponents=(-2, -1, -0.5, 0.5, 1, 2), rounds=4):
    import torch

    import benchmarks_gb300 as mf
    from .learned import cell_error_reduction, cell_lambda
    mesh = mf.BoxMesh(n, n, n, degree=p, amplitude=a)
    A = mf.LaplaceOperator(mesh)
    M = mf.MGPreconditioner(mesh, precision=32, operator=A)
    M64 = mf.MGPreconditioner(mesh, precision=64, operator=A)
    b = A.rhs_uniform(3)
    out = {"mesh": f"{n}^3 cells, p = {p}, amplitude {a}", "plain": _iterations(mf, A, M, b)}
    rho = cell_error_reduction(A, M64)
    lam = cell_lambda(A, 200)
    lr, ll = torch.log(rho), torch.log(lam)
    out["log_corr_rho_lambda"] = float(torch.corrcoef(torch.stack([lr, ll]))[0, 1])
    for g in exponents:
        keep = _set_weights(M, (rho / rho.mean()) ** g)
        out[f"rho^{g}"] = _iterations(mf, A, M, b)
    keep = _set_weights(M, lam ** 0.5)
    out["lambda^0.5"] = _iterations(mf, A, M, b)
    w = torch.ones(A.n_cells, dtype=torch.float64, device="cuda")
    seq = []
    for k in range(rounds):
        keep64 = _set_weights(M64, w)
        rw = cell_error_reduction(A, M64, seed=20 + k)
        w = w * (rw / rw.mean()) ** -0.5
        keep = _set_weights(M, w)
        seq.append(_iterations(mf, A, M, b))
    out["iterated_rho^-0.5"] = seq
    _set_weights(M, None)
    _set_weights(M64, None)
    del keep, keep64
    return out


def main():
    import torch
    torch.cuda.set_device(0)
    for n, p, a in MESHES:
        print(json.dumps(study(n, p, a)), flush=True)


if __name__ == "__main__":
    main()
