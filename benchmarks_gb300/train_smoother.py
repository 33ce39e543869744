"""Trains the learned smoother network on the GPU and writes its weights.

Training data: every cell of 48 deformed box meshes (8 x 8 x 6 cells, degree
drawn from 2..7, amplitude from U[0, 0.12], seed 0), features from the corner
Jacobians, targets lambda_max(D_e^-1 A_e) from the FP64 operator (200 power
iterations per cell).  Adam, 6000 steps of 1024 samples, lr 2e-3.

Run: python -m benchmarks_gb300.train_smoother OUTPUT.bin
"""
from __future__ import annotations

import json
import sys

import numpy as np


def main(path):
    import torch

    import benchmarks_gb300 as mf
    from benchmarks_gb300.learned import LearnedSmoother, cell_features, cell_lambda
    torch.cuda.set_device(0)
    rng = np.random.default_rng(0)
    meshes = [mf.BoxMesh(8, 8, 6, degree=int(p), amplitude=float(a))
              for p, a in zip(rng.integers(2, 8, 48), rng.uniform(0.0, 0.12, 48))]
    X, t = LearnedSmoother.training_data(meshes)
    S = LearnedSmoother(seed=1)
    loss = S.train(X, t, steps=6000, batch=1024, lr=2e-3)
    A = mf.LaplaceOperator(mf.BoxMesh(8, 8, 8, degree=4, amplitude=0.12))
    r = (torch.abs(S.predict(cell_features(A)) - cell_lambda(A)) / cell_lambda(A)).cpu().numpy()
    S.save(path)
    print(json.dumps({"samples": int(X.shape[0]), "loss_first": float(loss[:10].mean()),
                      "loss_last": float(loss[-50:].mean()), "heldout_rel_median": float(np.median(r)),
                      "heldout_rel_max": float(r.max()), "weights": path}))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "smoother_mlp.bin")
