"""CPU oracle (test infrastructure only) for the learned smoother weights.

No counterpart in the reference; this restates in FP64 numpy what the CUDA
library computes, so that its kernels can be checked:

  features   per cell, the Jacobian dx/dxi at the 8 corner GLL points (9
             entries each, reference directions r, s, t = local i, j, k),
             divided by |mean corner det J|^(1/3), then p / 8: 73 inputs
  target     lambda_e = lambda_max(D_e^{-1} A_e), the largest eigenvalue of the
             cell matrix A_e scaled by its own diagonal D_e
  model      y = softplus(w3 . relu(W2 relu(W1 x + b1) + b2) + b3)
             (73 -> 64 -> 64 -> 1), loss = mean (y - t)^2
"""
from __future__ import annotations

import numpy as np

from . import oracle as orc

N_IN, N_HID = 73, 64


def cell_features(prob) -> np.ndarray:
    n = prob.n
    ng = (prob.geometry_degree or prob.degree) + 1
    xg, _ = orc.gll(ng)
    xl, _ = orc.gll(n)
    corners = [0, n - 1]
    # geometry basis derivative at the operator's corner GLL points (= +-1)
    V = np.array([[orc.lib().orc_lagrange_value(ng, orc._p(xg), a, float(xl[i])) for a in range(ng)]
                  for i in range(n)])
    Dv = np.array([[orc.lib().orc_lagrange_derivative(ng, orc._p(xg), a, float(xl[i]))
                    for a in range(ng)] for i in range(n)])
    F = np.zeros((prob.n_cells, N_IN))
    for e in range(prob.n_cells):
        X = prob.cell_nodes(e).reshape(ng, ng, ng, 3)
        Js, dets = [], []
        for i in corners:
            for j in corners:
                for k in corners:
                    Jr = np.einsum("a,b,c,abcd->d", Dv[i], V[j], V[k], X)
                    Jsv = np.einsum("a,b,c,abcd->d", V[i], Dv[j], V[k], X)
                    Jt = np.einsum("a,b,c,abcd->d", V[i], V[j], Dv[k], X)
                    J = np.stack([Jr, Jsv, Jt], axis=1)  # J[d][a]
                    Js.append(J)
                    dets.append(np.linalg.det(J))
        s = abs(np.mean(dets)) ** (1.0 / 3.0)
        F[e, :72] = np.concatenate([J.reshape(-1) for J in Js]) / s
        F[e, 72] = prob.degree / 8.0
    return F


def cell_lambda(prob) -> np.ndarray:
    """lambda_max(D_e^{-1} A_e) of every cell by dense eigenvalues."""
    n3 = prob.n ** 3
    lam = np.zeros(prob.n_cells)
    for e in range(prob.n_cells):
        G = prob.G[e * 6 * n3:(e + 1) * 6 * n3]
        A = np.zeros((n3, n3))
        for c in range(n3):
            u = np.zeros(n3); u[c] = 1.0
            A[:, c] = orc.evector(prob.n, prob.D, G, u)
        d = np.diag(A)
        S = A / np.sqrt(np.outer(d, d))
        lam[e] = np.linalg.eigvalsh(0.5 * (S + S.T))[-1]
    return lam


def softplus(z):
    return np.where(z > 20, z, np.log1p(np.exp(np.minimum(z, 20))))


def sigmoid(z):
    return 1.0 / (1.0 + np.exp(-z))


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    return {"W1": rng.normal(0, np.sqrt(2.0 / N_IN), (N_HID, N_IN)), "b1": np.zeros(N_HID),
            "W2": rng.normal(0, np.sqrt(2.0 / N_HID), (N_HID, N_HID)), "b2": np.zeros(N_HID),
            "w3": rng.normal(0, np.sqrt(1.0 / N_HID), N_HID), "b3": np.array([1.0])}


def forward(P, X):
    z1 = X @ P["W1"].T + P["b1"]
    h1 = np.maximum(z1, 0)
    z2 = h1 @ P["W2"].T + P["b2"]
    h2 = np.maximum(z2, 0)
    z3 = h2 @ P["w3"] + P["b3"][0]
    return softplus(z3), (X, z1, h1, z2, h2, z3)


def loss_and_grads(P, X, t):
    y, (X, z1, h1, z2, h2, z3) = forward(P, X)
    B = X.shape[0]
    L = np.mean((y - t) ** 2)
    dy = 2.0 * (y - t) / B
    dz3 = dy * sigmoid(z3)
    g = {"w3": h2.T @ dz3, "b3": np.array([dz3.sum()])}
    dh2 = np.outer(dz3, P["w3"]) * (z2 > 0)
    g["W2"] = dh2.T @ h1
    g["b2"] = dh2.sum(0)
    dh1 = (dh2 @ P["W2"]) * (z1 > 0)
    g["W1"] = dh1.T @ X
    g["b1"] = dh1.sum(0)
    return L, g


# flat parameter vector in the library's order: W1 (row-major 64x73), b1, W2, b2, w3, b3
ORDER = [("W1", (N_HID, N_IN)), ("b1", (N_HID,)), ("W2", (N_HID, N_HID)), ("b2", (N_HID,)),
         ("w3", (N_HID,)), ("b3", (1,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in ORDER)


def flatten(P):
    return np.concatenate([np.asarray(P[k], dtype=np.float64).reshape(-1) for k, _ in ORDER])


def unflatten(v):
    out, o = {}, 0
    for k, s in ORDER:
        m = int(np.prod(s))
        out[k] = np.asarray(v[o:o + m], dtype=np.float64).reshape(s)
        o += m
    return out
