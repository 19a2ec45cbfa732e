"""CPU reference of the learned QLT closure's network and its training targets.

TEST INFRASTRUCTURE ONLY: the checker for the GPU forward/backward kernels
and the fused tensor-core inference; the product never imports it.

Network: 5 -> H -> H -> 3 (H = 32 or 64), tanh hidden layers, linear output;
parameter block W1[H][5] b1[H] W2[H][H] b2[H] W3[3][H] b3[3] (1379 values for
H = 32, 4739 for H = 64; the width is read off the block's length).
Loss: mean over samples and outputs of the squared error.  Everything here
is float64 numpy, written from the definitions (backpropagation by the chain
rule), and is itself checked against central finite differences.

Targets follow the slab-QLT closure of include/LegencyModel.hpp:557-645
(pitch_angle_diffusion_coefficient / _derivative) and the driver's
kappa_parallel closure (src/main.cpp:1177-1193):
  y0 = ln D_mumu - ln(1 - mu^2)
  y1 = (gk - 1) - gk reg^gk / (reg^gk + xi^gk),  reg = |mu| + h0
  y2 = ln kappa_parallel
"""
from __future__ import annotations

import numpy as np

N_IN, N_OUT = 5, 3


def layout(hidden: int) -> dict:
    """Offsets of W1 b1 W2 b2 W3 b3 and the block length for width `hidden`."""
    w1 = 0
    b1 = w1 + hidden * N_IN
    w2 = b1 + hidden
    b2 = w2 + hidden * hidden
    w3 = b2 + hidden
    b3 = w3 + N_OUT * hidden
    return {"W1": w1, "B1": b1, "W2": w2, "B2": b2, "W3": w3, "B3": b3,
            "N_PARAMS": b3 + N_OUT, "hidden": hidden}


def hidden_of(count: int) -> int:
    for hidden in (32, 64):
        if layout(hidden)["N_PARAMS"] == count:
            return hidden
    raise ValueError(f"no network width has {count} parameters")


def unpack(params: np.ndarray):
    p = np.asarray(params, dtype=np.float64)
    h = hidden_of(p.size)
    o = layout(h)
    return (p[o["W1"]:o["B1"]].reshape(h, N_IN), p[o["B1"]:o["W2"]],
            p[o["W2"]:o["B2"]].reshape(h, h), p[o["B2"]:o["W3"]],
            p[o["W3"]:o["B3"]].reshape(N_OUT, h), p[o["B3"]:o["N_PARAMS"]])


def forward(params: np.ndarray, x: np.ndarray) -> np.ndarray:
    w1, b1, w2, b2, w3, b3 = unpack(params)
    h1 = np.tanh(x @ w1.T + b1)
    h2 = np.tanh(h1 @ w2.T + b2)
    return h2 @ w3.T + b3


def loss_and_gradient(params: np.ndarray, x: np.ndarray, t: np.ndarray):
    """Mean squared error and its gradient with respect to the parameter block."""
    x = np.asarray(x, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    w1, b1, w2, b2, w3, b3 = unpack(params)
    h1 = np.tanh(x @ w1.T + b1)
    h2 = np.tanh(h1 @ w2.T + b2)
    y = h2 @ w3.T + b3
    n = x.shape[0]
    err = y - t
    loss = float(np.mean(err * err))
    gy = 2.0 * err / (n * N_OUT)
    g2 = (gy @ w3) * (1.0 - h2 * h2)
    g1 = (g2 @ w2) * (1.0 - h1 * h1)
    grad = np.concatenate([(g1.T @ x).ravel(), g1.sum(0), (g2.T @ h1).ravel(), g2.sum(0),
                           (gy.T @ h2).ravel(), gy.sum(0)])
    return loss, grad


def finite_difference_gradient(params: np.ndarray, x: np.ndarray, t: np.ndarray,
                               indices, h: float = 1e-6) -> np.ndarray:
    out = []
    for k in indices:
        up = np.array(params, dtype=np.float64)
        dn = up.copy()
        up[k] += h
        dn[k] -= h
        out.append((loss_and_gradient(up, x, t)[0] - loss_and_gradient(dn, x, t)[0]) / (2 * h))
    return np.array(out)


def qlt_targets(mu, p, b, sigma2, gk, *, p0, particle_v0, qlt_omega0, qlt_lc, qlt_h0):
    """(D_mumu, dD_mumu/dmu, y0, y1) of the slab-QLT closure, vectorised."""
    mu = np.asarray(mu, dtype=np.float64)
    speed = particle_v0 * p / p0
    omega = qlt_omega0 * b / np.sqrt(1.0 + p * p)
    one_minus_mu2 = 1.0 - mu * mu
    reg = np.abs(mu) + qlt_h0
    xi = omega * qlt_lc / speed
    reg_gk = reg ** gk
    den = reg_gk + xi ** gk
    norm = gk * np.sin(np.pi / gk) / np.pi
    pref = 0.25 * np.pi * omega * sigma2 * norm
    d = pref * one_minus_mu2 * xi * reg ** (gk - 1.0) / den
    y0 = np.log(pref * xi) + (gk - 1.0) * np.log(reg) - np.log(den)
    y1 = (gk - 1.0) - gk * reg_gk / den
    dd = d * (-2.0 * mu / one_minus_mu2 + np.sign(mu) * ((gk - 1.0) / reg
                                                        - gk * reg ** (gk - 1.0) / den))
    return d, dd, y0, y1


def kappa_parallel(p, b, *, p0, kpara0, gamma_turb, magnetic_dependency=1,
                   momentum_dependency=1):
    k = kpara0 * np.ones_like(np.asarray(p, dtype=np.float64))
    if magnetic_dependency == 1:
        k = k * b ** (gamma_turb - 2.0)
    if momentum_dependency == 1:
        k = k * (p / p0) ** (3.0 - gamma_turb)
    return k


def evaluate(params, norm, inputs, *, p0, qlt_h0, particle_v0=None, qlt_omega0=None,
             qlt_lc=None, kpara0=None, gamma_turb=None):
    """Raw inputs (mu, ln p, ln|B|, sigma^2, gamma_k) -> (D, dD/dmu, ln kappa)
    through the FP64 network with the box normalisation of a trained net
    (inputs assumed inside the box).  With the physics constants given, the
    served values blend linearly into the plain closure over
    mu_cut <= |mu| < 2 mu_cut, as the push does."""
    inputs = np.asarray(inputs, dtype=np.float64)
    mu = inputs[:, 0]
    feat = np.stack([np.log(np.abs(mu)), inputs[:, 1], inputs[:, 2], np.log(inputs[:, 3]),
                     inputs[:, 4]], axis=1)
    lo, hi = norm["in_lo"], norm["in_hi"]
    x = 2.0 * (feat - lo) / (hi - lo) - 1.0
    y = forward(params, x) * norm["out_scale"] + norm["out_offset"]
    one_minus_mu2 = 1.0 - mu * mu
    d = one_minus_mu2 * np.exp(y[:, 0])
    dd = d * (np.sign(mu) * y[:, 1] / (np.abs(mu) + qlt_h0) - 2.0 * mu / one_minus_mu2)
    lk = y[:, 2]
    if particle_v0 is not None:
        cut = norm["mu_cut"]
        amu = np.abs(mu)
        blend = amu < 2.0 * cut
        p, b = np.exp(inputs[:, 1]), np.exp(inputs[:, 2])
        pd, pdd, _, _ = qlt_targets(mu, p, b, inputs[:, 3], inputs[:, 4], p0=p0,
                                    particle_v0=particle_v0, qlt_omega0=qlt_omega0,
                                    qlt_lc=qlt_lc, qlt_h0=qlt_h0)
        pk = kappa_parallel(p, b, p0=p0, kpara0=kpara0, gamma_turb=gamma_turb)
        w = (amu - cut) / cut
        dw = np.sign(mu) / cut
        dd = np.where(blend, pdd + w * (dd - pdd) + dw * (d - pd), dd)
        d = np.where(blend, pd + w * (d - pd), d)
        lk = np.where(blend, np.log(pk + w * (np.exp(lk) - pk)), lk)
    return np.stack([d, dd, lk], axis=1)
