"""TEST INFRASTRUCTURE ONLY: numpy restatement (float64) of the learned
warm-start network of the library (vfps_ws_forward / vfps_ws_backward in
include/vfps.h), the checker of its GPU gradients.  The network has no
counterpart in the reference; its equations are the ones documented in
include/vfps.h:
    h1 = tanh(W1 x + b1), h2 = tanh(W2 h1 + b2), z = W3 h2 + b3,
    y  = bd + sum_k z_k Wd[k],  L = sum (y - t)^2 / (B npix)
"""
import numpy as np


def forward(w, x):
    x = np.asarray(x, np.float64)
    h1 = np.tanh(x @ w["w1"].T + w["b1"])
    h2 = np.tanh(h1 @ w["w2"].T + w["b2"])
    z = h2 @ w["w3"].T + w["b3"]
    y = w["bd"] + z @ w["wd"]
    return h1, h2, z, y


def loss_and_grads(w, x, target):
    x = np.asarray(x, np.float64)
    t = np.asarray(target, np.float64).reshape(len(x), -1)
    h1, h2, z, y = forward(w, x)
    B, npix = y.shape
    d = y - t
    loss = float((d * d).sum() / (B * npix))
    g = 2.0 * d / (B * npix)
    gr = {"wd": z.T @ g, "bd": g.sum(0)}
    dz = g @ w["wd"].T
    gr["w3"] = dz.T @ h2
    gr["b3"] = dz.sum(0)
    d2 = (dz @ w["w3"]) * (1.0 - h2 * h2)
    gr["w2"] = d2.T @ h1
    gr["b2"] = d2.sum(0)
    d1 = (d2 @ w["w2"]) * (1.0 - h1 * h1)
    gr["w1"] = d1.T @ x
    gr["b1"] = d1.sum(0)
    return loss, gr
