"""CPU oracle of the continuation-guess network -- TEST INFRASTRUCTURE ONLY.

A float64 numpy restatement of the network that goma_gb300's CUDA kernels
train (goma_gb300/csrc/gb_mlp.cu): layers W_l [out][in], b_l [out] in one
flat parameter vector, tanh on hidden layers, linear output, loss
sum(mask (y - t)^2) / sum(mask).  Used to check the GPU forward pass and
gradients; never part of the product path.
"""
import numpy as np


def layout(widths):
    offs, off = [], 0
    for i in range(len(widths) - 1):
        wo = off
        off += widths[i] * widths[i + 1]
        bo = off
        off += widths[i + 1]
        offs.append((wo, bo))
    return offs, off


def unpack(params, widths):
    offs, _ = layout(widths)
    Ws, bs = [], []
    for i, (wo, bo) in enumerate(offs):
        fi, fo = widths[i], widths[i + 1]
        Ws.append(params[wo:wo + fi * fo].reshape(fo, fi).astype(np.float64))
        bs.append(params[bo:bo + fo].astype(np.float64))
    return Ws, bs


def forward(params, widths, X):
    Ws, bs = unpack(params, widths)
    H = [np.asarray(X, np.float64)]
    for l, (W, b) in enumerate(zip(Ws, bs)):
        Z = H[-1] @ W.T + b
        H.append(np.tanh(Z) if l + 1 < len(Ws) else Z)
    return H


def loss_and_grad(params, widths, X, T, mask):
    Ws, bs = unpack(params, widths)
    H = forward(params, widths, X)
    msum = mask.sum()
    d = (H[-1] - T) * mask
    loss = (d * d).sum() / msum
    dZ = 2.0 * d / msum
    offs, n = layout(widths)
    g = np.zeros(n)
    for l in range(len(Ws) - 1, -1, -1):
        wo, bo = offs[l]
        g[wo:wo + Ws[l].size] = (dZ.T @ H[l]).ravel()
        g[bo:bo + bs[l].size] = dZ.sum(axis=0)
        if l == 0:
            break
        dH = dZ @ Ws[l]
        dZ = dH * (1.0 - H[l] ** 2)
    return loss, g
