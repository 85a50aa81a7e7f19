"""FP64 CPU restatement of the surrogate network of include/se2nn.h -- TEST
INFRASTRUCTURE ONLY (the oracle that libse2nn.so is tested against; nothing in the
product imports it).

The network has no counterpart in the reference (se2wave.c has no learned
component): this restates, in numpy float64, exactly the architecture the
header documents, with the same flat parameter layout, and differentiates it
by hand (adjoints of every linear map, GELU'), so the GPU kernels' forward
values and gradients can be compared with it.  It is itself pinned by central
finite differences and by torch-CPU autograd over an independent rfft2/irfft2
formulation (tests/test_nn_oracle.py).
"""
from __future__ import annotations

import dataclasses

import numpy as np
from scipy.special import erf


@dataclasses.dataclass
class Config:
    ny: int = 128
    nx: int = 128
    cin: int = 16
    width: int = 64
    modes: int = 16
    layers: int = 4
    nrec: int = 16
    nout: int = 2048
    hidden: int = 128
    max_batch: int = 32


def layout(c: Config):
    """Offsets and shapes of the flat parameter vector (se2nn.h order)."""
    w, m = c.width, c.modes
    items = [("Wlift", (c.cin, w)), ("blift", (w,))]
    for l in range(c.layers):
        items += [(f"Wre{l}", (2 * m, m, w, w)), (f"Wim{l}", (2 * m, m, w, w)), (f"W{l}", (w, w)), (f"b{l}", (w,))]
    ns = c.nout // c.ny
    items += [("Wdec1", (w, c.hidden)), ("cdec1", (c.hidden,)), ("Wdec2", (c.hidden, ns)), ("cdec2", (ns,))]
    out, o = {}, 0
    for name, shape in items:
        n = int(np.prod(shape))
        out[name] = (o, shape)
        o += n
    return out, o


def unpack(p: np.ndarray, c: Config) -> dict:
    lay, n = layout(c)
    assert p.size == n, (p.size, n)
    return {k: p[o: o + int(np.prod(s))].reshape(s) for k, (o, s) in lay.items()}


def pack(d: dict, c: Config) -> np.ndarray:
    lay, n = layout(c)
    p = np.zeros(n)
    for k, (o, s) in lay.items():
        p[o: o + int(np.prod(s))] = np.asarray(d[k], dtype=np.float64).reshape(-1)
    return p


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def dft_mats(c: Config):
    m, ny, nx = c.modes, c.ny, c.nx
    ky = np.array([j if j < m else ny - 2 * m + j for j in range(2 * m)])
    Ey = np.exp(-2j * np.pi * np.outer(ky, np.arange(ny)) / ny)          # [2m, ny]
    Ex = np.exp(-2j * np.pi * np.outer(np.arange(m), np.arange(nx)) / nx)  # [m, nx]
    wk = np.where(np.arange(m) == 0, 1.0, 2.0) / (nx * ny)                  # Hermitian weights and 1/(nx ny)
    return Ey, Ex, wk


def spectral(h, Wc, mats):
    """S = truncated-DFT spectral convolution of h [B, ny, nx, w] with complex weights Wc [2m, m, w, w]."""
    Ey, Ex, wk = mats
    Z = np.einsum("jy,kx,byxc->bjkc", Ey, Ex, h, optimize=True)
    Y = np.einsum("bjkc,jkcd->bjkd", Z, Wc, optimize=True)
    Yy = np.einsum("jy,bjkc->bykc", np.conj(Ey), Y, optimize=True)
    S = np.einsum("k,kx,bykc->byxc", wk, np.conj(Ex), Yy, optimize=True).real
    return S, Z


def spectral_adjoint(dS, Z, Wc, mats):
    """Gradients (dh, dWc) of spectral() for the output gradient dS; dWc = dL/dRe + i dL/dIm."""
    Ey, Ex, wk = mats
    dYy = np.einsum("k,kx,byxc->bykc", wk, Ex, dS, optimize=True)
    dY = np.einsum("jy,bykc->bjkc", Ey, dYy, optimize=True)
    dW = np.einsum("bjkc,bjkd->jkcd", np.conj(Z), dY, optimize=True)
    dZ = np.einsum("bjkd,jkcd->bjkc", dY, np.conj(Wc), optimize=True)
    dh = np.einsum("jy,kx,bjkc->byxc", np.conj(Ey), np.conj(Ex), dZ, optimize=True).real
    return dh, dW


def forward(p: np.ndarray, x: np.ndarray, c: Config, rec_x, keep: bool = False):
    """out [B, nrec, nout] of the network on x [B, ny, nx, cin]."""
    P = unpack(np.asarray(p, dtype=np.float64), c)
    mats = dft_mats(c)
    x = np.asarray(x, dtype=np.float64)
    rec_x = np.asarray(rec_x)
    h = x @ P["Wlift"] + P["blift"]
    Hs, As, Zs = [h], [], []
    for l in range(c.layers):
        Wc = P[f"Wre{l}"] + 1j * P[f"Wim{l}"]
        S, Z = spectral(h, Wc, mats)
        a = S + h @ P[f"W{l}"] + P[f"b{l}"]
        h = gelu(a) if l < c.layers - 1 else a
        As.append(a)
        Zs.append(Z)
        Hs.append(h)
    D0 = h[:, :, rec_x, :].transpose(0, 2, 1, 3)             # [B, nrec, ny, w]: each receiver's column
    D1pre = D0 @ P["Wdec1"] + P["cdec1"]
    D1 = gelu(D1pre)
    out = (D1 @ P["Wdec2"] + P["cdec2"]).reshape(x.shape[0], len(rec_x), -1)   # [B, nrec, ny * nsub]
    if keep:
        return out, dict(P=P, mats=mats, x=x, Hs=Hs, As=As, Zs=Zs, D0=D0, D1pre=D1pre, D1=D1, rec_x=rec_x)
    return out


def loss_grad(p: np.ndarray, x: np.ndarray, target: np.ndarray, c: Config, rec_x):
    """(loss, gradient, out) of loss = mean((out - target)^2)."""
    out, k = forward(p, x, c, rec_x, keep=True)
    P, mats = k["P"], k["mats"]
    diff = out - target
    loss = float(np.mean(diff * diff))
    g = {}
    dout = (2.0 * diff / diff.size).reshape(k["D1"].shape[:3] + (-1,))
    g["Wdec2"] = np.einsum("bryi,bryo->io", k["D1"], dout)
    g["cdec2"] = dout.sum(axis=(0, 1, 2))
    dD1pre = (dout @ P["Wdec2"].T) * gelu_grad(k["D1pre"])
    g["Wdec1"] = np.einsum("bryi,bryo->io", k["D0"], dD1pre)
    g["cdec1"] = dD1pre.sum(axis=(0, 1, 2))
    dD0 = dD1pre @ P["Wdec1"].T                                # [B, nrec, ny, w]
    B = x.shape[0]
    dh = np.zeros_like(k["Hs"][-1])
    for r, rx in enumerate(k["rec_x"]):
        dh[:, :, rx, :] += dD0[:, r]
    for l in reversed(range(c.layers)):
        a = k["As"][l]
        da = dh * gelu_grad(a) if l < c.layers - 1 else dh
        h = k["Hs"][l]
        g[f"W{l}"] = np.einsum("byxi,byxo->io", h, da)
        g[f"b{l}"] = da.sum(axis=(0, 1, 2))
        Wc = P[f"Wre{l}"] + 1j * P[f"Wim{l}"]
        dh_s, dW = spectral_adjoint(da, k["Zs"][l], Wc, mats)
        g[f"Wre{l}"] = dW.real
        g[f"Wim{l}"] = dW.imag
        dh = da @ P[f"W{l}"].T + dh_s
    g["Wlift"] = np.einsum("byxi,byxo->io", k["x"], dh)
    g["blift"] = dh.sum(axis=(0, 1, 2))
    assert B == x.shape[0]
    return loss, pack(g, c), out


def build_inputs(materials, src, idx, c: Config, sigma_cells: float):
    """Network input of se2nn_build_inputs: materials [N, ny, nx, 3] (row up from the bottom),
    src [N, 2] (cells, y up from the bottom); network row 0 is the top surface."""
    B = len(idx)
    x = np.zeros((B, c.ny, c.nx, c.cin))
    cy, cx = np.meshgrid(np.arange(c.ny) + 0.5, np.arange(c.nx) + 0.5, indexing="ij")
    for b, s in enumerate(idx):
        mt = materials[s][::-1]
        x[b, :, :, 0] = (mt[..., 0] - 5000.0) / 1500.0
        x[b, :, :, 1] = (mt[..., 1] - 2800.0) / 800.0
        x[b, :, :, 2] = (mt[..., 2] - 2500.0) / 500.0
        x[b, :, :, 3] = np.exp(-((cx - src[s][0]) ** 2 + (cy - (c.ny - src[s][1])) ** 2) / (2.0 * sigma_cells ** 2))
        x[b, :, :, 4] = (2.0 * np.floor(cx) + 1.0) / c.nx - 1.0
        x[b, :, :, 5] = (2.0 * np.floor(cy) + 1.0) / c.ny - 1.0
    return x


def adam(p, g, m, v, t, lr, b1, b2, eps, wd):
    """One step of se2nn_adam_step (bias-corrected, decoupled weight decay); returns (p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh, vh = m / (1 - b1 ** t), v / (1 - b2 ** t)
    return p - lr * (mh / (np.sqrt(vh) + eps) + wd * p), m, v
