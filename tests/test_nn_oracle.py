"""Pins of the FP64 network oracle (oracle/nn_oracle.py), on the CPU:
central finite differences of its loss, and torch-CPU autograd of an
independent formulation (torch.fft.rfft2 / irfft2 instead of DFT matrices)."""
import numpy as np
import pytest

from oracle import nn_oracle as NO

CFG = NO.Config(ny=8, nx=12, cin=16, width=4, modes=2, layers=2, nrec=3, nout=24, hidden=6, max_batch=4)
REC = [1, 5, 10]


def sample(c=CFG, B=2, seed=0):
    rng = np.random.default_rng(seed)
    _, n = NO.layout(c)
    p = rng.standard_normal(n) * 0.3
    x = rng.standard_normal((B, c.ny, c.nx, c.cin))
    t = rng.standard_normal((B, c.nrec, c.nout))
    return p, x, t


def test_layout_counts():
    lay, n = NO.layout(NO.Config())
    w, m = 64, 16
    assert n == 16 * w + w + 4 * (2 * 2 * m * m * w * w + w * w + w) + w * 128 + 128 + 128 * 16 + 16
    p = np.arange(n, dtype=np.float64)
    assert np.array_equal(NO.pack(NO.unpack(p, NO.Config()), NO.Config()), p)


def test_gradient_matches_finite_differences():
    p, x, t = sample()
    loss, g, _ = NO.loss_grad(p, x, t, CFG, REC)
    rng = np.random.default_rng(1)
    for _ in range(4):
        v = rng.standard_normal(p.size)
        eps = 1e-6
        lp = NO.loss_grad(p + eps * v, x, t, CFG, REC)[0]
        lm = NO.loss_grad(p - eps * v, x, t, CFG, REC)[0]
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g @ v) <= 1e-6 * max(1.0, abs(fd)), (fd, g @ v)
    # every parameter block gets a non-zero gradient
    lay, _ = NO.layout(CFG)
    for name, (o, s) in lay.items():
        assert np.any(g[o: o + int(np.prod(s))] != 0), name


def torch_forward(p, x, c, rec_x):
    import torch
    P = {k: torch.tensor(v) for k, v in NO.unpack(p, c).items()}
    for v in P.values():
        v.requires_grad_(True)
    xt = torch.tensor(x)
    m = c.modes
    h = xt @ P["Wlift"] + P["blift"]
    for l in range(c.layers):
        Wc = torch.complex(P[f"Wre{l}"], P[f"Wim{l}"])
        hf = torch.fft.rfft2(h, dim=(1, 2))                       # [B, ny, nx/2+1, w]
        of = torch.zeros_like(hf)
        of[:, :m, :m, :] = torch.einsum("bjkc,jkcd->bjkd", hf[:, :m, :m, :], Wc[:m])
        of[:, -m:, :m, :] = torch.einsum("bjkc,jkcd->bjkd", hf[:, -m:, :m, :], Wc[m:])
        S = torch.fft.irfft2(of, s=(c.ny, c.nx), dim=(1, 2))
        a = S + h @ P[f"W{l}"] + P[f"b{l}"]
        h = torch.nn.functional.gelu(a) if l < c.layers - 1 else a
    D0 = h[:, :, list(rec_x), :].permute(0, 2, 1, 3)
    out = torch.nn.functional.gelu(D0 @ P["Wdec1"] + P["cdec1"]) @ P["Wdec2"] + P["cdec2"]
    out = out.reshape(x.shape[0], len(rec_x), -1)
    return out, P


def test_oracle_matches_torch_autograd():
    torch = pytest.importorskip("torch")
    p, x, t = sample(seed=3)
    loss, g, out = NO.loss_grad(p, x, t, CFG, REC)
    tout, P = torch_forward(p, x, CFG, REC)
    tl = ((tout - torch.tensor(t)) ** 2).mean()
    tl.backward()
    np.testing.assert_allclose(out, tout.detach().numpy(), rtol=1e-10, atol=1e-12)
    assert abs(loss - tl.item()) <= 1e-12 * abs(loss)
    tg = NO.pack({k: v.grad.numpy() for k, v in P.items()}, CFG)
    np.testing.assert_allclose(g, tg, rtol=1e-8, atol=1e-12)


def test_adam_step_formula():
    p, g = np.array([1.0, -2.0]), np.array([0.5, 0.25])
    q, m, v = NO.adam(p, g, np.zeros(2), np.zeros(2), 1, 0.1, 0.9, 0.999, 1e-8, 0.0)
    np.testing.assert_allclose(q, p - 0.1 * np.sign(g), rtol=1e-6)
