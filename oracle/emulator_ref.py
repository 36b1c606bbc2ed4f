"""Oracle of the radiation emulator's MLP -- TEST INFRASTRUCTURE ONLY.

A numpy restatement of the forward pass, the mean-squared-error loss and the backward
pass that l-game_gb300/csrc/emulator.cu runs on the tensor cores, used by tests/ to check
the GPU gradients.  There is no reference counterpart: the reference has no emulator
(it calls RTE+RRTMGP, src/radiation/mo_rterrtmgp_coupler.F90:56-493), so the parity of
this oracle rests on its finite-difference check (tests/test_emulator.py) and on the
published definitions it restates:

    z_l = a_{l-1} W_l^T + b_l,  a_l = GELU(z_l) = z_l * Phi(z_l)  (l = 1..3),  y = a_3 W_4^T + b_4
    L = mean((y - t)^2) over batch x outputs (standardised targets t)

With bf16=True the operands of every GEMM are rounded to BF16 exactly where the GPU rounds
them (standardised inputs, weights, hidden activations, back-propagated errors), and the
products are accumulated in float64; with bf16=False everything is float64 (the form the
finite-difference check uses).
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf


def bf16_round(x: np.ndarray) -> np.ndarray:
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint32)
    return (b << 16).view(np.float32).astype(np.float64)


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def unflatten(p: np.ndarray, nin: int, hidden: int, nout: int):
    shapes = [(hidden, nin), (hidden,), (hidden, hidden), (hidden,), (hidden, hidden), (hidden,), (nout, hidden),
              (nout,)]
    out, off = [], 0
    for s in shapes:
        n = int(np.prod(s))
        out.append(np.asarray(p[off:off + n], dtype=np.float64).reshape(s))
        off += n
    return out


def _forward(params, x, nin, hidden, nout, norm, bf16):
    """Standardised outputs of the rows of x with the activations and pre-activations of the
    hidden layers; BF16 rounding of operands (and FP32 pre-activations) as on the GPU."""
    W1, b1, W2, b2, W3, b3, W4, b4 = unflatten(params, nin, hidden, nout)
    x = np.asarray(x, np.float64)
    if norm is not None:
        xm, xs = (np.asarray(v, np.float64) for v in norm[:2])
        x = (x - xm) / xs
    r = bf16_round if bf16 else (lambda a: np.asarray(a, np.float64))
    if bf16:  # the GPU standardises in float32 before rounding
        x = np.asarray(x, np.float32)
    a0 = r(x)
    Ws = [W1, W2, W3, W4]
    bs = [b1, b2, b3, b4]
    acts, zs = [a0], []
    for l in range(3):
        z = acts[-1] @ r(Ws[l]).T + bs[l]
        if bf16:
            z = np.asarray(z, np.float32).astype(np.float64)
        zs.append(z)
        acts.append(r(gelu(z)))
    out = acts[-1] @ r(Ws[3]).T + bs[3]
    return out, acts, zs, Ws, r


def predict(params: np.ndarray, x: np.ndarray, nin: int, hidden: int, nout: int, norm, bf16: bool = True):
    """Heating rates of the rows of x (inference): the network's outputs de-standardised with
    norm = (x_mean, x_std, y_mean, y_std)."""
    out = _forward(params, x, nin, hidden, nout, norm, bf16)[0]
    ym, ys = (np.asarray(v, np.float64) for v in norm[2:])
    return out * ys + ym


def loss_grad(params: np.ndarray, x: np.ndarray, y: np.ndarray, nin: int, hidden: int, nout: int,
              norm=None, bf16: bool = True):
    """(loss, flat gradient) of one batch; norm = (x_mean, x_std, y_mean, y_std) or None."""
    out, acts, zs, Ws, r = _forward(params, x, nin, hidden, nout, norm, bf16)
    y = np.asarray(y, np.float64)
    if norm is not None:
        ym, ys = (np.asarray(v, np.float64) for v in norm[2:])
        y = (y - ym) / ys
    B = x.shape[0]
    e = out - y
    loss = float(np.mean(e * e))
    d = 2.0 * e / (B * nout)
    grads = [None] * 8
    for l in range(3, -1, -1):
        grads[2 * l] = r(d).T @ acts[l]
        grads[2 * l + 1] = d.sum(0)
        if l == 0:
            break
        d = (r(d) @ r(Ws[l])) * gelu_grad(zs[l - 1])
        if bf16:
            d = np.asarray(d, np.float32).astype(np.float64)
    return loss, np.concatenate([g.ravel() for g in grads])
