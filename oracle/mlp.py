"""CPU oracle of the surrogate network (TEST INFRASTRUCTURE ONLY).

float64 numpy forward/backward of the MLP (x,y,z,t,p,D) -> 256 x 4 (SiLU) -> 18 that
rounds to BF16 at exactly the points where the tensor-core kernels hold BF16 values:
the normalised inputs, the weights, the hidden activations and the back-propagated
deltas.  Everything else (accumulation, biases, pre-activations, the loss) is kept in
high precision, so differences from the GPU come only from FP32 accumulation order and
from values that round to the other side of a BF16 boundary.
"""
import numpy as np

LAYERS = ((6, 256), (256, 256), (256, 256), (256, 256), (256, 18))


def bf16(a):
    a = np.asarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    out, o = [], 0
    for fi, fo in LAYERS:
        W = params[o:o + fi * fo].reshape(fo, fi).astype(np.float64)
        o += fi * fo
        b = params[o:o + fo].astype(np.float64)
        o += fo
        out.append((W, b))
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(params, X, shift=None, scale=None):
    layers = unpack(params)
    shift = np.zeros(6) if shift is None else np.asarray(shift, np.float64)
    scale = np.ones(6) if scale is None else np.asarray(scale, np.float64)
    H = bf16(((np.asarray(X, np.float64) - shift) * scale).astype(np.float32))
    Hs, Zs = [H], []
    for li, (W, b) in enumerate(layers):
        Z = H @ bf16(W.astype(np.float32)).T + b
        if li < len(layers) - 1:
            Zs.append(Z)
            H = bf16(silu(Z).astype(np.float32))
            Hs.append(H)
        else:
            return Z, Hs, Zs


def gradient(params, X, T, shift=None, scale=None):
    layers = unpack(params)
    Y, Hs, Zs = forward(params, X, shift, scale)
    P = X.shape[0]
    E = Y - T
    loss = 0.5 * np.sum(E * E) / P
    delta = bf16((E / P).astype(np.float32))
    grads = [None] * len(layers)
    for li in range(len(layers) - 1, -1, -1):
        W, _ = layers[li]
        grads[li] = (delta.T @ Hs[li], delta.sum(axis=0))
        if li > 0:
            dH = delta @ bf16(W.astype(np.float32))
            delta = bf16((dH * dsilu(Zs[li - 1])).astype(np.float32))
    flat = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
    return loss, flat
