"""TEST INFRASTRUCTURE ONLY: CPU restatement of the learned warm start network.

The network has no counterpart in the reference (it fills the zero start of a
contact without a cache entry, shapes/src/Physics/Solvers/Contact.hs:91-98).
This module restates what the tensor-core kernels compute — forward pass,
squared-error loss on normalised targets, back-propagation — with BF16
rounding (round to nearest even) at the same points as the kernels: the
normalised input, every weight, every hidden activation, the output error and
every back-propagated error before it enters a product.  Products of BF16
values are exact in float64, so the only differences left against the GPU are
FP32 accumulation order and the BF16 roundings those can flip.

`forward64` / `loss_grad64` are the same network in plain float64 without
rounding, used to check the back-propagation against finite differences.
Only tests use this module.
"""
from __future__ import annotations

import numpy as np

N_IN, N_HID, N_OUT = 16, 64, 2
OFF = {"W1": 0, "b1": 1024, "W2": 1088, "b2": 5184, "W3": 5248, "b3": 9344, "W4": 9408, "b4": 9536}
N_PARAMS = 9538
N_NORM = 36


def bf16(x) -> np.ndarray:
    """float32 -> nearest bfloat16 (ties to even), returned as float32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)
    return np.where(np.isnan(x), x, out).astype(np.float32)


def unpack(params: np.ndarray, dtype=np.float32) -> dict:
    p = np.asarray(params, dtype=dtype)
    return {
        "W1": p[OFF["W1"]:OFF["b1"]].reshape(N_HID, N_IN),
        "b1": p[OFF["b1"]:OFF["W2"]],
        "W2": p[OFF["W2"]:OFF["b2"]].reshape(N_HID, N_HID),
        "b2": p[OFF["b2"]:OFF["W3"]],
        "W3": p[OFF["W3"]:OFF["b3"]].reshape(N_HID, N_HID),
        "b3": p[OFF["b3"]:OFF["W4"]],
        "W4": p[OFF["W4"]:OFF["b4"]].reshape(N_OUT, N_HID),
        "b4": p[OFF["b4"]:N_PARAMS],
    }


def pack(g: dict) -> np.ndarray:
    out = np.zeros(N_PARAMS, dtype=np.float64)
    for k, v in g.items():
        out[OFF[k]:OFF[k] + v.size] = np.asarray(v, dtype=np.float64).reshape(-1)
    return out


def _mm(a, b):
    """float64 product of BF16-valued operands, rounded once to float32."""
    return (np.asarray(a, np.float64) @ np.asarray(b, np.float64)).astype(np.float32)


CLIP = 8.0  # normalised inputs are clipped to [-CLIP, CLIP] (fmin/fmax: a NaN becomes the bound)


def normalise_inputs(feat, norm):
    norm = np.asarray(norm, dtype=np.float32)
    f = np.asarray(feat, dtype=np.float32)
    x = (f - norm[:N_IN]) * norm[N_IN:2 * N_IN]
    return bf16(np.fmin(np.fmax(x, np.float32(-CLIP)), np.float32(CLIP)))


def forward(params, norm, feat):
    """Network outputs (normalised units) and the intermediates of backward()."""
    P = unpack(params)
    x = normalise_inputs(feat, norm)
    W = {k: bf16(P[k]) for k in ("W1", "W2", "W3", "W4")}
    z1 = _mm(x, W["W1"].T) + P["b1"]
    h1 = bf16(np.maximum(z1, 0))
    z2 = _mm(h1, W["W2"].T) + P["b2"]
    h2 = bf16(np.maximum(z2, 0))
    z3 = _mm(h2, W["W3"].T) + P["b3"]
    h3 = bf16(np.maximum(z3, 0))
    y = _mm(h3, W["W4"].T) + P["b4"]
    return y, dict(x=x, W=W, z1=z1, h1=h1, z2=z2, h2=h2, z3=z3, h3=h3)


def predict(params, norm, feat):
    """De-normalised predictions, as shapes_mlp_forward returns them."""
    norm = np.asarray(norm, dtype=np.float32)
    y, _ = forward(params, norm, feat)
    return y * norm[2 * N_IN + 2:2 * N_IN + 4] + norm[2 * N_IN:2 * N_IN + 2]


def loss_grad(params, norm, feat, tgt):
    """(mean squared error of the normalised outputs, its gradient) with the
    kernels' BF16 rounding points."""
    norm = np.asarray(norm, dtype=np.float32)
    n = len(feat)
    y, c = forward(params, norm, feat)
    t = (np.asarray(tgt, np.float32) - norm[2 * N_IN:2 * N_IN + 2]) / norm[2 * N_IN + 2:2 * N_IN + 4]
    dy = (y - t).astype(np.float32)
    loss = float(np.sum(dy.astype(np.float64) ** 2) / n)
    W = c["W"]
    e4 = bf16(dy)
    dz3 = bf16(_mm(e4, W["W4"]) * (c["z3"] > 0))
    dz2 = bf16(_mm(dz3, W["W3"]) * (c["z2"] > 0))
    dz1 = bf16(_mm(dz2, W["W2"]) * (c["z1"] > 0))
    g = {
        "W4": _mm(e4.T, c["h3"]), "b4": e4.astype(np.float64).sum(0),
        "W3": _mm(dz3.T, c["h2"]), "b3": dz3.astype(np.float64).sum(0),
        "W2": _mm(dz2.T, c["h1"]), "b2": dz2.astype(np.float64).sum(0),
        "W1": _mm(dz1.T, c["x"]), "b1": dz1.astype(np.float64).sum(0),
    }
    return loss, pack(g) * (2.0 / n)


def forward64(params, norm, feat):
    P = unpack(params, np.float64)
    norm = np.asarray(norm, np.float64)
    x = (np.asarray(feat, np.float64) - norm[:N_IN]) * norm[N_IN:2 * N_IN]
    x = np.fmin(np.fmax(x, -CLIP), CLIP)
    z1 = x @ P["W1"].T + P["b1"]
    h1 = np.maximum(z1, 0)
    z2 = h1 @ P["W2"].T + P["b2"]
    h2 = np.maximum(z2, 0)
    z3 = h2 @ P["W3"].T + P["b3"]
    h3 = np.maximum(z3, 0)
    y = h3 @ P["W4"].T + P["b4"]
    return y, dict(x=x, P=P, z1=z1, h1=h1, z2=z2, h2=h2, z3=z3, h3=h3)


def loss_grad64(params, norm, feat, tgt):
    """The same loss and gradient in float64 without rounding."""
    norm = np.asarray(norm, np.float64)
    n = len(feat)
    y, c = forward64(params, norm, feat)
    t = (np.asarray(tgt, np.float64) - norm[2 * N_IN:2 * N_IN + 2]) / norm[2 * N_IN + 2:2 * N_IN + 4]
    dy = y - t
    P = c["P"]
    dz3 = (dy @ P["W4"]) * (c["z3"] > 0)
    dz2 = (dz3 @ P["W3"]) * (c["z2"] > 0)
    dz1 = (dz2 @ P["W2"]) * (c["z1"] > 0)
    g = {"W4": dy.T @ c["h3"], "b4": dy.sum(0), "W3": dz3.T @ c["h2"], "b3": dz3.sum(0),
         "W2": dz2.T @ c["h1"], "b2": dz2.sum(0), "W1": dz1.T @ c["x"], "b1": dz1.sum(0)}
    return float(np.sum(dy ** 2) / n), pack(g) * (2.0 / n)


def identity_norm() -> np.ndarray:
    n = np.zeros(N_NORM, dtype=np.float32)
    n[N_IN:2 * N_IN] = 1.0
    n[2 * N_IN + 2:] = 1.0
    return n
