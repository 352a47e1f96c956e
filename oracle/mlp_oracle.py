"""FP64 restatement of the start-vector MLP (spin-ed_gb300/csrc/mlp.cu).

TEST INFRASTRUCTURE ONLY: the GPU gradient tests compare the library's
forward pass, loss and gradients with this numpy version; no product code
imports it. The network has no counterpart in the reference (SpinED passes
PRIMME no start vector, src/SpinED.hs:385-394), so this file pins the
library to its own definition, written out independently:

  x_j = +1 if bit j of the state is set else -1
  h1 = tanh(W1 x + b1), h2 = tanh(W2 h1 + b2), (a, s) = W3 h2 + b3
  y = |t_sign - parity(state & sign_mask)|
  L = mean[(a - t_abs)^2 + max(s, 0) - s y + log(1 + exp(-|s|))]

with the weight matrices rounded to BF16 (round to nearest even) and the
biases kept in FP32, as the library uses them.
"""
from __future__ import annotations

import numpy as np


def bf16(a: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), as float64."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p: np.ndarray, n: int, h: int) -> dict:
    out, o = {}, 0
    for name, shp in [("W1", (h, n)), ("b1", (h,)), ("W2", (h, h)), ("b2", (h,)), ("W3", (2, h)), ("b3", (2,))]:
        k = int(np.prod(shp))
        out[name] = np.asarray(p[o:o + k], dtype=np.float32).reshape(shp)
        o += k
    return out


def spins(states: np.ndarray, n: int) -> np.ndarray:
    bits = (states[:, None] >> np.arange(n, dtype=np.uint64)[None, :]) & np.uint64(1)
    return np.where(bits == 1, 1.0, -1.0)


def parity(states: np.ndarray, mask: int) -> np.ndarray:
    v = states & np.uint64(mask)
    c = np.zeros(len(states), dtype=np.int64)
    for j in range(64):
        c += ((v >> np.uint64(j)) & np.uint64(1)).astype(np.int64)
    return (c & 1).astype(np.float64)


def forward(p, n, h, states, act_bf16=False):
    """Activations and outputs. act_bf16 rounds h1 to BF16 before the second
    layer, as the tensor-core inference path stores it."""
    w = unpack(p, n, h)
    W1, W2, W3 = bf16(w["W1"]), bf16(w["W2"]), bf16(w["W3"])
    x = spins(states, n)
    h1 = np.tanh(x @ W1.T + w["b1"])
    if act_bf16:
        h1 = bf16(h1.astype(np.float32))
    h2 = np.tanh(h1 @ W2.T + w["b2"])
    out = h2 @ W3.T + w["b3"]
    return x, h1, h2, out


def loss_grad(p, n, h, states, t_abs, t_sign, sign_mask=0, act_bf16=False):
    """Loss and gradient with respect to the FP32 parameters (the BF16
    rounding of the weights is treated as the identity in the backward pass,
    as the library does).

    act_bf16 follows the tensor-core training step instead of the CUDA-core
    one: h1, h2 and the backward activations d2, d1 are rounded to BF16 where
    the GEMMs read them (h1 and h2 as stored, d2 before dW2 and d1, d1
    before dW1), while the bias gradients db2, db1 sum the unrounded d2, d1."""
    w = unpack(p, n, h)
    W1, W2, W3 = bf16(w["W1"]), bf16(w["W2"]), bf16(w["W3"])
    x = spins(states, n)
    r = (lambda a: bf16(a.astype(np.float32))) if act_bf16 else (lambda a: a)
    h1 = r(np.tanh(x @ W1.T + w["b1"]))
    h2 = r(np.tanh(h1 @ W2.T + w["b2"]))
    out = h2 @ W3.T + w["b3"]
    N = len(states)
    a, s = out[:, 0], out[:, 1]
    y = np.abs(t_sign.astype(np.float64) - parity(states, sign_mask))
    da = a - t_abs
    loss = np.mean(da * da + np.maximum(s, 0) - s * y + np.log1p(np.exp(-np.abs(s))))
    dout = np.stack([2 * da / N, (1 / (1 + np.exp(-s)) - y) / N], axis=1)
    dW3, db3 = dout.T @ h2, dout.sum(0)
    d2 = (dout @ W3) * (1 - h2 * h2)
    dW2, db2 = r(d2).T @ h1, d2.sum(0)
    d1 = (r(d2) @ W2) * (1 - h1 * h1)
    dW1, db1 = r(d1).T @ x, d1.sum(0)
    g = np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dW3.ravel(), db3])
    return loss, g


# ------------------------------------------------------------ patch network
# The size-independent variant (sed_mlp_create_patch): the same three layers
# applied to the P spins of each site's patch (patches[i] lists the sites of
# site i's patch, in a fixed order), summed over the N sites:
#   h1_i = tanh(W1 x_i + b1), h2_i = tanh(W2 h1_i + b2),
#   (a, s) = W3 sum_i h2_i + b3.
# The parameters do not depend on N, so a network trained on one lattice
# evaluates on another with the same patch shape.

def patch_spins(states: np.ndarray, patches: np.ndarray) -> np.ndarray:
    """[B, N, P] of +1/-1: spin patches[i][j] of each state."""
    sh = patches.astype(np.uint64)[None, :, :]
    bits = (states.astype(np.uint64)[:, None, None] >> sh) & np.uint64(1)
    return np.where(bits == 1, 1.0, -1.0)


def patch_forward(p, h, states, patches, act_bf16=False):
    """Activations ([B, N, H]) and outputs ([B, 2]) of the patch network;
    act_bf16 rounds h1 and h2 to BF16 as the tensor-core passes store them."""
    P = patches.shape[1]
    w = unpack(p, P, h)
    W1, W2, W3 = bf16(w["W1"]), bf16(w["W2"]), bf16(w["W3"])
    r = (lambda a: bf16(a.astype(np.float32))) if act_bf16 else (lambda a: a)
    x = patch_spins(states, patches)
    h1 = r(np.tanh(x @ W1.T + w["b1"]))
    h2 = r(np.tanh(h1 @ W2.T + w["b2"]))
    out = h2.sum(axis=1) @ W3.T + w["b3"]
    return x, h1, h2, out


def patch_loss_grad(p, h, states, patches, t_abs, t_sign, sign_mask=0, act_bf16=False):
    """Loss and gradient of the patch network, with loss_grad's loss and
    rounding conventions (act_bf16: the tensor-core step's rounding points)."""
    P = patches.shape[1]
    w = unpack(p, P, h)
    W2, W3 = bf16(w["W2"]), bf16(w["W3"])
    r = (lambda a: bf16(a.astype(np.float32))) if act_bf16 else (lambda a: a)
    x, h1, h2, out = patch_forward(p, h, states, patches, act_bf16)
    N = len(states)
    a, s = out[:, 0], out[:, 1]
    y = np.abs(t_sign.astype(np.float64) - parity(states, sign_mask))
    da = a - t_abs
    loss = np.mean(da * da + np.maximum(s, 0) - s * y + np.log1p(np.exp(-np.abs(s))))
    dout = np.stack([2 * da / N, (1 / (1 + np.exp(-s)) - y) / N], axis=1)
    dW3, db3 = dout.T @ h2.sum(axis=1), dout.sum(0)
    d2 = (dout @ W3)[:, None, :] * (1 - h2 * h2)
    rows2, rows1 = r(d2).reshape(-1, h), h1.reshape(-1, h)
    dW2, db2 = rows2.T @ rows1, d2.sum(axis=(0, 1))
    d1 = (r(d2) @ W2) * (1 - h1 * h1)
    dW1, db1 = r(d1).reshape(-1, h).T @ x.reshape(-1, P), d1.sum(axis=(0, 1))
    g = np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dW3.ravel(), db3])
    return loss, g
