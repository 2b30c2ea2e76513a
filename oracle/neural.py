"""CPU restatement of the learned texture decoder, for tests only (never imported by the library).

The decoder has no counterpart in the reference. What it reproduces is the plain sampler's point
sample of a texel (SampleLevel<SurfaceSampler> with nearest filtering, src/SwRast/Texture.h:412-459,
over the tiled layout of Texture.h:314-329); layer 1 holds NX, NY, M, R (src/SwRast/Scene.h:9,
Scene.cpp:31-34) and AO has no channel, so its target is the constant 1.

Model, as the device kernels compute it:
  taps:   texture level L reads latent level max(L-2, 0) (latent level k has texture level k+2's
          size) at x = (2 tx + 1) / (2 s) - 1/2, s = 4, 2, 1 for L = 0, 1, >= 2; wrap, bilinear;
  input:  x0 = ((c00 gx + c10 fx) gy + (c01 gx + c11 fx) fy) in float32 from FP16-rounded corners,
          rounded to BF16, followed by a constant 1 (the first bias), the flags L == 0 and L == 1,
          and five zeros;
  layers: z1 = X0 W1^T; h1 = bf16(gelu(z1)); z2 = h1 W2^T + b2; h2 = bf16(gelu(z2)); y = h2 W3^T + b3
          with BF16 weights and the tanh form of GELU (the device's tanh.approx.f32 differs from
          float64 tanh by a few 1e-4, so activations can round to a neighbouring BF16 value);
  loss:   per 128-sample tile, mean over its 128 x 8 outputs of (y - t)^2, summed over tiles;
  back:   dy = bf16(2/1024 (y - t)); dh2 = bf16((dy W3) gelu'(z2)); dh1 = bf16((dh2 W2) gelu'(z1));
          dx0 = dh1 W1; weight gradients from the BF16 activations; latent gradient = dx0 scattered
          at the bilinear weights (roundings treated as identity).
`exact=True` drops every rounding (float64 throughout) for finite-difference checks.
"""
from __future__ import annotations

import math

import numpy as np

PARAMS = 5704
PW1, PW2, PB2, PW3, PB3 = 0, 1024, 5120, 5184, 5696
GRAD_SCALE = 2.0 / 1024.0



def bf16(x: np.ndarray) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)


def f16(x: np.ndarray) -> np.ndarray:
    return np.asarray(x, dtype=np.float32).astype(np.float16).astype(np.float32)


GELU_A, GELU_B = math.sqrt(2.0 / math.pi), 0.044715


def gelu(x):
    """GELU, tanh form (Hendrycks & Gimpel, 2016), in float64 (the device uses tanh.approx.f32)."""
    return 0.5 * x * (1.0 + np.tanh(GELU_A * (x + GELU_B * x ** 3)))


def gelu_grad(x):
    t = np.tanh(GELU_A * (x + GELU_B * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * GELU_A * (1.0 + 3.0 * GELU_B * x * x)


def unpack_params(p: np.ndarray):
    p = np.asarray(p)
    return (p[PW1:PW2].reshape(64, 16), p[PW2:PB2].reshape(64, 64), p[PB2:PW3], p[PW3:PB3].reshape(8, 64), p[PB3:PARAMS])


def pack_params(W1, W2, b2, W3, b3) -> np.ndarray:
    return np.concatenate([np.asarray(W1).reshape(-1), np.asarray(W2).reshape(-1), b2, np.asarray(W3).reshape(-1), b3])


def unpack_texel(packed):
    packed = np.asarray(packed, dtype=np.uint32)
    return packed >> 28, packed & 0x3FFF, (packed >> 14) & 0x3FFF


# ------------------------------------------------------------------ plain texels (targets)
def texel_offset(x, y, stride):
    x = np.asarray(x, dtype=np.int64)
    y = np.asarray(y, dtype=np.int64)
    return (y & 7) | (x << 3) | ((y & ~7) << stride)


def plain_texels(data: np.ndarray, row_shift: int, mip_offsets, layer_stride: int, num_layers: int, level, x, y):
    """Raw RGBA8 words (layer 0, layer 1) of texels from a texture's storage (Texture2D::Data)."""
    level = np.asarray(level, dtype=np.int64)
    off = np.asarray(mip_offsets, dtype=np.int64)[level] + texel_offset(x, y, row_shift - level)
    a0 = data[off].astype(np.uint32)
    a1 = data[layer_stride + off].astype(np.uint32) if num_layers >= 2 else np.zeros_like(a0)
    return a0, a1


def targets_from_words(a0, a1) -> np.ndarray:
    t = np.stack([a0 & 255, (a0 >> 8) & 255, (a0 >> 16) & 255, a1 & 255, (a1 >> 8) & 255, (a1 >> 16) & 255, a1 >> 24],
                 axis=-1).astype(np.float32) * np.float32(1.0 / 255.0)
    return np.concatenate([t, np.ones(t.shape[:-1] + (1,), np.float32)], axis=-1)


# ------------------------------------------------------------------ latent taps and inputs
def latent_taps(level, tx, ty, level_w, level_h, level_offset):
    """Taps of texture level `level` texels on latent level max(level-2, 0) (sizes/offsets per latent level)."""
    level = np.asarray(level, dtype=np.int64)
    lat = np.maximum(level - 2, 0)
    inv = np.where(level == 0, np.float32(0.125), np.where(level == 1, np.float32(0.25), np.float32(0.5)))
    LW = np.asarray(level_w, dtype=np.int64)[lat]
    LH = np.asarray(level_h, dtype=np.int64)[lat]
    lx = (2 * np.asarray(tx, np.int64) + 1).astype(np.float32) * inv.astype(np.float32) - np.float32(0.5)
    ly = (2 * np.asarray(ty, np.int64) + 1).astype(np.float32) * inv.astype(np.float32) - np.float32(0.5)
    flx, fly = np.floor(lx), np.floor(ly)
    fx, fy = (lx - flx).astype(np.float32), (ly - fly).astype(np.float32)
    x0, y0 = flx.astype(np.int64), fly.astype(np.int64)
    x0 = np.where(x0 < 0, x0 + LW, x0)
    y0 = np.where(y0 < 0, y0 + LH, y0)
    x1 = np.where(x0 + 1 == LW, 0, x0 + 1)
    y1 = np.where(y0 + 1 == LH, 0, y0 + 1)
    b = np.asarray(level_offset, dtype=np.int64)[lat]
    idx = np.stack([b + y0 * LW + x0, b + y0 * LW + x1, b + y1 * LW + x0, b + y1 * LW + x1], axis=-1)
    return idx, fx, fy


def latent_inputs(latents: np.ndarray, idx, fx, fy, exact: bool = False) -> np.ndarray:
    if exact:
        c = latents.astype(np.float64)[idx]
        gx, gy = 1.0 - fx.astype(np.float64), 1.0 - fy.astype(np.float64)
        fxx, fyy = fx.astype(np.float64)[:, None], fy.astype(np.float64)[:, None]
        return (c[:, 0] * gx[:, None] + c[:, 1] * fxx) * gy[:, None] + (c[:, 2] * gx[:, None] + c[:, 3] * fxx) * fyy
    c = f16(latents[idx])
    gx, gy = (np.float32(1.0) - fx)[:, None], (np.float32(1.0) - fy)[:, None]
    fxx, fyy = fx[:, None], fy[:, None]
    return ((c[:, 0] * gx + c[:, 1] * fxx) * gy + (c[:, 2] * gx + c[:, 3] * fxx) * fyy).astype(np.float32)


def bilinear_weights(fx, fy):
    gx, gy = 1.0 - fx.astype(np.float64), 1.0 - fy.astype(np.float64)
    return np.stack([gx * gy, fx * gy, gx * fy, fx * fy], axis=-1)


# ------------------------------------------------------------------ network
def forward(params: np.ndarray, x0: np.ndarray, level=None, exact: bool = False) -> dict:
    """level: texture level of each row (its L == 0 / L == 1 flags feed W1 columns 9 and 10)."""
    W1, W2, b2, W3, b3 = unpack_params(params)
    rnd = (lambda a: np.asarray(a, np.float64)) if exact else (lambda a: bf16(a).astype(np.float64))
    n = x0.shape[0]
    X = np.zeros((n, 16))
    X[:, :8] = rnd(x0)
    X[:, 8] = 1.0
    if level is not None:
        level = np.asarray(level)
        X[:, 9] = level == 0
        X[:, 10] = level == 1
    W1b, W2b, W3b = rnd(W1), rnd(W2), rnd(W3)
    z1 = X @ W1b.T
    h1 = rnd(gelu(z1))
    z2 = h1 @ W2b.T + b2.astype(np.float64)
    h2 = rnd(gelu(z2))
    y = h2 @ W3b.T + b3.astype(np.float64)
    return {"X": X, "z1": z1, "h1": h1, "z2": z2, "h2": h2, "y": y, "W1": W1b, "W2": W2b, "W3": W3b}


def backward(params: np.ndarray, cache: dict, targets: np.ndarray, exact: bool = False):
    """Returns (param_grad[5704] float64, dx0[n, 8], loss) for the loss of the module docstring."""
    rnd = (lambda a: np.asarray(a, np.float64)) if exact else (lambda a: bf16(a).astype(np.float64))
    e = cache["y"] - targets.astype(np.float64)
    loss = float((e * e).sum())
    dy = np.zeros((e.shape[0], 16))
    dy[:, :8] = rnd(e * GRAD_SCALE)
    W3p = np.zeros((16, 64))
    W3p[:8] = cache["W3"]
    dh2 = rnd((dy @ W3p) * gelu_grad(cache["z2"]))
    dh1 = rnd((dh2 @ cache["W2"]) * gelu_grad(cache["z1"]))
    dx0 = (dh1 @ cache["W1"])[:, :8]
    g = np.zeros(PARAMS)
    g[PW1:PW2] = (dh1.T @ cache["X"]).reshape(-1)
    g[PW2:PB2] = (dh2.T @ cache["h1"]).reshape(-1)
    g[PB2:PW3] = dh2.sum(0)
    g[PW3:PB3] = (dy[:, :8].T @ cache["h2"]).reshape(-1)
    g[PB3:PARAMS] = dy[:, :8].sum(0)
    return g, dx0, loss


def latent_gradient(dx0: np.ndarray, idx, fx, fy, texels: int) -> np.ndarray:
    w = bilinear_weights(fx, fy)
    out = np.zeros((texels, 8))
    for k in range(4):
        np.add.at(out, idx[:, k], w[:, k:k + 1] * dx0)
    return out


def quantize(y: np.ndarray) -> np.ndarray:
    """Decoded outputs as the device stores them: unorm8 per channel, round to nearest."""
    return np.rint(np.clip(y, 0.0, 1.0) * 255.0).astype(np.int64)


def psnr(a: np.ndarray, b: np.ndarray, peak: float = 1.0) -> float:
    mse = float(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2))
    return float("inf") if mse == 0 else 10.0 * math.log10(peak * peak / mse)
