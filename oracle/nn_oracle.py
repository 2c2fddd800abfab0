"""CPU oracle of the neural IBL shader (test infrastructure only: the product's tensor-core kernels
in softglrender_gb300/csrc/sglc_nn.cu are checked against it; nothing in the product imports it).

It restates, in numpy, the network that softglrender_gb300/csrc/sglc_nn.cuh defines: the
6-frequency encoding of the 12 inputs (double-angle recurrence from sin/cos(pi x)), the
156 -> 64 -> 64 -> 3 ReLU MLP, the mean-squared-error loss, its gradient and the Adam update
(Kingma & Ba, "Adam: A Method for Stochastic Optimization", 2015, Algorithm 1 with bias-corrected
moments). With `bf16=True` the operands that the GPU feeds to the tensor cores (encoded inputs,
weights, hidden activations, dY, dH2, dH1) are rounded to BF16 (round to nearest even) and
products are accumulated in float64, so the only remaining difference to the device is FP32
accumulation order. With `bf16=False` it is the plain FP32 network the device approximates.

The network has no counterpart in the reference (SoftGLRender has no learned shader); what it
replaces is the IBL term of PbrSoft.h:291-309, whose own CPU restatement is the oracle library.
"""
from __future__ import annotations

import numpy as np

N_IN, N_FREQ, N_FEAT, N_HID, N_OUT = 12, 6, 156, 64, 3
SIZES = {"W1": (N_HID, N_FEAT), "b1": (N_HID,), "W2": (N_HID, N_HID), "b2": (N_HID,), "W3": (N_OUT, N_HID),
         "b3": (N_OUT,)}
ORDER = ("W1", "b1", "W2", "b2", "W3", "b3")
N_PARAMS = sum(int(np.prod(s)) for s in SIZES.values())   # 14403


def unflatten(flat: np.ndarray) -> dict:
    out, o = {}, 0
    for k in ORDER:
        n = int(np.prod(SIZES[k]))
        out[k] = np.asarray(flat[o:o + n], dtype=np.float32).reshape(SIZES[k])
        o += n
    return out


def flatten(p: dict) -> np.ndarray:
    return np.concatenate([np.asarray(p[k], dtype=np.float32).reshape(-1) for k in ORDER])


def bf16(a: np.ndarray) -> np.ndarray:
    """Round float32 to the nearest bfloat16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(a.shape)


def encode(x: np.ndarray) -> np.ndarray:
    """(n, 12) inputs -> (n, 156) features in the device order: feature 24k + 2i = sin(2^k pi x_i),
    24k + 2i + 1 = cos(2^k pi x_i) (k = 0..5), feature 144 + i = x_i. The double-angle recurrence is
    the device's (t = 2 s, s' = t c, c' = 1 - t s with one rounding)."""
    x = np.asarray(x, dtype=np.float32)
    n = x.shape[0]
    f = np.zeros((n, N_FEAT), dtype=np.float32)
    s = np.sin(np.pi * x.astype(np.float64)).astype(np.float32)
    c = np.cos(np.pi * x.astype(np.float64)).astype(np.float32)
    two = np.float32(2.0)
    for k in range(N_FREQ):
        f[:, 24 * k + 0:24 * k + 24:2] = s
        f[:, 24 * k + 1:24 * k + 24:2] = c
        t = two * s
        s, c = t * c, (1.0 - t.astype(np.float64) * s.astype(np.float64)).astype(np.float32)
    f[:, 144:156] = x
    return f


def _mm(a, b):
    return (a.astype(np.float64) @ b.astype(np.float64)).astype(np.float32)


def forward(p: dict, x: np.ndarray, use_bf16: bool = True):
    """Network outputs (n, 3) and the intermediates the backward pass needs."""
    r = bf16 if use_bf16 else (lambda a: np.asarray(a, dtype=np.float32))
    X = r(encode(x))
    W1, W2, W3 = r(p["W1"]), r(p["W2"]), r(p["W3"])
    a1 = _mm(X, W1.T) + p["b1"]
    h1 = np.maximum(a1, 0).astype(np.float32)
    H1 = r(h1)
    a2 = _mm(H1, W2.T) + p["b2"]
    h2 = np.maximum(a2, 0).astype(np.float32)
    H2 = r(h2)
    y = (_mm(H2, W3.T) + p["b3"]).astype(np.float32)
    return y, (X, H1, H2, h1 > 0, h2 > 0, W1, W2, W3)


def loss_and_grad(p: dict, x: np.ndarray, t: np.ndarray, use_bf16: bool = True):
    """Mean over records of the summed squared error of the 3 outputs, and its gradient (dict)."""
    n = x.shape[0]
    r = bf16 if use_bf16 else (lambda a: np.asarray(a, dtype=np.float32))
    y, (X, H1, H2, m1, m2, W1, W2, W3) = forward(p, x, use_bf16)
    e = (y - t).astype(np.float32)
    loss = float(np.sum(e.astype(np.float64) ** 2))
    dy = r((np.float32(2.0) * e) * np.float32(1.0 / n))
    dh2 = r(_mm(dy, W3) * m2)
    dh1 = r(_mm(dh2, W2) * m1)
    g = {
        "W3": _mm(dy.T, H2), "b3": dy.astype(np.float64).sum(0).astype(np.float32),
        "W2": _mm(dh2.T, H1), "b2": dh2.astype(np.float64).sum(0).astype(np.float32),
        "W1": _mm(dh1.T, X), "b1": dh1.astype(np.float64).sum(0).astype(np.float32),
    }
    return loss / n, g


def adam_step(p: dict, g: dict, m: dict, v: dict, step: int, lr: float, b1: float = 0.9, b2: float = 0.999,
              eps: float = 1e-8):
    """One Adam update (in place on p, m, v) at 1-based step `step`, FP32 arithmetic as on the device."""
    f = np.float32
    bc1 = f(1.0 - b1 ** step)
    bc2 = f(1.0 - b2 ** step)
    for k in ORDER:
        m[k] = f(b1) * m[k] + f(1.0 - b1) * g[k]
        v[k] = f(b2) * v[k] + f(1.0 - b2) * g[k] * g[k]
        p[k] = p[k] - f(lr) * (m[k] / bc1) / (np.sqrt(v[k] / bc2) + f(eps))


def mix64(z: np.ndarray) -> np.ndarray:
    """SplitMix64 finaliser (Steele, Lea & Flood 2014), as the device's record sampler uses it."""
    with np.errstate(over="ignore"):
        z = (z + np.uint64(0x9E3779B97F4A7C15)).astype(np.uint64)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def sample_indices(seed: int, step: int, batch: int, n_records: int) -> np.ndarray:
    """Record indices of training step `step` (0-based): mix64(seed ^ step << 32 ^ row) % n."""
    rows = np.arange(batch, dtype=np.uint64)
    key = np.uint64(seed) ^ (np.uint64(step) << np.uint64(32)) ^ rows
    return (mix64(key) % np.uint64(n_records)).astype(np.int64)


def psnr(a: np.ndarray, b: np.ndarray, peak: float = 255.0) -> float:
    d = a.astype(np.float64) - b.astype(np.float64)
    mse = float(np.mean(d * d))
    return float("inf") if mse == 0 else 10.0 * np.log10(peak * peak / mse)
