"""CPU oracle of the learned correction classifier (test infrastructure only).

The classifier is this project's own network (the reference's counterpart is
its forest/logistic-regression classifier, include/classification.hpp:51-157,
for which the project's learned decision stands in), so this oracle does not
restate reference code: it restates the device kernels' arithmetic in numpy
so that the tests can check them.

Network: 32 features -> 64 (ReLU) -> 64 (ReLU) -> 1 logit, sigmoid output.
Weights are BF16, biases FP32.  The device rounds to BF16 at the same points
as `forward`/`gradients` below: the input features, both hidden activations
after the ReLU, and the two hidden-layer gradients before they enter a matrix
product; everything else is FP32.  `forward64`/`gradients64` are the same
mathematics in float64 without any rounding, for the finite-difference check
of the gradient formulas.

Serialized model: 32-byte header {"CGMLP001", u32 32, 64, 64, payload bytes,
2 x u32 reserved}, payload w1 BF16[64][32], w2 BF16[64][64], w3 BF16[64],
b1 FP32[64], b2 FP32[64], b3 FP32, zero padding to a multiple of 16 bytes.
"""
from __future__ import annotations

import struct

import numpy as np

F, H = 32, 64
PAYLOAD = (F * H + H * H + H) * 2 + (2 * H + 1) * 4
PAYLOAD_PADDED = (PAYLOAD + 15) // 16 * 16
NPARAMS = F * H + H * H + H + 2 * H + 1


def bf16(x) -> np.ndarray:
    """Round float32 values to the nearest BF16 (ties to even), as float32."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def _from_bf16_bits(b: np.ndarray) -> np.ndarray:
    return (b.astype(np.uint32) << 16).view(np.float32)


def _to_bf16_bits(x: np.ndarray) -> np.ndarray:
    return (bf16(x).view(np.uint32) >> 16).astype(np.uint16)


def parse(model: bytes) -> dict:
    magic, f, h1, h2, payload = struct.unpack_from("<8s4I", model, 0)
    assert magic == b"CGMLP001" and (f, h1, h2) == (F, H, H) and payload == PAYLOAD_PADDED
    p = memoryview(model)[32:]
    off = 0

    def take_bf16(n):
        nonlocal off
        a = np.frombuffer(p[off:off + 2 * n], np.uint16)
        off += 2 * n
        return _from_bf16_bits(a)

    w1 = take_bf16(H * F).reshape(H, F)
    w2 = take_bf16(H * H).reshape(H, H)
    w3 = take_bf16(H)
    b = np.frombuffer(p[off:off + 4 * (2 * H + 1)], np.float32)
    return {"w1": w1, "w2": w2, "w3": w3, "b1": b[:H].copy(), "b2": b[H:2 * H].copy(), "b3": np.float32(b[2 * H])}


def serialize(m: dict) -> bytes:
    head = struct.pack("<8s4I2I", b"CGMLP001", F, H, H, PAYLOAD_PADDED, 0, 0)
    body = (_to_bf16_bits(m["w1"]).tobytes() + _to_bf16_bits(m["w2"]).tobytes() + _to_bf16_bits(m["w3"]).tobytes()
            + np.asarray(m["b1"], np.float32).tobytes() + np.asarray(m["b2"], np.float32).tobytes()
            + np.float32(m["b3"]).tobytes())
    return head + body + b"\0" * (PAYLOAD_PADDED - len(body))


def random_model(seed: int, scale: float = 1.0) -> dict:
    rng = np.random.default_rng(seed)

    def u(shape, fan):
        lim = np.sqrt(6.0 / fan) * scale
        return bf16(rng.uniform(-lim, lim, shape).astype(np.float32))

    return {"w1": u((H, F), F), "w2": u((H, H), H), "w3": u((H,), H),
            "b1": rng.normal(0, 0.1, H).astype(np.float32), "b2": rng.normal(0, 0.1, H).astype(np.float32),
            "b3": np.float32(rng.normal(0, 0.1))}


def forward(m: dict, x: np.ndarray):
    xb = bf16(x)
    z1 = xb @ m["w1"].T + m["b1"]
    h1 = bf16(np.maximum(z1, 0))
    z2 = h1 @ m["w2"].T + m["b2"]
    h2 = bf16(np.maximum(z2, 0))
    z = (h2 @ m["w3"] + m["b3"]).astype(np.float32)
    return z, xb, h1, h2


def _loss(z, y):
    return np.maximum(z, 0) + np.log1p(np.exp(-np.abs(z))) - y * z


def gradients(m: dict, x: np.ndarray, y: np.ndarray):
    """Mean BCE loss and its gradient in parameter order (w1, w2, w3, b1, b2, b3)."""
    y = np.asarray(y, np.float32)
    n = len(x)
    z, xb, h1, h2 = forward(m, x)
    p = 1.0 / (1.0 + np.exp(-z))
    dz = ((p - y) / np.float32(n)).astype(np.float32)
    gw3 = dz @ h2
    gb3 = dz.sum()
    d2 = (dz[:, None] * m["w3"][None, :]) * (h2 > 0)
    gb2 = d2.sum(0)
    d2b = bf16(d2)
    gw2 = d2b.T @ h1
    d1 = (d2b @ m["w2"]) * (h1 > 0)
    gb1 = d1.sum(0)
    d1b = bf16(d1)
    gw1 = d1b.T @ xb
    g = np.concatenate([gw1.ravel(), gw2.ravel(), gw3, gb1, gb2, [gb3]]).astype(np.float32)
    return float(_loss(z, y).mean()), g


def forward64(m: dict, x: np.ndarray):
    w1, w2, w3 = (np.asarray(m[k], np.float64) for k in ("w1", "w2", "w3"))
    z1 = x @ w1.T + m["b1"]
    h1 = np.maximum(z1, 0)
    z2 = h1 @ w2.T + m["b2"]
    h2 = np.maximum(z2, 0)
    return h2 @ w3 + float(m["b3"]), h1, h2


def loss64(m: dict, x: np.ndarray, y: np.ndarray) -> float:
    z, _, _ = forward64(m, np.asarray(x, np.float64))
    return float(_loss(z, np.asarray(y, np.float64)).mean())


def gradients64(m: dict, x: np.ndarray, y: np.ndarray) -> np.ndarray:
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    z, h1, h2 = forward64(m, x)
    dz = (1.0 / (1.0 + np.exp(-z)) - y) / len(x)
    w2, w3 = np.asarray(m["w2"], np.float64), np.asarray(m["w3"], np.float64)
    d2 = dz[:, None] * w3[None, :] * (h2 > 0)
    d1 = (d2 @ w2) * (h1 > 0)
    return np.concatenate([(d1.T @ x).ravel(), (d2.T @ h1).ravel(), dz @ h2, d1.sum(0), d2.sum(0), [dz.sum()]])


def unflatten(m: dict, v: np.ndarray) -> dict:
    """A model with the parameters of `v` (parameter order), in float64."""
    i = 0
    out = {}
    for k, shape in (("w1", (H, F)), ("w2", (H, H)), ("w3", (H,)), ("b1", (H,)), ("b2", (H,)), ("b3", ())):
        n = int(np.prod(shape)) if shape else 1
        out[k] = np.asarray(v[i:i + n], np.float64).reshape(shape) if shape else float(v[i])
        i += n
    return out


def flatten(m: dict) -> np.ndarray:
    return np.concatenate([np.ravel(m["w1"]), np.ravel(m["w2"]), np.ravel(m["w3"]), np.ravel(m["b1"]),
                           np.ravel(m["b2"]), [float(m["b3"])]]).astype(np.float64)
