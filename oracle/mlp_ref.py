"""CPU oracle of the warm-start MLP (test infrastructure only; nothing in the product imports it).

The network has no counterpart in the reference: SPG's VBD only knows the inertial initial
guess (spg/include/spg/sim/solver/vbd.h:22, spg/source/sim/solver/vbd.cpp:78-83). This module
restates the library's definition in numpy so the GPU kernels can be checked:

  h1 = gelu(x W1 + b1), h2 = gelu(h1 W2 + b2), h3 = gelu(h2 W3 + b3), y = h3 W4 + b4
  gelu(z) = 0.5 z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3)))   (tanh form)
  loss = mean over the n x 3 outputs of (y - t)^2

Weights are used BF16-rounded (round to nearest even) in the forward pass, biases in FP32;
the rounding is passed straight through in the backward pass. Flat layout: W1[24][128] b1
W2[128][128] b2 W3[128][128] b3 W4[128][3] b4, row-major.
"""
import numpy as np

N_IN, N_HID, N_OUT = 24, 128, 3
SHAPES = [("W1", (N_IN, N_HID)), ("b1", (N_HID,)), ("W2", (N_HID, N_HID)), ("b2", (N_HID,)),
          ("W3", (N_HID, N_HID)), ("b3", (N_HID,)), ("W4", (N_HID, N_OUT)), ("b4", (N_OUT,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def bf16_round(a) -> np.ndarray:
    """Round FP32 values to the nearest BF16 (ties to even), returned as FP32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32)
    return np.where(np.isfinite(a), out, a)


def unpack(w):
    w = np.asarray(w).reshape(-1)
    assert w.size == N_PARAMS, w.size
    out, o = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = w[o:o + n].reshape(shape)
        o += n
    return out


def pack(p) -> np.ndarray:
    return np.concatenate([np.asarray(p[name]).reshape(-1) for name, _ in SHAPES])


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(0.7978845608028654 * (z + 0.044715 * z ** 3)))


def gelu_grad(z):
    t = np.tanh(0.7978845608028654 * (z + 0.044715 * z ** 3))
    du = 0.7978845608028654 * (1.0 + 3 * 0.044715 * z * z)
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * du


def quantized(w, quantize=True):
    """The forward-pass weights: BF16-rounded matrices (unless quantize is False), FP32
    biases, as FP64."""
    if not quantize:
        return {k: v.astype(np.float64) for k, v in unpack(np.asarray(w, dtype=np.float64)).items()}
    p = unpack(np.asarray(w, dtype=np.float32))
    return {k: (bf16_round(v) if k.startswith("W") else v).astype(np.float64) for k, v in p.items()}


def forward(w, x, emulate_bf16_activations=False):
    """FP64 forward pass. With emulate_bf16_activations the inputs and hidden activations are
    rounded to BF16 like the tensor-core inference kernel's operands."""
    q = quantized(w)
    x = np.asarray(x, dtype=np.float64)
    r = (lambda a: bf16_round(a.astype(np.float32)).astype(np.float64)) if emulate_bf16_activations else (lambda a: a)
    h = r(x)
    for k in (1, 2, 3):
        h = r(gelu(h @ q[f"W{k}"] + q[f"b{k}"]))
    return h @ q["W4"] + q["b4"]


def loss_grad(w, x, t, quantize=True, emulate_bf16_operands=False):
    """FP64 mean-squared-error loss and its gradient with respect to the flat weights. With
    emulate_bf16_operands every operand of the eleven matrix products is rounded to BF16 first,
    as the tensor-core GEMMs of the device training take them (the FP32 values are kept for
    the bias, GELU and loss arithmetic)."""
    q = quantized(w, quantize)
    x = np.asarray(x, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    r = (lambda a: bf16_round(np.asarray(a, dtype=np.float32)).astype(np.float64)) if emulate_bf16_operands \
        else (lambda a: a)
    z1 = r(x) @ q["W1"] + q["b1"]
    a1 = gelu(z1)
    z2 = r(a1) @ q["W2"] + q["b2"]
    a2 = gelu(z2)
    z3 = r(a2) @ q["W3"] + q["b3"]
    a3 = gelu(z3)
    y = r(a3) @ q["W4"] + q["b4"]
    e = y - t
    loss = float(np.mean(e * e))
    dy = 2.0 * e / e.size
    g = {"W4": r(a3).T @ r(dy), "b4": dy.sum(0)}
    d3 = (r(dy) @ q["W4"].T) * gelu_grad(z3)
    g["W3"], g["b3"] = r(a2).T @ r(d3), d3.sum(0)
    d2 = (r(d3) @ q["W3"].T) * gelu_grad(z2)
    g["W2"], g["b2"] = r(a1).T @ r(d2), d2.sum(0)
    d1 = (r(d2) @ q["W2"].T) * gelu_grad(z1)
    g["W1"], g["b1"] = r(x).T @ r(d1), d1.sum(0)
    return loss, pack(g)
