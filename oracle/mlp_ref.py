"""Reference forward/backward of the denoiser MLP in numpy.  TEST
INFRASTRUCTURE ONLY (the checker of the GPU training kernels).

Same network and rounding points as the GPU path (compound-ray_gb300/csrc/
denoiser.cpp): bf16 copies of the weights, bf16 hidden activations after
ReLU, bf16 output gradient and bf16 back-propagated gradients after the ReLU
mask; everything else accumulates in float64 here (fp32 on the GPU).
"""
import numpy as np

FEAT = 112
HID = 128
OUT = 8
OFF_W1 = 0
OFF_B1 = OFF_W1 + FEAT * HID
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + HID * HID
OFF_W4 = OFF_B3 + HID
OFF_B4 = OFF_W4 + HID * OUT
N_PARAMS = OFF_B4 + OUT


def bf16(x):
    """Round float32 values to bfloat16 (nearest even) and back."""
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return rounded.astype(np.uint32).view(np.float32)


def bf16_bits(x):
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    return (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) & 0xFFFF).astype(np.uint16)


def unpack(params):
    p = np.asarray(params, np.float32)
    return (p[OFF_W1:OFF_B1].reshape(FEAT, HID), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(HID, HID),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3].reshape(HID, HID), p[OFF_B3:OFF_W4], p[OFF_W4:OFF_B4].reshape(HID, OUT),
            p[OFF_B4:N_PARAMS])


def forward_backward(params, X, base, target):
    """Loss and gradient vector (layout of the parameter vector)."""
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(params)
    W1b, W2b, W3b, W4b = (bf16(w).astype(np.float64) for w in (W1, W2, W3, W4))
    X = bf16(X).astype(np.float64)
    H1 = bf16(np.maximum(X @ W1b + b1, 0).astype(np.float32)).astype(np.float64)
    H2 = bf16(np.maximum(H1 @ W2b + b2, 0).astype(np.float32)).astype(np.float64)
    H3 = bf16(np.maximum(H2 @ W3b + b3, 0).astype(np.float32)).astype(np.float64)
    Y = H3 @ W4b + b4
    rows = len(X)
    pred = base + Y[:, :3]
    diff = pred - target
    loss = float((diff ** 2).mean())
    dY = np.zeros((rows, OUT))
    dY[:, :3] = 2.0 * diff / (3.0 * rows)
    dYb = bf16(dY.astype(np.float32)).astype(np.float64)
    g = np.zeros(N_PARAMS)
    g[OFF_W4:OFF_B4] = (H3.T @ dYb).ravel()
    g[OFF_B4:N_PARAMS] = dY.sum(0)
    dZ3 = bf16(((dYb @ W4b.T) * (H3 > 0)).astype(np.float32)).astype(np.float64)
    g[OFF_W3:OFF_B3] = (H2.T @ dZ3).ravel()
    g[OFF_B3:OFF_W4] = dZ3.sum(0)
    dZ2 = bf16(((dZ3 @ W3b.T) * (H2 > 0)).astype(np.float32)).astype(np.float64)
    g[OFF_W2:OFF_B2] = (H1.T @ dZ2).ravel()
    g[OFF_B2:OFF_W3] = dZ2.sum(0)
    dZ1 = bf16(((dZ2 @ W2b.T) * (H1 > 0)).astype(np.float32)).astype(np.float64)
    g[OFF_W1:OFF_B1] = (X.T @ dZ1).ravel()
    g[OFF_B1:OFF_W2] = dZ1.sum(0)
    return loss, g


def from_bits(bits):
    """bf16 bit patterns -> float32."""
    return (np.asarray(bits, np.uint16).astype(np.uint32) << 16).view(np.float32)


def predict(params, X, base):
    """base + network(X)[:, :3] with the GPU path's rounding points."""
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(params)
    W1b, W2b, W3b, W4b = (bf16(w).astype(np.float64) for w in (W1, W2, W3, W4))
    X = bf16(X).astype(np.float64)
    H1 = bf16(np.maximum(X @ W1b + b1, 0).astype(np.float32)).astype(np.float64)
    H2 = bf16(np.maximum(H1 @ W2b + b2, 0).astype(np.float32)).astype(np.float64)
    H3 = bf16(np.maximum(H2 @ W3b + b3, 0).astype(np.float32)).astype(np.float64)
    return base + (H3 @ W4b + b4)[:, :3]


def adam_step(w, g, m, v, lr, c1, c2, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (Kingma & Ba 2015) in float32, one correctly rounded
    operation at a time in the order of the GPU's adamKernel
    (compound-ray_gb300/csrc/mlp.cu): m = b1 m + (1 - b1) g,
    v = b2 v + ((1 - b2) g) g, w = w - (lr (m c1)) / (sqrt(v c2) + eps), with
    c1 = 1 / (1 - b1^t) and c2 = 1 / (1 - b2^t) given.  Returns (w, m, v,
    bf16 bit patterns of w)."""
    f = np.float32
    w, g, m, v = (np.asarray(a, np.float32) for a in (w, g, m, v))
    b1, b2, eps, lr, c1, c2 = f(b1), f(b2), f(eps), f(lr), f(c1), f(c2)
    with np.errstate(over="ignore", invalid="ignore", divide="ignore"):
        m = (b1 * m) + ((f(1) - b1) * g)
        v = (b2 * v) + (((f(1) - b2) * g) * g)
        w = w - ((lr * (m * c1)) / (np.sqrt(v * c2) + eps))
    return w.astype(np.float32), m.astype(np.float32), v.astype(np.float32), bf16_bits(w)


def forward_parts(params, X):
    """The forward pass with the GPU path's rounding points: the bf16 hidden
    activations H1..H3 (float64 values) and the output layer's inputs and
    weights, for error bounds of the GPU's fp32 sums."""
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(params)
    W1b, W2b, W3b, W4b = (bf16(w).astype(np.float64) for w in (W1, W2, W3, W4))
    X = bf16(X).astype(np.float64)
    H1 = bf16(np.maximum(X @ W1b + b1, 0).astype(np.float32)).astype(np.float64)
    H2 = bf16(np.maximum(H1 @ W2b + b2, 0).astype(np.float32)).astype(np.float64)
    H3 = bf16(np.maximum(H2 @ W3b + b3, 0).astype(np.float32)).astype(np.float64)
    return X, (H1, H2, H3), (W1b, W2b, W3b, W4b)


def gradient_magnitudes(params, X, base, target):
    """Per parameter, the sum of the absolute values of the terms its gradient
    adds up (weights: sum over rows of |input| * |upstream gradient|; biases:
    sum of |upstream gradient|): the scale against which bf16 rounding steps
    and fp32 summation order are measured.  The upstream gradients pass each
    ReLU where the reference's mask is open, and also where the
    pre-activation lies within a few bf16 steps (2^-6 relative to the sum of
    its absolute terms) of zero, where the GPU's mask may differ."""
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(params)
    Xb, (H1, H2, H3), (W1b, W2b, W3b, W4b) = forward_parts(params, X)
    rows = len(Xb)
    pred = base + (H3 @ W4b + b4)[:, :3]
    dY = np.zeros((rows, OUT))
    dY[:, :3] = 2.0 * (pred - target) / (3.0 * rows)

    def gate(Hin, Wb, b):
        z = Hin @ Wb + b
        scale = np.abs(Hin) @ np.abs(Wb) + np.abs(b)
        return (z > 0) | (np.abs(z) <= 2.0 ** -6 * scale)

    m1, m2, m3 = gate(Xb, W1b, b1), gate(H1, W2b, b2), gate(H2, W3b, b3)
    g = np.zeros(N_PARAMS)
    aY = np.abs(dY)
    g[OFF_W4:OFF_B4] = (np.abs(H3).T @ aY).ravel()
    g[OFF_B4:N_PARAMS] = aY.sum(0)
    a3 = (aY @ np.abs(W4b).T) * m3
    g[OFF_W3:OFF_B3] = (np.abs(H2).T @ a3).ravel()
    g[OFF_B3:OFF_W4] = a3.sum(0)
    a2 = (a3 @ np.abs(W3b).T) * m2
    g[OFF_W2:OFF_B2] = (np.abs(H1).T @ a2).ravel()
    g[OFF_B2:OFF_W3] = a2.sum(0)
    a1 = (a2 @ np.abs(W2b).T) * m1
    g[OFF_W1:OFF_B1] = (np.abs(Xb).T @ a1).ravel()
    g[OFF_B1:OFF_W2] = a1.sum(0)
    return g
