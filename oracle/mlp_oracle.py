"""CPU oracle of the learned-shading network (TEST INFRASTRUCTURE ONLY).

A float64 numpy restatement of what srp_gb300/csrc/k_mlp.cu computes, used by
tests/ as the checker of the GPU kernels; the product never imports it. The
network has no counterpart in kitrofimov/srp, so this restates the
library's own definition (srp_gb300/csrc/mlp.h):

  encoding   feature f of 108: component c = f // 12 of (position, unit
             normal, unit view direction), band b = (f % 12) // 2,
             sin (even f) / cos (odd f) of 2**b * pi * x_c
  network    H1 = relu(X W1 + b1), H2, H3 likewise, Y = H3 W4 + b4
  loss       mean over the batch and the 3 channels of (Y - T)**2
  Adam       beta1 0.9, beta2 0.999, eps 1e-8, rate lr * (1 + cos(pi (t-1)/T)) / 2
  batch      row i of step t takes sample mix(t * 0x9E3779B9 ^ mix(i + 0x632BE5AB)) % n
"""
import numpy as np

IN, HID, OUT = 108, 64, 3
SIZES = [("W1", (IN, HID)), ("b1", (HID,)), ("W2", (HID, HID)), ("b2", (HID,)),
         ("W3", (HID, HID)), ("b3", (HID,)), ("W4", (HID, OUT)), ("b4", (OUT,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(p):
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + n], dtype=np.float64).reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([d[name].reshape(-1) for name, _ in SIZES])


def encode(samples):
    x = np.asarray(samples, dtype=np.float64)[:, :9]
    cols = []
    for c in range(9):
        for b in range(6):
            a = np.float32(np.pi * (1 << b)) * x[:, c].astype(np.float32)
            cols.append(np.sin(a.astype(np.float64)))
            cols.append(np.cos(a.astype(np.float64)))
    return np.stack(cols, axis=1)


def forward(p, samples):
    w = unpack(p)
    X = encode(samples)
    H1 = np.maximum(X @ w["W1"] + w["b1"], 0)
    H2 = np.maximum(H1 @ w["W2"] + w["b2"], 0)
    H3 = np.maximum(H2 @ w["W3"] + w["b3"], 0)
    Y = H3 @ w["W4"] + w["b4"]
    return Y, (X, H1, H2, H3)


def loss_and_grad(p, samples):
    """Summed squared error and the gradient of the mean squared error."""
    w = unpack(p)
    Y, (X, H1, H2, H3) = forward(p, samples)
    T = np.asarray(samples, dtype=np.float64)[:, 9:12]
    B = len(samples)
    d = Y - T
    dY = 2.0 * d / (OUT * B)
    g = {"W4": H3.T @ dY, "b4": dY.sum(0)}
    dH3 = (dY @ w["W4"].T) * (H3 > 0)
    g["W3"], g["b3"] = H2.T @ dH3, dH3.sum(0)
    dH2 = (dH3 @ w["W3"].T) * (H2 > 0)
    g["W2"], g["b2"] = H1.T @ dH2, dH2.sum(0)
    dH1 = (dH2 @ w["W2"].T) * (H1 > 0)
    g["W1"], g["b1"] = X.T @ dH1, dH1.sum(0)
    return float((d * d).sum()), pack(g)


def mix(x):
    x = np.asarray(x, dtype=np.uint64) & 0xFFFFFFFF
    x ^= x >> 16
    x = (x * 0x7FEB352D) & 0xFFFFFFFF
    x ^= x >> 15
    x = (x * 0x846CA68B) & 0xFFFFFFFF
    x ^= x >> 16
    return x


def batch_indices(step, B, n):
    i = np.arange(B, dtype=np.uint64)
    h = mix(((np.uint64(step) * np.uint64(0x9E3779B9)) & np.uint64(0xFFFFFFFF)) ^ mix(i + np.uint64(0x632BE5AB)))
    return (h % np.uint64(n)).astype(np.int64)


def adam_step(p, g, m, v, t, total, lr):
    frac = min((t - 1) / total, 1.0) if total > 0 else 0.0
    rate = lr * 0.5 * (1.0 + np.cos(np.pi * frac))
    m = 0.9 * m + 0.1 * g
    v = 0.999 * v + 0.001 * g * g
    c1, c2 = 1 - 0.9 ** t, 1 - 0.999 ** t
    return p - rate * (m / c1) / (np.sqrt(v / c2) + 1e-8), m, v
