"""FP64 numpy restatement of the radiance-cache network (craystal_gb300
csrc/cr_mlp.cu): encoding, forward, relative-L2 loss, backward and Adam.

TEST INFRASTRUCTURE ONLY (the checker of the GPU kernels).  The network has
no counterpart in the reference; this is its definition.  Arithmetic is
float64; the FP16 roundings the GPU performs (weights, encoded features,
hidden activations, output gradients, hidden gradients) are applied at the
same points, so the two agree to FP32-accumulation error.
"""
import numpy as np

N_IN, N_FREQ, N_FEAT, N_HID, N_LAYERS = 7, 12, 176, 64, 6
SHAPES = [(N_FEAT, N_HID)] + [(N_HID, N_HID)] * 4 + [(N_HID, 3)]
N_PARAMS = sum(k * n for k, n in SHAPES)
GRAD_CLIP = 256.0  # per-sample |dL/dy| clip of the GPU training kernel


ROUND_FP16 = True  # the GPU's FP16 roundings; switched off to check the oracle by finite differences


def h16(x):
    if not ROUND_FP16:
        return np.asarray(x, np.float64)
    return np.asarray(x, np.float64).astype(np.float16).astype(np.float64)


def split_params(p):
    out, o = [], 0
    for k, n in SHAPES:
        out.append(np.asarray(p[o:o + k * n], np.float64).reshape(k, n))
        o += k * n
    return out


def encode(x):
    """Features j = d*24 + 2f + {0: sin, 1: cos} of (pi * 2^f * x_d), 168 of 176."""
    x = np.asarray(x, np.float64)
    n = len(x)
    feat = np.zeros((n, N_FEAT))
    for d in range(N_IN):
        for f in range(N_FREQ):
            y = np.ldexp(x[:, d].astype(np.float32), f).astype(np.float64)
            y = y - 2.0 * np.floor(y * 0.5)
            feat[:, d * 24 + 2 * f] = np.sin(np.pi * y)
            feat[:, d * 24 + 2 * f + 1] = np.cos(np.pi * y)
    return h16(feat)


def forward(params, x):
    W = [h16(w) for w in split_params(params)]
    acts = [encode(x)]
    a = acts[0]
    for l in range(N_LAYERS - 1):
        a = h16(np.maximum(a @ W[l], 0.0))
        acts.append(a)
    return a @ W[-1], acts


def loss_and_grads(params, x, t):
    y, acts = forward(params, x)
    W = [h16(w) for w in split_params(params)]
    t = np.asarray(t, np.float64)
    den = y * y + 0.01
    loss = np.mean((y - t) ** 2 / den)
    dy = h16(np.clip(2.0 * (y - t) / den, -GRAD_CLIP, GRAD_CLIP))
    scale = 1.0 / (3.0 * len(x))
    grads = [None] * N_LAYERS
    for l in range(N_LAYERS - 1, -1, -1):
        grads[l] = acts[l].T @ dy * scale
        if l > 0:
            dx = dy @ W[l].T
            dy = h16(np.where(acts[l] > 0, dx, 0.0))
    return loss, np.concatenate([g.reshape(-1) for g in grads])


def adam_step(params, m, v, grads, step, lr=1e-2, b1=0.9, b2=0.99, eps=1e-8):
    m = b1 * m + (1 - b1) * grads
    v = b2 * v + (1 - b2) * grads * grads
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return params - lr * mh / (np.sqrt(vh) + eps), m, v
