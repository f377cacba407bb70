"""CPU oracle of the learned-triage network — TEST INFRASTRUCTURE ONLY.

float64 numpy restatement of the library's MLP (saber_gb300/csrc/triage.cu):
inputs normalised with the model's mu / isd, weights rounded to bf16 (round
to nearest even) as the GPU forward pass uses them, ReLU hidden layers, one
logit, binary cross-entropy with positives weighted by pos_weight, mean over
the rows; gradients with respect to the (fp32 master) weights through the
bf16 rounding taken as the identity.  Used by the tests to check the GPU
forward and backward kernels; never by the library.
"""
import numpy as np

IN, FEAT, HID = 32, 24, 256
OFF_B1 = IN * HID
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + HID
OFF_MU = OFF_B3 + 1
OFF_ISD = OFF_MU + IN
NFLOAT = OFF_ISD + IN


def bf16_round(a):
    """float32 -> nearest bf16 (ties to even), returned as float64."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(model, bf16=True):
    m = np.asarray(model, np.float32)
    r = bf16_round if bf16 else (lambda a: np.asarray(a, np.float64))
    return dict(W1=r(m[:OFF_B1]).reshape(IN, HID), b1=m[OFF_B1:OFF_W2].astype(np.float64),
                W2=r(m[OFF_W2:OFF_B2]).reshape(HID, HID), b2=m[OFF_B2:OFF_W3].astype(np.float64),
                W3=r(m[OFF_W3:OFF_B3]), b3=float(m[OFF_B3]), mu=m[OFF_MU:OFF_ISD].astype(np.float64),
                isd=m[OFF_ISD:].astype(np.float64))


def normalize(p, X):
    x = np.asarray(X, np.float64).reshape(-1, IN).copy()
    x[:, :FEAT] = (x[:, :FEAT] - p["mu"][:FEAT]) * p["isd"][:FEAT]
    x[:, FEAT:] = 0.0
    return x


def forward(model, X, bf16=True):
    p = unpack(model, bf16)
    xn = normalize(p, X)
    h1 = np.maximum(xn @ p["W1"] + p["b1"], 0.0)
    h2 = np.maximum(h1 @ p["W2"] + p["b2"], 0.0)
    return h2 @ p["W3"] + p["b3"], (xn, h1, h2, p)


def loss_and_grads(model, X, y, pos_weight=1.0, bf16=True):
    z, (xn, h1, h2, p) = forward(model, X, bf16)
    y = np.asarray(y, np.float64)
    n = max(len(y), 1)
    w = np.where(y > 0, pos_weight, 1.0)
    loss = float(np.sum(w * (np.log1p(np.exp(-np.abs(z))) + np.maximum(z, 0.0) - y * z)) / n)
    dz = w * (1.0 / (1.0 + np.exp(-z)) - y) / n
    g = np.zeros(NFLOAT, np.float64)
    g[OFF_W3:OFF_B3] = h2.T @ dz
    g[OFF_B3] = dz.sum()
    dh2 = np.outer(dz, p["W3"]) * (h2 > 0)
    g[OFF_W2:OFF_B2] = (h1.T @ dh2).ravel()
    g[OFF_B2:OFF_W3] = dh2.sum(axis=0)
    dh1 = (dh2 @ p["W2"].T) * (h1 > 0)
    g[:OFF_B1] = (xn.T @ dh1).ravel()
    g[OFF_B1:OFF_W2] = dh1.sum(axis=0)
    return loss, g
