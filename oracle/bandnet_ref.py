"""CPU reference of the band-proposal MLP (features, forward, backward).

TEST INFRASTRUCTURE ONLY: the gradient check for the GPU kernels in
mauve-py_gb300/csrc/mlp.cu.  Float64 arithmetic with the same bf16
roundings the GPU applies between layers (weights, activations and the
backward GEMM operands), so the two agree to accumulation-order error.
"""
import numpy as np

N_IN, N_HID, N_OUT = 528, 256, 2


def bf16(x):
    """Round float values to bfloat16 (nearest-even), returned as float64."""
    f = np.ascontiguousarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def features(sa, oa, sb, ob):
    """4-mer spectra (counts * 256 / (L-3)) of both sequences and log(L)/5, bf16-rounded."""
    n = len(oa) - 1
    X = np.zeros((n, N_IN), np.float32)
    for p in range(n):
        for side, (s, o) in enumerate(((sa, oa), (sb, ob))):
            x = s[int(o[p]):int(o[p + 1])].astype(np.int64) & 3
            L = len(x)
            if L > 3:
                code = (x[:-3] << 6) | (x[1:-2] << 4) | (x[2:-1] << 2) | x[3:]
                cnt = np.bincount(code, minlength=256).astype(np.float32)
                X[p, side * 256:(side + 1) * 256] = cnt * np.float32(256.0 / (L - 3))
        X[p, 512] = np.float32(np.log(np.float32(oa[p + 1] - oa[p]))) * np.float32(0.2)
        X[p, 513] = np.float32(np.log(np.float32(ob[p + 1] - ob[p]))) * np.float32(0.2)
    return bf16(X)


def unpack(params):
    p = np.asarray(params, np.float64)
    dims = [(N_HID, N_IN), (N_HID, N_HID), (N_HID, N_HID), (N_OUT, N_HID)]
    out, k = [], 0
    for o, i in dims:
        W = p[k:k + o * i].reshape(o, i)
        k += o * i
        b = p[k:k + o]
        k += o
        out.append((W, b))
    return out


def _erf(x):
    from math import erf
    return np.vectorize(erf)(x)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + _erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2 * np.pi)


def loss_and_grads(params, X, T):
    """Mean over rows of sum_k (o_k - t_k)^2 and its gradient (flat layout)."""
    layers = unpack(params)
    Wb = [bf16(W) for W, _ in layers]
    h = X
    zs, hs = [], [X]
    for q in range(3):
        z = h @ Wb[q].T + layers[q][1]
        zs.append(z)
        h = bf16(gelu(z))
        hs.append(h)
    o = h @ Wb[3].T + layers[3][1]
    n = X.shape[0]
    diff = o - T
    loss = float(np.sum(diff * diff) / n)
    d = 2.0 * diff / n
    grads = [None] * 4
    db = d.sum(0)
    dq = bf16(d)
    grads[3] = (dq.T @ hs[3], db)
    dh = dq @ Wb[3]
    for q in (2, 1, 0):
        dz = dh * gelu_grad(zs[q])
        dzq = bf16(dz)
        grads[q] = (dzq.T @ hs[q], dz.sum(0))
        dh = dzq @ Wb[q]
    flat = np.concatenate([np.concatenate([g[0].ravel(), g[1]]) for g in grads])
    return loss, flat


def forward(params, X):
    layers = unpack(params)
    h = X
    for q in range(3):
        h = bf16(gelu(h @ bf16(layers[q][0]).T + layers[q][1]))
    return h @ bf16(layers[3][0]).T + layers[3][1]
