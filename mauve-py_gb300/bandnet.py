"""Learned band proposal for the gap DP.

A small MLP (528 -> 256 -> 256 -> 256 -> 2, GELU; kernels in csrc/mlp.cu,
BF16 tensor-core GEMMs with FP32 accumulation) predicts, for each gap, the
diagonal offset and half-width of a band for mvg_gapdp_banded.  The banded
DP keeps a result only when it provably equals the full DP, so a proposal
that is too narrow costs a fallback, never a wrong answer.

Labels come from the exact full DP run on the GPU: the optimal path's
envelope (extreme deviations from the diagonal j = i*LB/LA) gives the
offset, and the half-width is the larger of the envelope half-width and
an estimate of the width the exactness check needs.  The check bounds a
path leaving the band by its exit score plus the sum of the best per-base
scores of what remains; an exit k columns off the optimal path costs one
gap (400) and forgoes about 155 per skipped base, so bands need roughly
(best total - score - 400) / 155 columns each side, where best total =
min over the two sequences of the sum of each base's best NUC_SP + 60
entry.  Targets: offset / 100 and log(1 + half-width).
"""
import ctypes

import numpy as np

import mvg

N_IN, N_HID, N_OUT = 528, 256, 2
DELTA_SCALE = 100.0
DELTA_CLIP = 10.0
MAX_PAIR = 160
# best NUC_SP + 60 entry per base code A, C, G, T (MU/nucmx.cpp:8-25 diagonal + 60)
BASE_BEST = np.array([151, 160, 160, 151], np.int64)


def best_totals(seq, off):
    """Per problem: sum over its bases of BASE_BEST (the banded bound's total)."""
    seq = np.asarray(seq)
    off = np.asarray(off, np.int64)
    v = BASE_BEST[seq & 3]
    cs = np.concatenate([[0], np.cumsum(v)])
    return cs[off[1:]] - cs[off[:-1]]


def init_params(seed=0):
    """He-initialised flat fp32 parameters in the library's layout."""
    rng = np.random.default_rng(seed)
    parts = []
    dims = [(N_HID, N_IN), (N_HID, N_HID), (N_HID, N_HID), (N_OUT, N_HID)]
    for k, (o, i) in enumerate(dims):
        std = np.sqrt(2.0 / i) if k < 3 else np.sqrt(1.0 / i)
        parts.append(rng.normal(0, std, (o, i)).astype(np.float32).ravel())
        parts.append(np.zeros(o, np.float32))
    p = np.concatenate(parts)
    assert p.size == int(mvg.load_library().mvg_mlp_num_params())
    return p


def labels_from_full_dp(la, lb, scores, env, margin=8, totals=None):
    """(offset target, log(1 + half) target, offset, half) from full-DP
    results.  totals = (best_totals of A, of B); without them the need is
    estimated with 160 per base."""
    la = la.astype(np.int64)
    lb = lb.astype(np.int64)
    lo, hi = env[:, 0].astype(np.int64), env[:, 1].astype(np.int64)
    delta = (lo + hi) // 2
    half_env = (hi - lo + 1) // 2 + margin
    best = np.minimum(totals[0], totals[1]) if totals is not None else MAX_PAIR * np.minimum(la, lb)
    need = np.maximum(best - scores.astype(np.int64) - 400, 0) // 155 + margin
    half = np.maximum(half_env, need)
    half = np.clip(half, 0, np.maximum(la, lb))
    # offsets beyond +-1000 columns are clipped in the target: such gaps need a
    # band of most of the matrix and are decided by the half-width anyway
    t = np.stack([np.clip(delta / DELTA_SCALE, -DELTA_CLIP, DELTA_CLIP), np.log1p(half)], axis=1).astype(np.float32)
    return t, delta.astype(np.int32), half.astype(np.int32)


class BandNet:
    """The band-proposal network bound to one library context."""

    def __init__(self, ctx, params=None, seed=0):
        self.ctx = ctx
        self.step = 0
        self.set_params(init_params(seed) if params is None else params)

    def set_params(self, params):
        params = np.ascontiguousarray(params, np.float32)
        mvg._check(mvg.load_library().mvg_mlp_set_params(self.ctx.handle, mvg._ptr(params)))
        self.step = 0

    def get_params(self):
        p = np.zeros(int(mvg.load_library().mvg_mlp_num_params()), np.float32)
        mvg._check(mvg.load_library().mvg_mlp_get_params(self.ctx.handle, mvg._ptr(p)))
        return p

    # device-pointer calls (inputs resident on the GPU)
    def features_dev(self, d_sa, d_oa, d_sb, d_ob, n, d_x):
        mvg.wait_producers()
        mvg._check(mvg.load_library().mvg_band_features_dev(self.ctx.handle, d_sa, d_oa, d_sb, d_ob, n, d_x))

    def forward_dev(self, d_x, n, d_out):
        mvg.wait_producers()
        mvg._check(mvg.load_library().mvg_mlp_forward_dev(self.ctx.handle, d_x, n, d_out))

    def grad_dev(self, d_x, d_t, n):
        mvg.wait_producers()
        g = np.zeros(int(mvg.load_library().mvg_mlp_num_params()), np.float32)
        loss = ctypes.c_float(0)
        mvg._check(mvg.load_library().mvg_mlp_grad_dev(self.ctx.handle, d_x, d_t, n, mvg._ptr(g), ctypes.byref(loss)))
        return g, float(loss.value)

    def train_step_dev(self, d_x, d_t, n, lr):
        mvg.wait_producers()
        self.step += 1
        loss = ctypes.c_float(0)
        mvg._check(mvg.load_library().mvg_mlp_train_step_dev(self.ctx.handle, d_x, d_t, n, ctypes.c_float(lr),
                                                             self.step, ctypes.byref(loss)))
        return float(loss.value)

    def propose_dev(self, d_sa, d_oa, d_sb, d_ob, n, alpha=1.0, beta=8.0):
        mvg.wait_producers()
        delta = np.zeros(max(n, 1), np.int32)
        half = np.zeros(max(n, 1), np.int32)
        mvg._check(mvg.load_library().mvg_band_propose_dev(self.ctx.handle, d_sa, d_oa, d_sb, d_ob, n,
                                                           ctypes.c_float(alpha), ctypes.c_float(beta),
                                                           mvg._ptr(delta), mvg._ptr(half)))
        return delta[:n], half[:n]


def full_dp_labels_dev(ctx, d_sa, d_oa, d_sb, d_ob, n, margin=8, torch_device=None):
    """Runs the exact full DP on device inputs and returns (targets, delta, half, scores) on the host."""
    import torch
    d_sc = torch.zeros(n, dtype=torch.int32, device=torch_device)
    d_env = torch.zeros(2 * n, dtype=torch.int32, device=torch_device)
    mvg.wait_producers()
    mvg._check(mvg.load_library().mvg_gapdp_envelope_dev(ctx.handle, d_sa, d_oa, d_sb, d_ob, n, d_sc.data_ptr(),
                                                         d_env.data_ptr()))
    return d_sc.cpu().numpy(), d_env.cpu().numpy().reshape(-1, 2)


def heuristic_band(la, lb, frac=0.1, extra=32):
    """The band without the network: centred on the diagonal, half-width
    |LA - LB| + frac * min(LA, LB) + extra."""
    la = np.asarray(la, np.int64)
    lb = np.asarray(lb, np.int64)
    half = np.abs(la - lb) + (frac * np.minimum(la, lb)).astype(np.int64) + extra
    return np.zeros(len(la), np.int32), half.astype(np.int32)
