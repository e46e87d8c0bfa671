"""GPU tests of the band-proposal network's tcgen05 forward layers.

The tcgen05 path (TMA-fed tensor-core GEMMs with bias, GELU and the output
layer in the epilogue) is checked against the float64 CPU reference of the
network (same bf16 roundings of weights and activations) and against the
mma.sync path; the two GPU paths differ only in the order of fp32 sums, so
their outputs agree to bf16 rounding of the hidden activations.
"""
import numpy as np
import pytest

import bandnet
import bandnet_ref as REF
import mvg
import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import build as pkg_build
    pkg_build.build()
    c = mvg.Context(0)
    yield c
    c.close()


def _features(ctx, net, seed, n):
    import torch
    sa, oa, sb, ob = synth.gap_batch_recoded(seed=seed, nprob=n, lmin=20, lmax=800)
    t = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (sa, oa.astype(np.int64), sb, ob.astype(np.int64))]
    X = torch.zeros((n, bandnet.N_IN), dtype=torch.bfloat16, device=t[0].device)
    net.features_dev(*[x.data_ptr() for x in t], n, X.data_ptr())
    return t, X


def _forward(ctx, net, X, n, tc):
    import torch
    ctx.set_mlp_tcgen05(tc)
    before = ctx.mlp_tcgen05_passes()
    out = torch.zeros((n, 2), dtype=torch.float32, device=X.device)
    net.forward_dev(X.data_ptr(), n, out.data_ptr())
    ran_tc = ctx.mlp_tcgen05_passes() - before
    ctx.set_mlp_tcgen05(True)
    return out.cpu().numpy(), ran_tc


@pytest.mark.parametrize("n", [8, 128, 1000, 4104])
def test_forward_matches_cpu_reference_and_mma_path(ctx, n):
    """Tile edges: one partial tile, one whole tile, a ragged last tile,
    many tiles.  Tolerance: 2e-2 (relative and absolute) against the CPU
    reference, 1e-2 between the GPU paths."""
    net = bandnet.BandNet(ctx, seed=5)
    _, X = _features(ctx, net, 31 + n, n)
    out_tc, ran = _forward(ctx, net, X, n, True)
    assert ran == 1, "the tcgen05 path did not run"
    out_mma, ran = _forward(ctx, net, X, n, False)
    assert ran == 0
    ref = REF.forward(net.get_params(), X.float().cpu().numpy().astype(np.float64))
    np.testing.assert_allclose(out_tc, ref, rtol=2e-2, atol=2e-2)
    np.testing.assert_allclose(out_tc, out_mma, rtol=1e-2, atol=1e-2)
    assert np.abs(out_tc - out_mma).mean() < 1e-3


def test_trained_weights_forward(ctx):
    """The committed trained weights (larger activations than a fresh
    initialisation) through both paths."""
    import os
    path = os.path.join(os.path.dirname(mvg.__file__), "bandnet_weights.npz")
    if not os.path.exists(path):
        pytest.skip("no trained weights")
    w = np.load(path)
    net = bandnet.BandNet(ctx, params=w["params"])
    n = 2048
    _, X = _features(ctx, net, 77, n)
    out_tc, ran = _forward(ctx, net, X, n, True)
    assert ran == 1
    out_mma, _ = _forward(ctx, net, X, n, False)
    ref = REF.forward(net.get_params(), X.float().cpu().numpy().astype(np.float64))
    np.testing.assert_allclose(out_tc, ref, rtol=2e-2, atol=2e-2)
    np.testing.assert_allclose(out_tc, out_mma, rtol=1e-2, atol=1e-2)


def test_gradients_through_tcgen05_forward(ctx):
    """Training keeps the pre-activations the tcgen05 epilogue writes: every
    parameter block's gradient within 2e-2 (relative, in norm) of the
    float64 reference."""
    import torch
    net = bandnet.BandNet(ctx, seed=9)
    n = 264
    _, X = _features(ctx, net, 41, n)
    rng = np.random.default_rng(1)
    T = rng.normal(0, 1, (n, 2)).astype(np.float32)
    before = ctx.mlp_tcgen05_passes()
    g, loss = net.grad_dev(X.data_ptr(), torch.from_numpy(T).cuda().data_ptr(), n)
    assert ctx.mlp_tcgen05_passes() == before + 1
    rloss, rg = REF.loss_and_grads(net.get_params(), X.float().cpu().numpy().astype(np.float64), T.astype(np.float64))
    assert abs(loss - rloss) <= 2e-2 * abs(rloss) + 1e-6
    off = 0
    for s in [256 * 528, 256, 256 * 256, 256, 256 * 256, 256, 2 * 256, 2]:
        a, b = g[off:off + s], rg[off:off + s]
        assert np.linalg.norm(a - b) <= 2e-2 * np.linalg.norm(b) + 1e-7, (off, s)
        off += s


def test_ragged_caller_rows_take_the_mma_path(ctx):
    """A caller's input of n rows, n not a multiple of 8, cannot be given to
    TMA in 8-row groups without reading past it: that pass runs on mma.sync
    and still matches the reference."""
    net = bandnet.BandNet(ctx, seed=6)
    n = 1003
    _, X = _features(ctx, net, 51, n)
    out, ran = _forward(ctx, net, X, n, True)
    assert ran == 0
    ref = REF.forward(net.get_params(), X.float().cpu().numpy().astype(np.float64))
    np.testing.assert_allclose(out, ref, rtol=2e-2, atol=2e-2)


def test_band_proposals_agree_between_paths(ctx):
    """Band proposals (the library pads its own feature buffer, so a ragged
    count runs on tcgen05): integer bands equal on at least 99% of gaps and
    within a few units elsewhere."""
    import os
    path = os.path.join(os.path.dirname(mvg.__file__), "bandnet_weights.npz")
    w = np.load(path) if os.path.exists(path) else None
    net = bandnet.BandNet(ctx, params=w["params"]) if w is not None else bandnet.BandNet(ctx, seed=2)
    n = 5003
    t, _ = _features(ctx, net, 61, n)
    ptrs = [x.data_ptr() for x in t]
    before = ctx.mlp_tcgen05_passes()
    d1, h1 = net.propose_dev(*ptrs, n, 1.6, 16.0)
    assert ctx.mlp_tcgen05_passes() == before + 1
    ctx.set_mlp_tcgen05(False)
    d0, h0 = net.propose_dev(*ptrs, n, 1.6, 16.0)
    ctx.set_mlp_tcgen05(True)
    assert np.mean((d1 == d0) & (h1 == h0)) >= 0.99
    assert np.abs(d1.astype(np.int64) - d0).max() <= 3
    assert np.abs(h1.astype(np.int64) - h0).max() <= 0.02 * h0.max() + 3
