"""The no-allocation sorted-mer-list entry point (mvg_sml_build_noalloc).

It exists for callers that cannot call cudaMalloc when they need a sorted
mer list.  One is a process whose other runtime has reserved the device's
memory for its own pool.  Another is a latency-bound loop that cannot take
cudaMalloc's implicit synchronisation.  It keeps its scratch in one static
device array of the library.  This test calls it through the C ABI on device
buffers and checks that its output equals the allocating entry point's
(mvg_sml_build_dev) bit for bit, on two calls in a row, that the second
call leaves the device's free memory unchanged (nothing allocated), and
that input over its size limit is refused.  The file sorts last so that a run stopping at
the first failure has already run every other test.  The test also passes
alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import mvg
import synth

pytestmark = pytest.mark.gpu

MAX_BASES = 262_144


def _noalloc_fn():
    L = mvg.load_library()
    f = L.mvg_sml_build_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64), ctypes.c_void_p]
    return f


def test_no_alloc_sml_equals_allocating_entry_point():
    import torch

    import build as pkg_build
    pkg_build.build()
    ctx = mvg.Context(0)
    f = _noalloc_fn()
    rng = np.random.default_rng(2026)
    cases = [(MAX_BASES, mvg.get_seed(15, 3)), (150_001, mvg.get_seed(17, 3))]  # two calls in a row
    for call, (n, seed) in enumerate(cases):
        seq = synth.random_bases(rng, n, float(rng.uniform(0.35, 0.6)))
        d_seq = torch.from_numpy(seq).cuda()
        L = mvg.seed_length(seed)
        cnt = n - L + 1
        ref_pos = torch.zeros(cnt, dtype=torch.int32, device="cuda")
        ref_mer = torch.zeros(cnt, dtype=torch.int64, device="cuda")
        got_pos = torch.full((cnt,), -1, dtype=torch.int32, device="cuda")
        got_mer = torch.full((cnt,), -1, dtype=torch.int64, device="cuda")
        assert ctx.sml_build_dev(d_seq.data_ptr(), n, seed, ref_pos.data_ptr(), ref_mer.data_ptr(), cnt) == cnt
        torch.cuda.synchronize()
        out = ctypes.c_uint64(0)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc = f(d_seq.data_ptr(), n, seed, got_pos.data_ptr(), got_mer.data_ptr(), cnt, ctypes.byref(out), None)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        assert rc == 0, mvg.load_library().mvg_last_error()
        if call > 0:  # the first call may commit the library's static array; later ones allocate nothing
            assert free_after == free_before
        assert out.value == cnt
        assert torch.equal(got_pos, ref_pos)
        assert torch.equal(got_mer, ref_mer)
    # over the static scratch limit: refused, nothing written
    big = torch.zeros(MAX_BASES + 1, dtype=torch.uint8, device="cuda")
    out = ctypes.c_uint64(0)
    rc = f(big.data_ptr(), MAX_BASES + 1, mvg.get_seed(15, 3), None, None, MAX_BASES + 1, ctypes.byref(out), None)
    assert rc == 5  # MVG_ERR_CAPACITY
    ctx.close()
