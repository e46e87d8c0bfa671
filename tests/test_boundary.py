"""C-ABI boundary checks that need no GPU: the library builds for sm_103a,
loads, exports every symbol include/mauve_gb300.h declares, and its pure
host functions agree with the oracle."""
import os
import re

import numpy as np
import pytest

import build as pkg_build
import mvg
import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    pkg_build.build()
    return mvg.load_library()


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "mauve_gb300.h")).read()
    return sorted(set(re.findall(r"\b(mvg_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_binding_exports():
    assert declared_symbols() == sorted(mvg.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_seed_helpers_match_oracle(lib):
    for w in range(3, 32):
        for r in range(6):
            assert mvg.get_seed(w, r) == O.get_seed(w, r)
    assert mvg.get_seed(17, mvg.SOLID_SEED) == (1 << 17) - 1
    for n in [0, 1, 31, 32, 1000, 4_600_000, 12_000_000, 1 << 40]:
        assert mvg.default_seed_weight(n) == O.default_seed_weight(n)
    for s in [0x16DF6D, 0x1FFFF, 0x7954F, 0x6B]:
        assert mvg.seed_length(s) == O.seed_length(s)
        assert mvg.seed_weight(s) == O.seed_weight(s)


def test_create_without_gpu_fails_loudly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises((RuntimeError, MemoryError)):
        mvg.Context(0)


def test_oracle_gap_batch_matches_single_calls():
    import synth
    sa, oa, sb, ob = synth.gap_batch(seed=5, nprob=20, lmin=1, lmax=200)
    scores, plen, paths, poff = O.nw_batch(sa, oa, sb, ob, nthreads=2)
    for k in range(20):
        p, s = O.nw_align(sa[oa[k]:oa[k + 1]], sb[ob[k]:ob[k + 1]])
        assert s == scores[k]
        assert p == paths[int(poff[k]):int(poff[k]) + int(plen[k])].tobytes().decode()
