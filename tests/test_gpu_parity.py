"""GPU parity: the CUDA path (through the C ABI) against the reference's golden
fixtures and the CPU oracle.  Integer / index work, so every comparison is
bit-exact."""
import numpy as np
import pytest

import mvg
import oracle as O
import synth
from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import build as pkg_build
    pkg_build.build()
    c = mvg.Context(0)
    yield c
    c.close()


# ------------------------------------------------------------------ SML

def test_sml_matches_reference_fixtures(ctx):
    g = load_golden("sml.npz")
    for k in range(int(g["count"])):
        seq, seed = g["seq%d" % k], int(g["seed%d" % k])
        pos, mer = ctx.sml_build(seq, seed)
        rpos, rmer = g["pos%d" % k], g["mer%d" % k]
        np.testing.assert_array_equal(mer, rmer)
        np.testing.assert_array_equal(pos, rpos[np.lexsort((rpos, rmer))])


@pytest.mark.parametrize("n,weight,rank", [(200_000, 15, 3), (150_000, 17, 3), (100_000, 11, 0), (5, 15, 3),
                                           (21, 15, 3), (22, 15, 3), (65_537, 9, 0)])
def test_sml_matches_oracle(ctx, n, weight, rank):
    rng = np.random.default_rng(n + weight)
    seq = synth.random_bases(rng, n, 0.45)
    seed = mvg.get_seed(weight, rank)
    pos, mer = ctx.sml_build(seq, seed)
    opos, omer = O.sml_build(seq, seed)
    np.testing.assert_array_equal(pos, opos)
    np.testing.assert_array_equal(mer, omer)


def test_sml_rejects_gap_character(ctx):
    with pytest.raises(ValueError):
        ctx.sml_build(b"ACGTACGTACGTACGTACGTACG-ACGTACGT", mvg.get_seed(15, 3))


def test_sml_unaligned_input_and_iupac(ctx):
    rng = np.random.default_rng(3)
    buf = synth.random_bases(rng, 50_001, 0.5)
    buf[rng.choice(50_001, 500, replace=False)] = np.frombuffer(b"NnRYacgtKMSWBb" * 36, np.uint8)[:500]
    seq = buf[1:]  # not 16-byte aligned
    seed = mvg.get_seed(15, 3)
    pos, mer = ctx.sml_build(seq, seed)
    opos, omer = O.sml_build(seq, seed)
    np.testing.assert_array_equal(pos, opos)
    np.testing.assert_array_equal(mer, omer)


# -------------------------------------------------------------- matches

def test_matches_reference_fixtures(ctx):
    g = load_golden("matches.npz")
    for k in range(int(g["count"])):
        m = ctx.pairwise_matches(g["a%d" % k], g["b%d" % k], int(g["seed%d" % k]))
        np.testing.assert_array_equal(m, g["m%d" % k], err_msg="case %d" % k)


@pytest.mark.parametrize("seed_id", range(6))
def test_matches_oracle_random_pairs(ctx, seed_id):
    rng = np.random.default_rng(100 + seed_id)
    n = int(rng.integers(20_000, 120_000))
    b = synth.random_bases(rng, n, float(rng.uniform(0.35, 0.65)))
    if seed_id % 2:
        b = synth.insert_repeats(rng, b, int(rng.integers(100, 2000)), int(rng.integers(2, 30)))
    a = synth.mutate(rng, b, float(rng.uniform(0, 0.1)), int(rng.integers(0, 80)), 4.0, int(rng.integers(0, 6)),
                     (200, 5000))
    w = mvg.default_seed_weight((len(a) + len(b)) // 2)
    seed = mvg.get_seed(w, 3 if seed_id < 4 else 0)
    m = ctx.pairwise_matches(a, b, seed)
    om = O.pairwise_matches(a, b, seed)
    np.testing.assert_array_equal(m, om)
    st = ctx.pairwise_stats()
    assert st["matches"] == len(m) and st["pairs"] == st["matches"] + st["collisions"]


def test_matches_genome_pair_small_config(ctx):
    """The 1 Mbp plain-method pair, end to end against the oracle."""
    a, b = synth.genome_pair_small()
    seed = mvg.get_seed(mvg.default_seed_weight((len(a) + len(b)) // 2), 3)
    m = ctx.pairwise_matches(a, b, seed)
    om = O.pairwise_matches(a, b, seed)
    np.testing.assert_array_equal(m, om)


def test_matches_reference_mds42_pair(ctx):
    """The reference's own recoded E. coli fixture pair (3.98 Mbp each,
    29,403 matches): the GPU match list equals the reference's, bit for bit,
    through the host and the device entry points."""
    import torch
    from conftest import load_mds42
    a, b, seed, want = load_mds42()
    np.testing.assert_array_equal(ctx.pairwise_matches(a, b, seed), want)
    st = ctx.pairwise_stats()
    assert st["pairs"] == st["matches"] + st["collisions"]
    da, db = torch.from_numpy(a.copy()).cuda(), torch.from_numpy(b.copy()).cuda()
    out = torch.zeros(3 * (len(want) + 16), dtype=torch.int64, device="cuda")
    n = ctx.pairwise_matches_dev(da.data_ptr(), len(a), db.data_ptr(), len(b), seed, out.data_ptr(), len(want) + 16)
    assert n == len(want)
    np.testing.assert_array_equal(out[:3 * n].cpu().numpy().reshape(-1, 3), want)


@pytest.mark.parametrize("n,sub", [(300000, 0.01), (300000, 0.05), (600000, 0.10)])
def test_matches_single_diagonal_buckets(ctx, n, sub):
    """Substitutions only: nearly every seed pair lands in one bucket (the
    cluster replay), with few or with more entries than a CTA's shared copy
    holds (the hand-back to the one-CTA replay)."""
    rng = np.random.default_rng(int(n * sub))
    acgt = np.frombuffer(b"ACGT", np.uint8)
    a = rng.choice(acgt, n)
    b = a.copy()
    m = rng.random(n) < sub
    b[m] = acgt[(np.searchsorted(acgt, b[m]) + rng.integers(1, 4, int(m.sum()))) % 4]
    seed = O.get_seed(O.default_seed_weight(n), 3)
    m = ctx.pairwise_matches(a, b, seed)
    np.testing.assert_array_equal(m, O.pairwise_matches(a, b, seed))
    st = ctx.pairwise_stats()  # every seed pair is either inserted or counted as contained
    assert st["matches"] == len(m) and st["pairs"] == st["matches"] + st["collisions"]


@pytest.mark.parametrize("cap", [32, 300])
def test_matches_bucket_sort_in_chunks(ctx, cap):
    """Seed-join buckets above the shared-memory capacity are sorted in
    chunks through global memory: forcing that for most buckets changes no
    match."""
    rng = np.random.default_rng(cap)
    b = synth.insert_repeats(rng, synth.random_bases(rng, 150_000), 500, 20)
    a = synth.mutate(rng, b, 0.03, 40, 4.0, 3, (200, 5000))
    seed = mvg.get_seed(15, 3)
    want = O.pairwise_matches(a, b, seed)
    ctx.set_pair_bucket_cap(cap)
    try:
        np.testing.assert_array_equal(ctx.pairwise_matches(a, b, seed), want)
    finally:
        ctx.set_pair_bucket_cap(3072)
    np.testing.assert_array_equal(ctx.pairwise_matches(a, b, seed), want)


@pytest.mark.parametrize("weight,rank", [(16, 0), (17, 3)])
def test_matches_wide_seed_keys(ctx, weight, rank):
    """Seeds of weight above 15 take 64-bit keys and the one-sort join."""
    rng = np.random.default_rng(weight)
    b = synth.random_bases(rng, 80_000)
    a = synth.mutate(rng, b, 0.04, 30, 4.0, 2, (200, 3000))
    seed = mvg.get_seed(weight, rank)
    np.testing.assert_array_equal(ctx.pairwise_matches(a, b, seed), O.pairwise_matches(a, b, seed))


def test_matches_recoded_pair_config(ctx):
    """The synthetic recoded-genome pair (4.6 Mbp, coding seed w=15): the GPU
    match list equals the oracle's, element by element."""
    a, b = synth.genome_pair_recoded()
    seed = mvg.get_seed(mvg.default_seed_weight((len(a) + len(b)) // 2), 3)
    np.testing.assert_array_equal(ctx.pairwise_matches(a, b, seed), O.pairwise_matches(a, b, seed))


def test_matches_large_pair_config(ctx):
    """The 12 Mbp, 16-contig pair at GC 0.38 with 300 repeat copies: weight
    17 has no coding seed, so the solid 17-mer and 64-bit keys (the one-sort
    join) are used; the match list equals the oracle's."""
    a, b = synth.genome_pair_large()
    w = mvg.default_seed_weight((len(a) + len(b)) // 2)
    seed = mvg.get_seed(w, 3)
    assert w == 17 and seed == (1 << 17) - 1
    np.testing.assert_array_equal(ctx.pairwise_matches(a, b, seed), O.pairwise_matches(a, b, seed))


def test_matches_gap_search_fixtures(ctx):
    """The reference's gap anchor search runs MemHash::FindMatches with the
    rank-0 seed of the gap's default weight (LM/ProgressiveAligner.cpp:590-679).
    On 44 gap pairs of 9 bp to 50 kbp its match list (before the overlap and
    length filters) equals the pairwise matcher's with the same seed."""
    g = load_golden("gapsearch.npz")
    tested = 0
    for k in range(int(g["count"])):
        w = int(g["w%d" % k])
        if w < 5:  # the reference does not search such gaps
            continue
        m = ctx.pairwise_matches(g["a%d" % k], g["b%d" % k], mvg.get_seed(w, 0))
        np.testing.assert_array_equal(m, g["mh%d" % k], err_msg="gap %d" % k)
        tested += 1
    assert tested >= 40


def test_matches_degenerate_inputs(ctx):
    seed = mvg.get_seed(15, 3)
    assert ctx.pairwise_matches(b"ACGT", b"ACGTACGT", seed).shape == (0, 3)
    rng = np.random.default_rng(9)
    x = synth.random_bases(rng, 3000)
    np.testing.assert_array_equal(ctx.pairwise_matches(x, x, seed), O.pairwise_matches(x, x, seed))
    poly = np.frombuffer(b"A" * 5000, np.uint8)  # one key repeated: no unique seeds
    assert ctx.pairwise_matches(poly, poly, seed).shape == (0, 3)


# --------------------------------------------------------------- gap DP

def _check_batch(ctx, sa, oa, sb, ob):
    scores, paths = ctx.gap_align_batch(sa, oa, sb, ob)
    oscores, oplen, opaths, opoff = O.nw_batch(sa, oa, sb, ob)
    np.testing.assert_array_equal(scores, oscores)
    raw = opaths.tobytes()
    for k in range(len(oa) - 1):
        assert paths[k] == raw[int(opoff[k]):int(opoff[k]) + int(oplen[k])].decode(), k


def test_gapdp_reference_fixtures(ctx):
    g = load_golden("gapdp.npz")
    scores, paths = ctx.gap_align_batch(g["seq_a"], g["off_a"], g["seq_b"], g["off_b"])
    for k in range(len(g["off_a"]) - 1):
        assert paths[k] == g["paths"][g["off_p"][k]:g["off_p"][k + 1]].tobytes().decode(), k


def test_gapdp_edge_shapes(ctx):
    rng = np.random.default_rng(21)
    shapes = [(1, 1), (1, 2), (2, 1), (1, 300), (300, 1), (127, 5), (128, 5), (129, 5), (256, 256), (257, 3),
              (5, 129), (33, 33), (2, 2), (3, 1000), (1000, 3)]
    a_list, b_list = [], []
    for la, lb in shapes:
        for _ in range(3):
            a_list.append(rng.integers(0, 4, la).astype(np.uint8))
            b_list.append(rng.integers(0, 4, lb).astype(np.uint8))
    oa = np.concatenate([[0], np.cumsum([len(x) for x in a_list])]).astype(np.uint64)
    ob = np.concatenate([[0], np.cumsum([len(x) for x in b_list])]).astype(np.uint64)
    _check_batch(ctx, np.concatenate(a_list), oa, np.concatenate(b_list), ob)


def test_gapdp_random_batch_vs_oracle(ctx):
    sa, oa, sb, ob = synth.gap_batch(seed=31, nprob=400, lmin=1, lmax=3000)
    _check_batch(ctx, sa, oa, sb, ob)


def test_gapdp_small_arena_waves_identical(ctx):
    sa, oa, sb, ob = synth.gap_batch(seed=32, nprob=60, lmin=200, lmax=2500)
    s1, p1 = ctx.gap_align_batch(sa, oa, sb, ob)
    ctx.set_tb_arena(4 << 20)  # forces many waves
    try:
        s2, p2 = ctx.gap_align_batch(sa, oa, sb, ob)
    finally:
        ctx.set_tb_arena(1 << 62)
    np.testing.assert_array_equal(s1, s2)
    assert p1 == p2


def test_gapdp_scores_only_equals_with_paths(ctx):
    sa, oa, sb, ob = synth.gap_batch(seed=33, nprob=100, lmin=1, lmax=1500)
    s1, _ = ctx.gap_align_batch(sa, oa, sb, ob, with_paths=True)
    s2, _ = ctx.gap_align_batch(sa, oa, sb, ob, with_paths=False)
    np.testing.assert_array_equal(s1, s2)


def test_gapdp_rejects_bad_codes_and_empty(ctx):
    with pytest.raises(ValueError):
        ctx.gap_align_batch(np.array([0, 5, 1], np.uint8), [0, 3], np.array([1, 2], np.uint8), [0, 2])
    with pytest.raises(ValueError):
        ctx.gap_align_batch(np.array([0, 1], np.uint8), [0, 0, 2], np.array([1, 2], np.uint8), [0, 1, 2])


def test_gapdp_whole_cta_mode_paths_vs_oracle(ctx):
    """Problems of at least 16 strips (A above 4,096 rows at 8 rows per lane)
    are solved by a whole CTA whose 8 warps pipeline the strips through a
    shared row buffer.  Scores and traceback paths equal the oracle's on 8
    pairs of 4.2-20 kbp at 0-30% divergence, one of them 20,000 x 20,000."""
    rng = np.random.default_rng(4020)
    pairs = []
    for la, d in zip([4200, 5000, 6500, 8000, 10000, 13000, 16000], np.linspace(0.0, 0.30, 7)):
        a = rng.integers(0, 4, la).astype(np.uint8)
        pairs.append((a, synth.mutate_codes(rng, a, 0.9 * d, int(0.1 * d * la / 3.0), 3.0)))
    a = rng.integers(0, 4, 20_000).astype(np.uint8)
    b = a.copy()
    m = rng.random(20_000) < 0.15  # substitutions only: 20,000 x 20,000
    b[m] = (b[m] + rng.integers(1, 4, int(m.sum()))).astype(np.uint8) % 4
    pairs.append((a, b))
    sa = np.concatenate([x for x, _ in pairs])
    sb = np.concatenate([y for _, y in pairs])
    oa = np.concatenate([[0], np.cumsum([len(x) for x, _ in pairs])]).astype(np.uint64)
    ob = np.concatenate([[0], np.cumsum([len(y) for _, y in pairs])]).astype(np.uint64)
    assert min(len(x) for x, _ in pairs) >= 16 * 32 * ctx.full_rows
    _check_batch(ctx, sa, oa, sb, ob)


def test_gapdp_whole_cta_mode_many_problems_vs_oracle(ctx):
    """More whole-CTA problems than resident CTAs, so each CTA claims
    several in turn (with the one-warp problems after them): 360 pairs of
    4.1-4.6 kbp plus 200 short ones, scores and paths equal to the oracle's."""
    rng = np.random.default_rng(4100)
    pairs = []
    for k in range(360):
        a = rng.integers(0, 4, int(rng.integers(4100, 4600))).astype(np.uint8)
        pairs.append((a, synth.mutate_codes(rng, a, float(rng.uniform(0, 0.27)), int(rng.integers(0, 40)), 3.0)))
    for k in range(200):
        a = rng.integers(0, 4, int(rng.integers(1, 900))).astype(np.uint8)
        pairs.append((a, synth.mutate_codes(rng, a, float(rng.uniform(0, 0.3)), int(rng.integers(0, 5)), 3.0)))
    order = rng.permutation(len(pairs))
    pairs = [pairs[i] for i in order]
    sa = np.concatenate([x for x, _ in pairs])
    sb = np.concatenate([y for _, y in pairs])
    oa = np.concatenate([[0], np.cumsum([len(x) for x, _ in pairs])]).astype(np.uint64)
    ob = np.concatenate([[0], np.cumsum([len(y) for _, y in pairs])]).astype(np.uint64)
    _check_batch(ctx, sa, oa, sb, ob)


def test_gapdp_watchdog_gives_up_and_handle_recovers(ctx):
    """The whole-CTA mode's waits are bounded.  With the limit at one poll a
    warp gives up waiting for its predecessor: the call returns
    MVG_ERR_DEVICE (a RuntimeError here) instead of hanging, and after the
    limit is restored the same handle solves the same batch exactly."""
    rng = np.random.default_rng(77)
    a = rng.integers(0, 4, 9000).astype(np.uint8)
    b = synth.mutate_codes(rng, a, 0.05, 20, 3.0)
    ctx.set_dp_spin_limit(1)
    try:
        with pytest.raises(RuntimeError, match="error 7"):
            ctx.gap_align_batch(a, [0, len(a)], b, [0, len(b)])
    finally:
        ctx.set_dp_spin_limit()
    scores, paths = ctx.gap_align_batch(a, [0, len(a)], b, [0, len(b)])
    p, s = O.nw_align(a, b)
    assert paths[0] == p and int(scores[0]) == s


def test_gapdp_long_pair_property(ctx):
    """A 12 kbp pair: path consumes both sequences, and the score re-derived
    from the path with NWSmall's scoring equals the returned score."""
    rng = np.random.default_rng(44)
    a = rng.integers(0, 4, 12_000).astype(np.uint8)
    b = synth.mutate_codes(rng, a, 0.2, 60, 3.0)
    scores, paths = ctx.gap_align_batch(a, [0, len(a)], b, [0, len(b)])
    p = paths[0]
    assert p.count("M") + p.count("D") == len(a) and p.count("M") + p.count("I") == len(b)
    assert int(scores[0]) == _path_score(a, b, p)
    assert int(scores[0]) == O.nw_score(a, b)


def _path_score(a, b, path):
    """Score of an edge path under NWSmall's model (open -200 / close -200 per
    gap, first-position open free, extend 0)."""
    sp = np.array([[91, -114, -31, -123], [-114, 100, -125, -31], [-31, -125, 100, -114], [-123, -31, -114, 91]]) + 60
    i = j = 0
    s = 0
    prev = None
    for e in path:
        if e == "M":
            if prev in ("D", "I"):
                s += -200  # close
            s += int(sp[a[i], b[j]])
            i += 1
            j += 1
        elif e == "D":
            if prev != "D":
                s += 0 if i == 0 else -200  # open at A position i
            i += 1
        else:
            if prev != "I":
                s += 0 if j == 0 else -200
            j += 1
        prev = e
    return s


def test_gapdp_checkpointed_equals_stored_bits(ctx):
    """Full-DP passes keep checkpoints and recompute the blocks the path
    crosses (default) or store every traceback bit: identical scores, paths
    and path envelopes, at both strip heights, on shapes around the block
    edges (strips of 32 * R rows, column blocks of 128), a whole-CTA pair and
    a random batch, with many waves (a small arena) too."""
    import torch
    import bandnet
    rng = np.random.default_rng(128)
    a_list, b_list = [], []
    for la in (1, 2, 127, 128, 129, 255, 256, 257, 513, 2100):
        for lb in (1, 2, 127, 128, 129, 255, 256, 257, 385, 1000):
            a = rng.integers(0, 4, la).astype(np.uint8)
            # a mutated copy of A cut or padded with random bases to exactly lb
            m = synth.mutate_codes(rng, a, 0.1, la // 100, 3.0)[:lb]
            b = np.concatenate([m, rng.integers(0, 4, lb - len(m)).astype(np.uint8)])
            a_list.append(a)
            b_list.append(b)
    a = rng.integers(0, 4, 4300).astype(np.uint8)
    a_list.append(a)
    b_list.append(synth.mutate_codes(rng, a, 0.2, 30, 3.0))
    sa2, oa2, sb2, ob2 = synth.gap_batch(seed=129, nprob=300, lmin=1, lmax=3000)
    sa = np.concatenate(a_list + [sa2])
    sb = np.concatenate(b_list + [sb2])
    oa = np.concatenate([[0], np.cumsum([len(x) for x in a_list])]).astype(np.uint64)
    ob = np.concatenate([[0], np.cumsum([len(x) for x in b_list])]).astype(np.uint64)
    oa = np.concatenate([oa, oa[-1] + oa2[1:].astype(np.uint64)])
    ob = np.concatenate([ob, ob[-1] + ob2[1:].astype(np.uint64)])
    n = len(oa) - 1
    dev = torch.device("cuda", 0)
    d = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in (sa, oa.astype(np.int64), sb, ob.astype(np.int64))]
    full0, band0 = ctx.full_rows, ctx.band_rows
    try:
        for rows in (4, 8):
            ctx.set_dp_rows(rows, band0)
            res = {}
            for ck in (True, False):
                ctx.set_dp_checkpoint(ck)
                sc, paths = ctx.gap_align_batch(sa, oa, sb, ob)
                lsc, env = bandnet.full_dp_labels_dev(ctx, *[x.data_ptr() for x in d], n, torch_device=dev)
                res[ck] = (sc, paths, lsc, env)
            np.testing.assert_array_equal(res[True][0], res[False][0])
            assert res[True][1] == res[False][1], rows
            np.testing.assert_array_equal(res[True][2], res[False][2])
            np.testing.assert_array_equal(res[True][3], res[False][3])
        ctx.set_dp_checkpoint(True)
        ctx.set_tb_arena(8 << 20)  # many waves
        try:
            s_w, p_w = ctx.gap_align_batch(sa, oa, sb, ob)
        finally:
            ctx.set_tb_arena(1 << 62)
        np.testing.assert_array_equal(s_w, res[True][0])
        assert p_w == res[True][1]
    finally:
        ctx.set_dp_checkpoint(True)
        ctx.set_dp_rows(full0, band0)


def test_gapdp_graph_and_direct_launches_identical(ctx):
    """The DP waves recorded into one CUDA graph (default) and launched one by
    one give identical scores and paths, across calls of different shapes
    (the kept executable graph updated or rebuilt), with many waves (a small
    traceback arena) and long paths (the warp walker on the side stream),
    and with stage timing on (event nodes inside the graph)."""
    sa, oa, sb, ob = synth.gap_batch(seed=57, nprob=300, lmin=50, lmax=6000)
    ctx.set_dp_graph(False)
    try:
        s_direct, p_direct = ctx.gap_align_batch(sa, oa, sb, ob)
    finally:
        ctx.set_dp_graph(True)
    for arena in (1 << 62, 64 << 20, 16 << 20):
        ctx.set_tb_arena(arena)
        try:
            s_graph, p_graph = ctx.gap_align_batch(sa, oa, sb, ob)
        finally:
            ctx.set_tb_arena(1 << 62)
        np.testing.assert_array_equal(s_graph, s_direct)
        assert p_graph == p_direct
    ctx.set_profiling(True)
    try:
        s_prof, p_prof = ctx.gap_align_batch(sa, oa, sb, ob)
        st = ctx.stage_times()
    finally:
        ctx.set_profiling(False)
    np.testing.assert_array_equal(s_prof, s_direct)
    assert p_prof == p_direct
    assert st.get("dp", 0) > 0 and st.get("traceback", 0) > 0
    oscores, _, _, _ = O.nw_batch(sa, oa, sb, ob, with_paths=False)
    np.testing.assert_array_equal(s_direct, oscores)


def _rows_from_path(a, b, path):
    ra, rb, i, j = [], [], 0, 0
    for e in path:
        ra.append(a[i] if e != "I" else ord("-"))
        rb.append(b[j] if e != "D" else ord("-"))
        i += e != "I"
        j += e != "D"
    return bytes(ra), bytes(rb)


def test_path_rows_reference_fixtures(ctx):
    """The gapped rows of the reference's own profile-profile alignments
    (gapdp.npz holds MUSCLE's rows as paths over A/C/G/T): the GPU's paths
    turned into rows by the batched AlignTwoMSAsGivenPath equal them."""
    g = load_golden("gapdp.npz")
    sa, sb, oa, ob = g["seq_a"], g["seq_b"], g["off_a"], g["off_b"]
    _, paths = ctx.gap_align_batch(sa, oa, sb, ob)
    acgt = np.frombuffer(b"ACGT", np.uint8)
    ta, tb = acgt[sa], acgt[sb]
    rows = ctx.path_rows(ta, oa, tb, ob, paths)
    for k in range(len(oa) - 1):
        ref_path = g["paths"][g["off_p"][k]:g["off_p"][k + 1]].tobytes().decode()
        want = _rows_from_path(ta[oa[k]:oa[k + 1]], tb[ob[k]:ob[k + 1]], ref_path)
        assert rows[k] == want, k


def test_path_rows_ascii_batch_and_bad_path(ctx):
    """Rows of a random batch with IUPAC/lower-case letters copied through,
    against rows built from the oracle's paths; a path that does not consume
    its sequences is refused."""
    sa, oa, sb, ob = synth.gap_batch(seed=88, nprob=500, lmin=1, lmax=4000)
    rng = np.random.default_rng(88)
    letters = np.frombuffer(b"acgtNRYKM", np.uint8)
    ta = np.frombuffer(b"ACGT", np.uint8)[sa].copy()
    tb = np.frombuffer(b"ACGT", np.uint8)[sb].copy()
    for t in (ta, tb):
        m = rng.random(len(t)) < 0.05
        t[m] = rng.choice(letters, int(m.sum()))
    _, oplen, opaths, opoff = O.nw_batch(sa, oa, sb, ob)
    raw = opaths.tobytes()
    paths = [raw[int(opoff[k]):int(opoff[k]) + int(oplen[k])].decode() for k in range(len(oa) - 1)]
    rows = ctx.path_rows(ta, oa, tb, ob, paths)
    for k in range(len(oa) - 1):
        assert rows[k] == _rows_from_path(ta[oa[k]:oa[k + 1]], tb[ob[k]:ob[k + 1]], paths[k]), k
    with pytest.raises(ValueError):
        ctx.path_rows(ta[:10], [0, 10], tb[:10], [0, 10], ["M" * 9])
