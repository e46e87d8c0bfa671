"""The multi-rank (replica) path of bench.py on CPU: two ranks over a gloo
process group.  Each rank aligns its own genome pair (weak scaling, no data
exchange); the job's time is the slowest rank's (all-reduce MAX).  The ranks
run the oracle's anchoring on a small pair of their own, so the test needs no
GPU: it checks the rank plumbing (environment, rank-specific inputs, the MAX
reduction) that the GPU run uses with NCCL."""
import os
import socket

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import sys
    for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests"), os.path.join(ROOT, "mauve-py_gb300")):
        sys.path.insert(0, p)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench
    import oracle as O
    import synth
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w_, r_, l_ = bench.dist_setup(world)
    rng = np.random.default_rng(bench.replica_pair_seed(r_))
    b = synth.random_bases(rng, 40_000)
    a = synth.mutate(rng, b, 0.01, 10, 4.0, 1, (500, 2000))
    seed, w = bench.seeds_for(a, b)
    m = O.pairwise_matches(a, b, seed)
    fake_ms = 10.0 * (rank + 1)  # rank-specific "time"
    job_ms = bench.max_over_ranks(fake_ms, w_, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    out.put((r_, w_, l_, int(len(m)), int(m[:, 2].sum()) if len(m) else 0, job_ms))


def test_two_replicas_over_gloo():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=240) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, l0, n0, s0, t0), (r1, w1, l1, n1, s1, t1) = res
    assert (r0, r1) == (0, 1) and w0 == w1 == 2 and (l0, l1) == (0, 1)
    assert n0 > 0 and n1 > 0 and (n0, s0) != (n1, s1)  # each rank aligned its own pair
    assert t0 == t1 == 20.0  # both ranks report the slowest rank's time
