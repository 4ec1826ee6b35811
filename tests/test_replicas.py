"""Multi-rank (replica) path on the CPU: two gloo ranks split a list of proof jobs with
whir_gb300.replicas.shard, prove their shares (with the CPU oracle, so no GPU is needed), and the
gathered proofs equal the ones a single process makes; the max-over-ranks timing reduction works."""

import hashlib
import os
import socket

import pytest
import torch.multiprocessing as mp

from whir_gb300.replicas import max_over_ranks, shard

JOBS = [("Goldilocks2", 8, 1), ("Goldilocks2", 9, 2), ("Goldilocks3", 8, 3), ("Goldilocks1", 10, 4),
        ("Goldilocks2", 10, 5)]


def _prove(job):
    import oracle
    from test_oracle_pins import make_statement
    field, nv, seed = job
    p = oracle.make_params(unique_decoding=True, security_level=40, pow_bits=5, initial_folding_factor=2,
                           folding_factor=2)
    f, vecs, pts, covs, evals = make_statement(oracle, field, nv, 1, 1, 1, False, seed=seed)
    pr = oracle.whir_prove(f, p, nv, "replica-%d" % seed, vecs, pts, covs, evals)
    return hashlib.sha256(pr.narg + pr.hints).hexdigest()


def _worker(rank, world, port, out_dir):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = {i: _prove(JOBS[i]) for i in shard(len(JOBS), rank, world)}
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    t = max_over_ranks(dist, float(rank + 1))
    if rank == 0:
        merged = {}
        for part in gathered:
            for k, v in part.items():
                assert k not in merged
                merged[k] = v
        with open(os.path.join(out_dir, "result.txt"), "w") as f:
            f.write("%s\n%r\n" % (t, [merged[i] for i in range(len(JOBS))]))
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_shard_partitions_jobs():
    for n in range(0, 11):
        for world in (1, 2, 3, 8):
            seen = sorted(i for r in range(world) for i in shard(n, r, world))
            assert seen == list(range(n))
    with pytest.raises(ValueError):
        shard(4, 2, 2)


def test_two_gloo_ranks_match_single_process(tmp_path):
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
        assert p.exitcode == 0
    t, hashes = open(os.path.join(tmp_path, "result.txt")).read().split("\n")[:2]
    assert float(t) == 2.0
    assert eval(hashes) == [_prove(j) for j in JOBS]
