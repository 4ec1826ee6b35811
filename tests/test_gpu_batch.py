"""Multi-job launches and the autotuner. A batched commit (whir_commit_batch: one encode column pass,
one row pass and one Merkle launch per tile step over a table of jobs of uneven sizes) yields the same
roots and proofs as committing each job alone, and as the CPU oracle; every encode plan the
autotuner may choose gives the same codeword and leaf digests as the default plan."""

import numpy as np
import pytest

import whir_gb300 as W
from whir_gb300 import serving
from whir_gb300.inputs import Rng, field_elements

pytestmark = pytest.mark.gpu


def _uneven_jobs(ctx, field, sizes, ud, seed, hash_id="Blake3", k=4):
    params = W.ProtocolParameters(unique_decoding=ud, security_level=64, pow_bits=12, initial_folding_factor=k,
                                  folding_factor=k, starting_log_inv_rate=1, hash_id=hash_id)
    return [serving.make_job(field, d, params, 1 + i % 2, seed * 100 + i, ctx, session="batch-%d" % i)
            for i, d in enumerate(sizes)]


def _alone(ctx, jobs):
    out = []
    for j in jobs:
        c = serving.ProofJob(j.field, j.nv, j.params, j.vectors, j.points, j.evaluations, j.session)
        serving.prove_job(ctx, c)
        out.append((c.narg, c.hints))
    return out


def _oracle(orc, job):
    p = job.params
    op = orc.make_params(unique_decoding=p.unique_decoding, security_level=p.security_level, pow_bits=p.pow_bits,
                         initial_folding_factor=p.initial_folding_factor, folding_factor=p.folding_factor,
                         starting_log_inv_rate=p.starting_log_inv_rate, hash_id=p.hash_id)
    f = orc.FIELD_IDS[job.field]
    pr = orc.whir_prove(f, op, job.nv, job.session, job.vectors.reshape(1, -1), job.points, [], job.evaluations)
    return pr.narg, pr.hints, pr.roots


@pytest.mark.parametrize("field,sizes,ud,hash_id", [
    ("Goldilocks3", (14, 8, 16, 10, 12, 18), False, "Blake3"),  # four-step and single-pass encodes mixed
    ("Goldilocks2", (9, 13, 11, 16, 8), True, "Sha3"),
    ("Goldilocks1", (8, 12, 10), True, "Keccak"),
])
def test_commit_batch_matches_single_commits_and_oracle(ctx, orc, field, sizes, ud, hash_id):
    jobs = _uneven_jobs(ctx, field, sizes, ud, seed=len(sizes) + int(ud), hash_id=hash_id)
    ref = _alone(ctx, jobs)
    cfgs = [W.Config(j.field, j.size, j.params) for j in jobs]
    states = [W.ProverState(c, j.session) for c, j in zip(cfgs, jobs)]
    flats = [j.vectors.reshape(-1) for j in jobs]
    wits = W.commit_batch(ctx, cfgs, states, flats)
    for j, c, ps, flat, w, (narg, hints) in zip(jobs, cfgs, states, flats, wits, ref):
        root = w.root()
        c.prove(ctx, ps, flat, [w], j.points, [], j.evaluations)
        w.free()
        got = ps.proof()
        assert got == (narg, hints), j.session
        on, oh, oroots = _oracle(orc, j)
        assert got == (on, oh) and root == oroots[:32]


def test_batch_prover_with_batched_commits_equals_alone(ctx):
    jobs = _uneven_jobs(ctx, "Goldilocks3", (8, 14, 10, 12, 16, 9, 11, 13), False, seed=21)
    ref = _alone(ctx, jobs)
    bp = serving.BatchProver(device=0, workers=3, batch_commit=True)
    try:
        bp.prove_all(jobs)
    finally:
        bp.close()
    for j, r in zip(jobs, ref):
        assert (j.narg, j.hints) == r, j.session


def test_commit_batch_rejects_mixed_fields(ctx):
    a = _uneven_jobs(ctx, "Goldilocks2", (8,), True, seed=31)[0]
    b = _uneven_jobs(ctx, "Goldilocks3", (8,), True, seed=32)[0]
    cfgs = [W.Config(j.field, j.size, j.params) for j in (a, b)]
    states = [W.ProverState(c, j.session) for c, j in zip(cfgs, (a, b))]
    with pytest.raises(W.WhirError) as e:
        W.commit_batch(ctx, cfgs, states, [a.vectors.reshape(-1), b.vectors.reshape(-1)])
    assert e.value.code == -1


@pytest.mark.parametrize("field,nv", [("Goldilocks2", 16), ("Goldilocks3", 12), ("Field192", 10)])
def test_autotune_choices_are_bit_exact(ctx, orc, field, nv):
    # Every candidate plan of every commitment shape the tuner measured, forced one at a time through
    # the import path, encodes to the default plan's codeword; the tuned proof equals the oracle's.
    W.autotune_clear()
    params = W.ProtocolParameters(unique_decoding=True, security_level=64, pow_bits=12, hash_id="Blake3")
    cfg = W.Config(field, 1 << nv, params)
    rep = W.autotune(ctx, cfg, reps=1)
    assert len(rep["shapes"]) == 1 + len(cfg.json()["rounds"])
    fid = W.FIELDS[field]
    base = {"Goldilocks2": "Goldilocks1", "Goldilocks3": "Goldilocks1"}.get(field, field)
    try:
        for si, shape in enumerate(rep["shapes"][:2]):
            assert shape["candidates"] and shape["pick_ms"] > 0
            n_msgs, msg_len, cw = shape["n_msgs"], shape["msg_len"], shape["codeword_len"]
            ename = base if si == 0 else field
            efid = W.FIELDS[ename]
            msgs = field_elements(ename, n_msgs * msg_len, rng=Rng(nv + si)).reshape(n_msgs, msg_len, -1)
            W.autotune_clear()
            want = W.interleaved_encode(ctx, efid, msgs, cw)
            for mode, logc2, w, g, _ in shape["candidates"]:
                W.autotune_import("encode %d %d %d %d %d %d %d %d\n" % (n_msgs, msg_len, cw, shape["elem_bytes"],
                                                                      mode, logc2, w, g))
                assert np.array_equal(W.interleaved_encode(ctx, efid, msgs, cw), want), (mode, logc2, w, g)
        W.autotune_clear()
        W.autotune(ctx, cfg, reps=1)
        table = W.autotune_export()
        assert "encode " in table and "merkle " in table
        job = serving.make_job(field, nv, params, 1, 77, ctx, session="tuned")
        serving.prove_job(ctx, job)
        on, oh, _ = _oracle(orc, job)
        assert (job.narg, job.hints) == (on, oh)
        W.autotune_clear()
        W.autotune_import(table)
        assert W.autotune_export() == table
    finally:
        W.autotune_clear()
