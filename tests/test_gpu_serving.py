"""Batched proving and the continuous-batching server: every proof made while other proofs share the
GPU (several contexts/streams, admission by a memory budget) is byte-identical to the proof of the same
job made alone, and to the CPU oracle's proof. Also checks whir_multilinear_evaluate, which computes
the statements' evaluations on the device."""

import numpy as np
import pytest

import whir_gb300 as W
from whir_gb300 import serving
from whir_gb300.inputs import Rng, field_elements

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fname,fid", [("Goldilocks1", 0), ("Goldilocks2", 1), ("Goldilocks3", 2)])
@pytest.mark.parametrize("nv,n", [(0, 1), (1, 2), (5, 32), (5, 17), (12, 4096), (20, 1 << 20)])
def test_multilinear_evaluate_parity(ctx, orc, fname, fid, nv, n):
    rng = Rng(nv * 7 + n + fid)
    x = rng.goldilocks(n)
    pt = field_elements(fname, nv, rng=rng).reshape(-1)
    assert np.array_equal(W.multilinear_evaluate(ctx, fid, x, pt), orc.multilinear_extend(fid, x, pt))


def _max_pow_bits(params, field, nv):
    c = W.Config(field, 1 << nv, params).json()
    thr = [c["initial_sumcheck"]["round_pow_threshold"], c["initial_skip_pow_threshold"], c["final_pow_threshold"],
           c["final_sumcheck"]["round_pow_threshold"]]
    for r in c["rounds"]:
        thr += [r["pow_threshold"], r["sumcheck"]["round_pow_threshold"]]
    return max(64 - np.log2(float(t)) for t in thr)


def _small_jobs(ctx, count, seed):
    r = Rng(seed)
    jobs = []
    for k in range(count):
        field = ("Goldilocks2", "Goldilocks3", "Goldilocks1")[k % 3]
        nv = 8 + int(r.raw(1)[0] % 7)
        # A 64-bit field with list decoding needs ~40-bit fold proofs of work: Goldilocks1 jobs use
        # unique decoding.
        ud = bool(k % 2) or field == "Goldilocks1"
        params = W.ProtocolParameters(unique_decoding=ud, security_level=64, pow_bits=12,
                                      initial_folding_factor=2 + k % 3, folding_factor=2 + k % 2,
                                      starting_log_inv_rate=1 + k % 2, hash_id="Blake3")
        assert _max_pow_bits(params, field, nv) <= 24, (field, nv, ud)
        jobs.append(serving.make_job(field, nv, params, 1 + k % 2, seed * 100 + k, ctx, session="mix-%d" % k))
    return jobs


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
    return pr.narg, pr.hints


def test_batched_proofs_identical_to_alone(ctx, orc):
    jobs = _small_jobs(ctx, 12, seed=11)
    ref = _alone(ctx, jobs)
    bp = serving.BatchProver(device=0, workers=4)
    try:
        bp.prove_all(jobs)
    finally:
        bp.close()
    for j, (narg, hints) in zip(jobs, ref):
        assert j.narg == narg and j.hints == hints, j.session
    for j in jobs[:4]:
        assert (j.narg, j.hints) == _oracle(orc, j)


def test_served_proofs_identical_to_alone(ctx):
    jobs = _small_jobs(ctx, 12, seed=12)
    ref = _alone(ctx, jobs)
    budget = max(j.memory_estimate() for j in jobs) * 2  # forces admission waits
    srv = serving.ProofServer(device=0, workers=3, hbm_budget=budget)
    try:
        lat = srv.run(jobs, serving.poisson_arrivals(len(jobs), 400.0, seed=3))
    finally:
        srv.close()
    assert len(lat) == len(jobs) and all(x > 0 for x in lat)
    for j, (narg, hints) in zip(jobs, ref):
        assert j.narg == narg and j.hints == hints, j.session


@pytest.mark.parametrize("policy", [dict(priority_workers=1), dict(priority_workers=1, priority_large=True),
                                    dict(max_work=3 << 12)])
def test_served_proofs_identical_with_other_policies(ctx, policy):
    # One size class on raised-priority contexts, or a cap on the work in service: proofs are unchanged.
    jobs = _small_jobs(ctx, 10, seed=14)
    ref = _alone(ctx, jobs)
    srv = serving.ProofServer(device=0, workers=3, hbm_budget=1 << 40, large_nv=12, **policy)
    try:
        srv.run(jobs, serving.poisson_arrivals(len(jobs), 800.0, seed=4))
    finally:
        srv.close()
    for j, (narg, hints) in zip(jobs, ref):
        assert j.narg == narg and j.hints == hints, j.session


def test_server_rejects_request_over_budget(ctx):
    jobs = _small_jobs(ctx, 1, seed=13)
    srv = serving.ProofServer(device=0, workers=1, hbm_budget=1024)
    try:
        with pytest.raises(ValueError):
            srv.run(jobs, [0.0])
    finally:
        srv.close()
