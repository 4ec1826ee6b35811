"""End-to-end parity of the GPU prover: commit + prove through the C ABI produce the same Merkle roots,
NARG string and hints as the CPU oracle prover for the same inputs, the oracle verifier (a
restatement of whir::Config::verify) accepts every GPU proof, and the final claims agree."""

import hashlib

import numpy as np
import pytest

import whir_gb300 as W
from whir_gb300.inputs import Rng, field_elements

pytestmark = pytest.mark.gpu


def statement(orc, field, nv, npts, bs, nw, cov, seed):
    from test_oracle_pins import make_statement
    return make_statement(orc, field, nv, npts, bs, nw, cov, seed=seed)


def gpu_prove(ctx, field, params, nv, session, vecs, pts, covs, evals, nw):
    cfg = W.Config(field, 1 << nv, params)
    ps = W.ProverState(cfg, session)
    bs = params.batch_size
    L = W.SOURCE_LIMBS[cfg.field]
    flat = np.ascontiguousarray(vecs, dtype=np.uint64).reshape(nw, bs * (1 << nv) * L)
    wits = [cfg.commit(ctx, ps, flat[w]) for w in range(nw)]
    claim = cfg.prove(ctx, ps, np.ascontiguousarray(vecs, dtype=np.uint64), wits, pts, covs, evals)
    narg, hints = ps.proof()
    return narg, hints, claim, [w.root() for w in wits]


CASES = [
    # field, nv, unique, k0, k, points, pow_bits, hash, security, batch, witnesses, rate, covector
    ("Goldilocks2", 8, True, 2, 2, 1, 5, "Sha2", 32, 1, 1, 1, False),
    ("Goldilocks2", 10, False, 2, 2, 2, 5, "Blake3", 32, 1, 1, 1, False),
    ("Goldilocks3", 9, False, 3, 3, 1, 0, "Blake3", 32, 1, 1, 1, True),
    ("Goldilocks1", 8, True, 4, 4, 0, 0, "Keccak", 32, 1, 1, 1, False),
    ("Goldilocks1", 11, False, 3, 2, 2, 8, "Sha3", 40, 1, 1, 2, False),
    ("Goldilocks3", 8, False, 2, 2, 1, 5, "Blake3", 32, 2, 2, 1, False),
    ("Goldilocks2", 12, True, 4, 4, 1, 10, "Blake3", 100, 1, 1, 1, False),
    ("Goldilocks2", 14, True, 4, 4, 0, 10, "Blake3", 60, 1, 1, 1, False),
    ("Goldilocks2", 16, True, 4, 4, 3, 20, "Blake3", 100, 1, 1, 1, False),
    ("Goldilocks3", 16, False, 4, 4, 2, 20, "Blake3", 100, 1, 1, 1, False),
    ("Goldilocks2", 13, True, 1, 3, 1, 10, "Blake3", 64, 1, 1, 2, False),
    ("Field192", 8, False, 4, 4, 2, 10, "Sha3", 32, 1, 1, 1, False),
    ("Field256", 8, False, 4, 4, 1, 5, "Sha3", 32, 1, 2, 1, False),
    ("Field192", 9, True, 3, 2, 1, 0, "Blake3", 40, 2, 1, 1, True),
    ("Field256", 12, False, 4, 4, 4, 16, "Sha3", 128, 1, 1, 2, False),
    ("Field192", 14, False, 4, 4, 4, 20, "Keccak", 128, 1, 1, 2, False),
    ("Field256", 11, True, 2, 3, 2, 8, "Sha2", 64, 1, 1, 3, False),
]


@pytest.mark.parametrize("case", CASES, ids=["%s-nv%d-%d" % (c[0], c[1], i) for i, c in enumerate(CASES)])
def test_gpu_proof_equals_oracle_proof(ctx, orc, case):
    field, nv, ud, k0, k, npts, powb, h, sec, bs, nw, rate, cov = case
    params = W.ProtocolParameters(unique_decoding=ud, security_level=sec, pow_bits=powb, hash_id=h,
                                  initial_folding_factor=k0, folding_factor=k, starting_log_inv_rate=rate,
                                  batch_size=bs)
    op = orc.make_params(unique_decoding=ud, security_level=sec, pow_bits=powb, hash_id=W.ENGINES[h],
                         initial_folding_factor=k0, folding_factor=k, starting_log_inv_rate=rate, batch_size=bs)
    f, vecs, pts, covs, evals = statement(orc, field, nv, npts, bs, nw, cov, seed=nv + 17)
    session = "gpu parity %s" % field
    narg, hints, claim, roots = gpu_prove(ctx, field, params, nv, session, vecs, pts, covs, evals, nw)
    ref = orc.whir_prove(f, op, nv, session, vecs, pts, covs, evals)
    assert b"".join(roots) == ref.roots
    assert narg == ref.narg
    assert hints == ref.hints
    assert np.array_equal(claim.evaluation_point.reshape(-1), ref.evaluation_point)
    assert np.array_equal(claim.rlc_coefficients.reshape(-1), ref.rlc_coefficients)
    assert orc.whir_verify(f, op, nv, session, nw, narg, hints, pts, covs, evals)
    assert W.Config(field, 1 << nv, params).verify(session, narg, hints, nw, pts, covs, evals)


def test_gpu_proof_is_identical_across_runs_and_contexts(ctx, orc):
    params = W.ProtocolParameters(unique_decoding=True, security_level=100, pow_bits=20)
    f, vecs, pts, covs, evals = statement(orc, "Goldilocks2", 14, 1, 1, 1, False, seed=3)
    a = gpu_prove(ctx, "Goldilocks2", params, 14, "s", vecs, pts, covs, evals, 1)
    b = gpu_prove(ctx, "Goldilocks2", params, 14, "s", vecs, pts, covs, evals, 1)
    ctx2 = W.Context(0)
    c = gpu_prove(ctx2, "Goldilocks2", params, 14, "s", vecs, pts, covs, evals, 1)
    ctx2.close()
    assert a[0] == b[0] == c[0] and a[1] == b[1] == c[1]


def test_d20_goldilocks2_matches_oracle(ctx, orc):
    params = W.ProtocolParameters(unique_decoding=True, security_level=100, pow_bits=20)
    op = orc.make_params(unique_decoding=True, security_level=100, pow_bits=20)
    r = Rng(20)
    vec = r.goldilocks(1 << 20).reshape(1, 1 << 20)
    pt = field_elements("Goldilocks2", 20, rng=r).reshape(20, 2)
    ev = orc.multilinear_extend(orc.GOLDILOCKS2, vec.reshape(-1), pt.reshape(-1))
    narg, hints, claim, roots = gpu_prove(ctx, "Goldilocks2", params, 20, "d20", vec, [pt], [], [[ev]], 1)
    ref = orc.whir_prove(orc.GOLDILOCKS2, op, 20, "d20", vec, [pt], [], [[ev]])
    assert narg == ref.narg and hints == ref.hints
    assert orc.whir_verify(orc.GOLDILOCKS2, op, 20, "d20", 1, narg, hints, [pt], [], [[ev]])


@pytest.mark.parametrize("field", ["Field256", "Field192"])
def test_d20_montgomery_fields_match_oracle(ctx, orc, field):
    # Multi-limb workload shape: d=20, SHA3 Merkle, rate 1/4, k=4, list decoding, security 128,
    # pow 20, 4 uniform random evaluation points; byte-identical to the oracle and accepted by it.
    params = W.ProtocolParameters(unique_decoding=False, security_level=128, pow_bits=20, hash_id="Sha3",
                                  starting_log_inv_rate=2)
    op = orc.make_params(unique_decoding=False, security_level=128, pow_bits=20, hash_id=orc.ENGINE_SHA3,
                         starting_log_inv_rate=2)
    f = orc.FIELD_IDS[field]
    r = Rng(f * 20)
    vec = field_elements(field, 1 << 20, rng=r).reshape(1, 1 << 20, -1)
    pts = [field_elements(field, 20, rng=r).reshape(20, -1) for _ in range(4)]
    evs = [[W.multilinear_evaluate(ctx, f, vec.reshape(-1), p.reshape(-1))] for p in pts]
    for p, e in zip(pts, evs):
        assert np.array_equal(e[0], orc.multilinear_extend(f, vec.reshape(-1), p.reshape(-1)))
    narg, hints, claim, roots = gpu_prove(ctx, field, params, 20, "d20 " + field, vec, pts, [], evs, 1)
    ref = orc.whir_prove(f, op, 20, "d20 " + field, vec, pts, [], evs)
    assert b"".join(roots) == ref.roots
    assert narg == ref.narg and hints == ref.hints
    assert orc.whir_verify(f, op, 20, "d20 " + field, 1, narg, hints, pts, [], evs)


def test_d24_goldilocks2_matches_oracle_and_verifies(ctx, orc):
    # Headline workload: d=24 Goldilocks2, Blake3, rate 1/2, k=4, unique decoding, sec 100, pow 20,
    # one random evaluation point (the seed the benchmark uses). The GPU proof is byte-identical to
    # the oracle prover's (roots, NARG string, hints, final claim), both verifiers accept it, and a
    # proof with a flipped bit is rejected.
    params = W.ProtocolParameters(unique_decoding=True, security_level=100, pow_bits=20)
    op = orc.make_params(unique_decoding=True, security_level=100, pow_bits=20)
    r = Rng(2)
    vec = r.goldilocks(1 << 24).reshape(1, 1 << 24)
    pt = field_elements("Goldilocks2", 24, rng=r).reshape(24, 2)
    ev = orc.multilinear_extend(orc.GOLDILOCKS2, vec.reshape(-1), pt.reshape(-1))
    narg, hints, claim, roots = gpu_prove(ctx, "Goldilocks2", params, 24, "d24", vec, [pt], [], [[ev]], 1)
    ref = orc.whir_prove(orc.GOLDILOCKS2, op, 24, "d24", vec, [pt], [], [[ev]])
    assert b"".join(roots) == ref.roots
    assert narg == ref.narg
    assert hints == ref.hints
    assert np.array_equal(claim.evaluation_point.reshape(-1), ref.evaluation_point)
    assert np.array_equal(claim.rlc_coefficients.reshape(-1), ref.rlc_coefficients)
    assert orc.whir_verify(orc.GOLDILOCKS2, op, 24, "d24", 1, narg, hints, [pt], [], [[ev]])
    cfg = W.Config("Goldilocks2", 1 << 24, params)
    assert cfg.verify("d24", narg, hints, 1, [pt], [], [[ev]])
    bad = bytearray(hints)
    bad[100] ^= 4
    assert not orc.whir_verify(orc.GOLDILOCKS2, op, 24, "d24", 1, narg, bytes(bad), [pt], [], [[ev]])
    assert not cfg.verify("d24", narg, bytes(bad), 1, [pt], [], [[ev]])
    assert hashlib.sha256(narg).hexdigest() != hashlib.sha256(hints).hexdigest()


@pytest.mark.parametrize("field,nv,bs,ud", [("Goldilocks2", 22, 1, True), ("Goldilocks3", 20, 7, False)])
def test_staged_host_upload_matches_device_input(ctx, orc, field, nv, bs, ud):
    # Host inputs of at least 16 MiB are copied in message groups on a second stream while the
    # encode's first pass runs (32 MiB: 2 groups of 8 messages; 56 MiB: 3 uneven groups of 112
    # messages). The proof equals the one made from a device-resident copy and the oracle's.
    params = W.ProtocolParameters(unique_decoding=ud, security_level=100, pow_bits=16, batch_size=bs)
    op = orc.make_params(unique_decoding=ud, security_level=100, pow_bits=16, batch_size=bs)
    f, vecs, pts, covs, evals = statement(orc, field, nv, 1, bs, 1, False, seed=nv + bs)
    narg_h, hints_h, _, _ = gpu_prove(ctx, field, params, nv, "staged", vecs, pts, covs, evals, 1)
    flat = np.ascontiguousarray(vecs, dtype=np.uint64).reshape(-1)
    dptr = ctx.alloc(flat.nbytes)
    try:
        ctx.upload(dptr, flat)
        cfg = W.Config(field, 1 << nv, params)
        ps = W.ProverState(cfg, "staged")
        w = cfg.commit(ctx, ps, dptr, on_device=True)
        cfg.prove(ctx, ps, dptr, [w], pts, covs, evals, on_device=True)
        narg_d, hints_d = ps.proof()
    finally:
        ctx.free(dptr)
    assert narg_h == narg_d and hints_h == hints_d
    ref = orc.whir_prove(f, op, nv, "staged", vecs, pts, covs, evals)
    assert narg_h == ref.narg and hints_h == ref.hints
