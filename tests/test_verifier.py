"""The library's host-side verifier (whir_verify, a restatement of Config::verify + FinalClaim::verify)
accepts the CPU oracle's proofs — the GPU prover's proofs are byte-identical to those, which the GPU
parity tests check — and rejects tampered proof strings, tampered hints, another session and a wrong
statement. Needs no GPU: verification runs on the host."""

import numpy as np
import pytest

import whir_gb300 as W
from test_oracle_pins import CASES, make_statement

ENGINE_NAMES = {"BLAKE3": "Blake3", "SHA2": "Sha2", "SHA3": "Sha3", "KECCAK": "Keccak"}


def _configs(orc, case):
    field, nv, ud, k, npts, powb, h, sec, bs, nw, rate, cov = case
    params = W.ProtocolParameters(unique_decoding=ud, security_level=sec, pow_bits=powb, hash_id=ENGINE_NAMES[h],
                                  initial_folding_factor=k, folding_factor=k, starting_log_inv_rate=rate,
                                  batch_size=bs)
    op = orc.make_params(unique_decoding=ud, security_level=sec, pow_bits=powb, hash_id=getattr(orc, "ENGINE_" + h),
                         initial_folding_factor=k, folding_factor=k, starting_log_inv_rate=rate, batch_size=bs)
    return W.Config(field, 1 << nv, params), op


@pytest.mark.parametrize("case", CASES, ids=[c[0] + "-nv%d-%d" % (c[1], i) for i, c in enumerate(CASES)])
def test_verifier_accepts_oracle_proofs_and_rejects_tampering(orc, case):
    field, nv, ud, k, npts, powb, h, sec, bs, nw, rate, cov = case
    cfg, op = _configs(orc, case)
    f, vecs, pts, covs, evals = make_statement(orc, field, nv, npts, bs, nw, cov, seed=nv + 5)
    session = "verifier test"
    pr = orc.whir_prove(f, op, nv, session, vecs, pts, covs, evals)
    assert cfg.verify(session, pr.narg, pr.hints, nw, pts, covs, evals)
    bad = bytearray(pr.narg)
    bad[len(bad) // 2] ^= 0x04
    assert not cfg.verify(session, bytes(bad), pr.hints, nw, pts, covs, evals)
    assert "" != W.last_verify_reason()
    if pr.hints:
        badh = bytearray(pr.hints)
        badh[len(badh) - 5] ^= 0x01
        assert not cfg.verify(session, pr.narg, bytes(badh), nw, pts, covs, evals)
    assert not cfg.verify("another session", pr.narg, pr.hints, nw, pts, covs, evals)
    assert not cfg.verify(session, pr.narg[:-1], pr.hints, nw, pts, covs, evals)
    if len(evals):
        wrong = np.array(evals, dtype=np.uint64).copy()
        wrong.reshape(-1)[0] = (int(wrong.reshape(-1)[0]) + 1) % 0xFFFFFFFF00000001
        assert not cfg.verify(session, pr.narg, pr.hints, nw, pts, covs, wrong)


def test_verifier_rejects_noncanonical_statement(orc):
    case = CASES[0]
    field, nv, ud, k, npts, powb, h, sec, bs, nw, rate, cov = case
    cfg, op = _configs(orc, case)
    f, vecs, pts, covs, evals = make_statement(orc, field, nv, npts, bs, nw, cov, seed=3)
    pr = orc.whir_prove(f, op, nv, "s", vecs, pts, covs, evals)
    big = np.array(pts, dtype=np.uint64).copy()
    big.reshape(-1)[0] = np.uint64(0xFFFFFFFFFFFFFFFF)
    with pytest.raises(W.WhirError):
        cfg.verify("s", pr.narg, pr.hints, nw, big, covs, evals)


def test_verifier_rejects_every_single_byte_corruption_and_truncation(orc):
    # Robustness of the host verifier on malformed proofs: 96 single-byte corruptions spread over the
    # proof string and the hints, truncations at arbitrary lengths and appended bytes are all
    # rejected (WHIR_REJECT, never an exception or an acceptance).
    case = ("Goldilocks2", 10, False, 2, 2, 10, "BLAKE3", 32, 1, 1, 1, False)
    field, nv, ud, k, npts, powb, h, sec, bs, nw, rate, cov = case
    cfg, op = _configs(orc, case)
    f, vecs, pts, covs, evals = make_statement(orc, field, nv, npts, bs, nw, cov, seed=99)
    pr = orc.whir_prove(f, op, nv, "fuzz", vecs, pts, covs, evals)
    assert cfg.verify("fuzz", pr.narg, pr.hints, nw, pts, covs, evals)
    rng = np.random.default_rng(5)
    for buf_name in ("narg", "hints"):
        buf = getattr(pr, buf_name)
        for pos in rng.choice(len(buf), size=48, replace=False):
            bad = bytearray(buf)
            bad[pos] ^= int(rng.integers(1, 256))
            args = (bytes(bad), pr.hints) if buf_name == "narg" else (pr.narg, bytes(bad))
            assert not cfg.verify("fuzz", *args, nw, pts, covs, evals), (buf_name, int(pos))
        for cut in sorted(set(int(c) for c in rng.integers(0, len(buf), size=8))) + [0]:
            args = (buf[:cut], pr.hints) if buf_name == "narg" else (pr.narg, buf[:cut])
            assert not cfg.verify("fuzz", *args, nw, pts, covs, evals), (buf_name, "cut", cut)
        args = (buf + b"\0", pr.hints) if buf_name == "narg" else (pr.narg, buf + b"\0")
        assert not cfg.verify("fuzz", *args, nw, pts, covs, evals), (buf_name, "appended")
