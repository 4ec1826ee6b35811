"""Pins the CPU oracle against the reference crate's own known answers (tests/golden/reference_kats.json,
extracted from the reference sources by tests/golden/make_reference_kats.py) and against hashlib."""

import hashlib
import json
import os

import numpy as np
import pytest

from whir_gb300.inputs import GOLDILOCKS_P as P, Rng, field_elements

import blake3_spec

KATS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))


def test_engine_ids_match_reference_and_hashlib(orc):
    # mod.rs:88-103: EngineId = SHA3-256("whir::hash" || oid or name)
    for name, pre in KATS["engine_id_preimages"].items():
        tail = bytes.fromhex(pre["oid_der_body"]) if "oid_der_body" in pre else pre["name"].encode()
        assert hashlib.sha3_256(b"whir::hash" + tail).hexdigest() == KATS["engine_ids"][name]["hex"]
    assert orc.ENGINE_BLAKE3.hex() == KATS["engine_ids"]["BLAKE3"]["hex"]
    assert orc.ENGINE_SHA2.hex() == KATS["engine_ids"]["SHA2"]["hex"]
    assert orc.ENGINE_SHA3.hex() == KATS["engine_ids"]["SHA3"]["hex"]
    assert orc.ENGINE_KECCAK.hex() == KATS["engine_ids"]["KECCAK"]["hex"]
    assert orc.ENGINE_COPY.hex() == KATS["engine_ids"]["COPY"]["hex"]


def test_blake3_empty_hash(orc):
    # blake3_engine.rs:23 EMPTY_HASH pins the compression function, IV and flags
    assert orc.hash_many(orc.ENGINE_BLAKE3, 0, b"", 3) == bytes.fromhex(KATS["blake3_empty_hash"]["hex"]) * 3


@pytest.mark.parametrize("n", [1, 63, 64, 65, 128, 200, 576, 1023, 1024, 1025, 2048, 2049, 3072, 4096, 4097, 9000])
def test_blake3_against_spec_restatement(orc, n):
    # Several blocks per chunk, partial last blocks and the parent-node tree above one chunk, checked
    # against a plain-Python restatement of the BLAKE3 specification, itself pinned by EMPTY_HASH.
    assert blake3_spec.blake3(b"") == bytes.fromhex(KATS["blake3_empty_hash"]["hex"])
    rng = np.random.default_rng(1000 + n)
    for count in (1, 2):
        msgs = rng.integers(0, 256, size=n * count, dtype=np.uint8).tobytes()
        exp = b"".join(blake3_spec.blake3(msgs[i * n:(i + 1) * n]) for i in range(count))
        assert orc.hash_many(orc.ENGINE_BLAKE3, n, msgs, count) == exp


@pytest.mark.parametrize("n", [0, 1, 3, 31, 32, 64, 100, 135, 136, 137, 271, 272, 500, 1024])
def test_sha2_sha3_against_hashlib(orc, n):
    rng = np.random.default_rng(n)
    for count in (1, 3):
        msgs = rng.integers(0, 256, size=n * count, dtype=np.uint8).tobytes()
        got = orc.hash_many(orc.ENGINE_SHA3, n, msgs, count)
        exp = b"".join(hashlib.sha3_256(msgs[i * n:(i + 1) * n]).digest() for i in range(count))
        assert got == exp
        got = orc.hash_many(orc.ENGINE_SHA2, n, msgs, count)
        exp = b"".join(hashlib.sha256(msgs[i * n:(i + 1) * n]).digest() for i in range(count))
        assert got == exp


def test_keccak256_padding(orc):
    # Keccak-256 shares the permutation with SHA3-256 (pinned above); its empty-input digest is the
    # widely published constant c5d2...a470.
    assert orc.hash_many(orc.ENGINE_KECCAK, 0, b"", 1).hex() == \
        "c5d2460186f7233c927e7db2dcc703c0e500b653ca82273b7bfad8045d85a470"


def test_copy_engine(orc):
    out = orc.hash_many(orc.ENGINE_COPY, 5, b"abcdefghij", 2)
    assert out == b"abcde" + b"\0" * 27 + b"fghij" + b"\0" * 27
    with pytest.raises(RuntimeError):
        orc.hash_many(orc.ENGINE_COPY, 33, b"x" * 33, 1)


def test_sha3_512_against_hashlib(orc):
    for n in (0, 7, 71, 72, 73, 200):
        m = bytes(range(n % 256)) * (n // 256 + 1)
        m = m[:n]
        assert orc.sha3_512(m) == hashlib.sha3_512(m).digest()


def test_goldilocks_roots(orc):
    g = KATS["goldilocks"]
    assert g["modulus"] == P
    order = g["engine_order"]
    w = int(orc.ntt_root(0, order)[0])
    assert w == pow(g["generator"], (P - 1) // order, P)  # cooley_tukey.rs:583-595
    for n in (2, 4, 8, 16, 3, 6, 12, 1 << 20):
        r = int(orc.ntt_root(0, n)[0])
        assert pow(r, n, P) == 1
        for p in (2, 3):
            if n % p == 0:
                assert pow(r, n // p, P) != 1
    # root(16)^2 == root(8) etc. (cooley_tukey.rs:611-621)
    r16 = int(orc.ntt_root(0, 16)[0])
    assert pow(r16, 2, P) == int(orc.ntt_root(0, 8)[0])
    assert pow(r16, 8, P) == int(orc.ntt_root(0, 2)[0]) == P - 1
    assert orc.next_order(0, 5) == 6 and orc.next_order(0, 7) == 8 and orc.next_order(0, 1 << 20) == 1 << 20


def naive_poly_eval(coeffs, x):
    v = 0
    for c in reversed(coeffs):
        v = (v * x + c) % P
    return v


@pytest.mark.parametrize("msg_len,codeword_len", [(1, 2), (2, 4), (3, 8), (4, 8), (5, 12), (6, 6), (8, 32), (16, 32),
                                                  (9, 24), (7, 24), (3, 96)])
def test_encode_matches_polynomial_evaluation(orc, msg_len, codeword_len):
    # ntt/mod.rs:158-222 property: codeword row i = message evaluated at evaluation_points(i)
    rng = Rng(msg_len * 100 + codeword_len)
    msgs = rng.goldilocks(3 * msg_len).reshape(3, msg_len)
    cw = orc.interleaved_encode(orc.GOLDILOCKS1, msgs, None, codeword_len)
    pts = orc.evaluation_points(orc.GOLDILOCKS1, msg_len, codeword_len, list(range(codeword_len)))
    for i in range(codeword_len):
        for m in range(3):
            assert int(cw[i, m]) == naive_poly_eval([int(c) for c in msgs[m]], int(pts[i]))
    assert len(set(int(p) for p in pts)) == codeword_len  # evaluation points are unique


def test_challenge_indices_mock_sponge_kats(orc):
    for case in KATS["challenge_indices"]:
        got = orc.challenge_indices_replay(bytes(case["squeeze"]), case["num_leaves"], case["count"], case["dedup"])
        assert got == case["expected"], case["name"]


def test_pow_threshold_and_difficulty_kats(orc):
    for bits, thr in KATS["pow_threshold"]:
        assert orc.pow_threshold(bits) == thr
    for thr, bits in KATS["pow_difficulty"]:
        assert orc.pow_difficulty(thr) == bits


def test_layers_for_size(orc):
    for n, layers in KATS["layers_for_size"]:
        assert orc.layers_for_size(n) == layers


def test_pow_grind_lowest_nonce(orc):
    chal = bytes(range(32))
    thr = 1 << 56  # 8 bits
    nonce = orc.pow_grind(orc.ENGINE_BLAKE3, chal, thr)
    for k in range(nonce + 1):
        h = orc.hash_many(orc.ENGINE_BLAKE3, 64, chal + k.to_bytes(8, "little") + b"\0" * 24, 1)
        ok = int.from_bytes(h[:8], "little") <= thr
        assert ok == (k == nonce)


def _zero_pad(v, L):
    n = v.shape[0]
    m = 1 << max(0, (n - 1).bit_length()) if n else 0
    out = np.zeros((m, L), np.uint64)
    out[:n] = v.reshape(n, L)
    return out


@pytest.mark.parametrize("length", [0, 1, 2, 3, 5, 8, 13, 64, 100])
def test_sumcheck_and_fold_zero_padding(orc, length):
    # algebra/sumcheck.rs:160-188: implicit zero padding equals explicit padding
    f = orc.GOLDILOCKS2
    rng = Rng(length + 7)
    a = field_elements("Goldilocks2", length, rng=rng).reshape(length, 2)
    b = field_elements("Goldilocks2", length, rng=rng).reshape(length, 2)
    pa, pb = _zero_pad(a, 2), _zero_pad(b, 2)
    e0, e2 = orc.sumcheck_poly(f, pa, pb)
    c0, c2 = orc.sumcheck_poly(f, a, b)
    assert (c0 == e0).all() and (c2 == e2).all()
    w = field_elements("Goldilocks2", 1, rng=rng).reshape(2)
    assert (orc.fold(f, a, w) == orc.fold(f, pa, w)).all()


def test_eval_eq_matches_definition(orc):
    f = orc.GOLDILOCKS1
    rng = Rng(3)
    pt = rng.goldilocks(4)
    s = rng.goldilocks(1)
    acc = orc.eval_eq(f, np.zeros(16, np.uint64), pt, s)
    for i in range(16):
        v = int(s[0])
        for k in range(4):
            bit = (i >> (3 - k)) & 1
            v = v * (int(pt[k]) if bit else (1 - int(pt[k])) % P) % P
        assert int(acc[i]) == v


def test_geometric_accumulate_matches_definition(orc):
    f = orc.GOLDILOCKS1
    rng = Rng(9)
    acc0 = rng.goldilocks(37)
    s = rng.goldilocks(5)
    x = rng.goldilocks(5)
    acc = orc.geometric_accumulate(f, acc0, s, x)
    for i in range(37):
        v = int(acc0[i])
        for j in range(5):
            v = (v + int(s[j]) * pow(int(x[j]), i, P)) % P
        assert int(acc[i]) == v


def test_config_schedule_d24(orc):
    # Round schedule for d=24 Goldilocks2, unique decoding, sec 100, pow 20, rate 1/2, k=4:
    # q = 193, 88, 81, 81, 81, 81; codewords 2^21, 2^20 .. 2^16 (irs_commit.rs:125-196, config.rs:65-122)
    p = orc.make_params(unique_decoding=True, security_level=100, pow_bits=20)
    c = orc.whir_config_json(orc.GOLDILOCKS2, p, 24)
    assert c["initial_committer"]["in_domain_samples"] == 193
    assert c["initial_committer"]["codeword_length"] == 1 << 21
    assert [r["irs"]["in_domain_samples"] for r in c["rounds"]] == [88, 81, 81, 81, 81]
    assert [r["irs"]["codeword_length"] for r in c["rounds"]] == [1 << 20, 1 << 19, 1 << 18, 1 << 17, 1 << 16]
    assert c["final_sumcheck"]["initial_size"] == 1 and c["final_sumcheck"]["num_rounds"] == 0
    assert all(r["sumcheck"]["round_pow_threshold"] == 2**64 - 1 for r in c["rounds"])
    for r in c["rounds"]:
        assert 19.0 <= orc.pow_difficulty(r["pow_threshold"]) <= 20.0


def test_config_list_decoding_pow_infeasible_goldilocks2(orc):
    # Goldilocks2 with list decoding at security 100 needs ~38.8 fold-PoW bits in the first round.
    p = orc.make_params(unique_decoding=False, security_level=100, pow_bits=20)
    c = orc.whir_config_json(orc.GOLDILOCKS2, p, 24)
    assert 38 < orc.pow_difficulty(c["initial_sumcheck"]["round_pow_threshold"]) < 39.5


CASES = [
    # field, nv, unique, k, points, pow_bits, hash, security, batch, witnesses, rate, covector
    ("Goldilocks2", 8, True, 2, 1, 5, "SHA2", 32, 1, 1, 1, False),
    ("Goldilocks2", 10, False, 2, 2, 5, "BLAKE3", 32, 1, 1, 1, False),
    ("Goldilocks3", 9, False, 3, 1, 0, "BLAKE3", 32, 1, 1, 1, True),
    ("Goldilocks1", 8, True, 4, 0, 0, "KECCAK", 32, 1, 1, 1, False),
    ("Field192", 8, False, 4, 2, 10, "SHA3", 32, 1, 1, 1, False),
    ("Field256", 8, False, 4, 1, 5, "SHA3", 32, 1, 1, 2, False),
    ("Goldilocks3", 8, False, 2, 1, 5, "BLAKE3", 32, 2, 2, 1, False),
    ("Goldilocks2", 12, True, 4, 1, 10, "BLAKE3", 100, 1, 1, 1, False),
]


def make_statement(orc, field, nv, npts, bs, nw, cov, seed=7):
    f = orc.FIELD_IDS[field]
    base = {"Goldilocks2": "Goldilocks1", "Goldilocks3": "Goldilocks1"}.get(field, field)
    r = Rng(seed)
    vecs = field_elements(base, nw * bs * (1 << nv), rng=r).reshape(nw * bs, 1 << nv, -1)
    pts = [field_elements(field, nv, rng=r).reshape(nv, -1) for _ in range(npts)]
    covs = [field_elements(field, 1 << nv, rng=r).reshape(1 << nv, -1)] if cov else []
    evals = [[orc.multilinear_extend(f, v.reshape(-1), pt.reshape(-1)) for v in vecs] for pt in pts]
    L, SL = orc.TARGET_LIMBS[f], orc.SOURCE_LIMBS[f]
    for c in covs:
        row = []
        for v in vecs:
            lifted = np.zeros((1 << nv, L), np.uint64)
            lifted[:, :SL] = v.reshape(1 << nv, SL)
            prod = orc.field_op(f, "mul", c.reshape(-1), lifted.reshape(-1)).reshape(1 << nv, L)
            acc = np.zeros(L, np.uint64)
            for x in prod:
                acc = orc.field_op(f, "add", acc, x)
            row.append(acc)
        evals.append(row)
    return f, vecs, pts, covs, evals


@pytest.mark.parametrize("case", CASES, ids=[c[0] + "-nv%d" % c[1] for c in CASES])
def test_oracle_prove_verify_roundtrip(orc, case):
    # whir/mod.rs:176-303 end to end: commit -> prove -> verify -> FinalClaim::verify, and a
    # tampered NARG string is rejected (whir/mod.rs:521-617 negative test).
    field, nv, ud, k, npts, powb, h, sec, bs, nw, rate, cov = case
    p = orc.make_params(unique_decoding=ud, security_level=sec, pow_bits=powb, hash_id=getattr(orc, "ENGINE_" + h),
                        initial_folding_factor=k, folding_factor=k, starting_log_inv_rate=rate, batch_size=bs)
    f, vecs, pts, covs, evals = make_statement(orc, field, nv, npts, bs, nw, cov)
    pr = orc.whir_prove(f, p, nv, "oracle test", vecs, pts, covs, evals)
    assert orc.whir_verify(f, p, nv, "oracle test", nw, pr.narg, pr.hints, pts, covs, evals)
    bad = bytearray(pr.narg)
    bad[len(bad) // 3] ^= 0x10
    assert not orc.whir_verify(f, p, nv, "oracle test", nw, bytes(bad), pr.hints, pts, covs, evals)
    assert not orc.whir_verify(f, p, nv, "other session", nw, pr.narg, pr.hints, pts, covs, evals)
    if evals:
        wrong = np.array(evals, dtype=np.uint64).copy()
        wrong.reshape(-1)[0] ^= 1
        assert not orc.whir_verify(f, p, nv, "oracle test", nw, pr.narg, pr.hints, pts, covs, wrong)


def test_oracle_proof_fixture(orc):
    # Regression pin of the oracle's own transcript bytes (tests/golden/oracle_proofs.json).
    fx = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "oracle_proofs.json")))
    for case in fx["cases"]:
        p = orc.make_params(**case["params"], hash_id=bytes.fromhex(case["hash_id"]))
        f, vecs, pts, covs, evals = make_statement(orc, case["field"], case["nv"], case["points"], 1, 1, False,
                                                   seed=case["seed"])
        pr = orc.whir_prove(f, p, case["nv"], case["session"], vecs, pts, covs, evals)
        assert hashlib.sha256(pr.narg).hexdigest() == case["narg_sha256"]
        assert hashlib.sha256(pr.hints).hexdigest() == case["hints_sha256"]
