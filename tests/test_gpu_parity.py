"""GPU parity: every kernel of the prover path, called through the C ABI, against the CPU oracle on
the same seeded inputs. Integer / finite-field work: the bar is bit-exact equality."""

import hashlib

import numpy as np
import pytest

import whir_gb300 as W
from whir_gb300.inputs import Rng, field_elements

pytestmark = pytest.mark.gpu

FIELDS = [("Goldilocks1", W.GOLDILOCKS1), ("Goldilocks2", W.GOLDILOCKS2), ("Goldilocks3", W.GOLDILOCKS3),
          ("Field192", W.FIELD192), ("Field256", W.FIELD256)]
BASE_NAME = {"Goldilocks1": "Goldilocks1", "Goldilocks2": "Goldilocks1", "Goldilocks3": "Goldilocks1",
             "Field192": "Field192", "Field256": "Field256"}


@pytest.mark.parametrize("fname,fid", FIELDS)
@pytest.mark.parametrize("n_msgs,msg_len,codeword_len", [
    (1, 1, 1), (2, 1, 64), (16, 1, 1 << 10), (16, 16, 1 << 12), (16, 256, 1 << 12), (4, 8, 8),
    (16, 1 << 10, 1 << 11), (16, 1 << 12, 1 << 16), (8, 1 << 14, 1 << 15), (16, 3, 64), (2, 1 << 16, 1 << 17),
    (3, 5, 32),
])
def test_encode_parity(ctx, orc, fname, fid, n_msgs, msg_len, codeword_len):
    rng = Rng(n_msgs * 1000 + msg_len + codeword_len)
    L = W.TARGET_LIMBS[fid]
    msgs = field_elements(fname, n_msgs * msg_len, rng=rng).reshape(n_msgs, msg_len, L) if L > 1 else \
        field_elements(fname, n_msgs * msg_len, rng=rng).reshape(n_msgs, msg_len)
    got = W.interleaved_encode(ctx, fid, msgs, codeword_len)
    exp = orc.interleaved_encode(fid, msgs, None, codeword_len)
    assert np.array_equal(got, exp)


@pytest.mark.parametrize("fname,fid", FIELDS)
@pytest.mark.parametrize("n_msgs,msg_len,mask_len,codeword_len", [
    (1, 1, 1, 4), (4, 6, 2, 16), (16, 1000, 24, 1 << 12), (3, 0, 5, 8), (16, 1 << 12, 3, 1 << 14),
])
def test_encode_with_masks_parity(ctx, orc, fname, fid, n_msgs, msg_len, mask_len, codeword_len):
    # ReedSolomon::interleaved_encode with masks: message m is msgs[m] followed by masks[m], so the
    # coset size follows msg_len + mask_len.
    rng = Rng(n_msgs * 7 + msg_len * 3 + mask_len)
    L = W.TARGET_LIMBS[fid]
    msgs = field_elements(fname, n_msgs * msg_len, rng=rng).reshape(n_msgs, msg_len, L)
    masks = field_elements(fname, n_msgs * mask_len, rng=rng).reshape(n_msgs, mask_len, L)
    if L == 1:
        msgs, masks = msgs.reshape(n_msgs, msg_len), masks.reshape(n_msgs, mask_len)
    got = W.interleaved_encode(ctx, fid, msgs, codeword_len, masks=masks)
    exp = orc.interleaved_encode(fid, msgs, masks, codeword_len)
    assert np.array_equal(got, exp)


def test_encode_rejects_unsupported_and_invalid_shapes(ctx):
    # Non-power-of-two codewords (valid for the reference's mixed-radix engine, unused by WHIR) are
    # refused with WHIR_ERR_UNSUPPORTED; a message longer than the codeword with WHIR_ERR_INVALID.
    msgs = np.ones((2, 4), np.uint64)
    with pytest.raises(W.WhirError) as e:
        W.interleaved_encode(ctx, W.GOLDILOCKS1, msgs, 12)
    assert e.value.code == -2
    with pytest.raises(W.WhirError) as e:
        W.interleaved_encode(ctx, W.GOLDILOCKS1, np.ones((2, 40), np.uint64), 32)
    assert e.value.code == -1
    with pytest.raises(W.WhirError):
        W.interleaved_encode(ctx, W.GOLDILOCKS1, msgs, 16, masks=np.ones((3, 2), np.uint64))


@pytest.mark.parametrize("fname,fid", FIELDS[3:])
def test_encode_montgomery_fields_four_step(ctx, orc, fname, fid):
    # Field192/Field256 rows are 24/32 bytes per element: the d=20, rate-1/4 initial shape (16 messages
    # of 2^16 -> 2^18 rows) runs the four-step path; checked at spot rows against the oracle's
    # univariate evaluation at the row's evaluation point.
    rng = Rng(fid * 77)
    L = W.TARGET_LIMBS[fid]
    msgs = field_elements(fname, 16 << 16, rng=rng).reshape(16, 1 << 16, L)
    cw = W.interleaved_encode(ctx, fid, msgs, 1 << 18)
    rows = [0, 1, 5, 77777, (1 << 16) - 1, 1 << 16, (1 << 18) - 1]
    pts = orc.evaluation_points(fid, 1 << 16, 1 << 18, np.array(rows, np.uint64))
    for r, x in zip(rows, pts.reshape(len(rows), L)):
        for m in (0, 9, 15):
            v = orc.univariate_evaluate(fid, msgs[m].reshape(-1), x)
            assert np.array_equal(cw[r, m], v)


def test_encode_d24_initial_shape_properties(ctx, orc):
    # Full d=24 initial commitment shape (16 x 2^20 -> 2^21 x 16): size-independent checks —
    # spot rows equal the polynomial evaluation at evaluation_points(row) computed by the oracle.
    rng = Rng(24)
    msgs = rng.goldilocks(16 << 20).reshape(16, 1 << 20)
    cw = W.interleaved_encode(ctx, W.GOLDILOCKS1, msgs, 1 << 21)
    rows = [0, 1, 2, 12345, (1 << 20) - 1, 1 << 20, (1 << 21) - 1, 1777777]
    pts = orc.evaluation_points(orc.GOLDILOCKS1, 1 << 20, 1 << 21, rows)
    for r, x in zip(rows, pts):
        for m in (0, 7, 15):
            v = orc.univariate_evaluate(orc.GOLDILOCKS1, msgs[m], np.array([x], np.uint64))
            assert int(cw[r, m]) == int(v[0])


@pytest.mark.parametrize("fname,fid", FIELDS)
@pytest.mark.parametrize("n", [1, 7, 4096, 100003])
def test_lift_parity(ctx, orc, fid, fname, n):
    # lift maps each source element into the target field (Embedding::map, embedding.rs:141-153):
    # the constant coefficient of a Goldilocks extension with zeros above it, the identity for the
    # prime fields (canonical limbs in and out, also for the Montgomery-form fields).
    rng = Rng(n + 5 * fid)
    src = field_elements(BASE_NAME[fname], n, rng=rng).reshape(n, -1)
    got = W.lift(ctx, fid, src).reshape(n, -1)
    L, S = W.TARGET_LIMBS[fid], W.SOURCE_LIMBS[fid]
    want = np.zeros((n, L), np.uint64)
    want[:, :S] = src
    assert np.array_equal(got, want)


@pytest.mark.parametrize("engine", ["Blake3", "Sha2", "Sha3", "Keccak"])
@pytest.mark.parametrize("size", [0, 4, 32, 60, 64, 128, 132, 256, 384, 512, 1020, 1024])
def test_hash_many_parity(ctx, orc, engine, size):
    count = 37
    data = np.random.default_rng(size).integers(0, 256, size=size * count, dtype=np.uint8).tobytes()
    got = W.hash_many(ctx, engine, size, data, count)
    exp = orc.hash_many(W.ENGINES[engine], size, data, count)
    assert got == exp
    if engine == "Sha3":
        assert got[:32] == hashlib.sha3_256(data[:size]).digest()
    if engine == "Sha2":
        assert got[:32] == hashlib.sha256(data[:size]).digest()


@pytest.mark.parametrize("engine", ["Blake3", "Sha2", "Sha3", "Keccak"])
@pytest.mark.parametrize("n", [1, 2, 3, 5, 512, 513, 1 << 12, (1 << 14) + 3])
def test_merkle_parity(ctx, orc, engine, n):
    leaves = np.random.default_rng(n).integers(0, 256, size=32 * n, dtype=np.uint8).tobytes()
    assert W.merkle_nodes(ctx, engine, leaves) == orc.merkle_commit(W.ENGINES[engine], leaves)


@pytest.mark.parametrize("fname,fid", FIELDS)
@pytest.mark.parametrize("n", [1, 2, 4, 8, 1 << 10, 1 << 16, 1 << 18, 1 << 20])
def test_sumcheck_fold_parity(ctx, orc, fname, fid, n):
    rng = Rng(n + fid)
    L = W.TARGET_LIMBS[fid]
    a = field_elements(fname, n, rng=rng).reshape(-1)
    b = field_elements(fname, n, rng=rng).reshape(-1)
    w = field_elements(fname, 1, rng=rng).reshape(-1)
    c0, c2 = W.sumcheck_polynomial(ctx, fid, a, b)
    e0, e2 = orc.sumcheck_poly(fid, a, b)
    assert np.array_equal(c0, e0) and np.array_equal(c2, e2)
    assert np.array_equal(W.fold(ctx, fid, a, w), orc.fold(fid, a, w))


@pytest.mark.parametrize("fname,fid", FIELDS)
@pytest.mark.parametrize("nv", [0, 1, 2, 5, 11, 16, 20])
def test_eval_eq_parity(ctx, orc, fname, fid, nv):
    rng = Rng(nv * 3 + fid)
    acc = field_elements(fname, 1 << nv, rng=rng).reshape(-1)
    pt = field_elements(fname, nv, rng=rng).reshape(-1)
    s = field_elements(fname, 1, rng=rng).reshape(-1)
    assert np.array_equal(W.eval_eq(ctx, fid, acc, pt, s), orc.eval_eq(fid, acc, pt, s))


@pytest.mark.parametrize("fname,fid", FIELDS)
@pytest.mark.parametrize("n,m", [(1, 1), (37, 5), (4096, 1), (5000, 70), (1 << 16, 193), (1 << 18, 88)])
def test_geometric_accumulate_parity(ctx, orc, fname, fid, n, m):
    rng = Rng(n + m + fid)
    acc = field_elements(fname, n, rng=rng).reshape(-1)
    s = field_elements(fname, m, rng=rng).reshape(-1)
    x = field_elements(fname, m, rng=rng).reshape(-1)
    assert np.array_equal(W.geometric_accumulate(ctx, fid, acc, s, x), orc.geometric_accumulate(fid, acc, s, x))


@pytest.mark.parametrize("fname,fid", FIELDS)
@pytest.mark.parametrize("n", [1, 2, 31, 32, 33, 8192, 100000, 1 << 20])
def test_univariate_parity(ctx, orc, fid, fname, n):
    rng = Rng(n + 11 * fid)
    c = field_elements(BASE_NAME[fname], n, rng=rng).reshape(-1)
    x = field_elements(fname, 1, rng=rng).reshape(-1)
    assert np.array_equal(W.univariate_evaluate(ctx, fid, c, x), orc.univariate_evaluate(fid, c, x))


@pytest.mark.parametrize("engine", ["Blake3", "Sha2", "Sha3", "Keccak"])
@pytest.mark.parametrize("bits", [1, 8, 16, 20])
def test_pow_lowest_nonce_parity(ctx, orc, engine, bits):
    chal = hashlib.sha256(b"%s-%d" % (engine.encode(), bits)).digest()
    thr = orc.pow_threshold(float(bits))
    assert W.pow_grind(ctx, engine, chal, thr) == orc.pow_grind(W.ENGINES[engine], chal, thr)


@pytest.mark.parametrize("seed", range(6))
def test_pow_blake3_split_round_parity(ctx, orc, seed):
    # The Blake3 search computes the nonce-independent part of round 1 once per challenge; lowest
    # nonces over several challenges and difficulties equal the oracle's full compressions.
    chal = hashlib.sha256(b"split-%d" % seed).digest()
    for bits in (3, 12, 18):
        thr = orc.pow_threshold(float(bits))
        assert W.pow_grind(ctx, "Blake3", chal, thr) == orc.pow_grind(W.ENGINES["Blake3"], chal, thr)


def test_evaluation_points_parity(orc):
    for masked, cw in ((1, 2), (16, 64), (1 << 16, 1 << 20), (4, 1 << 16)):
        idx = np.array([0, 1, cw // 3, cw - 1], np.uint64)
        for fname, fid in FIELDS:
            assert np.array_equal(W.evaluation_points(fid, masked, cw, idx), orc.evaluation_points(fid, masked, cw, idx))
