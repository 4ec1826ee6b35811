"""Row hints of an opening are ark-serialize's compressed encoding of the opened submatrix
(`prover_hint_ark(&submatrix)`, irs_commit.rs:425 -> CanonicalSerialize::serialize_compressed,
transcript/mod.rs:224-233). No GPU needed: the proofs come from the oracle prover, which the GPU
prover matches byte for byte in the -m gpu tests.

ark-serialize 0.5 (a dependency absent from this container) writes, for `Vec<T>` with compression:
the length as a little-endian u64, then each element; a prime-field element (`Fp`, no flags) as its
canonical integer in little-endian over ceil(MODULUS_BIT_SIZE / 8) bytes; an extension element
(`QuadExtField` / `CubicExtField`) as its coefficients c0, c1[, c2] in that order. The test restates
that format in Python and checks the first hint of a proof against the committed codeword: its
length prefix is queries x columns, and every opened row it carries is a row of the initial
codeword (computed by the oracle's encoder), element by element."""

import numpy as np
import pytest

from whir_gb300.inputs import field_elements

MODULUS_BITS = {"Goldilocks1": 64, "Field192": 192, "Field256": 254}


def ark_compressed_vec(elements, limbs, modulus_bits):
    """CanonicalSerialize::serialize_compressed of a Vec of prime-field elements given as canonical
    u64 limbs (little-endian)."""
    width = (modulus_bits + 7) // 8
    out = bytearray(len(elements).to_bytes(8, "little"))
    for e in elements:
        v = 0
        for i in range(limbs):
            v |= int(e[i]) << (64 * i)
        out += v.to_bytes(width, "little")
    return bytes(out)


CASES = [
    # field, nv, unique decoding, folding factor, hash, security, pow bits, rate
    ("Goldilocks2", 10, True, 4, "BLAKE3", 60, 8, 1),
    ("Goldilocks3", 9, False, 3, "SHA3", 40, 5, 1),
    ("Goldilocks1", 8, True, 2, "SHA2", 32, 0, 2),
    ("Field192", 8, False, 2, "KECCAK", 32, 5, 1),
    ("Field256", 8, True, 4, "SHA3", 32, 5, 1),
]


@pytest.mark.parametrize("field,nv,ud,k,h,sec,powb,rate", CASES)
def test_first_row_hint_is_ark_compressed_submatrix(orc, field, nv, ud, k, h, sec, powb, rate):
    from test_oracle_pins import make_statement
    p = orc.make_params(unique_decoding=ud, security_level=sec, pow_bits=powb, hash_id=getattr(orc, "ENGINE_" + h),
                        initial_folding_factor=k, folding_factor=k, starting_log_inv_rate=rate)
    f, vecs, pts, covs, evals = make_statement(orc, field, nv, 1, 1, 1, False, seed=nv + 3)
    proof = orc.whir_prove(f, p, nv, "hint format", vecs, pts, covs, evals)
    cfg = orc.whir_config_json(f, p, nv)["initial_committer"]
    base = {"Goldilocks2": "Goldilocks1", "Goldilocks3": "Goldilocks1"}.get(field, field)
    limbs = orc.SOURCE_LIMBS[f]
    width = (MODULUS_BITS[base] + 7) // 8
    n_msgs, cw = cfg["num_cols"], cfg["codeword_length"]
    msgs = vecs.reshape(n_msgs, (1 << nv) // n_msgs, limbs)
    code = orc.interleaved_encode(orc.BASE_FIELD[f], msgs, None, cw).reshape(cw, n_msgs, limbs)
    rows = {ark_compressed_vec(code[r], limbs, MODULUS_BITS[base])[8:]: r for r in range(cw)}
    q = cfg["in_domain_samples"]
    hints = proof.hints
    count = int.from_bytes(hints[:8], "little")
    assert count == q * n_msgs, "length prefix is the number of opened elements"
    body = hints[8:8 + count * width]
    assert len(body) == count * width
    opened = [body[i * n_msgs * width:(i + 1) * n_msgs * width] for i in range(q)]
    assert all(r in rows for r in opened), "every opened row is a codeword row in ark's element encoding"
    # the restated writer reproduces the hint exactly from the rows it names
    again = ark_compressed_vec([code[rows[r]][c] for r in opened for c in range(n_msgs)], limbs, MODULUS_BITS[base])
    assert hints[:8 + count * width] == again


def test_ark_writer_restatement_known_answers():
    # Known answers of the restated format: a u64 length prefix, then fixed-width little-endian
    # canonical integers (8 bytes for Goldilocks, 32 for the 254-bit Field256).
    assert ark_compressed_vec([], 1, 64) == bytes(8)
    assert ark_compressed_vec([[1]], 1, 64) == bytes([1, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0])
    x = field_elements("Field256", 1).reshape(-1)
    enc = ark_compressed_vec([x], 4, 254)
    assert len(enc) == 8 + 32 and enc[:8] == (1).to_bytes(8, "little")
    assert int.from_bytes(enc[8:], "little") == sum(int(x[i]) << (64 * i) for i in range(4))
    assert np.uint64(0xFFFFFFFF00000000).tobytes() == ark_compressed_vec([[0xFFFFFFFF00000000]], 1, 64)[8:]
