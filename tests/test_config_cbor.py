"""The protocol id preimage: ciborium's CBOR of the serde form of whir::Config
(transcript/mod.rs:111-121). No GPU needed.

The library and the oracle each write it with their own encoder; both must produce the same bytes,
those bytes must decode (with the strict decoder below, itself checked against the RFC 8949
Appendix A examples) into maps whose keys are the reference's struct field names in declaration
order (extracted from the reference sources into golden/reference_kats.json), and the values must be
the derived configuration's values."""

import hashlib
import json
import os
import struct

import numpy as np
import pytest

import whir_gb300 as W

KATS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))
LAYOUT = KATS["serde_config_layout"]
GL_P = 0xFFFFFFFF00000001
F192_P = 3801539170989320091464968600173246866371124347557388484609
F256_P = 21888242871839275222246405745257275088548364400416034343698204186575808495617


class Decoder:
    """Strict CBOR decoder for the subset ciborium writes for serde data: every head must use its
    shortest form, lengths are definite, floats must use the narrowest exact width."""

    def __init__(self, data):
        self.d = data
        self.i = 0

    def byte(self):
        b = self.d[self.i]
        self.i += 1
        return b

    def take(self, n):
        b = self.d[self.i:self.i + n]
        assert len(b) == n, "truncated"
        self.i += n
        return b

    def head(self):
        ib = self.byte()
        major, info = ib >> 5, ib & 31
        if major == 7:
            return major, info, None
        if info < 24:
            return major, info, info
        n = {24: 1, 25: 2, 26: 4, 27: 8}[info]
        v = int.from_bytes(self.take(n), "big")
        assert v >= {1: 24, 2: 256, 4: 65536, 8: 1 << 32}[n], "non-shortest head"
        return major, info, v

    def item(self):
        major, info, v = self.head()
        if major == 0:
            return v
        if major == 1:
            return -1 - v
        if major == 2:
            return bytes(self.take(v))
        if major == 3:
            return self.take(v).decode()
        if major == 4:
            return [self.item() for _ in range(v)]
        if major == 5:
            out = []
            for _ in range(v):
                k = self.item()
                out.append((k, self.item()))
            return out  # ordered (key, value) pairs
        if major == 7:
            if info == 20:
                return False
            if info == 21:
                return True
            if info == 25:
                h = struct.unpack(">e", self.take(2))[0]
                return ("f16", h)
            if info == 26:
                f = struct.unpack(">f", self.take(4))[0]
                assert not _half_exact(f), "binary32 used where binary16 is exact"
                return ("f32", f)
            if info == 27:
                f = struct.unpack(">d", self.take(8))[0]
                assert not _half_exact(f) and not _single_exact(f), "binary64 used where a narrower width is exact"
                return ("f64", f)
        raise AssertionError("unexpected CBOR item %d/%d" % (major, info))

    def whole(self):
        v = self.item()
        assert self.i == len(self.d), "trailing bytes"
        return v


def _half_exact(f):
    try:
        return struct.unpack(">e", struct.pack(">e", f))[0] == f
    except OverflowError:
        return False


def _single_exact(f):
    try:
        return struct.unpack(">f", struct.pack(">f", f))[0] == f
    except OverflowError:
        return False


def decode(data):
    return Decoder(bytes(data)).whole()


# RFC 8949 Appendix A examples (unsigned integers, floats, strings, arrays, maps).
RFC_EXAMPLES = [
    ("00", 0), ("01", 1), ("0a", 10), ("17", 23), ("1818", 24), ("1819", 25), ("1864", 100), ("1903e8", 1000),
    ("1a000f4240", 1000000), ("1b000000e8d4a51000", 1000000000000), ("1bffffffffffffffff", 18446744073709551615),
    ("f90000", ("f16", 0.0)), ("f93c00", ("f16", 1.0)), ("fb3ff199999999999a", ("f64", 1.1)),
    ("f93e00", ("f16", 1.5)), ("f97bff", ("f16", 65504.0)), ("fa47c35000", ("f32", 100000.0)),
    ("fa7f7fffff", ("f32", 3.4028234663852886e38)), ("fb7e37e43c8800759c", ("f64", 1.0e300)),
    ("f90001", ("f16", 5.960464477539063e-8)), ("f90400", ("f16", 0.00006103515625)), ("f9c400", ("f16", -4.0)),
    ("fbc010666666666666", ("f64", -4.1)), ("f4", False), ("f5", True), ("40", b""), ("4401020304", b"\x01\x02\x03\x04"),
    ("60", ""), ("6161", "a"), ("6449455446", "IETF"), ("80", []), ("83010203", [1, 2, 3]),
    ("8301820203820405", [1, [2, 3], [4, 5]]), ("a0", []), ("a201020304", [(1, 2), (3, 4)]),
    ("a26161016162820203", [("a", 1), ("b", [2, 3])]),
]


@pytest.mark.parametrize("hexs,value", RFC_EXAMPLES)
def test_decoder_on_rfc8949_examples(hexs, value):
    assert decode(bytes.fromhex(hexs)) == value


@pytest.mark.parametrize("hexs", ["1800", "190017", "f93c", "fa3f800000", "fb3ff0000000000000"])
def test_decoder_rejects_non_shortest_forms(hexs):
    with pytest.raises(AssertionError):
        decode(bytes.fromhex(hexs))


def keys(pairs):
    return [k for k, _ in pairs]


def as_dict(pairs):
    return dict(pairs)


def check_field_info(pairs, prime, degree):
    assert keys(pairs) == LAYOUT["field_info"]["fields"]
    d = as_dict(pairs)
    p_be = prime.to_bytes((prime.bit_length() + 7) // 8, "big")
    assert d["characteristic"] == p_be and d["characteristic"][0] != 0
    assert d["extension_degree"] == degree


def check_engine(value, engine_id):
    assert value == list(engine_id)


def check_pow(pairs, engine_id, threshold):
    assert keys(pairs) == LAYOUT["pow_config"]["fields"]
    d = as_dict(pairs)
    check_engine(d["hash_id"], engine_id)
    assert d["threshold"] == threshold


def check_sumcheck(pairs, js, prime, degree, engine_id):
    assert keys(pairs) == LAYOUT["sumcheck_config"]["fields"]
    d = as_dict(pairs)
    check_field_info(d["field"], prime, degree)
    assert d["initial_size"] == js["initial_size"] and d["num_rounds"] == js["num_rounds"]
    assert d["mask_length"] == 0
    check_pow(d["round_pow"], engine_id, js["round_pow_threshold"])


def check_irs(pairs, js, prime, degree, engine_id, basefield):
    assert keys(pairs) == LAYOUT["irs_config"]["fields"]
    d = as_dict(pairs)
    emb = d["embedding"]
    assert keys(emb) == LAYOUT["typed_value"]["fields"]
    emb = as_dict(emb)
    kind = "basefield" if basefield else "identity"
    assert emb["type"] == LAYOUT[kind + "_type_info"]["value"]
    assert keys(emb["value"]) == LAYOUT[kind]["fields"]
    check_field_info(emb["value"][0][1], prime, degree)
    for k in ("num_vectors", "vector_size", "codeword_length", "interleaving_depth", "in_domain_samples",
              "out_domain_samples"):
        assert d[k] == js[k], k
    assert d["mask_length"] == 0 and d["deduplicate_in_domain"] is False
    width, slack = d["johnson_slack"]
    assert slack == js["johnson_slack"]
    mc = d["matrix_commit"]
    assert keys(mc) == LAYOUT["matrix_config"]["fields"]
    mc = as_dict(mc)
    check_field_info(mc["element_type"], prime, 1 if basefield else degree)
    assert mc["num_cols"] == js["num_cols"]
    check_engine(mc["leaf_hash_id"], engine_id)
    mt = mc["merkle_tree"]
    assert keys(mt) == LAYOUT["merkle_config"]["fields"]
    mt = as_dict(mt)
    assert mt["num_leaves"] == js["codeword_length"]
    assert len(mt["layers"]) == js["merkle_layers"]
    for layer in mt["layers"]:
        assert keys(layer) == LAYOUT["merkle_layer"]["fields"]
        check_engine(layer[0][1], engine_id)


CONFIGS = [
    ("Goldilocks2", 24, True, 100, 20, 1, 4, "Blake3"),
    ("Goldilocks2", 18, True, 100, 20, 1, 4, "Blake3"),
    ("Goldilocks3", 20, False, 128, 20, 1, 4, "Blake3"),
    ("Goldilocks1", 16, True, 80, 16, 2, 3, "Sha3"),
    ("Field256", 20, False, 128, 20, 2, 4, "Sha3"),
    ("Field192", 20, False, 128, 20, 2, 4, "Keccak"),
    ("Field192", 12, True, 64, 10, 3, 2, "Sha2"),
]


@pytest.mark.parametrize("field,nv,ud,sec,powb,rate,k,h", CONFIGS)
def test_config_cbor_matches_reference_layout_and_oracle(orc, field, nv, ud, sec, powb, rate, k, h):
    params = W.ProtocolParameters(unique_decoding=ud, security_level=sec, pow_bits=powb, starting_log_inv_rate=rate,
                                  initial_folding_factor=k, folding_factor=k, hash_id=h)
    cfg = W.Config(field, 1 << nv, params)
    mine = cfg.cbor()
    op = orc.make_params(unique_decoding=ud, security_level=sec, pow_bits=powb, starting_log_inv_rate=rate,
                         initial_folding_factor=k, folding_factor=k, hash_id=W.ENGINES[h])
    assert mine == orc.whir_config_bytes(orc.FIELD_IDS[field], op, nv)
    js = cfg.json()
    eid = W.ENGINES[h]
    prime = {"Field192": F192_P, "Field256": F256_P}.get(field, GL_P)
    degree = {"Goldilocks2": 2, "Goldilocks3": 3}.get(field, 1)
    top = decode(mine)
    assert keys(top) == LAYOUT["whir_config"]["fields"]
    d = as_dict(top)
    check_irs(d["initial_committer"], js["initial_committer"], prime, degree, eid, basefield=degree > 1)
    check_sumcheck(d["initial_sumcheck"], js["initial_sumcheck"], prime, degree, eid)
    check_pow(d["initial_skip_pow"], eid, js["initial_skip_pow_threshold"])
    assert len(d["round_configs"]) == len(js["rounds"])
    for rc, rj in zip(d["round_configs"], js["rounds"]):
        assert keys(rc) == LAYOUT["round_config"]["fields"]
        r = as_dict(rc)
        check_irs(r["irs_committer"], rj["irs"], prime, degree, eid, basefield=False)
        check_sumcheck(r["sumcheck"], rj["sumcheck"], prime, degree, eid)
        check_pow(r["pow"], eid, rj["pow_threshold"])
    check_sumcheck(d["final_sumcheck"], js["final_sumcheck"], prime, degree, eid)
    check_pow(d["final_pow"], eid, js["final_pow_threshold"])


def test_unique_decoding_slack_is_a_half_precision_zero():
    # johnson_slack = 0.0 in unique decoding: ciborium writes the binary16 zero f9 00 00.
    params = W.ProtocolParameters(unique_decoding=True, security_level=100, pow_bits=20)
    b = W.Config("Goldilocks2", 1 << 16, params).cbor()
    key = b"\x6djohnson_slack"
    assert b.count(key) == 1 + len(W.Config("Goldilocks2", 1 << 16, params).json()["rounds"])
    i = b.index(key) + len(key)
    assert b[i:i + 3] == b"\xf9\x00\x00"


def test_protocol_id_separates_configurations():
    # The protocol id (SHA3-512 of the CBOR) differs between configurations that differ in any field.
    ids = set()
    for field, nv, ud, sec, powb, rate, k, h in CONFIGS:
        params = W.ProtocolParameters(unique_decoding=ud, security_level=sec, pow_bits=powb,
                                      starting_log_inv_rate=rate, initial_folding_factor=k, folding_factor=k,
                                      hash_id=h)
        ids.add(hashlib.sha3_512(W.Config(field, 1 << nv, params).cbor()).digest())
    assert len(ids) == len(CONFIGS)
    assert np.all([len(x) == 64 for x in ids])
