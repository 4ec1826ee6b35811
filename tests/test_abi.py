"""C-ABI checks that need no GPU: the library builds for sm_103a, loads, exports every entry point
include/whir_gb300.h declares, and fails loudly (no CPU fallback) when no device is present."""

import ctypes
import os
import re

import numpy as np
import pytest

import whir_gb300 as W

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "whir_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(whir_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("whir_ctx_create", "whir_config_new", "whir_commit", "whir_prove", "whir_rs_interleaved_encode",
                     "whir_hash_many", "whir_merkle_nodes", "whir_sumcheck_polynomial", "whir_fold", "whir_eval_eq",
                     "whir_geometric_accumulate", "whir_univariate_evaluate", "whir_pow_grind"):
        assert required in names


def test_library_exports_every_declared_symbol():
    lib = W.load_library()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_config_and_transcript_without_device():
    # Parameter selection and the transcript are host code and work without a GPU.
    p = W.ProtocolParameters(unique_decoding=True, security_level=100, pow_bits=20)
    c = W.Config("Goldilocks2", 1 << 24, p)
    j = c.json()
    assert j["initial_committer"]["in_domain_samples"] == 193
    assert [r["irs"]["in_domain_samples"] for r in j["rounds"]] == [88, 81, 81, 81, 81]
    ps = W.ProverState(c, "session")
    narg, hints = ps.proof()
    assert narg == b"" and hints == b""


def test_config_matches_oracle(orc):
    # The library's Config::new restatement and the oracle's agree on every derived value.
    for field in ("Goldilocks1", "Goldilocks2", "Goldilocks3", "Field192", "Field256"):
        for ud in (True, False):
            for nv, k, sec, powb, rate in ((10, 2, 32, 5, 1), (16, 4, 100, 20, 1), (20, 4, 128, 20, 2),
                                           (24, 4, 100, 20, 1), (13, 3, 80, 10, 3)):
                try:
                    p = W.ProtocolParameters(unique_decoding=ud, security_level=sec, pow_bits=powb,
                                             initial_folding_factor=k, folding_factor=k, starting_log_inv_rate=rate)
                    mine = W.Config(field, 1 << nv, p).json()
                except W.WhirError as e:
                    with pytest.raises(RuntimeError):
                        orc.whir_config_json(orc.FIELD_IDS[field], orc.make_params(
                            unique_decoding=ud, security_level=sec, pow_bits=powb, initial_folding_factor=k,
                            folding_factor=k, starting_log_inv_rate=rate), nv)
                    continue
                op = orc.make_params(unique_decoding=ud, security_level=sec, pow_bits=powb, initial_folding_factor=k,
                                     folding_factor=k, starting_log_inv_rate=rate)
                theirs = orc.whir_config_json(orc.FIELD_IDS[field], op, nv)
                assert mine == theirs, (field, ud, nv)


def test_config_bytes_match_oracle(orc):
    # The protocol id hashes identical configuration bytes in both implementations (the CBOR of the
    # configuration, a map of six entries), so a GPU transcript and an oracle transcript with the same
    # session start from the same sponge state.
    p = W.ProtocolParameters(unique_decoding=True, security_level=100, pow_bits=20)
    c = W.Config("Goldilocks2", 1 << 12, p)
    ob = orc.whir_config_bytes(orc.GOLDILOCKS2, orc.make_params(unique_decoding=True, security_level=100,
                                                                pow_bits=20), 12)
    assert ob == c.cbor()
    assert ob[:1] == b"\xa6" and ob[1:19] == b"\x71initial_committer"


def test_no_device_fails_loudly():
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a CUDA device is present")
    with pytest.raises(W.WhirError) as e:
        W.Context(0)
    assert e.value.code in (-4, -3)


def test_invalid_arguments_return_error_codes():
    # Host-side argument checks of the boundary return negative statuses (never abort): a size that is
    # not a power of two, unknown field and engine ids, a null parameter block and a null
    # configuration; an empty proof is a rejection, not an error.
    lib = W.load_library()
    p = W.ProtocolParameters(unique_decoding=True, security_level=100, pow_bits=20)
    with pytest.raises(W.WhirError) as e:
        W.Config("Goldilocks2", 3 << 10, p)
    assert e.value.code < 0
    params = W._Params()
    params.unique_decoding = 1
    params.starting_log_inv_rate = 1
    params.initial_folding_factor = 4
    params.folding_factor = 4
    params.security_level = 100
    params.pow_bits = 20
    params.batch_size = 1
    out = ctypes.c_void_p()
    assert lib.whir_config_new(ctypes.c_int(7), ctypes.byref(params), ctypes.c_uint64(1 << 12), ctypes.byref(out)) < 0
    params.hash_id = (ctypes.c_uint8 * 32)(*([0xAB] * 32))
    assert lib.whir_config_new(ctypes.c_int(W.GOLDILOCKS2), ctypes.byref(params), ctypes.c_uint64(1 << 12),
                               ctypes.byref(out)) < 0
    assert lib.whir_config_new(ctypes.c_int(W.GOLDILOCKS2), None, ctypes.c_uint64(1 << 12), ctypes.byref(out)) < 0
    c = W.Config("Goldilocks2", 1 << 10, p)
    pt = np.zeros((10, 2), np.uint64)
    assert not c.verify("s", b"", b"", 1, [pt], [], [[np.zeros(2, np.uint64)]])  # empty proof: rejected
    assert lib.whir_verify(None, None, 0, None, 0, None, 0, 1, None, 0, None, 0, None) < 0


def test_autotune_table_import_export_without_device():
    # The tuning table is host state: import validates each line (a plan the kernels cannot run is
    # refused), export writes it back in a canonical order, clear empties it.
    W.autotune_clear()
    try:
        W.autotune_import("encode 16 1048576 2097152 8 1 9 4 1\nmerkle 21 9\n")
        assert W.autotune_export() == "encode 16 1048576 2097152 8 1 9 4 1\nmerkle 21 9\n"
        for bad in ("encode 16 1048576 2097152 8 1 9 64 1\n",  # column-pass tile over the shared-memory budget
                    "encode 16 1048576 2097152 8 0 0 0 1\n",   # a whole 2^20-point coset in one CTA
                    "merkle 21 11\n", "nonsense\n"):
            with pytest.raises(W.WhirError):
                W.autotune_import(bad)
        assert W.autotune_export() == "encode 16 1048576 2097152 8 1 9 4 1\nmerkle 21 9\n"
        W.autotune_clear()
        assert W.autotune_export() == ""
    finally:
        W.autotune_clear()
