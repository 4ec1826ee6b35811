"""ORACLE — test infrastructure only.

ctypes bindings for the C++ CPU restatement of the WHIR reference (liboracle.so, built from the
sources in this directory by ``make``). Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of bench.py import this package; the product library (whir_gb300) never does.
"""

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lock = threading.Lock()
_lib = None

GOLDILOCKS1, GOLDILOCKS2, GOLDILOCKS3, FIELD192, FIELD256 = 0, 1, 2, 4, 5
FIELD_IDS = {
    "Goldilocks1": GOLDILOCKS1,
    "Goldilocks2": GOLDILOCKS2,
    "Goldilocks3": GOLDILOCKS3,
    "Field192": FIELD192,
    "Field256": FIELD256,
}
# u64 limbs per element of the target field and of the source field of each embedding id.
TARGET_LIMBS = {GOLDILOCKS1: 1, GOLDILOCKS2: 2, GOLDILOCKS3: 3, FIELD192: 3, FIELD256: 4}
SOURCE_LIMBS = {GOLDILOCKS1: 1, GOLDILOCKS2: 1, GOLDILOCKS3: 1, FIELD192: 3, FIELD256: 4}
BASE_FIELD = {GOLDILOCKS1: GOLDILOCKS1, GOLDILOCKS2: GOLDILOCKS1, GOLDILOCKS3: GOLDILOCKS1,
              FIELD192: FIELD192, FIELD256: FIELD256}

ENGINE_BLAKE3 = bytes.fromhex("03e01749ebcc0477924254eb482066b864a8dd4d77252464ca6f5b6f5cc05b4c")
ENGINE_SHA2 = bytes.fromhex("018eaa247cb8957ab1e9fdac885450403c5e7bda1acaaa504e4cc8f2f76bb076")
ENGINE_SHA3 = bytes.fromhex("aa802dcdabad8ea8a1430919893b96c30e31ff5734b385999108aa202d27dc12")
ENGINE_KECCAK = bytes.fromhex("ddd248964e320312a66775aee8e16c88c927734be59aca09b7af6deb0ad00e8c")
ENGINE_COPY = bytes.fromhex("09459020f451874a1b399819d079632cc0f9263b1486c423173c6e15d8e2d61d")


class OracleParams(ctypes.Structure):
    _fields_ = [
        ("unique_decoding", ctypes.c_int32),
        ("starting_log_inv_rate", ctypes.c_uint64),
        ("initial_folding_factor", ctypes.c_uint64),
        ("folding_factor", ctypes.c_uint64),
        ("security_level", ctypes.c_uint64),
        ("pow_bits", ctypes.c_uint64),
        ("batch_size", ctypes.c_uint64),
        ("hash_id", ctypes.c_uint8 * 32),
    ]


def make_params(unique_decoding=True, starting_log_inv_rate=1, initial_folding_factor=4, folding_factor=4,
                security_level=100, pow_bits=20, batch_size=1, hash_id=ENGINE_BLAKE3):
    p = OracleParams()
    p.unique_decoding = int(bool(unique_decoding))
    p.starting_log_inv_rate = starting_log_inv_rate
    p.initial_folding_factor = initial_folding_factor
    p.folding_factor = folding_factor
    p.security_level = security_level
    p.pow_bits = pow_bits
    p.batch_size = batch_size
    p.hash_id[:] = list(hash_id)
    return p


def build(force=False):
    """Compile liboracle.so with make (a few seconds per source file)."""
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            _lib = ctypes.CDLL(_LIB_PATH)
            _declare(_lib)
    return _lib


def _declare(L):
    P = ctypes.POINTER
    u64p, u8p = P(ctypes.c_uint64), P(ctypes.c_uint8)
    sz = ctypes.c_size_t
    L.oracle_last_error.restype = ctypes.c_char_p
    L.oracle_pow_difficulty.restype = ctypes.c_double
    L.oracle_pow_difficulty.argtypes = [ctypes.c_uint64]
    L.oracle_pow_threshold.argtypes = [ctypes.c_double, u64p]
    L.oracle_field_size_bits.restype = ctypes.c_double
    L.oracle_proof_narg.restype = sz
    L.oracle_proof_hints.restype = sz
    L.oracle_proof_eval_point.restype = sz
    L.oracle_proof_rlc.restype = sz
    L.oracle_proof_roots.restype = sz
    L.oracle_proof_free.argtypes = [ctypes.c_void_p]
    for name in ("oracle_proof_narg", "oracle_proof_hints", "oracle_proof_roots"):
        getattr(L, name).argtypes = [ctypes.c_void_p, P(u8p)]
    for name in ("oracle_proof_eval_point", "oracle_proof_rlc"):
        getattr(L, name).argtypes = [ctypes.c_void_p, P(u64p)]


def _check(rc):
    if rc != 0:
        raise RuntimeError("oracle: %s (rc=%d)" % (lib().oracle_last_error().decode(), rc))


def _u64(a):
    a = np.ascontiguousarray(a, dtype=np.uint64)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))


def _u8(b):
    a = np.frombuffer(bytes(b), dtype=np.uint8).copy() if not isinstance(b, np.ndarray) else np.ascontiguousarray(b, dtype=np.uint8)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))


def field_op(field, op, a, b=None):
    ops = {"add": 0, "sub": 1, "mul": 2, "inv": 3, "neg": 4}
    a, pa = _u64(a)
    if b is not None:
        b, pb = _u64(b)
    else:
        pb = None
    out = np.zeros_like(a)
    n = a.size // TARGET_LIMBS[field]
    _check(lib().oracle_field_op(field, ops[op], pa, pb, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                 ctypes.c_size_t(n)))
    return out


def ntt_root(field, order):
    out = np.zeros(TARGET_LIMBS[field], dtype=np.uint64)
    _check(lib().oracle_ntt_root(field, ctypes.c_uint64(order), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))))
    return out


def next_order(field, size):
    out = ctypes.c_uint64()
    rc = lib().oracle_next_order(field, ctypes.c_uint64(size), ctypes.byref(out))
    return None if rc else out.value


def interleaved_encode(field, msgs, masks, codeword_len):
    """msgs: (n_msgs, msg_len[, limbs]) array; returns codeword_len x n_msgs (x limbs)."""
    L = TARGET_LIMBS[field]
    msgs = np.ascontiguousarray(msgs, dtype=np.uint64)
    n_msgs, msg_len = msgs.shape[0], msgs.shape[1]
    masks = np.ascontiguousarray(masks if masks is not None else np.zeros((n_msgs, 0, L)), dtype=np.uint64)
    mask_len = masks.shape[1] if masks.ndim > 1 else 0
    out = np.zeros(codeword_len * n_msgs * L, dtype=np.uint64)
    _, pm = _u64(msgs)
    _, pk = _u64(masks)
    _check(lib().oracle_interleaved_encode(field, pm, ctypes.c_size_t(n_msgs), ctypes.c_size_t(msg_len), pk,
                                           ctypes.c_size_t(mask_len), ctypes.c_size_t(codeword_len),
                                           out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))))
    return out.reshape(codeword_len, n_msgs, L) if L > 1 else out.reshape(codeword_len, n_msgs)


def evaluation_points(field, masked_len, codeword_len, indices):
    L = TARGET_LIMBS[field]
    idx, pidx = _u64(indices)
    out = np.zeros(idx.size * L, dtype=np.uint64)
    _check(lib().oracle_evaluation_points(field, ctypes.c_size_t(masked_len), ctypes.c_size_t(codeword_len), pidx,
                                          ctypes.c_size_t(idx.size),
                                          out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))))
    return out.reshape(idx.size, L) if L > 1 else out


def hash_many(engine_id, size, data, count):
    d, pd = _u8(data) if len(data) else (np.zeros(1, np.uint8), None)
    if pd is None:
        pd = d.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
    out = np.zeros(32 * max(count, 1), dtype=np.uint8)
    _, pid = _u8(engine_id)
    _check(lib().oracle_hash_many(pid, ctypes.c_size_t(size), pd, ctypes.c_size_t(count),
                                  out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))
    return out[: 32 * count].tobytes()


def sha3_512(data):
    d, pd = _u8(data if len(data) else b"\0")
    out = np.zeros(64, dtype=np.uint8)
    _check(lib().oracle_sha3_512(pd, ctypes.c_size_t(len(data)), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))
    return out.tobytes()


def merkle_commit(engine_id, leaves):
    """leaves: bytes of n*32; returns all nodes (num_nodes*32 bytes)."""
    n = len(leaves) // 32
    nn = ctypes.c_size_t()
    _, pid = _u8(engine_id)
    l, pl = _u8(leaves if n else b"\0" * 32)
    _check(lib().oracle_merkle_commit(pid, pl, ctypes.c_size_t(n), None, ctypes.byref(nn)))
    out = np.zeros(nn.value * 32, dtype=np.uint8)
    _check(lib().oracle_merkle_commit(pid, pl, ctypes.c_size_t(n), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                      ctypes.byref(nn)))
    return out.tobytes()


def layers_for_size(n):
    return lib().oracle_layers_for_size(ctypes.c_size_t(n))


def hash_rows(field, engine_id, matrix, rows, cols):
    m, pm = _u64(matrix)
    out = np.zeros(rows * 32, dtype=np.uint8)
    _, pid = _u8(engine_id)
    _check(lib().oracle_hash_rows(field, pid, pm, ctypes.c_size_t(rows), ctypes.c_size_t(cols),
                                  out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))
    return out.tobytes()


def sumcheck_poly(field, a, b):
    L = TARGET_LIMBS[field]
    a, pa = _u64(a)
    b, pb = _u64(b)
    c0 = np.zeros(L, np.uint64)
    c2 = np.zeros(L, np.uint64)
    _check(lib().oracle_sumcheck_poly(field, pa, ctypes.c_size_t(a.size // L), pb, ctypes.c_size_t(b.size // L),
                                      c0.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                      c2.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))))
    return c0, c2


def fold(field, v, w):
    L = TARGET_LIMBS[field]
    v = np.array(v, dtype=np.uint64).copy()
    w, pw = _u64(w)
    nl = ctypes.c_size_t()
    _check(lib().oracle_fold(field, v.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), ctypes.c_size_t(v.size // L),
                             pw, ctypes.byref(nl)))
    return v.reshape(-1)[: nl.value * L]


def eval_eq(field, acc, point, scalar):
    L = TARGET_LIMBS[field]
    acc = np.array(acc, dtype=np.uint64).copy()
    point, pp = _u64(point)
    scalar, ps = _u64(scalar)
    _check(lib().oracle_eval_eq(field, acc.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), pp,
                                ctypes.c_size_t(point.size // L), ps))
    return acc


def geometric_accumulate(field, acc, scalars, points):
    L = TARGET_LIMBS[field]
    acc = np.array(acc, dtype=np.uint64).copy()
    s, ps = _u64(scalars)
    p, pp = _u64(points)
    _check(lib().oracle_geometric_accumulate(field, acc.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                             ctypes.c_size_t(acc.size // L), ps, pp, ctypes.c_size_t(s.size // L)))
    return acc


def univariate_evaluate(field, coeffs, point):
    c, pc = _u64(coeffs)
    p, pp = _u64(point)
    out = np.zeros(TARGET_LIMBS[field], np.uint64)
    _check(lib().oracle_univariate_evaluate(field, pc, ctypes.c_size_t(c.size // SOURCE_LIMBS[field]), pp,
                                            out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))))
    return out


def multilinear_extend(field, evals, point):
    e, pe = _u64(evals)
    p, pp = _u64(point)
    out = np.zeros(TARGET_LIMBS[field], np.uint64)
    _check(lib().oracle_multilinear_extend(field, pe, ctypes.c_size_t(e.size // SOURCE_LIMBS[field]), pp,
                                           ctypes.c_size_t(p.size // TARGET_LIMBS[field]),
                                           out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))))
    return out


def pow_threshold(bits):
    out = ctypes.c_uint64()
    _check(lib().oracle_pow_threshold(ctypes.c_double(bits), ctypes.byref(out)))
    return out.value


def pow_difficulty(threshold):
    return lib().oracle_pow_difficulty(ctypes.c_uint64(threshold))


def pow_grind(engine_id, challenge, threshold):
    out = ctypes.c_uint64()
    _, pid = _u8(engine_id)
    _, pc = _u8(challenge)
    _check(lib().oracle_pow_grind(pid, pc, ctypes.c_uint64(threshold), ctypes.byref(out)))
    return out.value


def challenge_indices_replay(squeezed, num_leaves, count, dedup):
    b, pb = _u8(squeezed)
    out = np.zeros(max(count, 1), np.uint64)
    n = ctypes.c_size_t()
    _check(lib().oracle_challenge_indices_replay(pb, ctypes.c_size_t(len(squeezed)), ctypes.c_size_t(num_leaves),
                                                 ctypes.c_size_t(count), int(dedup),
                                                 out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                                 ctypes.byref(n)))
    return [int(x) for x in out[: n.value]]


def sponge_squeeze(absorb, n_out):
    a, pa = _u8(absorb if len(absorb) else b"\0")
    out = np.zeros(n_out, np.uint8)
    lib().oracle_sponge_squeeze(pa, ctypes.c_size_t(len(absorb)), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                ctypes.c_size_t(n_out))
    return out.tobytes()


def whir_config_json(field, params, num_variables):
    import json
    buf = ctypes.create_string_buffer(1 << 16)
    _check(lib().oracle_whir_config_json(field, ctypes.byref(params), ctypes.c_size_t(num_variables), buf,
                                         ctypes.c_size_t(1 << 16)))
    return json.loads(buf.value.decode())


def whir_config_bytes(field, params, num_variables):
    n = ctypes.c_size_t()
    _check(lib().oracle_whir_config_bytes(field, ctypes.byref(params), ctypes.c_size_t(num_variables), None,
                                          ctypes.c_size_t(0), ctypes.byref(n)))
    out = np.zeros(n.value, np.uint8)
    _check(lib().oracle_whir_config_bytes(field, ctypes.byref(params), ctypes.c_size_t(num_variables),
                                          out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), n, ctypes.byref(n)))
    return out.tobytes()


def field_size_bits(field):
    return lib().oracle_field_size_bits(field)


class Proof:
    def __init__(self, narg, hints, evaluation_point, rlc_coefficients, roots):
        self.narg = narg
        self.hints = hints
        self.evaluation_point = evaluation_point
        self.rlc_coefficients = rlc_coefficients
        self.roots = roots


def _get_bytes(fn, h):
    p = ctypes.POINTER(ctypes.c_uint8)()
    n = fn(h, ctypes.byref(p))
    return ctypes.string_at(p, n) if n else b""


def _get_u64(fn, h):
    p = ctypes.POINTER(ctypes.c_uint64)()
    n = fn(h, ctypes.byref(p))
    return np.ctypeslib.as_array(p, shape=(n,)).copy() if n else np.zeros(0, np.uint64)


def whir_prove(field, params, num_variables, session, vectors, points=(), covectors=(), evaluations=()):
    """vectors: (n_vectors, 2^nv[, source limbs]); points: (n_points, nv, target limbs);
    covectors: (n_cov, 2^nv, target limbs); evaluations: (forms, vectors, target limbs)."""
    L = lib()
    bs = params.batch_size
    vectors = np.ascontiguousarray(vectors, dtype=np.uint64)
    n_vec = vectors.shape[0]
    assert n_vec % bs == 0
    pts = np.ascontiguousarray(np.asarray(points, dtype=np.uint64).reshape(-1))
    cov = np.ascontiguousarray(np.asarray(covectors, dtype=np.uint64).reshape(-1))
    ev = np.ascontiguousarray(np.asarray(evaluations, dtype=np.uint64).reshape(-1))
    n_points = len(points)
    n_cov = len(covectors)
    h = ctypes.c_void_p()
    u64p = ctypes.POINTER(ctypes.c_uint64)
    pp = pts.ctypes.data_as(u64p) if pts.size else None
    cp = cov.ctypes.data_as(u64p) if cov.size else None
    ep = ev.ctypes.data_as(u64p) if ev.size else None
    _check(L.oracle_whir_prove(field, ctypes.byref(params), ctypes.c_size_t(num_variables), session.encode(),
                               ctypes.c_size_t(n_vec // bs), vectors.ctypes.data_as(u64p), ctypes.c_size_t(n_points),
                               pp, ctypes.c_size_t(n_cov), cp, ep, ctypes.byref(h)))
    try:
        return Proof(_get_bytes(L.oracle_proof_narg, h), _get_bytes(L.oracle_proof_hints, h),
                     _get_u64(L.oracle_proof_eval_point, h), _get_u64(L.oracle_proof_rlc, h),
                     _get_bytes(L.oracle_proof_roots, h))
    finally:
        L.oracle_proof_free(h)


def whir_verify(field, params, num_variables, session, n_commitments, narg, hints, points=(), covectors=(),
                evaluations=()):
    """Returns True when the proof is accepted (and the final claim checks), False when rejected."""
    L = lib()
    pts = np.ascontiguousarray(np.asarray(points, dtype=np.uint64).reshape(-1))
    cov = np.ascontiguousarray(np.asarray(covectors, dtype=np.uint64).reshape(-1))
    ev = np.ascontiguousarray(np.asarray(evaluations, dtype=np.uint64).reshape(-1))
    u64p = ctypes.POINTER(ctypes.c_uint64)
    nb, pn = _u8(narg if narg else b"\0")
    hb, ph = _u8(hints if hints else b"\0")
    rc = L.oracle_whir_verify(field, ctypes.byref(params), ctypes.c_size_t(num_variables), session.encode(),
                              ctypes.c_size_t(n_commitments), ctypes.c_size_t(len(points)),
                              pts.ctypes.data_as(u64p) if pts.size else None, ctypes.c_size_t(len(covectors)),
                              cov.ctypes.data_as(u64p) if cov.size else None,
                              ev.ctypes.data_as(u64p) if ev.size else None, pn, ctypes.c_size_t(len(narg)), ph,
                              ctypes.c_size_t(len(hints)))
    if rc < 0:
        raise RuntimeError("oracle verify error: " + L.oracle_last_error().decode())
    return rc == 0
