"""whir_gb300 — GB300 (sm_103a) WHIR prover path behind the reference crate's interfaces.

Python mirror of the reference's API for the prover path (WizardOfMenlo/whir):

* ``ProtocolParameters``           — src/parameters.rs:9-24
* ``Config(field, size, params)``  — whir::Config::new (src/protocols/whir/config.rs:16-152)
* ``ProverState(config, session)`` — transcript::ProverState::new_std + DomainSeparator
                                     (src/transcript/mod.rs:110-181)
* ``Config.commit``                — whir::Config::commit (src/protocols/whir/mod.rs:79-92)
* ``Config.prove``                 — whir::Config::prove (src/protocols/whir/prover.rs:50-315)
* operator functions               — ReedSolomon::interleaved_encode / evaluation_points,
                                     HashEngine::hash_many, Merkle layers, sumcheck / fold /
                                     eval_eq / geometric_accumulate / univariate evaluation, PoW

Every call goes through the C ABI of libwhir_gb300.so (include/whir_gb300.h) and runs CUDA kernels.
There is no CPU fallback: without the library or a CUDA device the calls raise.
"""

import ctypes
import os
import threading

import numpy as np

from . import build as _build

__all__ = [
    "ProtocolParameters", "Config", "ProverState", "Context", "Witness", "FinalClaim", "WhirError",
    "FIELDS", "ENGINES", "load_library", "library_path",
]

GOLDILOCKS1, GOLDILOCKS2, GOLDILOCKS3, FIELD192, FIELD256 = 0, 1, 2, 4, 5
FIELDS = {"Goldilocks1": GOLDILOCKS1, "Goldilocks2": GOLDILOCKS2, "Goldilocks3": GOLDILOCKS3,
          "Field192": FIELD192, "Field256": FIELD256}
TARGET_LIMBS = {GOLDILOCKS1: 1, GOLDILOCKS2: 2, GOLDILOCKS3: 3, FIELD192: 3, FIELD256: 4}
SOURCE_LIMBS = {GOLDILOCKS1: 1, GOLDILOCKS2: 1, GOLDILOCKS3: 1, FIELD192: 3, FIELD256: 4}

# EngineIds (src/hash/blake3_engine.rs:19, digest_engine.rs:11-19, copy_engine.rs:9)
ENGINES = {
    "Blake3": bytes.fromhex("03e01749ebcc0477924254eb482066b864a8dd4d77252464ca6f5b6f5cc05b4c"),
    "Sha2": bytes.fromhex("018eaa247cb8957ab1e9fdac885450403c5e7bda1acaaa504e4cc8f2f76bb076"),
    "Sha3": bytes.fromhex("aa802dcdabad8ea8a1430919893b96c30e31ff5734b385999108aa202d27dc12"),
    "Keccak": bytes.fromhex("ddd248964e320312a66775aee8e16c88c927734be59aca09b7af6deb0ad00e8c"),
    "Copy": bytes.fromhex("09459020f451874a1b399819d079632cc0f9263b1486c423173c6e15d8e2d61d"),
}

DEVICE_PTRS = 1

_lib = None
_lock = threading.Lock()


class WhirError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("whir_gb300 error %d: %s" % (code, msg))
        self.code = code


class _Params(ctypes.Structure):
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


def library_path():
    return _build.LIB


def load_library():
    """Load (building first if the sources are newer) libwhir_gb300.so."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            lib = ctypes.CDLL(path)
            lib.whir_last_error.restype = ctypes.c_char_p
            lib.whir_ctx_launch_count.restype = ctypes.c_uint64
            lib.whir_ctx_launch_count.argtypes = [ctypes.c_void_p]
            for name in ("whir_ctx_destroy", "whir_config_free", "whir_prover_state_free", "whir_witness_free",
                         "whir_ctx_synchronize"):
                getattr(lib, name).argtypes = [ctypes.c_void_p]
            _lib = lib
    return _lib


def last_verify_reason():
    """Why the calling thread's last verification was rejected (or failed)."""
    lib = load_library()
    lib.whir_verify_last_reason.restype = ctypes.c_char_p
    return lib.whir_verify_last_reason().decode()


def _check(rc):
    if rc != 0:
        raise WhirError(rc, load_library().whir_last_error().decode())


def _u64ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))


def _u8ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))


def _as_u64(a):
    return np.ascontiguousarray(a, dtype=np.uint64)


class ProtocolParameters:
    """ProtocolParameters (src/parameters.rs:9-24)."""

    def __init__(self, unique_decoding=False, starting_log_inv_rate=1, initial_folding_factor=4, folding_factor=4,
                 security_level=128, pow_bits=20, batch_size=1, hash_id=ENGINES["Blake3"]):
        self.unique_decoding = bool(unique_decoding)
        self.starting_log_inv_rate = int(starting_log_inv_rate)
        self.initial_folding_factor = int(initial_folding_factor)
        self.folding_factor = int(folding_factor)
        self.security_level = int(security_level)
        self.pow_bits = int(pow_bits)
        self.batch_size = int(batch_size)
        self.hash_id = bytes(ENGINES.get(hash_id, hash_id))

    def _c(self):
        p = _Params()
        p.unique_decoding = int(self.unique_decoding)
        p.starting_log_inv_rate = self.starting_log_inv_rate
        p.initial_folding_factor = self.initial_folding_factor
        p.folding_factor = self.folding_factor
        p.security_level = self.security_level
        p.pow_bits = self.pow_bits
        p.batch_size = self.batch_size
        p.hash_id[:] = list(self.hash_id)
        return p


class Context:
    """A CUDA device, its stream and memory pool (one whir_ctx); priority > 0 raises the streams'
    scheduling priority."""

    def __init__(self, device=0, priority=0):
        lib = load_library()
        h = ctypes.c_void_p()
        _check(lib.whir_ctx_create_priority(ctypes.c_int(device), ctypes.c_int(priority), ctypes.byref(h)))
        self._h = h
        self.device = device

    def synchronize(self):
        _check(load_library().whir_ctx_synchronize(self._h))

    def launch_count(self):
        return int(load_library().whir_ctx_launch_count(self._h))

    def stream_handle(self):
        """The context's cudaStream_t as an integer (for torch.cuda.ExternalStream)."""
        lib = load_library()
        lib.whir_ctx_stream.restype = ctypes.c_void_p
        lib.whir_ctx_stream.argtypes = [ctypes.c_void_p]
        return int(lib.whir_ctx_stream(self._h) or 0)

    def transfer_bytes(self):
        h = ctypes.c_uint64()
        d = ctypes.c_uint64()
        _check(load_library().whir_ctx_transfer_bytes(self._h, ctypes.byref(h), ctypes.byref(d)))
        return h.value, d.value

    PROFILE_FAMILIES = ("encode", "merkle", "sumcheck", "eq", "geometric", "lift", "pow", "gather", "univariate")

    def set_profiling(self, enabled):
        _check(load_library().whir_ctx_set_profiling(self._h, ctypes.c_int(int(bool(enabled)))))

    def profile(self):
        """{family: (milliseconds, calls)} accumulated since set_profiling(True)."""
        n = len(self.PROFILE_FAMILIES)
        ms = (ctypes.c_double * n)()
        calls = (ctypes.c_uint64 * n)()
        rc = load_library().whir_ctx_profile(self._h, ms, calls, ctypes.c_size_t(n))
        if rc < 0:
            _check(rc)
        return {f: (ms[i], int(calls[i])) for i, f in enumerate(self.PROFILE_FAMILIES)}

    def alloc(self, nbytes):
        p = ctypes.c_void_p()
        _check(load_library().whir_device_alloc(self._h, ctypes.c_size_t(nbytes), ctypes.byref(p)))
        return p.value

    def free(self, ptr):
        _check(load_library().whir_device_free(self._h, ctypes.c_void_p(ptr)))

    def upload(self, dev_ptr, array):
        a = np.ascontiguousarray(array)
        _check(load_library().whir_memcpy_h2d(self._h, ctypes.c_void_p(dev_ptr), a.ctypes.data_as(ctypes.c_void_p),
                                              ctypes.c_size_t(a.nbytes)))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            load_library().whir_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _PinnedBuffer:
    """Owner of a page-locked host allocation (whir_host_alloc), freed when the last view dies."""

    def __init__(self, nbytes):
        lib = load_library()
        ptr = ctypes.c_void_p()
        _check(lib.whir_host_alloc(ctypes.c_size_t(max(nbytes, 1)), ctypes.byref(ptr)))
        self.ptr = ptr.value
        self.nbytes = max(nbytes, 1)

    def __del__(self):
        try:
            if self.ptr:
                load_library().whir_host_free(ctypes.c_void_p(self.ptr))
                self.ptr = None
        except Exception:
            pass


def pinned_empty(count, dtype=np.uint64):
    """A numpy array of `count` elements in page-locked host memory (whir_host_alloc): commit / prove
    inputs in such memory are uploaded by DMA while the encode runs."""
    dt = np.dtype(dtype)
    buf = _PinnedBuffer(count * dt.itemsize)
    raw = (ctypes.c_uint8 * buf.nbytes).from_address(buf.ptr)
    raw._owner = buf  # keeps the allocation alive as long as any view of it
    return np.frombuffer(raw, dtype=dt, count=count)


class Witness:
    """irs_commit::Witness with the codeword and Merkle tree resident on the device."""

    def __init__(self, handle, ctx):
        self._h = handle
        self._ctx = ctx

    def root(self):
        out = (ctypes.c_uint8 * 32)()
        _check(load_library().whir_witness_root(self._h, out))
        return bytes(out)

    def free(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            load_library().whir_witness_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class FinalClaim:
    def __init__(self, evaluation_point, rlc_coefficients):
        self.evaluation_point = evaluation_point
        self.rlc_coefficients = rlc_coefficients


class ProverState:
    """Prover transcript: NARG string + hints (src/transcript/mod.rs:72-93)."""

    def __init__(self, config, session=""):
        lib = load_library()
        h = ctypes.c_void_p()
        s = session.encode()
        _check(lib.whir_prover_state_new(config._h, s, ctypes.c_size_t(len(s)), ctypes.byref(h)))
        self._h = h
        self._config = config

    def proof(self):
        """Returns (narg_string, hints) bytes."""
        n = ctypes.POINTER(ctypes.c_uint8)()
        h = ctypes.POINTER(ctypes.c_uint8)()
        nl = ctypes.c_size_t()
        hl = ctypes.c_size_t()
        _check(load_library().whir_prover_state_proof(self._h, ctypes.byref(n), ctypes.byref(nl), ctypes.byref(h),
                                                      ctypes.byref(hl)))
        return (ctypes.string_at(n, nl.value) if nl.value else b"",
                ctypes.string_at(h, hl.value) if hl.value else b"")

    def __del__(self):
        try:
            if self._h is not None and self._h.value:
                load_library().whir_prover_state_free(self._h)
                self._h = None
        except Exception:
            pass


class Config:
    """whir::Config for an embedding ('Goldilocks1' | 'Goldilocks2' | 'Goldilocks3')."""

    def __init__(self, field, size, params):
        lib = load_library()
        self.field_name = field
        self.field = FIELDS[field] if isinstance(field, str) else int(field)
        self.size = int(size)
        self.params = params
        h = ctypes.c_void_p()
        cp = params._c()
        _check(lib.whir_config_new(ctypes.c_int(self.field), ctypes.byref(cp), ctypes.c_uint64(self.size),
                                   ctypes.byref(h)))
        self._h = h

    @property
    def num_variables(self):
        return self.size.bit_length() - 1

    def json(self):
        import json
        buf = ctypes.create_string_buffer(1 << 16)
        _check(load_library().whir_config_json(self._h, buf, ctypes.c_size_t(1 << 16)))
        return json.loads(buf.value.decode())

    def cbor(self):
        """CBOR of the configuration's serde form (ciborium::into_writer): the protocol-id preimage."""
        lib = load_library()
        n = ctypes.c_size_t()
        _check(lib.whir_config_cbor(self._h, None, ctypes.c_size_t(0), ctypes.byref(n)))
        buf = (ctypes.c_uint8 * max(n.value, 1))()
        _check(lib.whir_config_cbor(self._h, buf, ctypes.c_size_t(n.value), ctypes.byref(n)))
        return bytes(buf[: n.value])

    def commit(self, ctx, prover_state, vectors, on_device=False):
        """vectors: batch_size x size source elements (numpy uint64), or a device pointer (int) with
        on_device=True."""
        lib = load_library()
        out = ctypes.c_void_p()
        if on_device:
            ptr = ctypes.cast(ctypes.c_void_p(int(vectors)), ctypes.POINTER(ctypes.c_uint64))
            _check(lib.whir_commit(ctx._h, self._h, prover_state._h, ptr, ctypes.c_uint32(DEVICE_PTRS),
                                   ctypes.byref(out)))
        else:
            v = _as_u64(vectors)
            _check(lib.whir_commit(ctx._h, self._h, prover_state._h, _u64ptr(v), ctypes.c_uint32(0), ctypes.byref(out)))
        return Witness(out, ctx)

    def prove(self, ctx, prover_state, vectors, witnesses, points=(), covectors=(), evaluations=(), on_device=False):
        lib = load_library()
        L = TARGET_LIMBS[self.field]
        nv = self.num_variables
        pts = _as_u64(np.asarray(points, dtype=np.uint64).reshape(-1)) if len(points) else None
        cov = _as_u64(np.asarray(covectors, dtype=np.uint64).reshape(-1)) if len(covectors) else None
        ev = _as_u64(np.asarray(evaluations, dtype=np.uint64).reshape(-1)) if len(evaluations) else None
        wh = (ctypes.c_void_p * len(witnesses))(*[w._h.value for w in witnesses])
        ep = np.zeros(nv * L, dtype=np.uint64)
        rl = np.zeros(max(1, (len(points) + len(covectors))) * L, dtype=np.uint64)
        if on_device:
            vptr = ctypes.cast(ctypes.c_void_p(int(vectors)), ctypes.POINTER(ctypes.c_uint64))
            flags = DEVICE_PTRS
        else:
            varr = _as_u64(vectors)
            vptr = _u64ptr(varr)
            flags = 0
        _check(lib.whir_prove(ctx._h, self._h, prover_state._h, vptr, ctypes.c_uint32(flags),
                              ctypes.cast(wh, ctypes.POINTER(ctypes.c_void_p)), ctypes.c_size_t(len(witnesses)),
                              _u64ptr(pts) if pts is not None else None, ctypes.c_size_t(len(points)),
                              _u64ptr(cov) if cov is not None else None, ctypes.c_size_t(len(covectors)),
                              _u64ptr(ev) if ev is not None else None, _u64ptr(ep), _u64ptr(rl)))
        return FinalClaim(ep.reshape(nv, L) if L > 1 else ep, rl[: (len(points) + len(covectors)) * L])

    def verify(self, session, narg, hints, n_commitments, points=(), covectors=(), evaluations=()):
        """Config::verify + FinalClaim::verify on the host: True when the proof is accepted, False when
        a check fails (reason in `last_verify_reason()`); raises WhirError on bad arguments."""
        lib = load_library()
        s = session.encode()
        pts = _as_u64(np.asarray(points, dtype=np.uint64).reshape(-1)) if len(points) else None
        cov = _as_u64(np.asarray(covectors, dtype=np.uint64).reshape(-1)) if len(covectors) else None
        ev = _as_u64(np.asarray(evaluations, dtype=np.uint64).reshape(-1)) if len(evaluations) else None
        nb = np.frombuffer(bytes(narg) or b"\0", dtype=np.uint8).copy()
        hb = np.frombuffer(bytes(hints) or b"\0", dtype=np.uint8).copy()
        rc = lib.whir_verify(self._h, s, ctypes.c_size_t(len(s)), _u8ptr(nb), ctypes.c_size_t(len(narg)), _u8ptr(hb),
                             ctypes.c_size_t(len(hints)), ctypes.c_size_t(n_commitments),
                             _u64ptr(pts) if pts is not None else None, ctypes.c_size_t(len(points)),
                             _u64ptr(cov) if cov is not None else None, ctypes.c_size_t(len(covectors)),
                             _u64ptr(ev) if ev is not None else None)
        if rc == 1:
            return False
        if rc != 0:
            raise WhirError(rc, last_verify_reason())
        return True

    def __del__(self):
        try:
            if self._h is not None and self._h.value:
                load_library().whir_config_free(self._h)
                self._h = None
        except Exception:
            pass


def commit_batch(ctx, configs, prover_states, vectors, on_device=False):
    """Config.commit for several jobs in shared device launches (whir_commit_batch): configs,
    prover_states and vectors (host numpy arrays, or device pointers with on_device=True) are
    parallel lists; all configs share one embedding and one hash engine. Returns the witnesses."""
    lib = load_library()
    n = len(configs)
    if not (len(prover_states) == len(vectors) == n):
        raise WhirError(-1, "configs, prover_states and vectors must have the same length")
    cfg_h = (ctypes.c_void_p * max(n, 1))(*[c._h.value for c in configs])
    ps_h = (ctypes.c_void_p * max(n, 1))(*[s._h.value for s in prover_states])
    keep = []
    vp = (ctypes.POINTER(ctypes.c_uint64) * max(n, 1))()
    for i, v in enumerate(vectors):
        if on_device:
            vp[i] = ctypes.cast(ctypes.c_void_p(int(v)), ctypes.POINTER(ctypes.c_uint64))
        else:
            a = _as_u64(v).reshape(-1)
            keep.append(a)
            vp[i] = _u64ptr(a)
    out = (ctypes.c_void_p * max(n, 1))()
    _check(lib.whir_commit_batch(ctx._h, ctypes.c_size_t(n), cfg_h, ps_h, vp,
                                 ctypes.c_uint32(DEVICE_PTRS if on_device else 0), out))
    return [Witness(ctypes.c_void_p(out[i]), ctx) for i in range(n)]


def autotune(ctx, config, reps=3):
    """Times every valid encode plan and Merkle tile height for the commitment shapes of `config` on
    the context's device and records the fastest (whir_autotune); returns the JSON report."""
    import json
    buf = ctypes.create_string_buffer(1 << 20)
    _check(load_library().whir_autotune(ctx._h, config._h, ctypes.c_int(reps), buf, ctypes.c_size_t(1 << 20)))
    return json.loads(buf.value.decode())


def autotune_export():
    """The process-wide tuned choices as text lines (whir_autotune_export)."""
    lib = load_library()
    n = ctypes.c_size_t()
    _check(lib.whir_autotune_export(None, ctypes.c_size_t(0), ctypes.byref(n)))
    buf = ctypes.create_string_buffer(n.value + 1)
    _check(lib.whir_autotune_export(buf, ctypes.c_size_t(n.value + 1), ctypes.byref(n)))
    return buf.value.decode()


def autotune_import(text):
    """Loads tuned choices written by autotune_export (whir_autotune_import)."""
    _check(load_library().whir_autotune_import(text.encode()))


def autotune_clear():
    _check(load_library().whir_autotune_clear())


# ----------------------------------------------------------------------------------------------
# Operator-level functions (host numpy in, host numpy out)
# ----------------------------------------------------------------------------------------------
def interleaved_encode(ctx, field, msgs, codeword_len, masks=None):
    """ntt::interleaved_rs_encode: msgs (n_msgs, msg_len[, limbs]) and optional masks (n_msgs, mask_len[, limbs])
    -> (codeword_len, n_msgs[, limbs]); message m is encoded as msgs[m] followed by masks[m]."""
    L = TARGET_LIMBS[field]
    m = _as_u64(msgs)
    n_msgs, msg_len = m.shape[0], m.shape[1]
    mk = _as_u64(masks) if masks is not None else None
    mask_len = mk.shape[1] if mk is not None else 0
    if mk is not None and mk.shape[0] != n_msgs:
        raise WhirError(-1, "masks must have one row per message")
    out = np.zeros(codeword_len * n_msgs * L, dtype=np.uint64)
    _check(load_library().whir_rs_interleaved_encode(ctx._h, ctypes.c_int(field), _u64ptr(m), ctypes.c_size_t(n_msgs),
                                                     ctypes.c_size_t(msg_len), _u64ptr(mk) if mask_len else None,
                                                     ctypes.c_size_t(mask_len), ctypes.c_size_t(codeword_len),
                                                     _u64ptr(out), ctypes.c_uint32(0)))
    return out.reshape(codeword_len, n_msgs, L) if L > 1 else out.reshape(codeword_len, n_msgs)


def evaluation_points(field, masked_len, codeword_len, indices):
    L = TARGET_LIMBS[field]
    idx = _as_u64(indices)
    out = np.zeros(idx.size * L, dtype=np.uint64)
    _check(load_library().whir_rs_evaluation_points(ctypes.c_int(field), ctypes.c_size_t(masked_len),
                                                    ctypes.c_size_t(codeword_len), _u64ptr(idx),
                                                    ctypes.c_size_t(idx.size), _u64ptr(out)))
    return out.reshape(idx.size, L) if L > 1 else out


def hash_many(ctx, engine, size, data, count):
    eid = np.frombuffer(ENGINES.get(engine, engine), dtype=np.uint8).copy()
    d = np.frombuffer(bytes(data) if len(data) else b"\0", dtype=np.uint8).copy()
    out = np.zeros(32 * max(count, 1), dtype=np.uint8)
    _check(load_library().whir_hash_many(ctx._h, _u8ptr(eid), ctypes.c_size_t(size), _u8ptr(d),
                                         ctypes.c_size_t(count), _u8ptr(out), ctypes.c_uint32(0)))
    return out[: 32 * count].tobytes()


def merkle_nodes(ctx, engine, leaves):
    n = len(leaves) // 32
    layers = (n - 1).bit_length() if n else 0
    nn = (2 << layers) - 1
    eid = np.frombuffer(ENGINES.get(engine, engine), dtype=np.uint8).copy()
    l = np.frombuffer(bytes(leaves) if n else b"\0" * 32, dtype=np.uint8).copy()
    out = np.zeros(nn * 32, dtype=np.uint8)
    _check(load_library().whir_merkle_nodes(ctx._h, _u8ptr(eid), _u8ptr(l), ctypes.c_size_t(n), _u8ptr(out),
                                            ctypes.c_uint32(0)))
    return out.tobytes()


def sumcheck_polynomial(ctx, field, a, b):
    L = TARGET_LIMBS[field]
    a = _as_u64(a)
    b = _as_u64(b)
    c0 = np.zeros(L, np.uint64)
    c2 = np.zeros(L, np.uint64)
    _check(load_library().whir_sumcheck_polynomial(ctx._h, ctypes.c_int(field), _u64ptr(a), _u64ptr(b),
                                                   ctypes.c_size_t(a.size // L), _u64ptr(c0), _u64ptr(c2),
                                                   ctypes.c_uint32(0)))
    return c0, c2


def fold(ctx, field, v, weight):
    L = TARGET_LIMBS[field]
    v = _as_u64(v).reshape(-1).copy()
    w = _as_u64(weight)
    n = v.size // L
    _check(load_library().whir_fold(ctx._h, ctypes.c_int(field), _u64ptr(v), ctypes.c_size_t(n), _u64ptr(w),
                                    ctypes.c_uint32(0)))
    return v[: max(n // 2, min(n, 1)) * L]


def eval_eq(ctx, field, acc, point, scalar):
    L = TARGET_LIMBS[field]
    acc = _as_u64(acc).reshape(-1).copy()
    p = _as_u64(point).reshape(-1)
    s = _as_u64(scalar)
    _check(load_library().whir_eval_eq(ctx._h, ctypes.c_int(field), _u64ptr(acc), _u64ptr(p),
                                       ctypes.c_size_t(p.size // L), _u64ptr(s), ctypes.c_uint32(0)))
    return acc


def geometric_accumulate(ctx, field, acc, scalars, points):
    L = TARGET_LIMBS[field]
    acc = _as_u64(acc).reshape(-1).copy()
    s = _as_u64(scalars).reshape(-1)
    p = _as_u64(points).reshape(-1)
    _check(load_library().whir_geometric_accumulate(ctx._h, ctypes.c_int(field), _u64ptr(acc),
                                                    ctypes.c_size_t(acc.size // L), _u64ptr(s), _u64ptr(p),
                                                    ctypes.c_size_t(s.size // L), ctypes.c_uint32(0)))
    return acc


def univariate_evaluate(ctx, field, coeffs, point):
    c = _as_u64(coeffs).reshape(-1)
    p = _as_u64(point).reshape(-1)
    out = np.zeros(TARGET_LIMBS[field], np.uint64)
    _check(load_library().whir_univariate_evaluate(ctx._h, ctypes.c_int(field), _u64ptr(c),
                                                   ctypes.c_size_t(c.size // SOURCE_LIMBS[field]), _u64ptr(p),
                                                   _u64ptr(out), ctypes.c_uint32(0)))
    return out


def lift(ctx, field, src):
    """lift (algebra/mod.rs:51-59): source elements of the embedding -> target elements."""
    s = _as_u64(src).reshape(-1)
    n = s.size // SOURCE_LIMBS[field]
    out = np.zeros(max(n, 1) * TARGET_LIMBS[field], dtype=np.uint64)
    _check(load_library().whir_lift(ctx._h, ctypes.c_int(field), _u64ptr(s), ctypes.c_size_t(n), _u64ptr(out),
                                    ctypes.c_uint32(0)))
    return out[: n * TARGET_LIMBS[field]]


def multilinear_evaluate(ctx, field, coeffs, point):
    """MultilinearExtension(point).evaluate(embedding, coeffs) on the device."""
    c = _as_u64(coeffs).reshape(-1)
    p = _as_u64(point).reshape(-1)
    L = TARGET_LIMBS[field]
    out = np.zeros(L, np.uint64)
    _check(load_library().whir_multilinear_evaluate(ctx._h, ctypes.c_int(field), _u64ptr(c),
                                                    ctypes.c_size_t(c.size // SOURCE_LIMBS[field]), _u64ptr(p),
                                                    ctypes.c_size_t(p.size // L), _u64ptr(out), ctypes.c_uint32(0)))
    return out


def pow_grind(ctx, engine, challenge, threshold):
    eid = np.frombuffer(ENGINES.get(engine, engine), dtype=np.uint8).copy()
    ch = np.frombuffer(bytes(challenge), dtype=np.uint8).copy()
    out = ctypes.c_uint64()
    _check(load_library().whir_pow_grind(ctx._h, _u8ptr(eid), _u8ptr(ch), ctypes.c_uint64(threshold),
                                         ctypes.byref(out)))
    return out.value
