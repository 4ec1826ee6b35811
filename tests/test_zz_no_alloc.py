"""whir_eval_eq_noalloc, the entry point for callers that cannot allocate device memory (for
example code running inside a CUDA stream capture, or hosts that embed the prover behind their own
allocator): called through the C ABI with caller-owned device buffers, two calls in a row, each
checked bit for bit against the regular whir_eval_eq entry point. This file is collected last so a
run that stops at the first failure has already run every other test."""

import ctypes

import numpy as np
import pytest

import whir_gb300 as W
from whir_gb300.inputs import Rng, field_elements

pytestmark = pytest.mark.gpu


def _noalloc(lib, field, acc_dev, point_dev, nvars, scalar, stream):
    lib.whir_eval_eq_noalloc.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                         ctypes.POINTER(ctypes.c_uint64), ctypes.c_void_p]
    lib.whir_noalloc_last_error.restype = ctypes.c_char_p
    s = np.ascontiguousarray(scalar, dtype=np.uint64)
    rc = lib.whir_eval_eq_noalloc(field, ctypes.c_void_p(acc_dev), ctypes.c_void_p(point_dev), nvars,
                                  s.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), ctypes.c_void_p(stream))
    return rc, lib.whir_noalloc_last_error().decode()


@pytest.mark.parametrize("fname,fid,nvars", [("Goldilocks2", W.GOLDILOCKS2, 16), ("Goldilocks3", W.GOLDILOCKS3, 11),
                                            ("Goldilocks1", W.GOLDILOCKS1, 20)])
def test_noalloc_eval_eq_matches_regular_entry_point(fname, fid, nvars):
    lib = W.load_library()
    ctx = W.Context(0)
    L = W.TARGET_LIMBS[fid]
    n = 1 << nvars
    rng = Rng(77 + nvars)
    acc_dev = ctx.alloc(n * L * 8)
    point_dev = ctx.alloc(nvars * L * 8)
    try:
        acc = field_elements(fname, n, rng=rng).reshape(-1)
        expected = acc.copy()
        for call in range(2):  # two calls in a row: the second reuses the scratch of the first
            point = field_elements(fname, nvars, rng=rng).reshape(-1)
            scalar = field_elements(fname, 1, rng=rng).reshape(-1)
            ctx.upload(acc_dev, acc)
            ctx.upload(point_dev, point)
            rc, err = _noalloc(lib, fid, acc_dev, point_dev, nvars, scalar, ctx.stream_handle())
            assert rc == 0, err
            ctx.synchronize()
            got = np.zeros(n * L, dtype=np.uint64)
            _copy_back(lib, ctx, got, acc_dev)
            expected = W.eval_eq(ctx, fid, expected, point, scalar)
            assert np.array_equal(got, expected), "call %d differs from whir_eval_eq" % call
            acc = got
    finally:
        ctx.free(acc_dev)
        ctx.free(point_dev)
        ctx.close()


@pytest.mark.parametrize("fname,fid,max_nvars", [("Goldilocks1", W.GOLDILOCKS1, 28), ("Goldilocks2", W.GOLDILOCKS2, 26),
                                                 ("Goldilocks3", W.GOLDILOCKS3, 24)])
def test_noalloc_size_limits(fname, fid, max_nvars):
    # The largest nvars whose eq tables fit the 256 KiB scratch is accepted and agrees bit for bit
    # with whir_eval_eq on the same device buffers; one more variable is rejected before any work.
    torch = pytest.importorskip("torch")
    lib = W.load_library()
    lib.whir_eval_eq_noalloc_max_scratch.restype = ctypes.c_size_t
    assert lib.whir_eval_eq_noalloc_max_scratch() == 256 * 1024
    L = W.TARGET_LIMBS[fid]
    rng = Rng(500 + fid)
    point = torch.from_numpy(field_elements(fname, max_nvars, rng=rng).reshape(-1).view(np.int64)).cuda()
    scalar = field_elements(fname, 1, rng=rng).reshape(-1)
    gen = torch.Generator(device="cuda").manual_seed(fid)
    acc = torch.randint(0, 1 << 62, ((1 << max_nvars) * L,), dtype=torch.int64, device="cuda", generator=gen)
    ref = acc.clone()
    torch.cuda.synchronize()
    ctx = W.Context(0)
    try:
        rc, err = _noalloc(lib, fid, acc.data_ptr(), point.data_ptr(), max_nvars, scalar, ctx.stream_handle())
        assert rc == 0, err
        s = np.ascontiguousarray(scalar, dtype=np.uint64)
        rc = lib.whir_eval_eq(ctx._h, ctypes.c_int(fid), ctypes.c_void_p(ref.data_ptr()),
                              ctypes.c_void_p(point.data_ptr()), ctypes.c_size_t(max_nvars),
                              s.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), ctypes.c_uint32(W.DEVICE_PTRS))
        assert rc == 0, lib.whir_last_error().decode()
        ctx.synchronize()
        assert torch.equal(acc, ref)
        before = acc.clone()
        torch.cuda.synchronize()
        rc, err = _noalloc(lib, fid, acc.data_ptr(), point.data_ptr(), max_nvars + 1, scalar, ctx.stream_handle())
        assert rc == -1 and "scratch" in err
        ctx.synchronize()
        assert torch.equal(acc, before)
        rc, err = _noalloc(lib, fid, acc.data_ptr(), point.data_ptr(), 1, scalar, ctx.stream_handle())
        assert rc == 0 and err == "", "a successful call leaves no error message behind"
        ctx.synchronize()
    finally:
        ctx.close()


def test_noalloc_rejects_bad_arguments():
    lib = W.load_library()
    ctx = W.Context(0)
    dummy = ctx.alloc(64)
    try:
        rc, err = _noalloc(lib, W.GOLDILOCKS3, dummy, dummy, 27, np.zeros(3, np.uint64), ctx.stream_handle())
        assert rc == -1 and "scratch" in err
        rc, err = _noalloc(lib, W.GOLDILOCKS2, dummy, dummy, 0, np.zeros(2, np.uint64), ctx.stream_handle())
        assert rc == -1
        rc, err = _noalloc(lib, W.FIELD192, dummy, dummy, 2, np.zeros(3, np.uint64), ctx.stream_handle())
        assert rc == -1 and "field" in err
    finally:
        ctx.free(dummy)
        ctx.close()


def _copy_back(lib, ctx, host, dev):
    rc = lib.whir_memcpy_d2h(ctx._h, host.ctypes.data_as(ctypes.c_void_p), ctypes.c_void_p(dev),
                             ctypes.c_size_t(host.nbytes))
    assert rc == 0
