"""lbm_drag_lift_f64_noalloc against lbm_drag_lift_f64 (GPU, C-ABI).

The no-allocation variant exists for callers that cannot give the library
device memory -- their device memory belongs to another allocator, or they
must not allocate once set up.  It keeps its reduction partials in a fixed
array inside the library, so this test checks, through the C-ABI, that
calls in a row (different inputs, each reusing what the one before left in
the shared array; the first at exactly the fixed limit) give the same
drag/lift as the entry point that takes a caller buffer, and that a link
count above the fixed limit is refused.

This file is collected last on purpose; it must pass alone in a fresh
process as well as after the other tests.
"""
import ctypes

import numpy as np
import pytest
import torch

from lbm_gb300 import _lib

pytestmark = pytest.mark.gpu

MAX_LINKS = 1048576  # LBM_DRAG_NOALLOC_MAX_LINKS in include/lbm_gb300.h


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _inputs(nx, ny, n_links, seed):
    rng = np.random.default_rng(seed)
    g = torch.from_numpy(rng.random((9, nx, ny))).cuda()
    g_up = torch.from_numpy(rng.random((9, nx, ny))).cuda()
    links = np.stack([rng.integers(-1, nx, n_links), rng.integers(-1, ny, n_links),
                      rng.integers(1, 9, n_links)], axis=1).astype(np.int32)
    return g, g_up, torch.from_numpy(links).cuda()


def _with_buffer(links, n, g_up, g, nx, ny, stream):
    L = _lib.load()
    scratch = torch.zeros(L.lbm_drag_lift_scratch_bytes(n), dtype=torch.uint8, device="cuda")
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    _lib.call("lbm_drag_lift_f64", _ptr(links), n, _ptr(g_up), _ptr(g), nx, ny, _ptr(out),
              _ptr(scratch), stream)
    return out.cpu().numpy()


def _no_alloc(links, n, g_up, g, nx, ny, stream):
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    _lib.call("lbm_drag_lift_f64_noalloc", _ptr(links), n, _ptr(g_up), _ptr(g), nx, ny,
              _ptr(out), stream)
    return out.cpu().numpy()


def test_no_alloc_matches_buffered_entry_point_twice():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # First call: exactly the limit, so every slot of the fixed array (the
    # last one included) is written and the size check's boundary is run;
    # then fewer links each time, so a stale partial left by the call before
    # would change the sum if it were read.
    for (nx, ny, n, seed) in ((300, 200, MAX_LINKS, 3), (300, 200, 200_000, 1),
                              (64, 48, 3_000, 2)):
        g, g_up, links = _inputs(nx, ny, n, seed)
        ref = _with_buffer(links, n, g_up, g, nx, ny, stream)
        got = _no_alloc(links, n, g_up, g, nx, ny, stream)
        # Same kernels and summation order: the tolerance of the drag tests
        # (1e-13 relative) holds, and in practice the sums are identical.
        assert np.all(np.abs(got - ref) <= 1e-13 * np.abs(ref) + 1e-300), (got, ref)


def test_no_alloc_rejects_more_links_than_its_fixed_scratch():
    L = _lib.load()
    dummy = ctypes.c_void_p(256)  # never dereferenced: the size check comes first
    rc = L.lbm_drag_lift_f64_noalloc(dummy, MAX_LINKS + 1, dummy, dummy, 16, 16, dummy, None)
    assert rc == _lib.LBM_ERR_ARG
    assert b"limit" in L.lbm_last_error_string()
