"""The no-allocation moments entry point against the context-based one.

lbgpu_moments_noalloc serves callers that cannot let the library allocate device memory: their
populations already live on the GPU under their own allocator, or their loop runs under a fixed
device-memory budget.  It takes device pointers for every input and output and keeps its
reduction scratch in a fixed device array shared by all calls.  Here it must give the same
density, flux and l2err as lbgpu_moments (which copies host arrays through a context's own
buffers) -- bit for bit, the tolerance of the FP64 flow tests -- on two calls in a row of
different sizes, so that nothing left in the shared scratch by one call leaks into the next.
This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from laboetie_gb300 import Box, library

pytestmark = pytest.mark.gpu


def _case(shape, seed):
    rng = np.random.default_rng(seed)
    nat = (rng.random(shape) < 0.3).astype(np.int8)
    nat.flat[0] = 0
    n = (1.0 / 19) * (1.0 + 0.05 * rng.standard_normal((19,) + shape))
    f = [1e-4 * rng.standard_normal(shape) for _ in range(3)]
    jold = [1e-3 * rng.standard_normal(shape) for _ in range(3)]
    return nat, n, f, jold


def _noalloc(torch, n, f, jold):
    L = library()
    lz, ly, lx = n.shape[1:]
    dev = torch.device("cuda:0")
    dn = torch.from_numpy(np.ascontiguousarray(n)).to(dev)
    df = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in f]
    dj = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in jold]
    drho = torch.empty((lz, ly, lx), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    err = ctypes.c_double(-1.0)
    rc = L.lbgpu_moments_noalloc(lx, ly, lz, dn.data_ptr(), *(x.data_ptr() for x in df),
                                 drho.data_ptr(), *(x.data_ptr() for x in dj), ctypes.byref(err),
                                 None)
    torch.cuda.synchronize()
    return rc, drho.cpu().numpy(), [x.cpu().numpy() for x in dj], err.value


def test_noalloc_moments_match_the_context_entry_point_on_two_calls():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device visible to torch")
    for shape, seed in (((9, 7, 11), 1), ((5, 6, 4), 2)):
        nat, n, f, jold = _case(shape, seed)
        rc, rho, j, err = _noalloc(torch, n, f, jold)
        with Box(nat) as box:
            st, rho_r, j_r, err_r = box.moments(n, f, jold)
        assert rc == 0 and st == 0
        assert np.array_equal(rho, rho_r)
        for d in range(3):
            assert np.array_equal(j[d], j_r[d])
        assert err == err_r


def test_noalloc_moments_match_the_context_entry_point_on_non_finite_input():
    """A NaN population and an infinite one: both entry points raise LBGPU_ERR_NONFINITE, write
    the same (partly non-finite) moments and return the same l2err -- NaN for the NaN (a maximum
    over bit patterns keeps the NaN that fmax would drop), +Inf for the infinity; then a finite
    call on the same scratch is clean again."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device visible to torch")
    nonfinite = 1 << 3
    for bad in (np.nan, np.inf):
        nat, n, f, jold = _case((6, 5, 7), 3)
        n[4, 2, 3, 1] = bad
        rc, rho, j, err = _noalloc(torch, n, f, jold)
        with Box(nat) as box:
            st, rho_r, j_r, err_r = box.moments(n, f, jold)
        assert rc == st == nonfinite
        assert np.array_equal(rho, rho_r, equal_nan=True) and not np.isfinite(rho[2, 3, 1])
        for d in range(3):
            assert np.array_equal(j[d], j_r[d], equal_nan=True)
        if np.isnan(bad):
            assert np.isnan(err) and np.isnan(err_r)
        else:
            assert err == err_r == np.inf
    nat, n, f, jold = _case((6, 5, 7), 4)
    rc, rho, j, err = _noalloc(torch, n, f, jold)
    with Box(nat) as box:
        st, rho_r, j_r, err_r = box.moments(n, f, jold)
    assert rc == st == 0 and np.isfinite(err) and err == err_r


def test_noalloc_moments_reject_boxes_beyond_the_scratch():
    L = library()
    one = ctypes.c_void_p(1)  # never dereferenced: the size check comes first
    rc = L.lbgpu_moments_noalloc(257, 256, 256, *([one] * 8), None, None)
    assert rc == 1
    buf = ctypes.create_string_buffer(256)
    L.lbgpu_last_error(None, buf, 256)
    assert b"16777216" in buf.value
