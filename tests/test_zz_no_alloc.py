"""The allocation-free FCT_positivity entry point against the context-based one.

Callers that manage device memory themselves (their own pool or arena, or a
driver that forbids further cudaMalloc calls) pass device buffers to
swe_fct_positivity_noalloc, which keeps its R^- scratch in a fixed array
compiled into the library.  Its output must equal swe_fct_positivity (FP64,
same arithmetic: bit for bit) on two calls in a row, since the scratch array
is shared between calls and keeps the previous call's contents; also at the
largest accepted size, and on a stream other than the default one.
"""
import ctypes

import numpy as np
import pytest

from swe import cases as C, lib as L, mesh as M
from swe.update import from_case

pytestmark = pytest.mark.gpu


def _fn():
    lib = L.load()
    fn = lib.swe_fct_positivity_noalloc
    fn.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def _context_reference(mesh, htiny, rng):
    """f_ij, (lumped/dt) h^L and the context entry point's l_ij on a mesh."""
    npts = mesh["rr"].shape[1]
    case = C.Case("fct", mesh, C.Params(htiny=htiny, dt=1e-3), np.zeros(npts),
                  np.zeros((3, npts), order="F"), 1.0)
    upd = from_case(case)
    mt = upd.matrices()
    nnz = len(mt["ja"])
    hs = rng.random(npts) * 2e-3                    # straddles the htiny test
    f = rng.normal(size=nnz)
    ref = upd.fct_positivity(hs, f)
    upd.close()
    return mt, hs, f, ref


def _call(fn, torch, mt, hs, f, htiny, stream=None):
    dev = torch.device("cuda:0")
    d_ia = torch.from_numpy(mt["ia"].astype(np.int32)).to(dev)
    d_ja = torch.from_numpy(mt["ja"].astype(np.int32)).to(dev)
    d_u = torch.from_numpy(hs).to(dev)
    d_f = torch.from_numpy(f).to(dev)
    d_l = torch.full((len(f),), -7.0, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    handle = None if stream is None else stream.cuda_stream
    rc = fn(len(hs), d_ia.data_ptr(), d_ja.data_ptr(), d_u.data_ptr(), d_f.data_ptr(), htiny, d_l.data_ptr(),
            handle)
    return rc, d_l.cpu().numpy()


def test_noalloc_fct_positivity_matches_context_entry_point():
    torch = pytest.importorskip("torch")
    fn = _fn()
    rng = np.random.default_rng(12)
    htiny = 1e-3
    for call, n in enumerate((17, 23)):                  # two calls in a row, different sizes
        mesh = M.jittered_mesh(n, n, 0.0, 1.0, 0.0, 1.0, seed=call)
        mt, hs, f, ref = _context_reference(mesh, htiny, rng)
        rc, got = _call(fn, torch, mt, hs, f, htiny)
        assert rc == L.SWE_OK
        np.testing.assert_array_equal(got, ref)


def test_noalloc_largest_size_on_a_side_stream():
    """np = SWE_NOALLOC_MAX_NODES (a 1024 x 1024 lattice), launched on a
    torch side stream, then a small mesh again on the default stream."""
    torch = pytest.importorskip("torch")
    fn = _fn()
    rng = np.random.default_rng(5)
    htiny = 1e-3
    mesh = M.lattice_mesh(1024, 1024)
    assert mesh["rr"].shape[1] == L.NOALLOC_MAX_NODES
    mt, hs, f, ref = _context_reference(mesh, htiny, rng)
    side = torch.cuda.Stream()
    rc, got = _call(fn, torch, mt, hs, f, htiny, stream=side)
    assert rc == L.SWE_OK
    np.testing.assert_array_equal(got, ref)
    small = M.jittered_mesh(19, 19, 0.0, 1.0, 0.0, 1.0, seed=4)
    mt, hs, f, ref = _context_reference(small, htiny, rng)
    rc, got = _call(fn, torch, mt, hs, f, htiny)
    assert rc == L.SWE_OK
    np.testing.assert_array_equal(got, ref)


def test_noalloc_rejects_out_of_range_columns():
    """A column index outside 1..np is found by the kernels, which do not
    read through it: the call returns SWE_ERR_ARG; the next valid call is
    unaffected."""
    torch = pytest.importorskip("torch")
    fn = _fn()
    rng = np.random.default_rng(8)
    htiny = 1e-3
    mesh = M.jittered_mesh(13, 13, 0.0, 1.0, 0.0, 1.0, seed=2)
    mt, hs, f, ref = _context_reference(mesh, htiny, rng)
    for bad in (0, len(hs) + 1):
        ja = mt["ja"].copy()
        ja[len(ja) // 2] = bad
        rc, _ = _call(fn, torch, dict(mt, ja=ja), hs, f, htiny)
        assert rc == L.SWE_ERR_ARG, bad
    rc, got = _call(fn, torch, mt, hs, f, htiny)
    assert rc == L.SWE_OK
    np.testing.assert_array_equal(got, ref)


def test_noalloc_rejects_sizes_beyond_the_scratch_array():
    fn = _fn()
    dummy = ctypes.c_void_p(16)   # never dereferenced: the size check comes first
    assert fn(L.NOALLOC_MAX_NODES + 1, dummy, dummy, dummy, dummy, 1e-3, dummy, None) == L.SWE_ERR_ARG
