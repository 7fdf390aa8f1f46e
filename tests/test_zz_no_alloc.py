"""The allocation-free FCT_positivity entry point against the context-based one.

Callers that manage device memory themselves (their own pool or arena, or a
driver that forbids further cudaMalloc calls) pass device buffers to
swe_fct_positivity_noalloc, which keeps its R^- scratch in a fixed array
compiled into the library.  Its output must equal swe_fct_positivity (FP64,
same arithmetic: bit for bit) on two calls in a row, since the scratch array
is shared between calls and keeps the previous call's contents.
"""
import ctypes

import numpy as np
import pytest

from swe import cases as C, lib as L, mesh as M
from swe.update import from_case

pytestmark = pytest.mark.gpu


def test_noalloc_fct_positivity_matches_context_entry_point():
    torch = pytest.importorskip("torch")
    lib = L.load()
    fn = lib.swe_fct_positivity_noalloc
    fn.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    rng = np.random.default_rng(12)
    for call, n in enumerate((17, 23)):                  # two calls in a row, different sizes
        mesh = M.jittered_mesh(n, n, 0.0, 1.0, 0.0, 1.0, seed=call)
        npts = n * n
        htiny = 1e-3
        case = C.Case("fct", mesh, C.Params(htiny=htiny, dt=1e-3), np.zeros(npts),
                      np.zeros((3, npts), order="F"), 1.0)
        upd = from_case(case)
        mt = upd.matrices()
        nnz = len(mt["ja"])
        hs = rng.random(npts) * 2e-3                    # straddles the htiny test
        f = rng.normal(size=nnz)
        ref = upd.fct_positivity(hs, f)
        dev = torch.device("cuda:0")
        d_ia = torch.from_numpy(mt["ia"].astype(np.int32)).to(dev)
        d_ja = torch.from_numpy(mt["ja"].astype(np.int32)).to(dev)
        d_u = torch.from_numpy(hs).to(dev)
        d_f = torch.from_numpy(f).to(dev)
        d_l = torch.full((nnz,), -7.0, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc = fn(npts, d_ia.data_ptr(), d_ja.data_ptr(), d_u.data_ptr(), d_f.data_ptr(), htiny, d_l.data_ptr(), None)
        assert rc == L.SWE_OK
        np.testing.assert_array_equal(d_l.cpu().numpy(), ref)
        upd.close()


def test_noalloc_rejects_sizes_beyond_the_scratch_array():
    lib = L.load()
    fn = lib.swe_fct_positivity_noalloc
    fn.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    dummy = ctypes.c_void_p(16)   # never dereferenced: the size check comes first
    assert fn(L.NOALLOC_MAX_NODES + 1, dummy, dummy, dummy, dummy, 1e-3, dummy, None) == L.SWE_ERR_ARG
