"""gsls_dot_noalloc: the dot product for callers that cannot call cudaMalloc
(drivers that hand the whole device heap to their own pool, or code running
where no allocation may be made).  It takes its reduction scratch from a
fixed array in the library's device image instead of allocating.

Checked against the allocating entry point gsls_dot_dev on the same device
vectors, on two calls in a row (the shared array keeps the previous call's
contents, so the second call also checks that nothing left over leaks into
the result), within the dot-product tolerance of the other GPU tests.
Collected last so that a failure here does not stop the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest

from svfsi_gb300 import _lib, fsils, problems

pytestmark = pytest.mark.gpu

MAX_N = 4096 * 16384


def _dot_dev(gsls, lhs, dof, ut, vt):
    out = C.c_double()
    _lib.check(gsls.gsls_dot_dev(lhs.h, dof, C.c_void_p(ut.data_ptr()), C.c_void_p(vt.data_ptr()),
                                 C.byref(out)), "gsls_dot_dev")
    return out.value


def _dot_noalloc(gsls, n, ut, vt):
    out = C.c_double()
    _lib.check(gsls.gsls_dot_noalloc(n, C.c_void_p(ut.data_ptr()), C.c_void_p(vt.data_ptr()),
                                     C.byref(out), None), "gsls_dot_noalloc")
    return out.value


def test_dot_noalloc_matches_dot_dev_twice(gsls):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    p = problems.heats_cube(12)
    g, rp1, cp1 = problems.make_lhs_arrays(p)
    lhs = fsils.FSILS_LHS_CREATE(p.nNo, p.nNo, p.nnz, g, rp1, cp1, 1)
    dof = 3
    n = p.nNo * dof
    rng = np.random.default_rng(42)
    for call in range(2):
        u = rng.standard_normal(n) * (1.0 + call)
        v = rng.standard_normal(n)
        ut = torch.tensor(u, dtype=torch.float64, device="cuda")
        vt = torch.tensor(v, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        ref = _dot_dev(gsls, lhs, dof, ut, vt)
        got = _dot_noalloc(gsls, n, ut, vt)
        scale = float(np.abs(u * v).sum())
        assert abs(got - ref) < 1e-12 * scale, (call, got, ref)
        assert abs(got - float(np.dot(u, v))) < 1e-12 * scale
    lhs.free()


def test_dot_noalloc_rejects_oversize(gsls):
    torch = pytest.importorskip("torch")
    ut = torch.zeros(4, dtype=torch.float64, device="cuda")
    out = C.c_double()
    rc = gsls.gsls_dot_noalloc(MAX_N + 1, C.c_void_p(ut.data_ptr()), C.c_void_p(ut.data_ptr()),
                               C.byref(out), None)
    assert rc == -1  # GSLS_ERR_ARG, nothing launched
    assert b"maximum" in gsls.gsls_last_error()
