"""gsls_dot_noalloc: the dot product for callers that cannot call cudaMalloc
(drivers that hand the whole device heap to their own pool, or code running
where no allocation may be made).  It takes its reduction scratch from a
fixed array in the library's device image instead of allocating.

Checked against the allocating entry point gsls_dot_dev on the same device
vectors, on two calls in a row (the shared array keeps the previous call's
contents, so the second call also checks that nothing left over leaks into
the result), within the dot-product tolerance of the other GPU tests; at
sizes that use one reduction group, several groups, the largest accepted n
and n = 0; and the free device memory is the same before and after a call.
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


@pytest.mark.parametrize("nodes", [358_425, 0])
def test_dot_noalloc_several_groups_and_empty(gsls, nodes):
    """n = 3 x 358,425 (263 blocks in 9 reduction groups) against
    gsls_dot_dev on an lhs of that many nodes, twice; and n = 0 gives 0."""
    torch = pytest.importorskip("torch")
    if nodes == 0:
        ut = torch.zeros(1, dtype=torch.float64, device="cuda")
        for _ in range(2):
            assert _dot_noalloc(gsls, 0, ut, ut) == 0.0
        return
    nNo, dof = nodes, 3
    rp1 = np.arange(1, nNo + 2, dtype=np.int32)          # diagonal pattern
    cp1 = np.arange(1, nNo + 1, dtype=np.int32)
    lhs = fsils.FSILS_LHS_CREATE(nNo, nNo, nNo, np.arange(1, nNo + 1, dtype=np.int32), rp1, cp1,
                                 1)
    n = nNo * dof
    rng = np.random.default_rng(7)
    for call in range(2):
        u = rng.standard_normal(n)
        v = rng.standard_normal(n) * (3.0 - call)
        ut = torch.tensor(u, dtype=torch.float64, device="cuda")
        vt = torch.tensor(v, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        ref = _dot_dev(gsls, lhs, dof, ut, vt)
        got = _dot_noalloc(gsls, n, ut, vt)
        scale = float(np.abs(u * v).sum())
        assert abs(got - ref) < 1e-12 * scale, (call, got, ref)
    lhs.free()


def test_dot_noalloc_largest_n_allocates_nothing(gsls):
    """The largest accepted n (16,384 blocks in 512 groups), twice, against
    a float64 torch sum; the free device memory is unchanged by a call."""
    torch = pytest.importorskip("torch")
    n = MAX_N
    g = torch.Generator(device="cuda").manual_seed(11)
    ut = torch.rand(n, dtype=torch.float64, device="cuda", generator=g) - 0.5
    vt = torch.rand(n, dtype=torch.float64, device="cuda", generator=g) - 0.5
    ref = float((ut * vt).sum())
    scale = float((ut * vt).abs().sum())
    torch.cuda.synchronize()
    got1 = _dot_noalloc(gsls, n, ut, vt)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    got2 = _dot_noalloc(gsls, n, ut, vt)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0
    assert got1 == got2                    # same grid, same order: same bits
    assert abs(got1 - ref) < 1e-12 * scale, (got1, ref)
    del ut, vt
