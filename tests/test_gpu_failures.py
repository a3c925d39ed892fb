"""Failure paths of the C ABI, each reached by a fault made on the host:
bad numbers or arguments handed to the library, or a short poll limit that
makes a bounded device wait run out.  Nothing here faults, traps or hangs
the GPU; after every failure the test checks that the library still works.

Reference behaviour where one exists: the reference STOPs on bad arguments
(Code/Source/svFSILS/LHS.f:67-71), signals non-convergence only through
RI%suc = .FALSE. (CGRAD.f:146-182) and takes W = 1 for a zero diagonal
entry in PRECONDDIAG (PRECOND.f:104-109); the library returns a status
instead of stopping (include/gsls.h).
"""
import ctypes as C

import numpy as np
import pytest

from svfsi_gb300 import _lib, fsils, problems

pytestmark = pytest.mark.gpu

GSLS_ERR_ARG, GSLS_ERR_CUDA, GSLS_ERR_NAN, GSLS_ERR_JAC = -1, -2, -4, -5


def rel(a, b):
    a, b = np.asarray(a, float).ravel(), np.asarray(b, float).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _status(exc):
    return int(str(exc.value).split("status ")[1].split(":")[0])


def _heat_system(orc, seed=1):
    p = problems.heats_cube(6)
    rng = np.random.default_rng(seed)
    A = 1e-3 * rng.standard_normal((p.nNo, 1))
    Y = 1e-3 * rng.standard_normal((p.nNo, 1))
    R, Val = orc.assemble(p, A, Y)
    return p, R, Val


def _lhs_with_dir(p):
    g, rp1, cp1 = problems.make_lhs_arrays(p)
    lhs = fsils.FSILS_LHS_CREATE(p.nNo, p.nNo, p.nnz, g, rp1, cp1, 1)
    dirn = p.dirichlet[0].nodes
    fsils.FSILS_BC_CREATE(lhs, 1, dirn.size, 3, fsils.BC_TYPE_DIR, dirn + 1,
                          np.zeros((dirn.size, 3)))
    return lhs


def _oracle_solver(orc, p):
    s = orc.OracleSolver(p.nNo, p.rowPtr, p.colPtr, 1)
    dirn = p.dirichlet[0].nodes
    s.bc_create(1, dirn, 3, 0, np.zeros((dirn.size, 3)))
    return s


def _solve_ok_after(gsls, orc, p, R0, V0):
    """The library still solves correctly after a failed call."""
    lhs = _lhs_with_dir(p)
    ls = fsils.FSILS_LS_CREATE(fsils.LS_TYPE_CG, relTol=1e-8, maxItr=2000)
    R, Val = R0.copy(), V0.copy()
    fsils.FSILS_SOLVE(lhs, ls, p.dof, R, Val, fsils.PRECOND_FSILS)
    s = _oracle_solver(orc, p)
    ols = orc.ls_create(orc.LS_TYPE_CG, relTol=1e-8, mItr=2000)
    Ro, Vo = R0.copy(), V0.copy()
    s.solve(ols, p.dof, Ro, Vo, orc.PRECOND_FSILS)
    assert ls.RI.suc == 1
    assert rel(R, Ro) < 1e-7
    lhs.free()


@pytest.mark.parametrize("where", ["Val", "R"])
def test_nan_input_returns_err_nan(gsls, orc, where):
    p, R0, V0 = _heat_system(orc)
    lhs = _lhs_with_dir(p)
    ls = fsils.FSILS_LS_CREATE(fsils.LS_TYPE_CG, relTol=1e-8, maxItr=500)
    R, Val = R0.copy(), V0.copy()
    interior = np.setdiff1d(np.arange(p.nNo), p.dirichlet[0].nodes)[5]
    if where == "Val":
        Val[p.rowPtr[interior] + 1, 0] = np.nan
    else:
        R[interior, 0] = np.nan
    with pytest.raises(_lib.GslsError) as exc:
        fsils.FSILS_SOLVE(lhs, ls, 1, R, Val, fsils.PRECOND_FSILS)
    assert _status(exc) == GSLS_ERR_NAN
    lhs.free()
    _solve_ok_after(gsls, orc, p, R0, V0)


def test_flat_tet_returns_err_jac(gsls, orc):
    """Two tets, the second flat (all four nodes in z = 0): its Jacobian is
    exactly zero, which the mesh records and every assembly returns."""
    x = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0]], dtype=float)
    ien = np.array([[0, 1, 2, 3], [1, 4, 2, 0]], dtype=np.int32)
    rp, cp = orc.lhsa(x.shape[0], ien)
    g = np.arange(1, x.shape[0] + 1, dtype=np.int32)
    lhs = fsils.FSILS_LHS_CREATE(x.shape[0], x.shape[0], cp.size, g, rp + 1, cp + 1, 1)
    mesh = fsils.Mesh(lhs, ien, x)
    p = problems.heats_cube(2)
    z = np.zeros((x.shape[0], 1))
    for _ in range(2):
        with pytest.raises(_lib.GslsError) as exc:
            mesh.assemble(p.eq_params(), z, z, z, 1)
        assert _status(exc) == GSLS_ERR_JAC
    mesh.free()
    lhs.free()
    q, R0, V0 = _heat_system(orc)
    _solve_ok_after(gsls, orc, q, R0, V0)


@pytest.mark.parametrize("lstype", ["cg", "gmres"])
def test_iteration_limit_is_not_an_error(gsls, orc, lstype):
    """maxItr = 2 at relTol 1e-12: the solve returns GSLS_OK with
    RI%suc = 0 and the oracle's iteration count and final norm."""
    p, R0, V0 = _heat_system(orc)
    lhs = _lhs_with_dir(p)
    t = fsils.LS_TYPE_CG if lstype == "cg" else fsils.LS_TYPE_GMRES
    kw = dict(relTol=1e-12, maxItr=2) if lstype == "cg" else dict(relTol=1e-12, maxItr=2,
                                                                    dimKry=3)
    ls = fsils.FSILS_LS_CREATE(t, **kw)
    R, Val = R0.copy(), V0.copy()
    fsils.FSILS_SOLVE(lhs, ls, 1, R, Val, fsils.PRECOND_FSILS)
    s = _oracle_solver(orc, p)
    ols = orc.ls_create(t, relTol=1e-12, mItr=2, sD=kw.get("dimKry"))
    Ro, Vo = R0.copy(), V0.copy()
    s.solve(ols, 1, Ro, Vo, orc.PRECOND_FSILS)
    assert ls.RI.suc == ols.RI.suc == 0
    assert ls.RI.itr == ols.RI.itr
    assert abs(ls.RI.fNorm - ols.RI.fNorm) <= 1e-10 * ols.RI.iNorm
    assert rel(R, Ro) < 1e-10
    lhs.free()


def test_zero_diagonal_takes_unit_scaling(gsls, orc):
    """A zero diagonal entry on an interior row: PRECONDDIAG takes W = 1
    there (no division by zero); the scaled matrix and the first iterations
    equal the oracle's."""
    p, R0, V0 = _heat_system(orc)
    interior = np.setdiff1d(np.arange(p.nNo), p.dirichlet[0].nodes)[7]
    row = slice(p.rowPtr[interior], p.rowPtr[interior + 1])
    diag = p.rowPtr[interior] + int(np.nonzero(p.colPtr[row] == interior)[0][0])
    V0 = V0.copy()
    V0[diag, 0] = 0.0
    lhs = _lhs_with_dir(p)
    ls = fsils.FSILS_LS_CREATE(fsils.LS_TYPE_CG, relTol=1e-12, maxItr=3)
    R, Val = R0.copy(), V0.copy()
    fsils.FSILS_SOLVE(lhs, ls, 1, R, Val, fsils.PRECOND_FSILS)
    s = _oracle_solver(orc, p)
    ols = orc.ls_create(orc.LS_TYPE_CG, relTol=1e-12, mItr=3)
    Ro, Vo = R0.copy(), V0.copy()
    s.solve(ols, 1, Ro, Vo, orc.PRECOND_FSILS)
    assert np.all(np.isfinite(Val))
    assert rel(Val, Vo) < 1e-15
    # W = 1 on that row: its off-diagonal entries are scaled by the column
    # factors only, so they keep their sign and stay finite
    assert Val[diag, 0] == 0.0
    assert ls.RI.itr == ols.RI.itr and ls.RI.suc == ols.RI.suc
    assert rel(R, Ro) < 1e-10
    lhs.free()


def test_inconsistent_nnz_is_rejected(gsls, orc):
    p = problems.heats_cube(3)
    g, rp1, cp1 = problems.make_lhs_arrays(p)
    with pytest.raises(_lib.GslsError) as exc:
        fsils.FSILS_LHS_CREATE(p.nNo, p.nNo, p.nnz - 1, g, rp1, cp1[:-1], 1)
    assert _status(exc) == GSLS_ERR_ARG
    bad = rp1.copy()
    bad[0] = 0                               # not 1-based
    with pytest.raises(_lib.GslsError) as exc:
        fsils.FSILS_LHS_CREATE(p.nNo, p.nNo, p.nnz, g, bad, cp1, 1)
    assert _status(exc) == GSLS_ERR_ARG
    q, R0, V0 = _heat_system(orc)
    _solve_ok_after(gsls, orc, q, R0, V0)


@pytest.mark.parametrize("mixed", [False, True])
def test_grid_barrier_timeout_returns_cleanly(gsls, orc, mixed):
    """The persistent Schur-complement CG of the NS solver waits on a grid
    barrier between its phases (FP64 and FP32 inner vectors).  With the
    poll limit cut to 2 the waits run out on a healthy launch: every block
    leaves, the solve returns GSLS_ERR_CUDA, and with the default limit back
    the same solve repeats the result of a solve made before the failure bit
    for bit and matches the oracle (the context is intact)."""
    p = problems.fluid_cylinder(h=0.1, nsteps=1)
    rng = np.random.default_rng(3)
    Y = np.zeros((p.nNo, 4))
    Y[:, 2] = 30.0 * np.clip(1.0 - (p.x[:, 0] ** 2 + p.x[:, 1] ** 2) / 0.25, 0.0, None)
    Y[:, 3] = rng.standard_normal(p.nNo)
    A = 1e3 * rng.standard_normal((p.nNo, 4))
    R0, V0 = orc.assemble(p, A, Y)
    faces = [d.nodes for d in p.dirichlet]

    def solve():
        g, rp1, cp1 = problems.make_lhs_arrays(p)
        lhs = fsils.FSILS_LHS_CREATE(p.nNo, p.nNo, p.nnz, g, rp1, cp1, len(faces))
        for k, nodes in enumerate(faces):
            fsils.FSILS_BC_CREATE(lhs, k + 1, nodes.size, 3, fsils.BC_TYPE_DIR, nodes + 1,
                                  np.zeros((nodes.size, 3)))
        ls = fsils.FSILS_LS_CREATE(fsils.LS_TYPE_NS, dimKry=100)
        try:
            if mixed:
                import torch
                dR = torch.tensor(R0, dtype=torch.float64, device="cuda")
                dV = torch.tensor(V0, dtype=torch.float32, device="cuda")
                torch.cuda.synchronize()
                _lib.check(gsls.gsls_solve_dev(lhs.h, C.byref(ls), 4, C.c_void_p(dR.data_ptr()),
                                               C.c_void_p(dV.data_ptr()), _lib.PREC_MIXED,
                                               fsils.PRECOND_RCS, None, None), "gsls_solve_dev")
                R = dR.cpu().numpy()
            else:
                R, Val = R0.copy(), V0.copy()
                fsils.FSILS_SOLVE(lhs, ls, 4, R, Val, fsils.PRECOND_RCS)
        finally:
            lhs.free()
        return ls, R

    ls0, R_before = solve()
    try:
        _lib.check(gsls.gsls_set_wait_limit(2), "gsls_set_wait_limit")
        with pytest.raises(_lib.GslsError) as exc:
            solve()
        assert _status(exc) == GSLS_ERR_CUDA
        assert "grid barrier" in str(exc.value)
    finally:
        _lib.check(gsls.gsls_set_wait_limit(0), "gsls_set_wait_limit")
    ls, R = solve()
    s = orc.OracleSolver(p.nNo, p.rowPtr, p.colPtr, len(faces))
    for k, nodes in enumerate(faces):
        s.bc_create(k + 1, nodes, 3, 0, np.zeros((nodes.size, 3)))
    ols = orc.ls_create(orc.LS_TYPE_NS, sD=100)
    Ro, Vo = R0.copy(), V0.copy()
    s.solve(ols, 4, Ro, Vo, orc.PRECOND_RCS)
    # the solve after the failure repeats the one before it bit for bit
    assert np.array_equal(R, R_before) and ls.RI.itr == ls0.RI.itr
    if mixed:
        # FP32 inner solves: the outer NS iteration stops within one
        # iteration of the oracle's
        assert ls.RI.suc == ols.RI.suc and abs(ls.RI.itr - ols.RI.itr) <= 1
    else:
        assert ls.RI.suc == ols.RI.suc and ls.RI.itr == ols.RI.itr
        assert rel(R, Ro) < 1e-8


def test_persistent_cg_barrier_timeout_returns_cleanly(gsls, orc):
    """Small CG solves run in one cooperative launch whose iterations meet
    at bounded grid barriers.  With the poll limit cut to 2 the waits run
    out: the solve returns GSLS_ERR_CUDA, and with the default limit back
    the library solves correctly (the context is intact)."""
    # the 20^3 heat cube: ~19 blocks meet at every barrier
    q = problems.heats_cube(20)
    rng = np.random.default_rng(4)
    Rq, Vq = orc.assemble(q, 1e-3 * rng.standard_normal((q.nNo, 1)),
                          1e-3 * rng.standard_normal((q.nNo, 1)))
    lhs = _lhs_with_dir(q)
    ls = fsils.FSILS_LS_CREATE(fsils.LS_TYPE_CG, relTol=1e-10, maxItr=2000)
    try:
        _lib.check(gsls.gsls_set_wait_limit(2), "gsls_set_wait_limit")
        R, Val = Rq.copy(), Vq.copy()
        with pytest.raises(_lib.GslsError) as exc:
            fsils.FSILS_SOLVE(lhs, ls, 1, R, Val, fsils.PRECOND_FSILS)
        assert _status(exc) == GSLS_ERR_CUDA
        assert "grid barrier" in str(exc.value)
    finally:
        _lib.check(gsls.gsls_set_wait_limit(0), "gsls_set_wait_limit")
        lhs.free()
    p, R0, V0 = _heat_system(orc)
    _solve_ok_after(gsls, orc, p, R0, V0)
