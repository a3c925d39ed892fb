"""Edge cases of the drop-in solve and of the time step, each against the
oracle on the same inputs: a zero right-hand side and an iteration limit
of one for CG, GMRES and BiCGStab (CGRAD.f:146-182, GMRES.f:273-431,
BICGS.f), the mixed-precision solve of a zero right-hand side, and a
one-element mesh stepped as a heat equation (the smallest CSR: one 4x4
row block per node)."""
import ctypes as C
import dataclasses

import numpy as np
import pytest

from svfsi_gb300 import _lib, fsils, problems

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, float).ravel(), np.asarray(b, float).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _system(orc):
    p = problems.heats_cube(4)
    rng = np.random.default_rng(1)
    R0, V0 = orc.assemble(p, 1e-3 * rng.standard_normal((p.nNo, 1)),
                          1e-3 * rng.standard_normal((p.nNo, 1)))
    return p, R0, V0


def _lhs(p):
    g, rp1, cp1 = problems.make_lhs_arrays(p)
    lhs = fsils.FSILS_LHS_CREATE(p.nNo, p.nNo, p.nnz, g, rp1, cp1, 1)
    dirn = p.dirichlet[0].nodes
    fsils.FSILS_BC_CREATE(lhs, 1, dirn.size, 3, fsils.BC_TYPE_DIR, dirn + 1,
                          np.zeros((dirn.size, 3)))
    return lhs


def _oracle_solve(orc, p, lt, mitr, R, V, rtol):
    s = orc.OracleSolver(p.nNo, p.rowPtr, p.colPtr, 1)
    dirn = p.dirichlet[0].nodes
    s.bc_create(1, dirn, 3, 0, np.zeros((dirn.size, 3)))
    ls = orc.ls_create(lt, relTol=rtol, mItr=mitr)
    s.solve(ls, 1, R, V, orc.PRECOND_FSILS)
    return ls


@pytest.mark.parametrize("case", ["zero", "one_iteration"])
@pytest.mark.parametrize("lstype", ["cg", "gmres", "bicgs"])
def test_degenerate_solves_match_oracle(gsls, orc, lstype, case):
    """Zero right-hand side: X = 0 with the reference's flags (CG and
    BiCGStab report success after no iteration; GMRES returns before its
    first restart with suc false).  maxItr = 1: one CG / BiCGStab iteration
    (suc false) or one GMRES restart (it converges inside it); counts,
    flags and solution as the oracle's.

    GMRES's stop test and its fNorm read the Givens residual estimate
    |err(i+1)| (GMRES.f:161), and the Pythagorean norm sqrt|v.v - sum
    h_j^2| resolves h_{i+1,i} only to about sqrt(eps)|v|.  On this system
    the oracle's estimates after 7..12 inner iterations are 3.4e-5, 5.5e-6,
    9.4e-7, 1.6e-7, 2.1e-8 and 9.1e-9 of the initial norm; from the 11th on
    they are at that resolution (the GPU, summing the dot products in
    another order, reads 3.0e-9 at the 11th), so the count and fNorm at a
    1e-8 threshold depend on rounding.  The GMRES restart therefore stops
    at 2.5e-6, after the 9th iteration, with the iterations either side a
    factor 2 or more from the threshold."""
    p, R0, V0 = _system(orc)
    t = {"cg": fsils.LS_TYPE_CG, "gmres": fsils.LS_TYPE_GMRES, "bicgs": fsils.LS_TYPE_BICGS}[lstype]
    mitr = 1 if case == "one_iteration" else 500
    rtol = 2.5e-6 if (lstype, case) == ("gmres", "one_iteration") else 1e-8
    Rin = np.zeros_like(R0) if case == "zero" else R0.copy()
    lhs = _lhs(p)
    ls = fsils.FSILS_LS_CREATE(t, relTol=rtol, maxItr=mitr)
    R, V = Rin.copy(), V0.copy()
    fsils.FSILS_SOLVE(lhs, ls, 1, R, V, fsils.PRECOND_FSILS)
    Ro = Rin.copy()
    ols = _oracle_solve(orc, p, t, mitr, Ro, V0.copy(), rtol)
    assert (ls.RI.itr, ls.RI.suc) == (ols.RI.itr, ols.RI.suc)
    if case == "zero":
        assert np.all(R == 0.0) and ls.RI.iNorm == 0.0
    else:
        # GMRES's classical Gram-Schmidt with the Pythagorean norm is
        # rounding-sensitive near convergence
        tol = 1e-8 if lstype == "gmres" else 1e-10
        assert abs(ls.RI.fNorm - ols.RI.fNorm) <= tol * ols.RI.iNorm
        assert rel(R, Ro) < tol
    lhs.free()


def test_mixed_solve_of_zero_rhs(gsls, orc):
    """gsls_solve_dev with an FP32 matrix and a zero right-hand side: no
    iteration, X = 0, success (the CG test before the first iteration)."""
    torch = pytest.importorskip("torch")
    p, _, V0 = _system(orc)
    lhs = _lhs(p)
    ls = fsils.FSILS_LS_CREATE(fsils.LS_TYPE_CG, relTol=1e-8, maxItr=500)
    dR = torch.zeros((p.nNo, 1), dtype=torch.float64, device="cuda")
    dV = torch.tensor(V0, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    _lib.check(gsls.gsls_solve_dev(lhs.h, C.byref(ls), 1, C.c_void_p(dR.data_ptr()),
                                   C.c_void_p(dV.data_ptr()), _lib.PREC_MIXED,
                                   fsils.PRECOND_FSILS, None, None), "gsls_solve_dev")
    assert ls.RI.itr == 0 and ls.RI.suc == 1
    assert torch.count_nonzero(dR).item() == 0
    lhs.free()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_one_element_heat_steps(gsls, orc, precision):
    """One tet, four nodes, T = 1 on node 0 and 0 on node 1 (Dirichlet),
    five implicit steps: the GPU state equals the oracle's (FP64 1e-12,
    mixed 1e-8)."""
    base = problems.heats_cube(2, nsteps=5)
    x = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=float)
    ien = np.array([[0, 1, 2, 3]], dtype=np.int32)
    rp, cp = orc.lhsa(4, ien)
    dirs = [problems.DirBC(np.array([0]), 1.0), problems.DirBC(np.array([1]), 0.0)]
    p = dataclasses.replace(base, name="one_tet", x=x, ien=ien, rowPtr=rp, colPtr=cp,
                            dirichlet=dirs)
    assert (p.nEl, p.nNo, p.nnz) == (1, 4, 16)
    prec = fsils.PREC_FP64 if precision == "fp64" else fsils.PREC_MIXED
    lhs, mesh, eq = problems.build_equation(p, precision=prec)
    oeq = orc.OracleEquation(p)
    oeq.set_state(*p.initial_state())
    for _ in range(p.nsteps):
        gi, oi = eq.step(), oeq.step()
        assert gi.newton_itr == oi.newton_itr
    _, Y, _ = eq.get_state()
    _, Yo, _ = oeq.state()
    assert rel(Y, Yo) < (1e-12 if precision == "fp64" else 1e-8)
    assert Y[0, 0] == 1.0 and Y[1, 0] == 0.0
    eq.free()
    mesh.free()
    lhs.free()
