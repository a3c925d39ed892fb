"""GPU parity of linear elasticity (LELAS3D, GSLS_PHYS_LELAS) against the
oracle: element assembly in FP64 (1e-12 relative) and with the FP32
tangent (1e-5 on Val, residual still 1e-12), and implicit time steps of the
clamped beam under end traction in FP64 (1e-9) and mixed precision (1e-8).
"""
import ctypes as C

import numpy as np
import pytest

from svfsi_gb300 import _lib, fsils, problems

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, float).ravel(), np.asarray(b, float).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _state(p, seed):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((p.nNo, 3))
    Y = 1e-2 * rng.standard_normal((p.nNo, 3))
    D = 1e-3 * rng.standard_normal((p.nNo, 3))
    return A, Y, D


def _lhs(p):
    g, rp1, cp1 = problems.make_lhs_arrays(p)
    return fsils.FSILS_LHS_CREATE(p.nNo, p.nNo, p.nnz, g, rp1, cp1, 1)


def test_lelas_assembly_fp64(gsls, orc):
    p = problems.lelas_beam(8, 3, 3, f=(0.0, 1.0, -2.0))
    A, Y, D = _state(p, 1)
    R0, V0 = orc.assemble(p, A, Y, D)
    lhs = _lhs(p)
    mesh = fsils.Mesh(lhs, p.ien, p.x)
    R, Val = mesh.assemble(p.eq_params(), A, Y, D, p.dof)
    assert rel(R, R0) < 1e-12
    assert rel(Val, V0) < 1e-12


def test_lelas_assembly_fp32_tangent(gsls, orc):
    torch = pytest.importorskip("torch")
    p = problems.lelas_beam(8, 3, 3)
    A, Y, D = _state(p, 2)
    R0, V0 = orc.assemble(p, A, Y, D)
    lhs = _lhs(p)
    mesh = fsils.Mesh(lhs, p.ien, p.x)
    dA, dY, dD = (torch.tensor(v, device="cuda") for v in (A, Y, D))
    dR = torch.zeros((p.nNo, 3), dtype=torch.float64, device="cuda")
    dV = torch.zeros((p.nnz, 9), dtype=torch.float32, device="cuda")
    prm = p.eq_params()
    _lib.check(gsls.gsls_assemble_dev(mesh.h, C.byref(prm), C.c_void_p(dA.data_ptr()),
                                      C.c_void_p(dY.data_ptr()), C.c_void_p(dD.data_ptr()),
                                      C.c_void_p(dR.data_ptr()), C.c_void_p(dV.data_ptr()),
                                      fsils.PREC_MIXED))
    torch.cuda.synchronize()
    assert rel(dR.cpu().numpy(), R0) < 1e-12
    assert rel(dV.cpu().numpy().astype(np.float64), V0) < 1e-5


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_lelas_steps(gsls, orc, precision):
    p = problems.lelas_beam(12, 3, 3, nsteps=3, traction=(0.0, 0.0, -5e3))
    prec = fsils.PREC_FP64 if precision == "fp64" else fsils.PREC_MIXED
    lhs, mesh, eq = problems.build_equation(p, precision=prec)
    oeq = orc.OracleEquation(p)
    for _ in range(p.nsteps):
        gi = eq.step()
        oi = oeq.step()
        assert gi.last_suc == 1 and oi.last_suc == 1
    A, Y, D = eq.get_state()
    Ao, Yo, Do = oeq.state()
    assert np.abs(Do).max() > 0
    tol = 1e-9 if precision == "fp64" else 1e-8
    assert rel(D, Do) < tol
    assert rel(Y, Yo) < 10 * tol


def test_lelas_rejects_bad_poisson_ratio(gsls):
    p = problems.lelas_beam(4, 2, 2, nu=0.5)
    A, Y, D = _state(p, 3)
    lhs = _lhs(p)
    mesh = fsils.Mesh(lhs, p.ien, p.x)
    with pytest.raises(RuntimeError):
        mesh.assemble(p.eq_params(), A, Y, D, p.dof)
