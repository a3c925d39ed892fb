"""GPU parity of heat transport in a fluid (HEATF3D, GSLS_PHYS_HEATF)
against the oracle: element assembly with a random velocity and
temperature state (FP64 1e-12; FP32 tangent 1e-5 with the FP64 residual at
1e-12) and implicit steps of the cylinder with a prescribed Poiseuille
flow.

The discontinuity-capturing diffusivity of HEATF3D, nu + |r| / (2 sqrt(Tx.ks.Tx))
with r the strong residual, is left out of the reference's tangent, so its
Newton loop is a fixed-point iteration that converges linearly; the step
test runs a fixed number of iterations (the same in both codes) with each
correction solved tightly by restarted GMRES(20) -- the reference's
classical Gram-Schmidt with the Pythagorean norm stalls near 2e-8 relative
over long cycles on this system, after which its basis grows without bound
-- so every iterate is a well-conditioned function of the previous one
(FP64, 4 iterations: 1e-9 on the temperature change).  The mixed path's
FP32 GMRES corrections (relTol 1e-6) are refined by the FP64 residual of
the next iterations: after the configuration's 10 iterations per step the
temperature change is within 1e-8 of the oracle's.
"""
import ctypes as C

import numpy as np
import pytest

from svfsi_gb300 import _lib, fsils, meshgen, problems

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, float).ravel(), np.asarray(b, float).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _state(p, seed):
    rng = np.random.default_rng(seed)
    Y = np.zeros((p.nNo, 5))
    Y[:, :3] = 5.0 * rng.standard_normal((p.nNo, 3))
    Y[:, 4] = rng.standard_normal(p.nNo)
    A = np.zeros_like(Y)
    A[:, 4] = 10.0 * rng.standard_normal(p.nNo)
    return A, Y


def _lhs(p):
    g, rp1, cp1 = problems.make_lhs_arrays(p)
    return fsils.FSILS_LHS_CREATE(p.nNo, p.nNo, p.nnz, g, rp1, cp1, 1)


def test_heatf_assembly_fp64(gsls, orc):
    p = problems.heatf_cylinder(h=0.1, nsteps=1)
    p.params["src"] = 0.3
    A, Y = _state(p, 1)
    R0, V0 = orc.assemble(p, A, Y)
    lhs = _lhs(p)
    mesh = fsils.Mesh(lhs, p.ien, p.x)
    R, Val = mesh.assemble(p.eq_params(), A, Y, np.zeros_like(Y), p.dof)
    assert rel(R, R0) < 1e-12
    assert rel(Val, V0) < 1e-12


def test_heatf_assembly_fp32_tangent(gsls, orc):
    torch = pytest.importorskip("torch")
    p = problems.heatf_cylinder(h=0.1, nsteps=1)
    A, Y = _state(p, 2)
    R0, V0 = orc.assemble(p, A, Y)
    lhs = _lhs(p)
    mesh = fsils.Mesh(lhs, p.ien, p.x)
    dA, dY = torch.tensor(A, device="cuda"), torch.tensor(Y, device="cuda")
    dD = torch.zeros_like(dY)
    dR = torch.zeros(p.nNo, dtype=torch.float64, device="cuda")
    dV = torch.zeros(p.nnz, dtype=torch.float32, device="cuda")
    prm = p.eq_params()
    _lib.check(gsls.gsls_assemble_dev(mesh.h, C.byref(prm), C.c_void_p(dA.data_ptr()),
                                      C.c_void_p(dY.data_ptr()), C.c_void_p(dD.data_ptr()),
                                      C.c_void_p(dR.data_ptr()), C.c_void_p(dV.data_ptr()),
                                      fsils.PREC_MIXED))
    torch.cuda.synchronize()
    assert rel(dR.cpu().numpy(), R0) < 1e-12
    assert rel(dV.cpu().numpy().astype(np.float64), V0) < 1e-5


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_heatf_steps(gsls, orc, precision):
    nit = 4 if precision == "fp64" else 10

    def make():
        q = problems.heatf_cylinder(h=0.1, nsteps=2, u_max=3.0, cond=1.0, T0_linear=True)
        q.maxItr, q.ls_sD, q.ls_mItr, q.ls_relTol = nit, 20, 20, 1e-12
        return q
    p = make()
    if precision == "mixed":
        p.ls_relTol = 1e-6
    prec = fsils.PREC_FP64 if precision == "fp64" else fsils.PREC_MIXED
    lhs, mesh, eq = problems.build_equation(p, precision=prec)
    q = make()
    oeq = orc.OracleEquation(q)
    oeq.set_state(*q.initial_state())
    for _ in range(p.nsteps):
        gi = eq.step()
        oi = oeq.step()
        assert gi.newton_itr == oi.newton_itr <= nit
    _, Y, _ = eq.get_state()
    _, Yo, _ = oeq.state()
    assert np.array_equal(Y[:, :3], Yo[:, :3])  # the flow is carried unchanged
    dT, dTo = Y[:, 4] - q.Y0[:, 4], Yo[:, 4] - q.Y0[:, 4]
    assert np.abs(dTo).max() > 1e-4  # the temperature moved
    assert rel(dT, dTo) < (1e-9 if precision == "fp64" else 1e-8)


@pytest.mark.parametrize("u_max,g", [(-3.0, 0.0), (3.0, 0.5)])
def test_heatf_outlet_neumann_face(gsls, orc, u_max, g):
    """A Neumann face on the outlet plane z = 5 (BASSEMNEUBC + BHEATF): with
    the flow reversed the backflow term min(u.n, 0) T and its tangent act,
    with forward flow the flux -g alone; the temperature change of one step
    (2 Newton iterations, GMRES(20)) matches the oracle to 1e-9 and differs
    from the step without the face."""
    def run(with_face):
        p = problems.heatf_cylinder(h=0.2, nsteps=1, u_max=u_max, cond=1.0, T0_linear=True)
        p.maxItr, p.ls_sD, p.ls_mItr, p.ls_relTol = 2, 20, 20, 1e-12
        if with_face:
            p.neumann = [problems.NeuBC(meshgen.faces_on_plane(p.x, p.ien, 2, 5.0), g)]
        _, _, eq = problems.build_equation(p)
        oeq = orc.OracleEquation(p)
        oeq.set_state(*p.initial_state())
        eq.step()
        oeq.step()
        return (eq.get_state()[1][:, 4] - p.Y0[:, 4], oeq.state()[1][:, 4] - p.Y0[:, 4])

    dT, dTo = run(True)
    assert rel(dT, dTo) < 1e-9
    dT0, _ = run(False)
    assert rel(dT, dT0) > 1e-6


def test_neumann_face_of_other_physics_is_unsupported(gsls):
    p = problems.heats_cube(3, nsteps=1)
    _, _, eq = problems.build_equation(p)
    with pytest.raises(_lib.GslsError, match="BHEATF"):
        eq.add_neumann(meshgen.faces_on_plane(p.x, p.ien, 0, 1.0), 1.0)
