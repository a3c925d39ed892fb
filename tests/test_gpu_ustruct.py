"""USTRUCT (velocity-pressure nonlinear solid, Code/Source/svFSI/USTRUCT.f)
on the GPU against the oracle: the element assembly into Val and the
displacement tangent Kd (FP64 1e-12; the mixed path forms both tangents in
FP32 arithmetic: Val 1e-5, Kd 1e-6 -- Kd enters only the first Newton
iteration's right-hand side, which the later iterations refine), and converged
implicit steps with USTRUCTR's first-iteration correction and the ustruct
predictor/corrector (FP64 1e-9, mixed 1e-8, equal Newton counts), for the
compressible ST91 solid and the incompressible one (Kpen = 0)."""
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
    A = 1e1 * rng.standard_normal((p.nNo, 4))
    Y = 1e-2 * rng.standard_normal((p.nNo, 4))
    Y[:, 3] = 1e3 * rng.standard_normal(p.nNo)
    D = 1e-3 * rng.standard_normal((p.nNo, 4))
    D[:, 3] = 0.0
    return A, Y, D


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("visc", [0.0, 50.0])
def test_ustruct_assembly_matches_oracle(gsls, orc, mixed, visc):
    torch = pytest.importorskip("torch")
    p = problems.ustruct_beam(8, 3, 3, visc=visc, ctC=0.1)
    A, Y, D = _state(p, 3)
    R0, V0, K0 = orc.assemble_ustruct(p, A, Y, D)
    g, rp1, cp1 = problems.make_lhs_arrays(p)
    lhs = fsils.FSILS_LHS_CREATE(p.nNo, p.nNo, p.nnz, g, rp1, cp1, 1)
    mesh = fsils.Mesh(lhs, p.ien, p.x)
    dA, dY, dD = (torch.tensor(a, device="cuda") for a in (A, Y, D))
    dR = torch.zeros((p.nNo, 4), dtype=torch.float64, device="cuda")
    dV = torch.zeros((p.nnz, 16), dtype=torch.float32 if mixed else torch.float64, device="cuda")
    dK = torch.zeros((p.nnz, 12), dtype=torch.float64, device="cuda")
    prm = p.eq_params()
    _lib.check(gsls.gsls_assemble_ustruct_dev(
        mesh.h, C.byref(prm), C.c_void_p(dA.data_ptr()), C.c_void_p(dY.data_ptr()),
        C.c_void_p(dD.data_ptr()), C.c_void_p(dR.data_ptr()), C.c_void_p(dV.data_ptr()),
        C.c_void_p(dK.data_ptr()), fsils.PREC_MIXED if mixed else fsils.PREC_FP64))
    torch.cuda.synchronize()
    assert rel(dR.cpu().numpy(), R0) < 1e-12
    assert rel(dK.cpu().numpy(), K0) < (1e-6 if mixed else 1e-12)
    assert rel(dV.cpu().numpy().astype(np.float64), V0) < (1e-5 if mixed else 1e-12)
    mesh.free()
    lhs.free()


@pytest.mark.parametrize("nu", [0.45, 0.5])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ustruct_steps_match_oracle(gsls, orc, nu, precision):
    p = problems.ustruct_beam(12, 3, 3, nsteps=3, nu=nu)
    p.tol = 1e-10
    p.maxItr = 14
    prec = fsils.PREC_FP64 if precision == "fp64" else fsils.PREC_MIXED
    lhs, mesh, eq = problems.build_equation(p, precision=prec)
    oeq = orc.OracleEquation(p)
    oeq.set_state(*p.initial_state())
    for _ in range(p.nsteps):
        gi = eq.step()
        oi = oeq.step()
        assert gi.last_suc == 1 and oi.last_suc == 1
        assert gi.newton_itr == oi.newton_itr
    A, Y, D = eq.get_state()
    Ao, Yo, Do = oeq.state()
    tol = 1e-9 if precision == "fp64" else 1e-8
    assert rel(D[:, :3], Do[:, :3]) < tol
    assert rel(Y[:, :3], Yo[:, :3]) < tol
    assert rel(Y[:, 3], Yo[:, 3]) < tol
    assert np.abs(D[:, :3]).max() > 1e-3          # the beam did bend


def test_ustruct_medium_beam_matches_oracle(gsls, orc):
    """The 66x16x16-hex beam (101,376 tets) at the benchmark's settings (the
    reference's default GMRES, Newton tol 1e-8 and limit 10): one step in
    FP64 and mixed precision against the oracle's step on all host cores
    (coloured OpenMP assembly), equal Newton counts, FP64 1e-10 and mixed
    1e-8 on the displacement and the pressure."""
    import os
    p = problems.ustruct_beam(66, 16, 16, nsteps=1)
    assert p.nEl == 101_376
    orc.set_threads(os.cpu_count() or 1)
    try:
        oeq = orc.OracleEquation(p, colored=True)
        oeq.set_state(*p.initial_state())
        no = oeq.step().newton_itr
    finally:
        orc.set_threads(1)
    Ao, Yo, Do = oeq.state()
    for precision, tol in (("fp64", 1e-10), ("mixed", 1e-8)):
        prec = fsils.PREC_FP64 if precision == "fp64" else fsils.PREC_MIXED
        lhs, mesh, eq = problems.build_equation(p, precision=prec)
        gi = eq.step()
        A, Y, D = eq.get_state()
        eq.free()
        mesh.free()
        lhs.free()
        print(f"ustruct 66x16x16 {precision}: newton {gi.newton_itr} (oracle {no}); rel D "
              f"{rel(D[:, :3], Do[:, :3]):.2e} p {rel(Y[:, 3], Yo[:, 3]):.2e}")
        assert gi.newton_itr == no
        assert rel(D[:, :3], Do[:, :3]) < tol
        assert rel(Y[:, 3], Yo[:, 3]) < tol


def test_ustruct_restart_is_rejected(gsls, tmp_path):
    p = problems.ustruct_beam(4, 2, 2, nsteps=1)
    lhs, mesh, eq = problems.build_equation(p)
    with pytest.raises(_lib.GslsError, match="USTRUCT"):
        eq.write_restart(str(tmp_path / "r.bin"), 1, 0.0)
