"""GPU parity of CEP with fibres (CEP3D's anisotropic diffusion,
Code/Source/svFSI/CEP.f:136-266, no electromechanical coupling): the
diffusion tensor of an element is D = Diso I + sum_i Dani_i f_i f_i^T with
the element's fibre directions.  On a slab with a helical fibre field
(problems.slab_fibers), one and two fibre families:

* element assembly against the oracle, FP64 1e-12 and the FP32 tangent
  1e-5 (residual 1e-12), on the default path (the cached conduction
  operator) and, in a fresh process, on the element loop
  (GSLS_HEATS_ASM=element);
* 40 implicit steps of the activation wave, FP64 1e-10 and mixed 1e-8
  against the oracle, and the wave differs from the isotropic one;
* fibres on another physics are an argument error.
"""
import ctypes as C
import dataclasses

import numpy as np
import pytest

from svfsi_gb300 import _lib, fsils, problems

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, float).ravel(), np.asarray(b, float).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _lhs(p):
    g, rp1, cp1 = problems.make_lhs_arrays(p)
    return fsils.FSILS_LHS_CREATE(p.nNo, p.nNo, p.nnz, g, rp1, cp1, 1)


def _isotropic(p):
    prm = {k: v for k, v in p.params.items() if k != "Dani"}
    return dataclasses.replace(p, fibers=None, params=prm)


def _state(p, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((p.nNo, 1)), -80.0 + 20.0 * rng.standard_normal((p.nNo, 1))


@pytest.mark.parametrize("nFn", [1, 2])
def test_cep_fibre_assembly_fp64(gsls, orc, nFn):
    p = problems.cep_slab(8, 8, 3, nsteps=1, nFn=nFn)
    A, Y = _state(p, nFn)
    R0, V0 = orc.assemble(p, A, Y)
    Ri, Vi = orc.assemble(_isotropic(p), A, Y)
    # the fibre term is well above the tolerances (the tangent is mostly mass)
    assert rel(V0, Vi) > 3e-3 and rel(R0, Ri) > 0.1
    lhs = _lhs(p)
    mesh = fsils.Mesh(lhs, p.ien, p.x)
    R, Val = mesh.assemble(p.eq_params(), A, Y, np.zeros_like(Y), p.dof)
    assert rel(R, R0) < 1e-12
    assert rel(Val, V0) < 1e-12
    mesh.free()
    lhs.free()


def test_cep_fibre_assembly_with_element_diffusivity(gsls, orc):
    """Fibres with a per-element Diso (the parameter of the CEP adjoint):
    D_e = Diso_e I + sum_i Dani_i f_i f_i^T, FP64 1e-12."""
    p = problems.cep_slab(8, 8, 3, nsteps=1, nFn=2)
    ep = np.exp(0.3 * np.random.default_rng(4).standard_normal(p.nEl)) * 0.1
    A, Y = _state(p, 5)
    R0, V0 = orc.assemble(p, A, Y, eparam=ep)
    lhs = _lhs(p)
    mesh = fsils.Mesh(lhs, p.ien, p.x)
    prm = p.eq_params()
    epc = np.ascontiguousarray(ep)
    prm.eparam = epc.ctypes.data_as(C.POINTER(C.c_double))
    R, Val = mesh.assemble(prm, A, Y, np.zeros_like(Y), p.dof)
    assert rel(R, R0) < 1e-12
    assert rel(Val, V0) < 1e-12
    mesh.free()
    lhs.free()


def test_cep_fibre_assembly_fp32_tangent(gsls, orc):
    torch = pytest.importorskip("torch")
    p = problems.cep_slab(8, 8, 3, nsteps=1, nFn=2)
    A, Y = _state(p, 7)
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
                                      fsils.PREC_MIXED), "gsls_assemble_dev")
    torch.cuda.synchronize()
    assert rel(dR.cpu().numpy(), R0) < 1e-12
    assert rel(dV.cpu().numpy().astype(np.float64), V0) < 1e-5
    mesh.free()
    lhs.free()


def test_cep_fibres_on_the_element_loop(gsls):
    """The same assembly and step tests with the per-Newton element loop
    (k_asm_heats) instead of the cached operators, in a fresh process."""
    import os
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    env = dict(os.environ, GSLS_HEATS_ASM="element", PYTHONPATH=str(root))
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-m", "gpu", "-p", "no:cacheprovider",
                        "-k", "fibre_assembly or fibre_steps", str(Path(__file__).resolve())],
                       cwd=root, env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert "6 passed" in r.stdout, r.stdout[-500:]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cep_fibre_steps(gsls, orc, precision):
    p = problems.cep_slab(16, 16, 3, nsteps=40, A=52.0, nFn=2)
    if precision == "mixed":
        p.tol, p.maxItr = 1e-12, 8
    prec = fsils.PREC_FP64 if precision == "fp64" else fsils.PREC_MIXED
    lhs, mesh, eq = problems.build_equation(p, precision=prec)
    oeq = orc.OracleEquation(p)
    oiso = orc.OracleEquation(_isotropic(p))
    for _ in range(p.nsteps):
        gi, oi = eq.step(), oeq.step()
        if precision == "fp64":
            assert gi.newton_itr == oi.newton_itr
        oiso.step()
    _, Y, _ = eq.get_state()
    _, Yo, _ = oeq.state()
    _, Yi, _ = oiso.state()
    X = eq.get_cep_state()
    v0 = p.cep["V0"]
    assert rel(Yo - v0, Yi - v0) > 1e-2  # the fibres steer the wave
    assert rel(Y - v0, Yo - v0) < (1e-10 if precision == "fp64" else 1e-8)
    assert rel(X[:, 1], oeq.Xion[:, 1]) < (1e-9 if precision == "fp64" else 1e-8)
    assert Y.max() > -60.0
    eq.free()
    mesh.free()
    lhs.free()


def test_fibres_outside_cep_are_rejected(gsls):
    p = problems.heats_cube(3, nsteps=1)
    p.params["Dani"] = (0.5,)
    p.fibers = np.tile([1.0, 0.0, 0.0], (p.nEl, 1))
    g, rp1, cp1 = problems.make_lhs_arrays(p)
    lhs = fsils.FSILS_LHS_CREATE(p.nNo, p.nNo, p.nnz, g, rp1, cp1, 1)
    mesh = fsils.Mesh(lhs, p.ien, p.x)
    with pytest.raises(_lib.GslsError):
        fsils.Equation(mesh, p.eq_params(), p.eq_solver())
    mesh.free()
    lhs.free()
