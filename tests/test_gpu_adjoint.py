"""Discrete adjoint (forward/backward pair of the C ABI) against central
finite differences of the objective, on the GPU FP64 path and on the oracle
(the CPU restatement with per-element parameters).

Objective: J = 1/2 |u_tip - u_target|^2 on the final displacement of the
x = L face (STRUCT, parameter C10 = mu/2 per element) or 1/2 |T - T_target|^2
on all nodes (HEATS, conductivity per element).  Checked to 1e-5 relative
along seeded random directions (relative perturbations of every element's
parameter), with Newton and the Krylov solves converged tightly so that the
finite differences resolve 1e-5.
"""
import numpy as np
import pytest

from svfsi_gb300 import fsils, meshgen, problems

pytestmark = pytest.mark.gpu

FD_H = 1e-4  # relative parameter perturbation of the central differences


def _struct(nsteps=6):
    p = problems.struct_beam(10, 3, 3, nsteps=nsteps, traction=(0.0, 0.0, -5e3))
    p.tol, p.maxItr, p.ls_relTol = 1e-13, 20, 1e-12
    rng = np.random.default_rng(7)
    ep = p.params["C10"] * np.exp(0.2 * rng.standard_normal(p.nEl))
    tip = meshgen.nodes_on_plane(p.x, 0, 4.0)
    return p, ep, tip


def _heats(nsteps=5):
    p = problems.heats_cube(5, nsteps=nsteps)
    p.tol, p.maxItr, p.ls_relTol = 1e-13, 20, 1e-13
    rng = np.random.default_rng(8)
    ep = np.exp(0.3 * rng.standard_normal(p.nEl))
    return p, ep, np.arange(p.nNo)


def _final(p, ep, field):
    lhs, mesh, eq = problems.build_equation(p)
    eq.set_eparam(ep)
    for _ in range(p.nsteps):
        eq.step()
    st = eq.get_state()
    return st[field]


def _J(u, sel, target):
    d = u[sel] - target
    return 0.5 * float(np.sum(d * d))


def _adjoint_grad(p, ep, sel, field, target, precision):
    lhs, mesh, eq = problems.build_equation(p, precision=precision)
    eq.set_eparam(ep)
    tape = eq.adjoint_forward(p.nsteps, every=4)
    st = eq.get_state()
    uN = st[field]
    bar = np.zeros_like(uN)
    bar[sel] = uN[sel] - target
    grad = tape.backward(Dbar=bar) if field == 2 else tape.backward(Ybar=bar)
    tape.free()
    # the equation is left at step N
    assert np.allclose(eq.get_state()[field], uN, rtol=0, atol=0)
    return uN, grad


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", ["struct", "heats"])
def test_adjoint_gradient_matches_central_fd(gsls, case, precision):
    """The mixed path runs the forward and recomputed steps with the FP32
    tangent and inner CG, and each transpose solve as iterative refinement
    (FP32 CG sweeps on FP64 residuals, to the FP64 solve's 1e-12): its
    gradient matches the FP64 adjoint's to 1e-8 and the same central
    differences to 1e-5."""
    p, ep, sel = _struct() if case == "struct" else _heats()
    field = 2 if case == "struct" else 1  # D (struct) or T = Y (heats)
    u0 = _final(p, ep, field)
    rng = np.random.default_rng(21)
    target = u0[sel] * (1.0 + 0.1 * rng.standard_normal(u0[sel].shape))
    prec = fsils.PREC_FP64 if precision == "fp64" else fsils.PREC_MIXED
    uN, grad = _adjoint_grad(p, ep, sel, field, target, prec)
    # the FP64 forward is u0 to rounding; the mixed one within the contract
    tol = 1e-12 if precision == "fp64" else 1e-9
    assert np.allclose(uN, u0, rtol=0, atol=tol * np.abs(u0).max())
    if precision == "mixed":
        _, g64 = _adjoint_grad(p, ep, sel, field, target, fsils.PREC_FP64)
        assert np.linalg.norm(grad - g64) <= 1e-8 * np.linalg.norm(g64)
    for k in range(3):
        r = rng.standard_normal(p.nEl)
        r /= np.linalg.norm(r)
        dp = ep * r  # relative direction
        Jp = _J(_final(p, ep + FD_H * dp, field), sel, target)
        Jm = _J(_final(p, ep - FD_H * dp, field), sel, target)
        fd = (Jp - Jm) / (2 * FD_H)
        ad = float(grad @ dp)
        assert abs(fd - ad) <= 1e-5 * abs(ad), (k, fd, ad)


def test_adjoint_matches_oracle_fd(gsls, orc):
    """The GPU adjoint gradient against a central finite difference of the
    CPU oracle (same algorithm, per-element C10) along one direction."""
    p, ep, sel = _struct(nsteps=3)
    lhs, mesh, eq = problems.build_equation(p)
    eq.set_eparam(ep)
    tape = eq.adjoint_forward(p.nsteps, every=2)
    uN = eq.get_state()[2]
    rng = np.random.default_rng(5)
    target = uN[sel] * 0.95
    bar = np.zeros_like(uN)
    bar[sel] = uN[sel] - target
    grad = tape.backward(Dbar=bar)
    tape.free()
    r = rng.standard_normal(p.nEl)
    r /= np.linalg.norm(r)
    dp = ep * r

    def J_oracle(e):
        oeq = orc.OracleEquation(p, eparam=e)
        for _ in range(p.nsteps):
            oeq.step()
        return _J(oeq.state()[2], sel, target)

    fd = (J_oracle(ep + FD_H * dp) - J_oracle(ep - FD_H * dp)) / (2 * FD_H)
    ad = float(grad @ dp)
    assert abs(fd - ad) <= 1e-5 * abs(ad), (fd, ad)


def test_adjoint_solve_and_dRdp_building_blocks(gsls):
    """gsls_adjoint_solve returns K^-T g (checked through the tangent itself:
    K lambda = g on the free rows) and gsls_dRdp is linear in lambda."""
    torch = pytest.importorskip("torch")
    import ctypes as C

    from svfsi_gb300 import _lib
    p, ep, sel = _struct(nsteps=1)
    lhs, mesh, eq = problems.build_equation(p)
    eq.set_eparam(ep)
    Ao, Yo, Do = eq.get_state()
    eq.step()
    An, Yn, Dn = eq.get_state()
    dev = [torch.tensor(a, device="cuda") for a in (Ao, Yo, Do, An, Yn, Dn)]
    pt = _lib.AdjPoint(*[C.c_void_p(t.data_ptr()) for t in dev])
    rng = np.random.default_rng(3)
    g = torch.tensor(rng.standard_normal((p.nNo, 3)), device="cuda")
    lam = torch.zeros_like(g)
    L = _lib.load()
    _lib.check(L.gsls_adjoint_solve(eq.h, C.byref(pt), C.c_void_p(g.data_ptr()),
                                    C.c_void_p(lam.data_ptr())))
    out1 = torch.zeros(p.nEl, dtype=torch.float64, device="cuda")
    out2 = torch.zeros_like(out1)
    _lib.check(L.gsls_dRdp(eq.h, C.byref(pt), C.c_void_p(lam.data_ptr()),
                           C.c_void_p(out1.data_ptr())))
    lam2 = 2.0 * lam
    _lib.check(L.gsls_dRdp(eq.h, C.byref(pt), C.c_void_p(lam2.data_ptr()),
                           C.c_void_p(out2.data_ptr())))
    torch.cuda.synchronize()
    o1, o2 = out1.cpu().numpy(), out2.cpu().numpy()
    assert np.abs(o1).max() > 0
    assert np.allclose(o2, 2.0 * o1, rtol=1e-14, atol=0)
    # K lambda = g on free rows: assemble the tangent at the same point
    am, af = p.params["am"], p.params["af"]
    Ag = (1 - am) * Ao + am * An
    Yg = (1 - af) * Yo + af * Yn
    Dg = (1 - af) * Do + af * Dn
    import oracle as O
    e = np.ascontiguousarray(ep)
    _, Vo = O.assemble(p, Ag, Yg, Dg, eparam=e)
    lh = lam.cpu().numpy()
    Kl = np.zeros_like(lh)
    for i in range(p.nNo):
        for j in range(p.rowPtr[i], p.rowPtr[i + 1]):
            Kl[i] += Vo[j].reshape(3, 3) @ lh[p.colPtr[j]]
    free = np.ones(p.nNo, bool)
    free[p.dirichlet[0].nodes] = False
    gh = g.cpu().numpy()
    assert np.allclose(Kl[free], gh[free], rtol=1e-8, atol=1e-8 * np.abs(gh).max())
    assert np.abs(lh[~free]).max() == 0.0


# ---------------------------------------------------------------------------
# CEP: gradient of an activation-time mismatch with respect to the
# per-element diffusivity.  A planar front (stimulus +52 on x <= 1.5: under
# the Aliev-Panfilov sign convention -52 would hyperpolarise and nothing
# would activate) crosses a 24x24x2-hex slab, D_e = exp(0.2 N(0,1)),
# dt = dt_ode = 0.1 ms, 120 steps.  T_a = sum_n dt (1 - s(V_n(a))) with
# s(V) = 1/(1 + exp(-(V + 30)/5)), J = 1/2 |T - T*|^2, T* from a run with
# D_e perturbed by exp(0.05 N(0,1)).

CEP_VTH, CEP_VW = -30.0, 5.0


def _cep(nsteps=120, ode=0, nFn=0, Dani=(0.5, 0.1)):
    p = problems.cep_slab(24, 24, 2, nsteps=nsteps, A=52.0, Diso=1.0, nFn=nFn, Dani=Dani)
    p.stim = (p.x[:, 0] <= 1.5).astype(np.int32)
    p.params["dt"] = 0.1
    p.cep["dt_ode"] = 0.1
    if ode:  # AP_INTEGRK with two substeps per step
        p.cep["ode"], p.cep["dt_ode"] = 1, 0.05
    p.tol, p.maxItr, p.ls_relTol = 1e-13, 8, 1e-11
    rng = np.random.default_rng(9)
    ep = np.exp(0.2 * rng.standard_normal(p.nEl))
    return p, ep


def _act(Y):
    return 1.0 - 1.0 / (1.0 + np.exp(-(Y - CEP_VTH) / CEP_VW))


def _cep_T_gpu(p, ep):
    lhs, mesh, eq = problems.build_equation(p)
    eq.set_eparam(ep)
    T = np.zeros(p.nNo)
    for _ in range(p.nsteps):
        eq.step()
        T += p.params["dt"] * _act(eq.get_state()[1][:, 0])
    eq.free()
    mesh.free()
    lhs.free()
    return T


def _cep_T_oracle(orc, p, ep):
    eq = orc.OracleEquation(p, eparam=ep)
    eq.set_state(*p.initial_state())
    T = np.zeros(p.nNo)
    for _ in range(p.nsteps):
        eq.step()
        T += p.params["dt"] * _act(eq.state()[1][:, 0])
    return T


def _cep_adjoint(p, ep, Tstar, precision):
    lhs, mesh, eq = problems.build_equation(p, precision=precision)
    eq.set_eparam(ep)
    T, tape = eq.cep_adjoint_forward(p.nsteps, every=25, vth=CEP_VTH, vw=CEP_VW)
    YN = eq.get_state()[1].copy()
    grad = tape.backward(T - Tstar)
    tape.free()
    assert np.array_equal(eq.get_state()[1], YN)       # left at step N
    return T, grad


@pytest.mark.parametrize("precision,ode,nFn", [("fp64", 0, 0), ("mixed", 0, 0), ("fp64", 1, 0),
                                               ("fp64", 0, 2)])
def test_cep_activation_adjoint_matches_fd(gsls, orc, precision, ode, nFn):
    """FP64: the gradient against central differences of the GPU's and the
    oracle's activation times.  Mixed (FP32 tangent and CG in the steps,
    refined transpose solves): against the FP64 gradient to 1e-8 and the
    same central differences.  ode = 1: the RK4 cell step (two substeps
    per step) reversed stage by stage.  nFn = 2: two fibre families on top
    of the per-element isotropic diffusivity being differentiated."""
    p, ep = _cep(ode=ode, nFn=nFn)
    rng = np.random.default_rng(31)
    Tstar = _cep_T_gpu(p, ep * np.exp(0.05 * rng.standard_normal(p.nEl)))
    prec = fsils.PREC_FP64 if precision == "fp64" else fsils.PREC_MIXED
    T, grad = _cep_adjoint(p, ep, Tstar, prec)
    # the front crossed part of the slab: activation times spread over the run
    assert T.min() < 2.0 and np.percentile(T, 50) < 0.9 * p.nsteps * p.params["dt"]
    tol_T = 1e-12 if precision == "fp64" else 1e-9
    assert np.allclose(T, _cep_T_gpu(p, ep), rtol=0, atol=tol_T * T.max())
    if precision == "mixed":
        _, g64 = _cep_adjoint(p, ep, Tstar, fsils.PREC_FP64)
        assert np.linalg.norm(grad - g64) <= 1e-8 * np.linalg.norm(g64)

    def J(Tx):
        d = Tx - Tstar
        return 0.5 * float(d @ d)

    errs = []
    for k in range(2):
        r = rng.standard_normal(p.nEl)
        r /= np.linalg.norm(r)
        dp = ep * r
        fd = (J(_cep_T_gpu(p, ep + FD_H * dp)) - J(_cep_T_gpu(p, ep - FD_H * dp))) / (2 * FD_H)
        ad = float(grad @ dp)
        errs.append(abs(fd - ad) / abs(ad))
        print(f"CEP adjoint ({precision}, ode {ode}, nFn {nFn}) direction {k}: fd {fd:.12e} "
              f"adjoint {ad:.12e} "
              f"rel {errs[-1]:.2e}")
        if k == 0 and precision == "fp64":
            # and against finite differences of the oracle's own steps
            fdo = (J(_cep_T_oracle(orc, p, ep + FD_H * dp)) -
                   J(_cep_T_oracle(orc, p, ep - FD_H * dp))) / (2 * FD_H)
            print(f"CEP adjoint oracle fd {fdo:.12e}")
            assert abs(fdo - ad) <= 1e-5 * abs(ad), (fdo, ad)
    assert max(errs) <= 1e-5, errs


def test_cep_adjoint_rejects_other_physics(gsls):
    p = problems.heats_cube(3, nsteps=1)
    lhs, mesh, eq = problems.build_equation(p)
    with pytest.raises(Exception, match="CEP"):
        eq.cep_adjoint_forward(1)
