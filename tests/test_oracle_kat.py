"""Known-answer tests pinning the oracle (CPU only).

The reference ships no tests or golden data and cannot be compiled here, so
the oracle is pinned by mathematics: exact P1 element matrices, the patch
test, material identities and finite differences, Krylov solves against a
dense solve, and the gen-alpha closed forms.
"""
import ctypes as C

import numpy as np
import pytest

from svfsi_gb300 import meshgen, problems


def test_kuhn_cube_counts():
    p = problems.heats_cube(20)
    assert (p.nNo, p.nEl, p.nnz) == (9261, 48000, 128581)
    assert meshgen.tet_jacobians(p.x, p.ien).min() > 0


def test_kuhn_beam_counts_small():
    b = problems.struct_beam(8, 2, 2)
    assert b.nNo == 9 * 3 * 3 and b.nEl == 8 * 2 * 2 * 6
    assert meshgen.tet_jacobians(b.x, b.ien).min() > 0
    # traction face covers the x=4 end exactly (area 1)
    f = b.traction[0].faces
    x = b.x
    area = 0.5 * np.linalg.norm(np.cross(x[f[:, 1]] - x[f[:, 0]], x[f[:, 2]] - x[f[:, 0]]), axis=1)
    assert abs(area.sum() - 1.0) < 1e-12


@pytest.mark.parametrize("n", [(2, 2, 2), (3, 2, 4)])
def test_lhsa_equals_sorted_unique(orc, n):
    x, ien = meshgen.kuhn_box(*n)
    rng = np.random.default_rng(1)
    ien = ien[rng.permutation(ien.shape[0])]
    rp, cp = orc.lhsa(x.shape[0], ien)
    rp2, cp2 = meshgen.csr_from_ien(x.shape[0], ien)
    assert np.array_equal(rp, rp2) and np.array_equal(cp, cp2)


def _unit_tet():
    # x1..x4 with det(x1-x4, x2-x4, x3-x4) = 1
    return np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 0, 0]], dtype=float)


def test_p1_laplacian_and_mass_kat(orc):
    p = problems.heats_cube(1)
    eqp = orc.eqp_from(p)
    xl = orc.f64(_unit_tet().ravel())
    al = np.zeros(4)
    yl = np.zeros(4)
    lR = np.zeros(4)
    lK = np.zeros(16)
    # conductivity only
    eqp.rho = 0.0
    eqp.cond = 2.0
    orc.load().orc_elem_heats(C.byref(eqp), orc.dp(xl), orc.dp(al), orc.dp(yl), orc.dp(lR), orc.dp(lK))
    T1 = eqp.af * eqp.gam * eqp.dt
    G = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [-1, -1, -1]], dtype=float)
    K = (1.0 / 6.0) * 2.0 * G @ G.T
    assert np.allclose(lK.reshape(4, 4) / T1, K, rtol=1e-14, atol=1e-15)
    # mass only: amd * V/20 (1 + delta_ab), amd = am*rho/T1
    eqp.rho = 1.0
    eqp.cond = 0.0
    orc.load().orc_elem_heats(C.byref(eqp), orc.dp(xl), orc.dp(al), orc.dp(yl), orc.dp(lR), orc.dp(lK))
    M = (1.0 / 6.0) / 20.0 * (np.ones((4, 4)) + np.eye(4))
    assert np.allclose(lK.reshape(4, 4), eqp.am * M, rtol=1e-13)


def test_heats_patch_test(orc):
    """Linear T = 1 - x with dT/dt = 0 is in the P1 space: the assembled
    residual vanishes at interior nodes."""
    p = problems.heats_cube(3)
    Y = (1.0 - p.x[:, 0]).reshape(-1, 1)
    A = np.zeros_like(Y)
    R, Val = orc.assemble(p, A, Y)
    interior = np.all((p.x > 1e-12) & (p.x < 1 - 1e-12), axis=1)
    assert np.abs(R[interior]).max() < 1e-14
    # Val is symmetric (the heat tangent is)
    n = p.nNo
    K = np.zeros((n, n))
    for i in range(n):
        for j in range(p.rowPtr[i], p.rowPtr[i + 1]):
            K[i, p.colPtr[j]] = Val[j, 0]
    assert np.allclose(K, K.T, rtol=0, atol=1e-15)


def test_heats_steady_state_kept(orc):
    """Starting from the steady profile, a time step keeps it (Newton + CG)."""
    p = problems.heats_cube(4, nsteps=1)
    eq = orc.OracleEquation(p)
    Y0 = (1.0 - p.x[:, 0]).reshape(-1, 1)
    eq.set_state(np.zeros_like(Y0), Y0, np.zeros_like(Y0))
    eq.step()
    _, Y, _ = eq.state()
    assert np.abs(Y - Y0).max() < 1e-9


def _pk2(orc, C10, K, F):
    S = np.zeros(9)
    Dm = np.zeros(36)
    orc.load().orc_pk2cc_nhk(C10, K, orc.dp(orc.f64(F.ravel())), orc.dp(S), orc.dp(Dm))
    return S.reshape(3, 3), Dm.reshape(6, 6)


def test_nhk_stress_free_reference(orc):
    S, Dm = _pk2(orc, 1.7e5, 3.3e6, np.eye(3))
    assert np.abs(S).max() < 1e-9
    assert np.allclose(Dm, Dm.T)
    # small-strain limit: Dm = lambda 1x1 + 2 mu I (mu = 2 C10, lambda = K - 2mu/3)
    mu, K = 3.4e5, 3.3e6
    lam = K - 2 * mu / 3
    ref = np.zeros((6, 6))
    ref[:3, :3] = lam
    ref[np.arange(3), np.arange(3)] += 2 * mu
    ref[np.arange(3, 6), np.arange(3, 6)] = mu
    assert np.allclose(Dm, ref, rtol=1e-12, atol=1e-6)


def test_nhk_tangent_matches_fd(orc):
    rng = np.random.default_rng(7)
    C10, K = 1.7e5, 3.3e6
    F = np.eye(3) + 0.15 * rng.standard_normal((3, 3))
    _, Dm = _pk2(orc, C10, K, F)
    voigt = [(0, 0), (1, 1), (2, 2), (0, 1), (1, 2), (2, 0)]
    for trial in range(4):
        dF = rng.standard_normal((3, 3))
        h = 1e-6
        Sp, _ = _pk2(orc, C10, K, F + h * dF)
        Sm, _ = _pk2(orc, C10, K, F - h * dF)
        dS = (Sp - Sm) / (2 * h)
        dC = F.T @ dF + dF.T @ F
        dCv = np.array([dC[i, j] * (1 if i == j else 2) for i, j in voigt])
        pred = 0.5 * Dm @ dCv
        got = np.array([dS[i, j] for i, j in voigt])
        assert np.allclose(got, pred, rtol=1e-6, atol=1e-6 * np.abs(pred).max())


def _laplace_1d(n):
    rp = [0]
    cp = []
    vals = []
    for i in range(n):
        for j in (i - 1, i, i + 1):
            if 0 <= j < n:
                cp.append(j)
                vals.append(2.0 if j == i else -1.0)
        rp.append(len(cp))
    return np.array(rp, np.int32), np.array(cp, np.int32), np.array(vals)


@pytest.mark.parametrize("lstype", ["cg", "gmres"])
def test_krylov_1d_laplacian_exact(orc, lstype):
    n = 40
    rp, cp, v = _laplace_1d(n)
    A = np.zeros((n, n))
    for i in range(n):
        A[i, cp[rp[i]:rp[i + 1]]] = v[rp[i]:rp[i + 1]]
    b = np.sin(np.arange(n) + 1.0)
    s = orc.OracleSolver(n, rp, cp, 0)
    if lstype == "cg":
        ls = orc.ls_create(orc.LS_TYPE_CG, relTol=1e-12, mItr=200)
    else:
        ls = orc.ls_create(orc.LS_TYPE_GMRES, relTol=1e-12, mItr=4, sD=60)
    R = b.copy().reshape(n, 1)
    Val = v.copy().reshape(-1, 1)
    s.solve(ls, 1, R, Val, orc.PRECOND_FSILS)
    x = np.linalg.solve(A, b)
    assert ls.RI.suc == 1
    assert np.allclose(R.ravel(), x, rtol=1e-9, atol=1e-9)
    if lstype == "cg":
        assert ls.RI.itr <= n


def test_bicgstab_solves_the_system(orc):
    """BICGSV on an assembled beam tangent against a dense solve."""
    p = problems.struct_beam(4, 2, 2)
    rng = np.random.default_rng(12)
    A = 1e-3 * rng.standard_normal((p.nNo, 3))
    Y = 1e-3 * rng.standard_normal((p.nNo, 3))
    D = 1e-2 * rng.standard_normal((p.nNo, 3))
    R, Val = orc.assemble(p, A, Y, D)
    n = p.nNo
    K = np.zeros((3 * n, 3 * n))
    for i in range(n):
        for j in range(p.rowPtr[i], p.rowPtr[i + 1]):
            c = p.colPtr[j]
            K[3 * i:3 * i + 3, 3 * c:3 * c + 3] = Val[j].reshape(3, 3)
    dirn = p.dirichlet[0].nodes
    free = np.ones(3 * n, bool)
    for a in dirn:
        free[3 * a:3 * a + 3] = False
    x = np.zeros(3 * n)
    x[free] = np.linalg.solve(K[np.ix_(free, free)], R.ravel()[free])
    s = orc.OracleSolver(n, p.rowPtr, p.colPtr, 1)
    s.bc_create(1, dirn, 3, 0, np.zeros((dirn.size, 3)))
    ls = orc.ls_create(orc.LS_TYPE_BICGS, relTol=1e-12, mItr=2000)
    Rs, Vs = R.copy(), Val.copy()
    s.solve(ls, 3, Rs, Vs, orc.PRECOND_FSILS)
    assert ls.RI.suc == 1
    assert np.abs(Rs.ravel() - x).max() < 1e-8 * np.abs(x).max()


@pytest.mark.parametrize("roInf", [0.0, 0.2, 0.5, 1.0])
def test_genalpha_closed_form(orc, roInf):
    out = [C.c_double() for _ in range(4)]
    for so in (0, 1):
        orc.load().orc_genalpha(roInf, so, *[C.byref(o) for o in out])
        am, af, beta, gam = (o.value for o in out)
        assert np.allclose((am, af, beta, gam), problems.genalpha(roInf, bool(so)), rtol=1e-15)
        assert abs(gam - (0.5 + am - af)) < 1e-15
        assert abs(af - 1 / (1 + roInf)) < 1e-15


def test_doassem_equals_dense_assembly(orc):
    p = problems.struct_beam(2, 1, 1)
    rng = np.random.default_rng(3)
    A = 1e-3 * rng.standard_normal((p.nNo, 3))
    Y = 1e-3 * rng.standard_normal((p.nNo, 3))
    D = 1e-2 * rng.standard_normal((p.nNo, 3))
    R, Val = orc.assemble(p, A, Y, D)
    # dense re-assembly from element matrices
    n = p.nNo
    Kd = np.zeros((3 * n, 3 * n))
    Rd = np.zeros(3 * n)
    eqp = orc.eqp_from(p)
    for e in range(p.nEl):
        nd = p.ien[e]
        lR = np.zeros(12)
        lK = np.zeros(144)
        xl = orc.f64(p.x[nd].ravel())
        al, yl, dl = (orc.f64(M[nd].ravel()) for M in (A, Y, D))
        orc.load().orc_elem_struct(C.byref(eqp), 0.0, orc.dp(xl), orc.dp(al), orc.dp(yl),
                                   orc.dp(dl), orc.dp(lR), orc.dp(lK))
        for a in range(4):
            Rd[3 * nd[a]:3 * nd[a] + 3] += lR[3 * a:3 * a + 3]
            for b in range(4):
                Kd[3 * nd[a]:3 * nd[a] + 3, 3 * nd[b]:3 * nd[b] + 3] += \
                    lK[(a * 4 + b) * 9:(a * 4 + b + 1) * 9].reshape(3, 3)
    Kc = np.zeros_like(Kd)
    for i in range(n):
        for j in range(p.rowPtr[i], p.rowPtr[i + 1]):
            c = p.colPtr[j]
            Kc[3 * i:3 * i + 3, 3 * c:3 * c + 3] = Val[j].reshape(3, 3)
    assert np.allclose(Kc, Kd, rtol=1e-13, atol=1e-9)
    assert np.allclose(R.ravel(), Rd, rtol=1e-13, atol=1e-12)


def test_struct_tangent_is_residual_derivative(orc):
    """The assembled tangent is d(residual)/d(A) through the gen-alpha
    chain (dD = af*beta*dt^2/am ...) -- checked by central differences."""
    p = problems.struct_beam(2, 1, 1)
    rng = np.random.default_rng(5)
    A0 = 1e-3 * rng.standard_normal((p.nNo, 3))
    Y0 = 1e-3 * rng.standard_normal((p.nNo, 3))
    D0 = 1e-2 * rng.standard_normal((p.nNo, 3))
    prm = p.params
    am, af, beta, gam, dt = prm["am"], prm["af"], prm["beta"], prm["gam"], prm["dt"]
    R0, Val = orc.assemble(p, A0, Y0, D0)
    n = p.nNo
    Kc = np.zeros((3 * n, 3 * n))
    for i in range(n):
        for j in range(p.rowPtr[i], p.rowPtr[i + 1]):
            c = p.colPtr[j]
            Kc[3 * i:3 * i + 3, 3 * c:3 * c + 3] = Val[j].reshape(3, 3)
    dA = rng.standard_normal((p.nNo, 3))
    h = 1e-4

    def R_at(s):
        # An += s dA -> Ag += am s dA, Yg += af gam dt s dA, Dg += af beta dt^2 s dA
        return orc.assemble(p, A0 + am * s * dA, Y0 + af * gam * dt * s * dA,
                            D0 + af * beta * dt * dt * s * dA)[0]

    fd = (R_at(h) - R_at(-h)).ravel() / (2 * h)
    pred = am * (Kc @ dA.ravel()) / am  # lK is scaled so that K dA = dR/dAn
    assert np.allclose(fd, pred, rtol=1e-5, atol=1e-6 * np.abs(pred).max())


def _ap_run(orc, rk4, dt, T, stim_A=52.0):
    import ctypes as C
    X = (C.c_double * 2)(-80.0, 1e-3)
    n = int(round(T / dt))
    for i in range(n):
        t = i * dt
        orc.load().orc_ap_step(X, C.c_double(t), C.c_double(dt), C.c_double(stim_A if t < 2.0 else 0.0),
                               C.c_double(0.0), rk4)
    return np.array([X[0], X[1]])


def test_aliev_panfilov_rest_and_convergence(orc):
    import ctypes as C
    L = orc.load()
    L.orc_ap_getf.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_double]
    L.orc_ap_step.argtypes = [C.POINTER(C.c_double), C.c_double, C.c_double, C.c_double,
                              C.c_double, C.c_int]
    X = (C.c_double * 2)(0.0, 0.0)
    f = (C.c_double * 2)()
    L.orc_ap_getf(X, f, 0.0)
    assert f[0] == 0.0 and f[1] == 0.0  # the (scaled) rest state is a fixed point
    # FE and RK4 trajectories converge to the same solution as dt -> 0:
    # FE first order (error halves with dt), RK4 high order (>= 16x from
    # dt 0.4 to 0.2, roundoff-level at the CEP step 0.01)
    ref = _ap_run(orc, 1, 0.0025, 20.0)
    e_fe = [np.abs(_ap_run(orc, 0, dt, 20.0) - ref).max() for dt in (0.02, 0.01)]
    assert 1.8 < e_fe[0] / e_fe[1] < 2.2
    e_rk = [np.abs(_ap_run(orc, 1, dt, 20.0) - ref).max() for dt in (0.4, 0.2, 0.01)]
    assert e_rk[0] / e_rk[1] > 16 and e_rk[2] < 1e-10


# ---------------------------------------------------------------- fluid / NS
def _fluid_box(n=3):
    """Small fluid problem on a Kuhn box (interior nodes exist for n >= 3)."""
    x, ien = meshgen.kuhn_box(n, n, n)
    rp, cp = meshgen.csr_from_ien(x.shape[0], ien)
    am, af, beta, gam = problems.genalpha(0.2, False)
    params = dict(am=am, af=af, beta=beta, gam=gam, dt=1e-3, rho=1.06, mu_f=0.04, ctM=1.0,
                  ctC=36.0, fb=(0.0, 0.0, 0.0))
    return problems.Problem(name="fluid_box", x=x, ien=ien, rowPtr=rp, colPtr=cp,
                            phys=problems.PHYS_FLUID, dof=4, tDof=4, params=params)


def _interior(x):
    return np.all((x > 1e-12) & (x < 1 - 1e-12), axis=1)


@pytest.mark.parametrize("flow", ["uniform", "couette"])
def test_fluid_exact_solutions_have_zero_interior_residual(orc, flow):
    """Uniform flow and plane Couette flow (u_x = y) with constant pressure
    are exact steady Navier-Stokes solutions represented by P1: the VMS
    residual vanishes at interior nodes (momentum and continuity)."""
    p = _fluid_box(3)
    Y = np.zeros((p.nNo, 4))
    if flow == "uniform":
        Y[:, :3] = (0.3, -0.2, 0.5)
    else:
        Y[:, 0] = p.x[:, 1]
    Y[:, 3] = 7.0
    R, Val = orc.assemble(p, np.zeros_like(Y), Y)
    inner = _interior(p.x)
    assert inner.sum() > 0
    scale = np.abs(R).max()
    assert scale > 0
    assert np.abs(R[inner]).max() < 1e-12 * max(scale, 1.0)


def test_fluid_element_blocks_match_reference_structure(orc):
    """At rest (u = a = p = 0) FLUID3D_M/C reduce to the Stokes blocks:
    K_uu = wl (mu Nx_b Nx_a^T + mu Nx.Nx I + tauC Nx_a Nx_b^T + rho amd M I),
    K_pp = wl tauM Nx.Nx, K_up = -wl Nx_a Ns_b, K_pu = wl (Ns_a Nx_b + rho amd tauM Nx_a)."""
    p = _fluid_box(1)
    eqp = orc.eqp_from(p)
    xl = orc.f64(_unit_tet().ravel())
    z = np.zeros(16)
    lR = np.zeros(16)
    lK = np.zeros(256)
    orc.load().orc_elem_fluid(C.byref(eqp), orc.dp(xl), orc.dp(z), orc.dp(z), orc.dp(lR), orc.dp(lK))
    assert np.abs(lR).max() == 0.0
    prm = p.params
    rho, mu, dt = prm["rho"], prm["mu_f"], prm["dt"]
    T1 = prm["af"] * prm["gam"] * dt
    amd = prm["am"] / T1
    w = 1.0 / 24.0
    wl = w * T1
    Nx = np.array([[1, 0, 0, -1], [0, 1, 0, -1], [0, 0, 1, -1]], float)  # unit tet: xiX = I
    K = np.eye(3)
    kT = 4.0 / dt ** 2
    kS = 36.0 * 3.0 * (mu / rho) ** 2
    tauM = 1.0 / (rho * np.sqrt(kT + kS))
    tauC = 1.0 / (tauM * 3.0)
    s, t = (5 + 3 * np.sqrt(5)) / 20, (5 - np.sqrt(5)) / 20
    N = np.full((4, 4), t) + np.eye(4) * (s - t)
    M = N.T @ N
    for a in range(4):
        for b in range(4):
            blk = lK[(a * 4 + b) * 16:(a * 4 + b + 1) * 16].reshape(4, 4)
            NN = Nx[:, a] @ Nx[:, b]
            Kuu = 4 * wl * (mu * np.outer(Nx[:, b], Nx[:, a]) + mu * NN * np.eye(3)
                            + tauC * np.outer(Nx[:, a], Nx[:, b])) + wl * rho * amd * M[a, b] * np.eye(3)
            assert np.allclose(blk[:3, :3], Kuu, rtol=1e-12, atol=1e-14)
            assert np.allclose(blk[3, 3], 4 * wl * tauM * NN, rtol=1e-12)
            assert np.allclose(blk[:3, 3], -wl * Nx[:, a] * 1.0, rtol=1e-12)
            assert np.allclose(blk[3, :3], wl * (Nx[:, b] + 4 * rho * amd * tauM * 0.25 * Nx[:, a]),
                               rtol=1e-12)


def test_ge_matches_dense_solve(orc):
    rng = np.random.default_rng(11)
    for n in (1, 2, 5, 12):
        Q = rng.standard_normal((n, n))
        A = Q @ Q.T + n * np.eye(n)
        nV = 20
        Af = np.zeros((nV, nV))
        Af[:n, :n] = A
        Acol = np.asfortranarray(Af).ravel(order="F").copy()
        b = rng.standard_normal(nV)
        x = b.copy()
        ok = orc.load().orc_ge(nV, n, orc.dp(Acol), orc.dp(x))
        assert ok == 1
        assert np.allclose(x[:n], np.linalg.solve(A, b[:n]), rtol=1e-10)


def test_ns_solver_with_tight_tolerances_solves_the_system(orc):
    """RCS + NSSOLVER with tight inner/outer tolerances returns the solution
    of the Dirichlet-masked block system (checked by a dense solve); the
    x = 1 face is left traction-free so that the pressure is determined."""
    p = _fluid_box(3)
    rng = np.random.default_rng(4)
    Y = np.zeros((p.nNo, 4))
    Y[:, :3] = 0.5 * rng.standard_normal((p.nNo, 3))
    Y[:, 3] = rng.standard_normal(p.nNo)
    A = rng.standard_normal((p.nNo, 4))
    R, Val = orc.assemble(p, A, Y)
    walls = np.nonzero(~_interior(p.x) & (p.x[:, 0] < 1 - 1e-12))[0].astype(np.int32)
    n = p.nNo
    Kd = np.zeros((4 * n, 4 * n))
    for i in range(n):
        for j in range(p.rowPtr[i], p.rowPtr[i + 1]):
            c = p.colPtr[j]
            Kd[4 * i:4 * i + 4, 4 * c:4 * c + 4] = Val[j].reshape(4, 4)
    mask = np.ones(4 * n)
    for a in walls:
        mask[4 * a:4 * a + 3] = 0.0
    Km = Kd * mask[:, None] * mask[None, :]
    Km[mask == 0, mask == 0] = 1.0
    x = np.linalg.solve(Km, R.ravel() * mask)
    s = orc.OracleSolver(n, p.rowPtr, p.colPtr, 1)
    s.bc_create(1, walls, 3, 0, np.zeros((walls.size, 3)))
    # the outer residual is iNorm^2 - xB.B (NSSOLVER.f:167), so relative
    # tolerances below ~1e-8 cannot be met; the inner solves are tight
    ls = orc.ls_create(orc.LS_TYPE_NS, relTol=1e-6, absTol=1e-30, mItr=10, sD=200)
    ls.GM.relTol = ls.CG.relTol = 1e-13
    ls.GM.absTol = ls.CG.absTol = 1e-30
    ls.CG.mItr = 2000
    Rs, Vs = R.copy(), Val.copy()
    s.solve(ls, 4, Rs, Vs, orc.PRECOND_RCS)
    assert ls.RI.suc == 1
    # CGRAD_SCHUR takes S = L - Gt G (K^-1 ~ I after scaling), so the outer
    # least-squares loop converges linearly; relTol 1e-6 at cond ~1e8
    assert np.abs(Rs.ravel() - x).max() < 1e-4 * np.abs(x).max()


def test_coupled_neumann_face_adds_rank_one_term(orc):
    """GMRES with a coupled Neumann face (ADDBCMUL) solves (K + res v v^T) x = b
    on the free rows, v the face's val vector (checked by a dense solve)."""
    p = problems.heats_cube(4)
    rng = np.random.default_rng(9)
    A = rng.standard_normal((p.nNo, 1))
    Y = rng.standard_normal((p.nNo, 1))
    R, Val = orc.assemble(p, A, Y)
    n = p.nNo
    K = np.zeros((n, n))
    for i in range(n):
        K[i, p.colPtr[p.rowPtr[i]:p.rowPtr[i + 1]]] = Val[p.rowPtr[i]:p.rowPtr[i + 1], 0]
    dirn = p.dirichlet[0].nodes
    face = meshgen.nodes_on_plane(p.x, 1, 1.0)
    face = face[~np.isin(face, dirn)].astype(np.int32)
    v = 0.5 + rng.random(face.size)
    res = 3.0
    s = orc.OracleSolver(n, p.rowPtr, p.colPtr, 2)
    s.bc_create(1, dirn, 3, 0, np.zeros((dirn.size, 3)))
    s.bc_create(2, face, 1, 1, v.reshape(-1, 1))
    ls = orc.ls_create(orc.LS_TYPE_GMRES, relTol=1e-12, mItr=10, sD=120)
    Rs, Vs = R.copy(), Val.copy()
    s.solve(ls, 1, Rs, Vs, orc.PRECOND_FSILS, res=np.array([0.0, res]))
    free = np.ones(n, bool)
    free[dirn] = False
    vv = np.zeros(n)
    vv[face] = v
    Kc = K + res * np.outer(vv, vv)
    x = np.zeros(n)
    x[free] = np.linalg.solve(Kc[np.ix_(free, free)], R[free, 0])
    assert ls.RI.suc == 1
    # GMRES stops on its Givens estimate, which classical Gram-Schmidt lets
    # drift from the true residual at tight tolerances (cond here ~5e4)
    assert np.abs(Rs[:, 0] - x).max() < 1e-4 * np.abs(x).max()
    # the coupled term matters: without it the solution is far away
    x0 = np.zeros(n)
    x0[free] = np.linalg.solve(K[np.ix_(free, free)], R[free, 0])
    assert np.abs(x0 - x).max() > 1e-2 * np.abs(x).max()


def _lelas_K(p, Val):
    n = p.nNo
    K = np.zeros((3 * n, 3 * n))
    for i in range(n):
        for j in range(p.rowPtr[i], p.rowPtr[i + 1]):
            c = p.colPtr[j]
            K[3 * i:3 * i + 3, 3 * c:3 * c + 3] = Val[j].reshape(3, 3)
    return K


def test_lelas_patch_test_and_uniaxial_stress(orc):
    """LELAS3D: an affine displacement (constant strain) at rest leaves no
    residual at interior nodes, and on a boundary face the residual is the
    traction of the Hooke stress sigma = lambda tr(eps) I + 2 mu eps."""
    p = problems.lelas_beam(4, 2, 2)
    E, nu = p.params["elM"], p.params["nu"]
    lam = E * nu / (1 + nu) / (1 - 2 * nu)
    mu = E / (2 * (1 + nu))
    G = np.array([[1e-3, 2e-4, 0.0], [0.0, -3e-4, 5e-4], [1e-4, 0.0, 2e-4]])
    D = p.x @ G.T
    A = np.zeros_like(D)
    R, Val = orc.assemble(p, A, np.zeros_like(D), D)
    lo, hi = p.x.min(0), p.x.max(0)
    interior = np.all((p.x > lo + 1e-12) & (p.x < hi - 1e-12), axis=1)
    scale = np.abs(R).max()
    assert scale > 0
    assert np.abs(R[interior]).max() < 1e-12 * scale
    # total force on the x = 4 face nodes = (sigma . n) * area (n = +x, area 1)
    eps = 0.5 * (G + G.T)
    sig = lam * np.trace(eps) * np.eye(3) + 2 * mu * eps
    right = np.isclose(p.x[:, 0], hi[0])
    assert np.allclose(R[right].sum(0), sig[:, 0] * 1.0, rtol=1e-12, atol=1e-12 * scale)
    # the tangent is symmetric
    K = _lelas_K(p, Val)
    assert np.allclose(K, K.T, rtol=0, atol=1e-12 * np.abs(K).max())


def test_lelas_tangent_is_residual_derivative(orc):
    """The LELAS tangent is dR/dA through the gen-alpha chain; the problem is
    linear, so one difference is exact up to rounding."""
    p = problems.lelas_beam(3, 1, 1, f=(0.5, -1.0, 2.0))
    rng = np.random.default_rng(6)
    A0 = rng.standard_normal((p.nNo, 3))
    D0 = 1e-3 * rng.standard_normal((p.nNo, 3))
    prm = p.params
    am, af, beta, dt = prm["am"], prm["af"], prm["beta"], prm["dt"]
    R0, Val = orc.assemble(p, A0, np.zeros_like(A0), D0)
    dA = rng.standard_normal((p.nNo, 3))
    R1 = orc.assemble(p, A0 + am * dA, np.zeros_like(A0), D0 + af * beta * dt * dt * dA)[0]
    K = _lelas_K(p, Val)
    pred = K @ dA.ravel()
    assert np.allclose((R1 - R0).ravel(), pred, rtol=1e-9, atol=1e-10 * np.abs(pred).max())
    # the body force enters as -rho f per unit volume: at rest and undeformed
    # the residual sums to -rho f V (V = 4)
    Rf = orc.assemble(p, np.zeros_like(A0), np.zeros_like(A0), np.zeros_like(A0))[0]
    assert np.allclose(Rf.sum(0), -4.0 * np.array([0.5, -1.0, 2.0]), rtol=1e-12)


def test_heatf_reduces_to_heats_without_flow(orc):
    """HEATF3D with no velocity, no source and dT/dt = 0 is the heat
    equation with unit density: the same residual and tangent as HEATS3D."""
    pf = problems.heatf_cylinder(h=0.2, nsteps=1)
    rng = np.random.default_rng(3)
    T = rng.standard_normal(pf.nNo)
    Y = np.zeros((pf.nNo, 5))
    Y[:, 4] = T
    Rf, Vf = orc.assemble(pf, np.zeros_like(Y), Y)
    ph = problems.heats_cube(2)
    ph.x, ph.ien, ph.rowPtr, ph.colPtr = pf.x, pf.ien, pf.rowPtr, pf.colPtr
    ph.params = dict(pf.params, rho=1.0)
    Rh, Vh = orc.assemble(ph, np.zeros((pf.nNo, 1)), T.reshape(-1, 1))
    assert np.allclose(Rf, Rh, rtol=1e-13, atol=1e-13 * np.abs(Rh).max())
    assert np.allclose(Vf, Vh, rtol=1e-13, atol=1e-13 * np.abs(Vh).max())


def test_heatf_linear_profile_across_the_flow_is_steady(orc):
    """A linear temperature T = a.x with a orthogonal to a constant velocity
    is a steady solution (u.grad T = 0, no diffusion term at interior nodes):
    the residual vanishes away from the boundary."""
    p = problems.heatf_cylinder(h=0.15, nsteps=1)
    Y = np.zeros((p.nNo, 5))
    Y[:, 2] = 3.0                               # u = (0, 0, 3)
    Y[:, 4] = 0.7 * p.x[:, 0] - 0.2 * p.x[:, 1]  # grad T = (0.7, -0.2, 0)
    R, _ = orc.assemble(p, np.zeros_like(Y), Y)
    r = np.hypot(p.x[:, 0], p.x[:, 1])
    interior = (r < 0.5 - 1e-9) & (p.x[:, 2] > 1e-9) & (p.x[:, 2] < 5.0 - 1e-9)
    assert interior.sum() > 10
    assert np.abs(R[interior]).max() < 1e-12 * np.abs(R).max()


def _cy_mu(g, mi, mo, lam, a, n):
    """Carreau-Yasuda viscosity and d mu / d gamma, written from the model:
    mu = mi + (mo - mi) (1 + (lam g)^a)^((n - 1)/a)."""
    T = 1.0 + (lam * g) ** a
    mu = mi + (mo - mi) * T ** ((n - 1.0) / a)
    dmu = (mo - mi) * (n - 1.0) * T ** ((n - 1.0) / a - 1.0) * lam ** a * g ** (a - 1.0)
    return mu, dmu


def _casson_mu(g, mi, mo, lam):
    """Casson viscosity (sqrt(mi) form of the input) and d mu / d gamma, with
    the shear rate held at the threshold lam below it."""
    g = max(g, lam)
    r = mo / np.sqrt(g)
    return (mi + r) ** 2, 2.0 * r * (r + mi) / g, g


@pytest.mark.parametrize("model", ["cy", "cassons", "cassons_above_threshold"])
def test_fluid_viscosity_models(orc, model):
    """tet4 velocity gradients are element constants, so with a shear-rate
    dependent viscosity (GETVISCOSITY) the element residual equals the
    constant-viscosity residual at mu(gamma_e), and the tangent differs from
    it by 4 wl mu_g esNx_i(a) esNx_j(b) (mu_g = mu'(gamma)/gamma)."""
    p = _fluid_box(1)
    rng = np.random.default_rng(7)
    xl = _unit_tet() + 0.1 * rng.standard_normal((4, 3))
    yl = rng.standard_normal((4, 4))
    al = rng.standard_normal((4, 4))
    G = np.linalg.inv((xl[:3] - xl[3]).T)          # G[a, i] = d xi_a / d x_i
    Nx = np.zeros((3, 4))                          # Nx[i, a] = d N_a / d x_i
    Nx[:, :3] = G.T
    Nx[:, 3] = -G.T.sum(axis=1)
    ux = Nx @ yl[:, :3]                            # ux[i, j] = d u_j / d x_i
    es = ux + ux.T
    gam = np.sqrt(0.5 * np.sum(es * es))
    if model == "cy":
        vp = problems.viscosity_params("cy", mu=0.0035, mu_o=0.16, lam=8.2, a=0.64, n=0.2128)
        mu, dmu = _cy_mu(gam, 0.0035, 0.16, 8.2, 0.64, 0.2128)
        g_used = gam
    else:
        lam = gam * (1.5 if model == "cassons" else 0.5)
        vp = problems.viscosity_params("cassons", mu=0.0536, mu_o=0.4, lam=lam)
        mu, dmu, g_used = _casson_mu(gam, 0.0536, 0.4, lam)
    mu_g = dmu / g_used

    def elem(params):
        eqp = orc.eqp_from(p)
        for k, v in params.items():
            setattr(eqp, k, v)
        lR, lK = np.zeros(16), np.zeros(256)
        orc.load().orc_elem_fluid(C.byref(eqp), orc.dp(orc.f64(xl.ravel())), orc.dp(orc.f64(al.ravel())),
                                  orc.dp(orc.f64(yl.ravel())), orc.dp(lR), orc.dp(lK))
        return lR, lK

    R1, K1 = elem(vp)
    R0, K0 = elem(problems.viscosity_params("constant", mu=mu))
    assert np.allclose(R1, R0, rtol=1e-12, atol=1e-12 * np.abs(R0).max())
    prm = p.params
    wl = abs(np.linalg.det((xl[:3] - xl[3]).T)) / 24.0 * prm["af"] * prm["gam"] * prm["dt"]
    esNx = es.T @ Nx                               # esNx[i, a] = sum_k es[k, i] Nx[k, a]
    for a in range(4):
        for b in range(4):
            d = (K1 - K0)[(a * 4 + b) * 16:(a * 4 + b + 1) * 16].reshape(4, 4)
            ref = 4 * wl * mu_g * np.outer(esNx[:, a], esNx[:, b])
            assert np.allclose(d[:3, :3], ref, rtol=1e-9, atol=1e-12 * np.abs(K0).max())
            assert np.abs(d[3, :]).max() <= 1e-12 * np.abs(K0).max()
            assert np.abs(d[:3, 3]).max() <= 1e-12 * np.abs(K0).max()


def test_viscosity_params_follow_the_input_rules():
    assert problems.viscosity_params("newtonian", mu=0.04) == {"viscType": 0, "mu_f": 0.04}
    assert problems.viscosity_params("cass", mu=1.0, mu_o=2.0)["vlam"] == 0.5
    with pytest.raises(ValueError):
        problems.viscosity_params("cy", mu=0.2, mu_o=0.1, lam=1, a=1, n=0.5)
    with pytest.raises(ValueError):
        problems.viscosity_params("power-law")


def test_bheatf_uniform_state_kat(orc):
    """BHEATF on one face of the unit tet with uniform velocity and
    temperature: every node gets area/3 (h - min(u.n, 0) T) with h = -g, the
    outward normal points away from the fourth node, and the tangent is
    -wl udn M_face (row sums area/3 af gam dt (-udn))."""
    x = _unit_tet()
    ien = np.array([[0, 1, 2, 3]], np.int32)
    rp, cp = meshgen.csr_from_ien(4, ien)
    p = problems.heatf_cylinder(h=0.5, nsteps=1)  # parameters only
    eqp = orc.eqp_from(p)
    # face (x1, x2, x4) = (1,0,0), (0,1,0), (0,0,0) lies in z = 0; its outward
    # normal is -z, away from x3 = (0,0,1)
    face = np.array([[0, 1, 3]], np.int32)
    T, g = 2.0, 0.3
    for uz, udn in ((1.0, -1.0), (-1.0, 0.0)):    # u.n = -uz
        Y = np.zeros((4, 5))
        Y[:, 2] = uz
        Y[:, 4] = T
        R = np.zeros(4)
        Val = np.zeros(cp.size)
        orc.load().orc_bheatf(C.byref(eqp), 1, orc.ip(orc.i32(face.ravel())), C.c_double(g), 1,
                              orc.ip(orc.i32(ien.ravel())), orc.dp(orc.f64(x.ravel())),
                              orc.dp(orc.f64(Y.ravel())), orc.ip(orc.i32(rp)), orc.ip(orc.i32(cp)),
                              orc.dp(R), orc.dp(Val))
        area = 0.5
        exp = area / 3.0 * (-g - udn * T)
        assert np.allclose(R[[0, 1, 3]], exp, rtol=1e-14, atol=1e-15)
        assert R[2] == 0.0
        T1 = eqp.af * eqp.gam * eqp.dt
        rows = np.zeros(4)
        for i in range(4):
            rows[i] = Val[rp[i]:rp[i + 1]].sum()
        assert np.allclose(rows[[0, 1, 3]], area / 3.0 * T1 * (-udn), rtol=1e-14, atol=1e-16)


def _one_tet_cep(nFn, Dani, fib):
    import dataclasses
    base = problems.cep_slab(2, 2, 1, nsteps=1)
    x = np.array([[0.1, 0.0, 0.0], [1.3, 0.2, 0.1], [0.2, 0.9, 0.3], [0.3, 0.2, 1.1]])
    ien = np.array([[0, 1, 2, 3]], dtype=np.int32)
    rp, cp = meshgen.csr_from_ien(4, ien)
    params = dict(base.params)
    if nFn:
        params["Dani"] = tuple(Dani[:nFn])
    return dataclasses.replace(base, x=x, ien=ien, rowPtr=rp, colPtr=cp, params=params,
                               fibers=fib, stim=np.zeros(4, np.int32))


@pytest.mark.parametrize("nFn", [1, 2])
def test_cep_fibre_diffusion_kat(orc, nFn):
    """CEP3D's anisotropic part (F/CEP.f:221-266): against the isotropic
    element, the tangent gains T1 V sum_i Dani_i (f_i.grad N_a)(f_i.grad N_b)
    and the residual V sum_i Dani_i (f_i.grad N_a)(f_i.grad V), with V the
    tet's volume and grad N from the inverse Jacobian (numpy)."""
    rng = np.random.default_rng(11)
    f = rng.standard_normal((nFn, 3))
    f /= np.linalg.norm(f, axis=1, keepdims=True)
    Dani = (0.4, 0.05, 0.02)
    p1 = _one_tet_cep(nFn, Dani, f.reshape(1, -1))
    p0 = _one_tet_cep(0, Dani, None)
    A = rng.standard_normal((4, 1))
    Y = rng.standard_normal((4, 1))
    R1, V1 = orc.assemble(p1, A, Y)
    R0, V0 = orc.assemble(p0, A, Y)
    x = p1.x
    J = np.stack([x[k] - x[3] for k in range(3)], axis=1)  # dx/dxi
    G = np.linalg.inv(J).T @ np.array([[1, 0, 0, -1], [0, 1, 0, -1], [0, 0, 1, -1]], float)
    vol = np.linalg.det(J) / 6.0
    fG = f @ G                            # (nFn, 4): f_i . grad N_a
    d = np.array(Dani[:nFn])
    K = vol * (fG.T * d) @ fG
    T1 = p1.params["af"] * p1.params["gam"] * p1.params["dt"]
    gradV = G @ Y[:, 0]
    dR = vol * (fG.T * d) @ (f @ gradV)
    # the single element's CSR rows hold columns 0..3 in order
    assert np.array_equal(p1.colPtr, np.tile(np.arange(4), 4))
    assert np.allclose((V1 - V0)[:, 0].reshape(4, 4), T1 * K, rtol=1e-12, atol=1e-15)
    assert np.allclose((R1 - R0)[:, 0], dR, rtol=1e-12, atol=1e-14)
    assert np.abs(K).max() > 1e-2


def test_precond_diag_kat(orc):
    """PRECONDDIAG (L/PRECOND.f:50-145) against numpy on a 3-dof block CSR:
    W = 1/sqrt|diag| per node and component, W = 1 where the diagonal is
    zero, then Val <- W Val W blockwise and R <- W R.  (The Dirichlet mask
    multiplies W only for the faces FSILS_SOLVE flags as included,
    SOLVE.f:70-84; it is compared through the solves.)"""
    p = problems.struct_beam(4, 2, 2, nsteps=1)
    rng = np.random.default_rng(21)
    d = 3
    Val = rng.standard_normal((p.nnz, d * d))
    rows = np.repeat(np.arange(p.nNo), np.diff(p.rowPtr))
    diag = np.nonzero(p.colPtr == rows)[0]
    for j in diag:
        Val[j, [0, 4, 8]] = rng.uniform(0.5, 3.0, 3) * rng.choice([-1.0, 1.0], 3)
    Val[diag[5], 4] = 0.0  # a zero diagonal entry: W = 1 there
    R = rng.standard_normal((p.nNo, d))
    s = orc.OracleSolver(p.nNo, p.rowPtr, p.colPtr, 1)
    L = orc.load()
    L.orc_precond_diag.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double),
                                   C.POINTER(C.c_double), C.POINTER(C.c_double)]
    Vo, Ro, W = Val.copy(), R.copy(), np.zeros((p.nNo, d))
    L.orc_precond_diag(C.c_void_p(s.h), d, orc.dp(Vo), orc.dp(Ro), orc.dp(W))
    dg = Val[diag].reshape(p.nNo, d, d)[:, [0, 1, 2], [0, 1, 2]]
    We = 1.0 / np.sqrt(np.abs(np.where(dg == 0.0, 1.0, dg)))
    assert W[5, 1] == 1.0
    assert np.allclose(W, We, rtol=1e-15, atol=0)
    Ve = (We[rows][:, :, None] * Val.reshape(-1, d, d) * We[p.colPtr][:, None, :]).reshape(-1, d * d)
    assert np.allclose(Vo, Ve, rtol=1e-14, atol=1e-300)
    assert np.allclose(Ro, We * R, rtol=1e-15, atol=1e-300)
    # the scaled diagonal is +-1 wherever the original was nonzero
    sd = Vo[diag].reshape(p.nNo, d, d)[:, [0, 1, 2], [0, 1, 2]]
    nz = dg != 0.0
    assert np.allclose(np.abs(sd[nz]), 1.0, rtol=1e-14)


def test_precond_rcs_kat(orc):
    """PRECONDRCS (L/PRECOND.f:150-368, no Dirichlet face flagged) against a
    dense numpy restatement: passes of row and column scaling by
    1/sqrt(max |a|) over every scalar row and column, the stop test
    max|1 - max| < 2 over rows and columns taken before each pass's scaling,
    at most 10 passes; W1, W2, Val <- W1 Val W2 and R <- W1 R."""
    p = problems.struct_beam(4, 2, 2, nsteps=1)
    rng = np.random.default_rng(22)
    d = 3
    Val = rng.standard_normal((p.nnz, d * d)) * np.exp(3.0 * rng.standard_normal((p.nnz, 1)))
    R = rng.standard_normal((p.nNo, d))
    rows = np.repeat(np.arange(p.nNo), np.diff(p.rowPtr))
    n = p.nNo * d
    Ad = np.zeros((n, n))
    for j in range(p.nnz):
        Ad[rows[j] * d:(rows[j] + 1) * d, p.colPtr[j] * d:(p.colPtr[j] + 1) * d] = Val[j].reshape(d, d)
    pattern = Ad != 0.0
    W1, W2 = np.ones(n), np.ones(n)
    for it in range(1, 11):
        wr, wc = np.abs(Ad).max(axis=1), np.abs(Ad).max(axis=0)
        stop = it >= 10 or (np.abs(1 - wr).max() < 2.0 and np.abs(1 - wc).max() < 2.0)
        wr, wc = 1 / np.sqrt(wr), 1 / np.sqrt(wc)
        Ad = wr[:, None] * Ad * wc[None, :]
        W1 *= wr
        W2 *= wc
        if stop:
            break
    s = orc.OracleSolver(p.nNo, p.rowPtr, p.colPtr, 1)
    L = orc.load()
    L.orc_precond_rcs.argtypes = [C.c_void_p, C.c_int] + [C.POINTER(C.c_double)] * 4
    Vo, Ro = Val.copy(), R.copy()
    w1, w2 = np.zeros((p.nNo, d)), np.zeros((p.nNo, d))
    L.orc_precond_rcs(C.c_void_p(s.h), d, orc.dp(Vo), orc.dp(Ro), orc.dp(w1), orc.dp(w2))
    assert it > 1  # the matrix needed more than one pass
    assert np.allclose(w1.ravel(), W1, rtol=1e-13) and np.allclose(w2.ravel(), W2, rtol=1e-13)
    got = np.zeros((n, n))
    for j in range(p.nnz):
        got[rows[j] * d:(rows[j] + 1) * d, p.colPtr[j] * d:(p.colPtr[j] + 1) * d] = Vo[j].reshape(d, d)
    assert np.allclose(got[pattern], Ad[pattern], rtol=1e-12)
    assert np.allclose(Ro.ravel(), W1 * R.ravel(), rtol=1e-13)


def test_isotropic_cep_is_heats(orc):
    """Without fibres CEP3D (F/CEP.f:136-266) is HEATS3D (F/HEATS.f:116-159)
    with unit density, no source and conductivity Diso: the oracle's two
    assemblies agree on a slab (and so CEP inherits the P1 and patch-test
    pinning of HEATS)."""
    import dataclasses
    pc = problems.cep_slab(5, 4, 2, nsteps=1, Diso=0.37)
    ph = problems.heats_cube(2, nsteps=1)
    ph = dataclasses.replace(ph, x=pc.x, ien=pc.ien, rowPtr=pc.rowPtr, colPtr=pc.colPtr,
                             params=dict(pc.params, rho=1.0, cond=0.37, src=0.0))
    rng = np.random.default_rng(23)
    A, Y = rng.standard_normal((pc.nNo, 1)), rng.standard_normal((pc.nNo, 1))
    Rc, Vc = orc.assemble(pc, A, Y)
    Rh, Vh = orc.assemble(ph, A, Y)
    assert np.allclose(Rc, Rh, rtol=1e-13, atol=1e-13 * np.abs(Rh).max())
    assert np.allclose(Vc, Vh, rtol=1e-13, atol=1e-13 * np.abs(Vh).max())


def test_parabolic_inflow_profile():
    """BCINI's parabolic profile (F/BAFINI.f:362-403) on the cylinder's
    circular inlet: zero on the perimeter, 1 - r^2/R^2 inside (the centre is
    the area-weighted centroid, 0 here by symmetry, and each node is scaled
    by the perimeter node along its direction: exact for nodes on a ray
    through a perimeter node, within the perimeter's angular spacing
    otherwise)."""
    R, h = 0.5, 0.1
    x, ien, info = meshgen.cylinder(R, 5.0, h)
    inlet, wall = info["inlet"], info["wall"]
    perim = np.intersect1d(inlet, wall)
    gx = meshgen.parabolic_profile(x, info["inlet_faces"], inlet, perim)
    r2 = (x[inlet, 0] ** 2 + x[inlet, 1] ** 2) / R ** 2
    on_rim = np.isin(inlet, perim)
    assert np.allclose(gx[on_rim], 0.0, atol=1e-12)
    assert np.all(gx >= -1e-12) and np.all(gx <= 1.0 + 1e-12)
    # the perimeter polygon's vertices are spaced ~h apart on the circle:
    # the scaling radius is R cos(dphi/2) at worst
    dphi = 2.0 * np.pi / perim.size
    assert np.max(np.abs(gx - (1.0 - r2))) <= 1.0 - np.cos(dphi) + 1e-12
    assert gx.max() > 0.95


def test_slab_fibre_field():
    """The synthetic fibre field: unit directions, family 1 at -60 degrees
    at the bottom of the slab and +60 at the top (in the x-y plane), family
    2 orthogonal to it in the plane, family 3 along z; element order."""
    x, ien = meshgen.kuhn_box(4, 4, 4, 10.0, 10.0, 2.0)
    f = problems.slab_fibers(x, ien, 3)
    assert f.shape == (ien.shape[0], 9)
    fam = f.reshape(-1, 3, 3)
    assert np.allclose(np.linalg.norm(fam, axis=2), 1.0, atol=1e-15)
    assert np.allclose(np.einsum("ei,ei->e", fam[:, 0], fam[:, 1]), 0.0, atol=1e-15)
    assert np.allclose(fam[:, 2], [0.0, 0.0, 1.0])
    zc = x[ien, 2].mean(axis=1)
    ang = np.rad2deg(np.arctan2(fam[:, 0, 1], fam[:, 0, 0]))
    assert np.allclose(ang, -60.0 + 120.0 * zc / 2.0, atol=1e-12)
    assert np.allclose(problems.slab_fibers(x, ien, 1), f[:, :3])


def test_oracle_ctypes_mirrors_match_its_header(orc, tmp_path):
    """The oracle's ctypes structures have the size and field offsets that a
    C compiler gives oracle/orc.h (gcc probe)."""
    import shutil
    import subprocess
    from pathlib import Path
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    mirrors = {"SubLs": "orc_subls", "Ls": "orc_ls", "EqP": "orc_eqp", "DirBC": "orc_dirbc",
               "TracBC": "orc_tracbc", "CepP": "orc_cep", "NeuBC": "orc_neubc", "Eq": "orc_eq",
               "StepInfo": "orc_stepinfo"}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "orc.h"', "int main(void) {"]
    expect = []
    for py, c in mirrors.items():
        cls = getattr(orc, py)
        lines.append(f'  printf("%zu\\n", sizeof({c}));')
        expect.append((py, "sizeof", C.sizeof(cls)))
        for f, _ in cls._fields_:
            lines.append(f'  printf("%zu\\n", offsetof({c}, {f}));')
            expect.append((py, f, getattr(cls, f).offset))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = Path(__file__).resolve().parents[1] / "oracle"
    subprocess.run(["gcc", "-std=c99", "-I", str(inc), str(src), "-o", str(exe)], check=True)
    got = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert len(got) == len(expect)
    for (py, f, off), g in zip(expect, got):
        assert off == int(g), (py, f, off, g)


@pytest.mark.parametrize("case", ["struct", "fluid"])
def test_coloured_oracle_step_matches_serial(orc, case):
    """The timed CPU baseline assembles colour by colour with OpenMP: the
    colouring is conflict-free (no two elements of a colour share a node) and
    the coloured steps equal the serial element loop to rounding, with the
    same Newton and Krylov counts."""
    if case == "struct":
        p = problems.struct_beam(12, 3, 3, nsteps=2)
    else:
        p = problems.fluid_cylinder(h=0.12, nsteps=1)
    nc, off, order = orc.color_elements(p.nNo, p.ien)
    assert off[0] == 0 and off[-1] == p.nEl
    assert np.array_equal(np.sort(order), np.arange(p.nEl))
    for c in range(nc):
        nodes = p.ien[order[off[c]:off[c + 1]]].ravel()
        assert np.unique(nodes).size == nodes.size
    orc.set_threads(4)
    a, b = orc.OracleEquation(p), orc.OracleEquation(p, colored=True)
    for eq in (a, b):
        eq.set_state(*p.initial_state())
    for _ in range(p.nsteps):
        ia, ib = a.step(), b.step()
        assert (ia.newton_itr, ia.ls_itr_total) == (ib.newton_itr, ib.ls_itr_total)
    k = 2 if case == "struct" else 1
    fa, fb = a.state()[k], b.state()[k]
    assert np.linalg.norm(fa - fb) <= 1e-12 * np.linalg.norm(fa)
    orc.set_threads(1)


def test_bfluid_uniform_state_kat(orc):
    """BFLUID on one face of the unit tet with a uniform velocity: every face
    node gets -area/3 (h + udn u.n) n with h = -g and udn = bstab rho
    min(u.n, 0) (backflow only); the velocity diagonal of the tangent has row
    sums -area/3 af gam dt udn, the pressure row and column stay zero."""
    x = _unit_tet()
    ien = np.array([[0, 1, 2, 3]], np.int32)
    rp, cp = meshgen.csr_from_ien(4, ien)
    p = problems.fluid_cylinder(h=0.5, nsteps=1)   # parameters only
    eqp = orc.eqp_from(p)
    assert eqp.bstab == 0.2
    face = np.array([[0, 1, 3]], np.int32)          # z = 0, outward normal -z
    g = 0.7
    for uz in (1.0, -2.0):                          # u.n = -uz: backflow for uz > 0
        Y = np.zeros((4, 4))
        Y[:, 2] = uz
        R = np.zeros((4, 4))
        Val = np.zeros((cp.size, 16))
        orc.load().orc_bfluid(C.byref(eqp), 1, orc.ip(orc.i32(face.ravel())), C.c_double(g), 1,
                              orc.ip(orc.i32(ien.ravel())), orc.dp(orc.f64(x.ravel())),
                              orc.dp(orc.f64(Y.ravel())), orc.ip(orc.i32(rp)), orc.ip(orc.i32(cp)),
                              orc.dp(R), orc.dp(Val))
        area, un = 0.5, -uz
        udn = eqp.bstab * eqp.rho * min(un, 0.0)
        # hc = h n + udn u = (h + udn * (u.n)) n, with n = -e_z and u = -un n
        exp_z = -area / 3.0 * (-g + udn * un) * (-1.0)
        assert np.allclose(R[[0, 1, 3], 2], exp_z, rtol=1e-14, atol=1e-15)
        assert np.abs(R[[0, 1, 3]][:, [0, 1, 3]]).max() <= 1e-15
        assert np.all(R[2] == 0.0)
        T1 = eqp.af * eqp.gam * eqp.dt
        for i in range(4):
            rows = Val[rp[i]:rp[i + 1]].sum(axis=0).reshape(4, 4)
            want = 0.0 if i == 2 else -area / 3.0 * T1 * udn
            assert np.allclose(np.diag(rows)[:3], want, rtol=1e-14, atol=1e-16)
            off = rows.copy()
            np.fill_diagonal(off, 0.0)
            assert np.all(off == 0.0) and rows[3, 3] == 0.0


def _ustruct_elem(orc, eqp, xl, al, yl, dl):
    lR, lK, lKd = np.zeros(16), np.zeros(256), np.zeros(192)
    orc.load().orc_elem_ustruct(C.byref(eqp), orc.dp(orc.f64(xl.ravel())),
                                orc.dp(orc.f64(al.ravel())), orc.dp(orc.f64(yl.ravel())),
                                orc.dp(orc.f64(dl.ravel())), orc.dp(lR), orc.dp(lK), orc.dp(lKd))
    return lR.reshape(4, 4), lK.reshape(4, 4, 4, 4), lKd.reshape(4, 4, 4, 3)


@pytest.mark.parametrize("volType", [0, 1, 2])
def test_ustruct_element_rest_and_momentum_tangent(orc, volType):
    """USTRUCT element (USTRUCT3D_M/_C): zero residual at rest, and the
    momentum rows of the tangents are the residual's derivatives (central
    differences): lKd = af' dR/dD and lK = am dR/dA + af' dR/dY + (af'/am)
    lKd, af' = af gam dt (the Newton increment moves A by 1, Y by af' and D
    by af'^2/am).  The continuity rows also carry tau_M(J) and tau_C(J)
    undifferentiated, as in the reference, so they are left out."""
    p = problems.ustruct_beam(2, 1, 1, nu=0.4, volType=volType, ctC=0.0, visc=0.0)
    eqp = orc.eqp_from(p)
    xl = _unit_tet() * np.array([1.1, 0.9, 1.2])
    z = np.zeros((4, 4))
    lR, _, _ = _ustruct_elem(orc, eqp, xl, z, z, z)
    assert np.abs(lR).max() <= 1e-15 * eqp.C10     # S(I) = 0 up to rounding
    rng = np.random.default_rng(5)
    st = [1e2 * rng.standard_normal((4, 4)), 1e-1 * rng.standard_normal((4, 4)),
          1e-2 * rng.standard_normal((4, 4))]
    st[1][:, 3] = 1e3 * rng.standard_normal(4)
    st[2][:, 3] = 0.0
    lR, lK, lKd = _ustruct_elem(orc, eqp, xl, *st)
    afp = eqp.af * eqp.gam * eqp.dt
    am = eqp.am

    def d(which, b, c, h):
        e = np.zeros((4, 4))
        e[b, c] = h
        P = [x + e if k == which else x for k, x in enumerate(st)]
        M = [x - e if k == which else x for k, x in enumerate(st)]
        return (_ustruct_elem(orc, eqp, xl, *P)[0] - _ustruct_elem(orc, eqp, xl, *M)[0]) / (2 * h)

    sK = np.abs(lK[:, :, :3]).max()
    for b in range(4):
        for c in range(4):
            h = 1e-3 if c == 3 else 1e-6
            if c < 3:
                kd = afp * d(2, b, c, 1e-7)
                assert np.abs(kd[:, :3] - lKd[:, b, :3, c]).max() <= 1e-6 * np.abs(lKd).max()
            mass = am * d(0, b, c, 1e-3) + afp * d(1, b, c, h)
            want = lK[:, b, :3, c] - (afp / am * lKd[:, b, :3, c] if c < 3 else 0.0)
            assert np.abs(mass[:, :3] - want).max() <= 1e-6 * sK, (b, c)


def test_ustruct_oracle_steps_converge(orc):
    """Three implicit USTRUCT steps of the oracle converge (Newton to 1e-8)
    for the compressible (ST91) and the incompressible (Kpen = 0) solid,
    and the beam bends the same way and by a similar amount as the STRUCT
    formulation of the same problem."""
    q = problems.struct_beam(12, 3, 3, nsteps=3)
    eq = orc.OracleEquation(q)
    eq.set_state(*q.initial_state())
    for _ in range(3):
        eq.step()
    Ds = eq.state()[2]
    for nu in (0.45, 0.5):
        p = problems.ustruct_beam(12, 3, 3, nsteps=3, nu=nu)
        eq = orc.OracleEquation(p)
        eq.set_state(*p.initial_state())
        for _ in range(3):
            i = eq.step()
            assert i.last_suc == 1 and i.r1_last <= p.tol * 10
        Du = eq.state()[2][:, :3]
        assert np.linalg.norm(Du - Ds) <= 0.2 * np.linalg.norm(Ds)
