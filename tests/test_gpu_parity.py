"""GPU parity: every kernel path through the C ABI against the oracle on the
same seeded inputs.

Tolerances (FP64 path): SpMV and assembly 1e-12 relative; one linear solve
1e-10 relative L2 on the solution; time steps 1e-10 relative L2 on the
state after N steps.  Mixed path: solution within 1e-8 relative L2 of the
FP64 oracle (the mixed-precision contract).
"""
import ctypes as C

import numpy as np
import pytest

from svfsi_gb300 import _lib, fsils, problems

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, float).ravel(), np.asarray(b, float).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def torch_dev():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    return torch


def _lhs_for(p, nFaces=1):
    g, rp1, cp1 = problems.make_lhs_arrays(p)
    return fsils.FSILS_LHS_CREATE(p.nNo, p.nNo, p.nnz, g, rp1, cp1, nFaces)


@pytest.mark.parametrize("dof", [1, 2, 3, 4])
@pytest.mark.parametrize("mixed", [False, True])
def test_spmv_block_csr(gsls, orc, dof, mixed):
    torch = torch_dev()
    p = problems.heats_cube(6)
    lhs = _lhs_for(p)
    rng = np.random.default_rng(dof)
    Val = rng.standard_normal((p.nnz, dof * dof))
    U = rng.standard_normal((p.nNo, dof))
    ref = orc.OracleSolver(p.nNo, p.rowPtr, p.colPtr, 0).spmv(dof, Val, U)
    vt = torch.tensor(Val, dtype=torch.float32 if mixed else torch.float64, device="cuda")
    ut = torch.tensor(U, dtype=torch.float64, device="cuda")
    yt = torch.zeros_like(ut)
    torch.cuda.synchronize()
    _lib.check(gsls.gsls_spmv_dev(lhs.h, dof, C.c_void_p(vt.data_ptr()),
                                  _lib.PREC_MIXED if mixed else _lib.PREC_FP64,
                                  C.c_void_p(ut.data_ptr()), C.c_void_p(yt.data_ptr())))
    y = yt.cpu().numpy()
    assert rel(y, ref) < (1e-5 if mixed else 1e-14)


def test_dot_norm(gsls, orc):
    torch = torch_dev()
    p = problems.heats_cube(5)
    lhs = _lhs_for(p)
    rng = np.random.default_rng(0)
    u, v = rng.standard_normal((p.nNo, 3)), rng.standard_normal((p.nNo, 3))
    ut = torch.tensor(u, device="cuda")
    vt = torch.tensor(v, device="cuda")
    out = C.c_double()
    _lib.check(gsls.gsls_dot_dev(lhs.h, 3, C.c_void_p(ut.data_ptr()), C.c_void_p(vt.data_ptr()),
                                 C.byref(out)))
    assert abs(out.value - float(np.sum(u * v))) < 1e-12 * np.abs(u * v).sum()
    _lib.check(gsls.gsls_norm_dev(lhs.h, 3, C.c_void_p(ut.data_ptr()), C.byref(out)))
    assert abs(out.value - np.linalg.norm(u)) < 1e-13 * np.linalg.norm(u)


def _assembled_system(p, seed=0):
    import oracle as O
    rng = np.random.default_rng(seed)
    A = 1e-3 * rng.standard_normal((p.nNo, p.tDof))
    Y = 1e-3 * rng.standard_normal((p.nNo, p.tDof))
    D = 1e-2 * rng.standard_normal((p.nNo, p.tDof))
    R, Val = O.assemble(p, A, Y, D)
    return A, Y, D, R, Val


@pytest.mark.parametrize("case", ["heats", "struct"])
def test_assembly_fp64(gsls, orc, case):
    p = problems.heats_cube(6) if case == "heats" else problems.struct_beam(8, 3, 3)
    A, Y, D, R0, V0 = _assembled_system(p)
    lhs = _lhs_for(p)
    mesh = fsils.Mesh(lhs, p.ien, p.x)
    assert mesh.ncolors >= 20
    R, Val = mesh.assemble(p.eq_params(), A, Y, D, p.dof)
    assert rel(R, R0) < 1e-12
    assert rel(Val, V0) < 1e-12


def test_assembly_per_element_parameter(gsls, orc):
    p = problems.struct_beam(4, 2, 2)
    rng = np.random.default_rng(11)
    ep = p.params["C10"] * np.exp(0.2 * rng.standard_normal(p.nEl))
    A, Y, D, _, _ = _assembled_system(p)
    import oracle as O
    R0, V0 = O.assemble(p, A, Y, D, eparam=ep)
    lhs = _lhs_for(p)
    mesh = fsils.Mesh(lhs, p.ien, p.x)
    prm = p.eq_params()
    e = np.ascontiguousarray(ep)
    prm.eparam = e.ctypes.data_as(_lib.c_double_p)
    R, Val = mesh.assemble(prm, A, Y, D, p.dof)
    assert rel(R, R0) < 1e-12 and rel(Val, V0) < 1e-12


@pytest.mark.parametrize("case,lstype", [("heats", "cg"), ("heats", "gmres"),
                                         ("struct", "cg"), ("struct", "gmres")])
def test_fsils_solve_matches_oracle(gsls, orc, case, lstype):
    p = problems.heats_cube(6) if case == "heats" else problems.struct_beam(8, 3, 3)
    _, _, _, R0, V0 = _assembled_system(p, seed=1)
    d = p.dof
    dirn = p.dirichlet[0].nodes
    # product
    lhs = _lhs_for(p, nFaces=1)
    fsils.FSILS_BC_CREATE(lhs, 1, dirn.size, 3, fsils.BC_TYPE_DIR, dirn + 1, np.zeros((dirn.size, 3)))
    t = fsils.LS_TYPE_CG if lstype == "cg" else fsils.LS_TYPE_GMRES
    # Classical Gram-Schmidt with the Pythagorean norm (the reference's
    # GMRES) makes the iteration count sensitive to rounding once
    # h(i+1,i) nears cancellation; at relTol 1e-5 the count is stable.
    relTol = 1e-8 if lstype == "cg" else 1e-5
    kw = dict(relTol=relTol, maxItr=2000) if lstype == "cg" else dict(relTol=relTol, maxItr=10, dimKry=40)
    ls = fsils.FSILS_LS_CREATE(t, **kw)
    R, Val = R0.copy(), V0.copy()
    fsils.FSILS_SOLVE(lhs, ls, d, R, Val, fsils.PRECOND_FSILS)
    # oracle
    s = orc.OracleSolver(p.nNo, p.rowPtr, p.colPtr, 1)
    s.bc_create(1, dirn, 3, 0, np.zeros((dirn.size, 3)))
    ols = orc.ls_create(t, relTol=relTol, mItr=kw["maxItr"], sD=kw.get("dimKry"))
    Ro, Vo = R0.copy(), V0.copy()
    s.solve(ols, d, Ro, Vo, orc.PRECOND_FSILS)
    assert rel(Val, Vo) < 1e-15
    assert ls.RI.suc == ols.RI.suc == 1
    assert abs(ls.RI.iNorm - ols.RI.iNorm) <= 1e-12 * ols.RI.iNorm
    assert abs(ls.RI.itr - ols.RI.itr) <= 1
    assert rel(R, Ro) < (1e-7 if lstype == "cg" else 1e-6)
    # the preconditioned residual reached the requested tolerance
    assert ls.RI.fNorm <= relTol * ls.RI.iNorm * 1.0001


@pytest.mark.parametrize("case", ["heats", "struct"])
def test_gmres_tight_tolerance_converges(gsls, orc, case):
    p = problems.heats_cube(6) if case == "heats" else problems.struct_beam(8, 3, 3)
    _, _, _, R0, V0 = _assembled_system(p, seed=1)
    dirn = p.dirichlet[0].nodes
    lhs = _lhs_for(p, nFaces=1)
    fsils.FSILS_BC_CREATE(lhs, 1, dirn.size, 3, fsils.BC_TYPE_DIR, dirn + 1, np.zeros((dirn.size, 3)))
    ls = fsils.FSILS_LS_CREATE(fsils.LS_TYPE_GMRES, relTol=1e-8, maxItr=10, dimKry=40)
    R, Val = R0.copy(), V0.copy()
    fsils.FSILS_SOLVE(lhs, ls, p.dof, R, Val, fsils.PRECOND_FSILS)
    s = orc.OracleSolver(p.nNo, p.rowPtr, p.colPtr, 1)
    s.bc_create(1, dirn, 3, 0, np.zeros((dirn.size, 3)))
    ols = orc.ls_create(orc.LS_TYPE_CG, relTol=1e-13, mItr=5000)
    Ro, Vo = R0.copy(), V0.copy()
    s.solve(ols, p.dof, Ro, Vo, orc.PRECOND_FSILS)
    assert ls.RI.suc == 1
    assert rel(R, Ro) < 1e-6


def test_heats_c1_ten_steps_fp64(gsls, orc):
    p = problems.heats_cube(20, nsteps=10)
    lhs, mesh, eq = problems.build_equation(p)
    oeq = orc.OracleEquation(p)
    for s in range(p.nsteps):
        gi = eq.step()
        oi = oeq.step()
        assert gi.newton_itr == oi.newton_itr
    A, Y, D = eq.get_state()
    Ao, Yo, Do = oeq.state()
    assert rel(Y, Yo) < 1e-10
    assert rel(A, Ao) < 1e-8


def test_heats_mixed_within_1e8(gsls, orc):
    p = problems.heats_cube(12, nsteps=5)
    p.tol = 1e-12
    p.maxItr = 8
    lhs, mesh, eq = problems.build_equation(p, precision=fsils.PREC_MIXED)
    oeq = orc.OracleEquation(p)
    for s in range(p.nsteps):
        eq.step()
        oeq.step()
    _, Y, _ = eq.get_state()
    _, Yo, _ = oeq.state()
    assert rel(Y, Yo) < 1e-8


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_struct_steps(gsls, orc, precision):
    p = problems.struct_beam(12, 3, 3, nsteps=3)
    prec = fsils.PREC_FP64 if precision == "fp64" else fsils.PREC_MIXED
    lhs, mesh, eq = problems.build_equation(p, precision=prec)
    oeq = orc.OracleEquation(p)
    for s in range(p.nsteps):
        gi = eq.step()
        oeq.step()
        assert gi.last_suc == 1
    A, Y, D = eq.get_state()
    Ao, Yo, Do = oeq.state()
    tol = 1e-9 if precision == "fp64" else 1e-8
    assert rel(D, Do) < tol
    assert rel(Y, Yo) < 10 * tol


def test_assembly_and_solve_deterministic(gsls):
    p = problems.struct_beam(8, 3, 3, nsteps=2)
    outs = []
    for _ in range(2):
        lhs, mesh, eq = problems.build_equation(p)
        for s in range(p.nsteps):
            eq.step()
        outs.append(eq.get_state()[2])
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("lstype", ["cg", "gmres"])
@pytest.mark.parametrize("case", ["heats", "struct"])
def test_solve_dev_mixed_fp32_inner(gsls, orc, case, lstype):
    """FP32 matrix values and FP32 inner Krylov through gsls_solve_dev: the
    solution agrees with the FP64 oracle to the inner tolerance."""
    torch = torch_dev()
    p = problems.heats_cube(6) if case == "heats" else problems.struct_beam(8, 3, 3)
    _, _, _, R0, V0 = _assembled_system(p, seed=2)
    d = p.dof
    dirn = p.dirichlet[0].nodes
    lhs = _lhs_for(p, nFaces=1)
    fsils.FSILS_BC_CREATE(lhs, 1, dirn.size, 3, fsils.BC_TYPE_DIR, dirn + 1, np.zeros((dirn.size, 3)))
    t = fsils.LS_TYPE_CG if lstype == "cg" else fsils.LS_TYPE_GMRES
    kw = dict(relTol=1e-5, maxItr=3000) if lstype == "cg" else dict(relTol=1e-5, maxItr=20, dimKry=50)
    ls = fsils.FSILS_LS_CREATE(t, **kw)
    Rt = torch.tensor(R0, dtype=torch.float64, device="cuda")
    Vt = torch.tensor(V0, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    _lib.check(gsls.gsls_solve_dev(lhs.h, C.byref(ls), d, C.c_void_p(Rt.data_ptr()),
                                   C.c_void_p(Vt.data_ptr()), _lib.PREC_MIXED,
                                   fsils.PRECOND_FSILS, None, None))
    s = orc.OracleSolver(p.nNo, p.rowPtr, p.colPtr, 1)
    s.bc_create(1, dirn, 3, 0, np.zeros((dirn.size, 3)))
    ols = orc.ls_create(orc.LS_TYPE_CG, relTol=1e-12, mItr=5000)
    Ro, Vo = R0.copy(), V0.copy()
    s.solve(ols, d, Ro, Vo, orc.PRECOND_FSILS)
    assert ls.RI.suc == 1
    x = Rt.cpu().numpy()
    # true FP64 residual of the Dirichlet-reduced system (free rows/columns)
    free = np.ones(p.nNo, bool)
    free[dirn] = False
    assert np.all(x[~free] == 0.0)
    Kx = s.spmv(d, V0, x)
    r = (R0 - Kx)[free]
    # FP32 Arnoldi/CG: the true residual sits within ~100x of the requested
    # preconditioned tolerance; the FP64 Newton residual corrects the rest
    assert np.linalg.norm(r) < 1e-3 * np.linalg.norm(R0[free])
    if lstype == "cg":
        assert rel(x, Ro) < 1e-3


@pytest.mark.parametrize("precision,ode,A", [("fp64", 0, -52.0), ("fp64", 1, 52.0),
                                             ("mixed", 0, 52.0)])
def test_cep_steps(gsls, orc, precision, ode, A):
    """Monodomain Aliev-Panfilov slab: reaction step + diffusion solve per
    step, against the oracle; the +52 amplitude fires an activation wave."""
    p = problems.cep_slab(16, 16, 3, nsteps=60, A=A, ode=ode)
    if precision == "mixed":
        p.tol, p.maxItr = 1e-12, 8
    prec = fsils.PREC_FP64 if precision == "fp64" else fsils.PREC_MIXED
    lhs, mesh, eq = problems.build_equation(p, precision=prec)
    oeq = orc.OracleEquation(p)
    for s in range(p.nsteps):
        eq.step()
        oeq.step()
    _, Y, _ = eq.get_state()
    _, Yo, _ = oeq.state()
    X = eq.get_cep_state()
    # the reaction step runs in FP64 on both paths; the mixed path's FP32
    # tangent and inner CG are refined by the FP64 Newton residual
    tol = 1e-10 if precision == "fp64" else 1e-8
    assert rel(Y, Yo) < tol
    assert rel(X[:, 1], oeq.Xion[:, 1]) < (1e-9 if precision == "fp64" else 1e-8)
    if A > 0:
        assert Y.max() > -60.0  # the stimulated corner depolarised well above rest (-80 mV)


def test_gmres_coupled_neumann_face_matches_oracle(gsls, orc):
    """GMRES with a coupled Neumann (resistance) face: ADDBCMUL's rank-one
    term after every SpMV, as in GMRESV."""
    p = problems.struct_beam(8, 3, 3)
    _, _, _, R0, V0 = _assembled_system(p, seed=4)
    dirn = p.dirichlet[0].nodes
    from svfsi_gb300 import meshgen
    face = meshgen.nodes_on_plane(p.x, 0, 4.0).astype(np.int32)
    rng = np.random.default_rng(6)
    val = rng.random((face.size, 3)) + 0.5
    res = np.array([0.0, 50.0])
    lhs = _lhs_for(p, nFaces=2)
    fsils.FSILS_BC_CREATE(lhs, 1, dirn.size, 3, fsils.BC_TYPE_DIR, dirn + 1, np.zeros((dirn.size, 3)))
    fsils.FSILS_BC_CREATE(lhs, 2, face.size, 3, fsils.BC_TYPE_NEU, face + 1, val)
    ls = fsils.FSILS_LS_CREATE(fsils.LS_TYPE_GMRES, relTol=1e-5, maxItr=10, dimKry=40)
    R, Val = R0.copy(), V0.copy()
    fsils.FSILS_SOLVE(lhs, ls, 3, R, Val, fsils.PRECOND_FSILS, res=res)
    s = orc.OracleSolver(p.nNo, p.rowPtr, p.colPtr, 2)
    s.bc_create(1, dirn, 3, 0, np.zeros((dirn.size, 3)))
    s.bc_create(2, face, 3, 1, val)
    ols = orc.ls_create(orc.LS_TYPE_GMRES, relTol=1e-5, mItr=10, sD=40)
    Ro, Vo = R0.copy(), V0.copy()
    s.solve(ols, 3, Ro, Vo, orc.PRECOND_FSILS, res=res)
    assert ls.RI.suc == ols.RI.suc == 1
    assert abs(ls.RI.itr - ols.RI.itr) <= 1
    assert rel(R, Ro) < 1e-6
    # without the coupling the answer differs
    R2, V2 = R0.copy(), V0.copy()
    ls2 = fsils.FSILS_LS_CREATE(fsils.LS_TYPE_GMRES, relTol=1e-5, maxItr=10, dimKry=40)
    fsils.FSILS_SOLVE(lhs, ls2, 3, R2, V2, fsils.PRECOND_FSILS, res=np.array([0.0, 0.0]))
    assert rel(R2, Ro) > 1e-4


@pytest.mark.parametrize("case", ["heats", "struct"])
@pytest.mark.parametrize("mixed", [False, True])
def test_bicgstab_matches_oracle(gsls, orc, case, mixed):
    """LS_TYPE_BICGS (BICGSS/BICGSV) through FSILS_SOLVE against the oracle;
    mixed precision runs FP32 vectors and values on the device."""
    torch = pytest.importorskip("torch")
    p = problems.heats_cube(6) if case == "heats" else problems.struct_beam(8, 3, 3)
    _, _, _, R0, V0 = _assembled_system(p, seed=8)
    d = p.dof
    dirn = p.dirichlet[0].nodes
    lhs = _lhs_for(p, nFaces=1)
    fsils.FSILS_BC_CREATE(lhs, 1, dirn.size, 3, fsils.BC_TYPE_DIR, dirn + 1, np.zeros((dirn.size, 3)))
    ls = fsils.FSILS_LS_CREATE(fsils.LS_TYPE_BICGS, relTol=1e-8, maxItr=2000)
    s = orc.OracleSolver(p.nNo, p.rowPtr, p.colPtr, 1)
    s.bc_create(1, dirn, 3, 0, np.zeros((dirn.size, 3)))
    ols = orc.ls_create(orc.LS_TYPE_BICGS, relTol=1e-8, mItr=2000)
    Ro, Vo = R0.copy(), V0.copy()
    s.solve(ols, d, Ro, Vo, orc.PRECOND_FSILS)
    if not mixed:
        R, Val = R0.copy(), V0.copy()
        fsils.FSILS_SOLVE(lhs, ls, d, R, Val, fsils.PRECOND_FSILS)
        assert ls.RI.suc == ols.RI.suc == 1
        assert abs(ls.RI.itr - ols.RI.itr) <= 1
        assert rel(R, Ro) < 1e-6
    else:
        dR = torch.tensor(R0, device="cuda")
        dV = torch.tensor(V0, device="cuda").to(torch.float32)
        _lib.check(gsls.gsls_solve_dev(lhs.h, C.byref(ls), d, C.c_void_p(dR.data_ptr()),
                                       C.c_void_p(dV.data_ptr()), fsils.PREC_MIXED,
                                       fsils.PRECOND_FSILS, None, None))
        torch.cuda.synchronize()
        assert ls.RI.suc == 1
        assert rel(dR.cpu().numpy(), Ro) < 1e-3


def _spd_block_system(p, dof, seed):
    """Symmetric positive definite block matrix on the mesh graph: random
    blocks with K_ji = K_ij^T, the diagonal shifted so that the spectrum
    spans [0.02, 1] x its width (condition number ~50)."""
    rng = np.random.default_rng(seed)
    rp, cp = np.asarray(p.rowPtr), np.asarray(p.colPtr)
    pos = {}
    for i in range(p.nNo):
        for j in range(rp[i], rp[i + 1]):
            pos[(i, int(cp[j]))] = j
    Val = np.zeros((p.nnz, dof, dof))
    for i in range(p.nNo):
        for j in range(rp[i], rp[i + 1]):
            c = int(cp[j])
            if c > i:
                b = rng.standard_normal((dof, dof))
                Val[j] = b
                Val[pos[(c, i)]] = b.T
            elif c == i:
                s = rng.standard_normal((dof, dof))
                Val[j] = 0.5 * (s + s.T)
    n = p.nNo * dof
    Kd = np.zeros((n, n))
    for i in range(p.nNo):
        for j in range(rp[i], rp[i + 1]):
            c = int(cp[j])
            Kd[i * dof:(i + 1) * dof, c * dof:(c + 1) * dof] = Val[j]
    ev = np.linalg.eigvalsh(Kd)
    shift = -ev[0] + 0.02 * (ev[-1] - ev[0])
    for i in range(p.nNo):
        Val[pos[(i, i)]] += shift * np.eye(dof)
    R = rng.standard_normal((p.nNo, dof))
    return R, Val.reshape(p.nnz, dof * dof)


@pytest.mark.parametrize("dof", [1, 2, 3, 4])
@pytest.mark.parametrize("mixed", [False, True])
def test_cg_block_sizes_matches_oracle(gsls, orc, dof, mixed):
    """CG (diagonal preconditioner) on SPD block systems of every block size;
    solves run past the first batch of iterations, so they switch to the
    sliced copy of the matrix."""
    torch = torch_dev()
    p = problems.heats_cube(6)
    R0, V0 = _spd_block_system(p, dof, seed=10 + dof)
    dirn = p.dirichlet[0].nodes
    lhs = _lhs_for(p)
    fsils.FSILS_BC_CREATE(lhs, 1, dirn.size, 3, fsils.BC_TYPE_DIR, dirn + 1, np.zeros((dirn.size, 3)))
    ls = fsils.FSILS_LS_CREATE(fsils.LS_TYPE_CG, relTol=1e-8, maxItr=2000)
    s = orc.OracleSolver(p.nNo, p.rowPtr, p.colPtr, 1)
    s.bc_create(1, dirn, 3, 0, np.zeros((dirn.size, 3)))
    ols = orc.ls_create(orc.LS_TYPE_CG, relTol=1e-8, mItr=2000)
    Ro, Vo = R0.copy(), V0.copy()
    s.solve(ols, dof, Ro, Vo, orc.PRECOND_FSILS)
    assert ols.RI.itr > 16  # past the first batch on the device
    if mixed:
        ls = fsils.FSILS_LS_CREATE(fsils.LS_TYPE_CG, relTol=1e-5, maxItr=2000)
        dR = torch.tensor(R0, dtype=torch.float64, device="cuda")
        dV = torch.tensor(V0, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        _lib.check(gsls.gsls_solve_dev(lhs.h, C.byref(ls), dof, C.c_void_p(dR.data_ptr()),
                                       C.c_void_p(dV.data_ptr()), _lib.PREC_MIXED,
                                       fsils.PRECOND_FSILS, None, None))
        R = dR.cpu().numpy()
        assert ls.RI.itr > 8
        assert rel(R, Ro) < 1e-4
    else:
        R, Val = R0.copy(), V0.copy()
        fsils.FSILS_SOLVE(lhs, ls, dof, R, Val, fsils.PRECOND_FSILS)
        assert rel(Val, Vo) < 1e-15
        assert abs(ls.RI.itr - ols.RI.itr) <= 1
        assert rel(R, Ro) < 1e-7
    assert ls.RI.suc == 1


def test_fp64_fma_rate_probe(gsls):
    """The FP64 FMA probe (the compute roof of the FP64 SpMV) returns a
    positive rate of a plausible size and counts its launches."""
    n0 = gsls.gsls_launch_count()
    r = C.c_double()
    _lib.check(gsls.gsls_fp64_fma_rate(C.byref(r)), "gsls_fp64_fma_rate")
    assert 1e10 < r.value < 1e14
    assert gsls.gsls_launch_count() - n0 == 4


def test_next_equation_on_the_same_lhs_claims_the_freed_faces(gsls):
    """gsls_eq_free releases the LS faces of its Dirichlet sets: a second
    equation on the same lhs and mesh can be set up and steps bit for bit
    like the first."""
    p = problems.struct_beam(8, 2, 2, nsteps=1)
    lhs, mesh, eq = problems.build_equation(p)
    eq.step()
    D1 = eq.get_state()[2]
    eq.free()
    eq2 = fsils.Equation(mesh, p.eq_params(), p.eq_solver())
    for d in p.dirichlet:
        eq2.add_dirichlet(d.nodes, d.g, d.gx, d.mask, d.nV)
    for t in p.traction:
        eq2.add_traction(t.faces, t.h)
    eq2.set_state(*p.initial_state())
    eq2.step()
    assert np.array_equal(eq2.get_state()[2], D1)
    # a second live equation finds no free face
    eq3 = fsils.Equation(mesh, p.eq_params(), p.eq_solver())
    with pytest.raises(_lib.GslsError, match="face"):
        for d in p.dirichlet:
            eq3.add_dirichlet(d.nodes, d.g, d.gx, d.mask, d.nV)
    eq3.free()
    eq2.free()


_LIN_REUSE_CODE = r"""
import hashlib, json, numpy as np
from svfsi_gb300 import _lib, fsils, problems
L = _lib.load(); _lib.check(L.gsls_init(0))
out = {}
for name, prec in (("fp64", fsils.PREC_FP64), ("mixed", fsils.PREC_MIXED)):
    p = problems.cep_slab(16, 16, 3, nsteps=9, A=52.0)
    lhs, mesh, eq = problems.build_equation(p, precision=prec)
    counts = [(s.newton_itr, s.ls_itr_total) for s in (eq.step() for _ in range(3))]
    # an unrelated solve on the same lhs overwrites its preconditioner
    rp, cp = np.asarray(p.rowPtr), np.asarray(p.colPtr)
    V = np.where(cp == np.repeat(np.arange(p.nNo), np.diff(rp)),
                 0.5 * np.repeat(np.diff(rp), np.diff(rp)), -0.5)[:, None].astype(float)
    R = np.random.default_rng(5).standard_normal((p.nNo, 1))
    fsils.FSILS_SOLVE(lhs, fsils.FSILS_LS_CREATE(fsils.LS_TYPE_CG, relTol=1e-6), 1, R, V,
                      fsils.PRECOND_FSILS)
    counts += [(s.newton_itr, s.ls_itr_total) for s in (eq.step() for _ in range(3))]
    # a new per-element diffusivity rebuilds the conduction operator
    eq.set_eparam(np.exp(0.2 * np.random.default_rng(6).standard_normal(p.nEl)) * 0.1)
    counts += [(s.newton_itr, s.ls_itr_total) for s in (eq.step() for _ in range(3))]
    A, Y, D = eq.get_state()
    out[name] = dict(counts=counts, h=hashlib.sha256(np.ascontiguousarray(Y).tobytes()).hexdigest())
print(json.dumps(out))
"""


def test_linear_tangent_reuse_is_bitwise_the_rebuilt_tangent(gsls):
    """HEATS/CEP: the preconditioned tangent kept from the last full solve
    (default) against rebuilding and rescaling it every Newton iteration
    (GSLS_LIN_REUSE=0), in two fresh processes: nine CEP steps in FP64 and
    mixed precision, with an unrelated solve on the same lhs after step 3
    (it overwrites the preconditioner) and a new per-element diffusivity
    after step 6 (it rebuilds the operator).  Same iteration counts, same
    bits."""
    import json
    import os
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    outs = []
    for reuse in ("1", "0"):
        env = dict(os.environ, GSLS_LIN_REUSE=reuse, PYTHONPATH=str(root))
        r = subprocess.run([sys.executable, "-c", _LIN_REUSE_CODE], cwd=root, env=env,
                           capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        outs.append(json.loads(r.stdout.strip().splitlines()[-1]))
    assert outs[0] == outs[1], outs


def test_batched_cg_path_on_small_systems(gsls):
    """Small systems take the persistent CG (one cooperative launch per
    solve); the batched path (CUDA graphs of SpMV/update/direction kernels,
    sliced copy after the first batch) is what the large ones run.  This
    re-runs the small-system CG parity tests with the persistent kernel
    switched off (GSLS_CG_PERSISTENT=0), in a fresh process."""
    import os
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    env = dict(os.environ, GSLS_CG_PERSISTENT="0", PYTHONPATH=str(root))
    sel = ("cg_block_sizes or struct_steps or heats_c1 or heats_mixed or cep_steps or "
           "iteration_limit or zero_diagonal or deterministic")
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-m", "gpu", "-p", "no:cacheprovider",
                        "-k", sel, str(root / "tests" / "test_gpu_parity.py"),
                        str(root / "tests" / "test_gpu_failures.py")],
                       cwd=root, env=env, capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
    assert " passed" in r.stdout
