"""Synthetic problem definitions (seeded; no external data).

Each builder returns a ``Problem``: mesh, CSR, equation parameters,
boundary conditions and solver settings for one equation, in the reference's
conventions.  The workloads follow the five benchmark configurations:

* ``heats_cube``   -- unsteady heat equation on a Kuhn-split unit cube
                      (20^3 hexes -> 48,000 tets, 9,261 nodes at full size).
* ``struct_beam``  -- neo-Hookean + ST91 elastodynamics of a 4x1x1 beam
                      (176x44x44 hexes -> 2,044,416 tets, 358,425 nodes).
* ``fluid_cylinder`` -- VMS incompressible Navier-Stokes in a cylinder
                      (R 0.5, L 5; ~1.2M tets, ~0.2M nodes at full size).
* ``cep_slab``     -- Aliev-Panfilov monodomain on a 10x10x2 slab.

and, on the same boundary, ``lelas_beam`` -- linear elastodynamics of the
struct beam -- and ``heatf_cylinder`` -- heat carried by a prescribed
Poiseuille flow in the fluid cylinder.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import meshgen
from ._lib import (LS_TYPE_CG, LS_TYPE_GMRES, LS_TYPE_NS, PHYS_CEP, PHYS_FLUID, PHYS_HEATF, PHYS_HEATS,
                   PHYS_LELAS, PHYS_STRUCT, PHYS_USTRUCT, PREC_FP64,
                   PRECOND_FSILS, PRECOND_RCS, EqParams, EqSolver)

SEED = 20261203


def genalpha(roInf: float, second_order: bool):
    """F/INITIALIZE.f:76-139: (am, af, beta, gam)."""
    am = (2.0 - roInf) / (1.0 + roInf) if second_order else 0.5 * (3.0 - roInf) / (1.0 + roInf)
    af = 1.0 / (1.0 + roInf)
    beta = 0.25 * (1.0 + am - af) ** 2
    gam = 0.5 + am - af
    return am, af, beta, gam


@dataclass
class DirBC:
    nodes: np.ndarray   # 0-based
    g: float
    gx: np.ndarray | None = None
    mask: int = 0       # 0 = all components
    nV: np.ndarray | None = None  # (n, 3) unit normals: value g*gx*nV


@dataclass
class TracBC:
    faces: np.ndarray   # (nFel, 3) 0-based
    h: tuple


@dataclass
class NeuBC:
    faces: np.ndarray   # (nFel, 3) 0-based
    g: float            # Neumann value (HEATF: flux g, backflow term added)


@dataclass
class Problem:
    name: str
    x: np.ndarray
    ien: np.ndarray          # (nEl, 4) 0-based
    rowPtr: np.ndarray       # 0-based
    colPtr: np.ndarray       # 0-based
    phys: int
    dof: int
    tDof: int
    params: dict
    dirichlet: list = field(default_factory=list)
    traction: list = field(default_factory=list)
    neumann: list = field(default_factory=list)
    LS_type: int = LS_TYPE_CG
    prec: int = PRECOND_FSILS
    ls_relTol: float = -1.0
    ls_absTol: float = -1.0
    ls_mItr: int = -1
    ls_sD: int = -1
    minItr: int = 1
    maxItr: int = 5
    tol: float = 1e-6
    absTol: float = 1e-15
    nsteps: int = 10
    eparam: np.ndarray | None = None
    fibers: np.ndarray | None = None  # CEP fibre directions, nEl x 3 nFn (params: Dani)
    cep: dict | None = None         # cell model and stimulus (CEP only)
    stim: np.ndarray | None = None  # per-node stimulus flag (CEP only)
    s: int = 0                      # first unknown of this equation in the state
    Y0: np.ndarray | None = None    # initial Y (nNo, tDof), e.g. a prescribed velocity

    @property
    def nNo(self):
        return self.x.shape[0]

    @property
    def nEl(self):
        return self.ien.shape[0]

    @property
    def nnz(self):
        return int(self.colPtr.size)

    def eq_params(self) -> EqParams:
        """gsls_eq_params of the problem; the fibre array its fN points to
        is held by the returned structure."""
        p = EqParams()
        p.phys, p.dof, p.tDof, p.s = self.phys, self.dof, self.tDof, self.s
        for k, v in self.params.items():
            if k in ("fb", "Dani"):
                for i, vi in enumerate(v):
                    getattr(p, k)[i] = vi
            else:
                setattr(p, k, v)
        if self.fibers is not None:
            p._fib = np.ascontiguousarray(self.fibers, dtype=np.float64)
            p.nFn = p._fib.shape[1] // 3
            p.fN = p._fib.ctypes.data_as(C.POINTER(C.c_double))
        return p

    def eq_solver(self, precision=PREC_FP64) -> EqSolver:
        s = EqSolver()
        s.LS_type, s.prec = self.LS_type, self.prec
        s.ls_relTol, s.ls_absTol = self.ls_relTol, self.ls_absTol
        s.ls_mItr, s.ls_sD = self.ls_mItr, self.ls_sD
        s.ls_relTolIn[0] = s.ls_relTolIn[1] = -1.0
        s.ls_mItrIn[0] = s.ls_mItrIn[1] = -1
        s.minItr, s.maxItr, s.tol, s.absTol = self.minItr, self.maxItr, self.tol, self.absTol
        s.precision = precision
        return s

    def initial_state(self):
        z = np.zeros((self.nNo, self.tDof))
        Y = z.copy() if self.Y0 is None else np.array(self.Y0, dtype=float)
        if self.cep:
            Y[:, 0] = self.cep["V0"]  # resting potential of the cell model
        return z.copy(), Y, z.copy()

    def algorithmic_bytes(self, s_A: int, s_v: int):
        """Per-call algorithmic bytes of one CG iteration and one assembly
        (B_cg and B_asm of the design notes)."""
        nnz, nNo, d = self.nnz, self.nNo, self.dof
        B_spmv = nnz * (d * d * s_A + 4) + 8 * nNo + 2 * nNo * d * s_v
        B_cg = nnz * (d * d * s_A + 4) + 8 * nNo + 11 * nNo * d * s_v
        fields = 3 if self.phys in (PHYS_STRUCT, PHYS_LELAS) else 2
        B_asm = 16 * self.nEl + 24 * nNo + fields * nNo * self.tDof * 8 + nnz * d * d * s_A + 8 * nNo * d
        return {"spmv": B_spmv, "cg_iter": B_cg, "assembly": B_asm}


def heats_cube(n: int = 20, nsteps: int = 10) -> Problem:
    """Config: unit cube, n^3 hexes x 6 tets, conductivity 1, source 0,
    density 1, T=1 at x=0 and T=0 at x=1, T0=0, rho_inf 0.5, dt 0.01,
    CG + diagonal preconditioner, LS tolerance 1e-10."""
    x, ien = meshgen.kuhn_box(n, n, n)
    rp, cp = meshgen.csr_from_ien(x.shape[0], ien)
    am, af, beta, gam = genalpha(0.5, second_order=False)
    params = dict(am=am, af=af, beta=beta, gam=gam, dt=0.01, rho=1.0, cond=1.0, src=0.0)
    left = meshgen.nodes_on_plane(x, 0, 0.0)
    right = meshgen.nodes_on_plane(x, 0, 1.0)
    return Problem(name=f"heats_cube_{n}", x=x, ien=ien, rowPtr=rp, colPtr=cp,
                   phys=PHYS_HEATS, dof=1, tDof=1, params=params,
                   dirichlet=[DirBC(left, 1.0), DirBC(right, 0.0)],
                   LS_type=LS_TYPE_CG, prec=PRECOND_FSILS, ls_relTol=1e-10,
                   minItr=1, maxItr=5, tol=1e-6, nsteps=nsteps)


def struct_beam(nx: int = 176, ny: int = 44, nz: int = 44, nsteps: int = 10,
                E: float = 1e6, nu: float = 0.45, traction=(0.0, 0.0, -1e3),
                eparam: np.ndarray | None = None) -> Problem:
    """Config: 4x1x1 beam, nHK + ST91, E=1e6, nu=0.45, rho=1, x=0 clamped,
    constant traction on x=4, dt=1e-3, Newton tolerance 1e-8, CG + diagonal
    preconditioner (the reference's default for struct)."""
    x, ien = meshgen.kuhn_box(nx, ny, nz, 4.0, 1.0, 1.0)
    rp, cp = meshgen.csr_from_ien(x.shape[0], ien)
    am, af, beta, gam = genalpha(0.2, second_order=True)
    mu = E * 0.5 / (1.0 + nu)                    # F/READFILES.f:2662
    kap = E / (1.0 - 2.0 * nu) / 3.0             # F/READFILES.f:2670
    params = dict(am=am, af=af, beta=beta, gam=gam, dt=1e-3, rho=1.0, C10=0.5 * mu, Kpen=kap,
                  visc=0.0, dmp=0.0, fb=(0.0, 0.0, 0.0))
    clamp = meshgen.nodes_on_plane(x, 0, 0.0)
    tface = meshgen.faces_on_plane(x, ien, 0, 4.0)
    return Problem(name=f"struct_beam_{nx}x{ny}x{nz}", x=x, ien=ien, rowPtr=rp, colPtr=cp,
                   phys=PHYS_STRUCT, dof=3, tDof=3, params=params,
                   dirichlet=[DirBC(clamp, 0.0)], traction=[TracBC(tface, tuple(traction))],
                   LS_type=LS_TYPE_CG, prec=PRECOND_FSILS, minItr=1, maxItr=10, tol=1e-8,
                   nsteps=nsteps, eparam=eparam)


def lelas_beam(nx: int = 176, ny: int = 44, nz: int = 44, nsteps: int = 10,
               E: float = 1e6, nu: float = 0.45, traction=(0.0, 0.0, -1e3),
               f=(0.0, 0.0, 0.0)) -> Problem:
    """Linear elasticity (LELAS3D) on the struct beam: E=1e6, nu=0.45,
    rho=1, domain force f, x=0 clamped, constant traction on x=4 (BLELAS),
    dt=1e-3, second-order generalized-alpha with rho_inf 0.2, CG + diagonal
    preconditioner (the reference's default for lElas)."""
    x, ien = meshgen.kuhn_box(nx, ny, nz, 4.0, 1.0, 1.0)
    rp, cp = meshgen.csr_from_ien(x.shape[0], ien)
    am, af, beta, gam = genalpha(0.2, second_order=True)
    params = dict(am=am, af=af, beta=beta, gam=gam, dt=1e-3, rho=1.0, elM=E, nu=nu,
                  fb=tuple(f))
    clamp = meshgen.nodes_on_plane(x, 0, 0.0)
    tface = meshgen.faces_on_plane(x, ien, 0, 4.0)
    return Problem(name=f"lelas_beam_{nx}x{ny}x{nz}", x=x, ien=ien, rowPtr=rp, colPtr=cp,
                   phys=PHYS_LELAS, dof=3, tDof=3, params=params,
                   dirichlet=[DirBC(clamp, 0.0)], traction=[TracBC(tface, tuple(traction))],
                   LS_type=LS_TYPE_CG, prec=PRECOND_FSILS, minItr=1, maxItr=10, tol=1e-8,
                   nsteps=nsteps)


VOL_QUAD, VOL_ST91, VOL_M94 = 0, 1, 2


def ustruct_beam(nx: int = 24, ny: int = 6, nz: int = 6, nsteps: int = 10,
                 E: float = 1e6, nu: float = 0.45, traction=(0.0, 0.0, -1e3),
                 visc: float = 0.0, volType: int = VOL_ST91, ctM: float = 1e-3,
                 ctC: float = 0.0) -> Problem:
    """USTRUCT (velocity-pressure solid, F/USTRUCT.f) on the beam mesh:
    state (v, p) with the displacement in D, neo-Hookean isochoric part
    (C10 = mu/2) and the volumetric penalty volType (kappa = E/3(1-2nu),
    0 for nu = 0.5: incompressible), rho 1, solid viscosity visc, VMS
    stabilisation with the input defaults ctM 1e-3 and ctC 0
    (F/READFILES.f:1099-1106), x = 0 clamped, constant traction on x = 4,
    dt 1e-3, first-order generalized-alpha with rho_inf 0.2 (the reference
    does not take the second-order am for ustruct, F/INITIALIZE.f:101-104),
    GMRES + diagonal preconditioner (its default, F/READFILES.f:628)."""
    x, ien = meshgen.kuhn_box(nx, ny, nz, 4.0, 1.0, 1.0)
    rp, cp = meshgen.csr_from_ien(x.shape[0], ien)
    am, af, beta, gam = genalpha(0.2, second_order=False)
    mu = E * 0.5 / (1.0 + nu)
    kap = 0.0 if abs(nu - 0.5) < 1e-15 else E / (1.0 - 2.0 * nu) / 3.0
    params = dict(am=am, af=af, beta=beta, gam=gam, dt=1e-3, rho=1.0, C10=0.5 * mu, Kpen=kap,
                  visc=visc, fb=(0.0, 0.0, 0.0), elM=E, nu=nu, ctM=ctM, ctC=ctC,
                  volType=volType)
    clamp = meshgen.nodes_on_plane(x, 0, 0.0)
    tface = meshgen.faces_on_plane(x, ien, 0, 4.0)
    return Problem(name=f"ustruct_beam_{nx}x{ny}x{nz}", x=x, ien=ien, rowPtr=rp, colPtr=cp,
                   phys=PHYS_USTRUCT, dof=4, tDof=4, params=params,
                   dirichlet=[DirBC(clamp, 0.0)], traction=[TracBC(tface, tuple(traction))],
                   LS_type=LS_TYPE_GMRES, prec=PRECOND_FSILS, minItr=1, maxItr=10, tol=1e-8,
                   nsteps=nsteps)


def slab_fibers(x: np.ndarray, ien: np.ndarray, nFn: int, depth: float = 2.0,
                angles=(-60.0, 60.0)) -> np.ndarray:
    """Synthetic myocardial fibre field on a slab, per element (nEl x 3 nFn):
    family 1 lies in the x-y plane at an angle turning linearly through the
    thickness (the element centroid's z) from angles[0] to angles[1]
    degrees; family 2, when asked for, is the in-plane direction normal to
    it; family 3 is z."""
    zc = x[ien, 2].mean(axis=1)
    th = np.deg2rad(angles[0] + (angles[1] - angles[0]) * np.clip(zc / depth, 0.0, 1.0))
    fam = [np.stack([np.cos(th), np.sin(th), np.zeros_like(th)], axis=1),
           np.stack([-np.sin(th), np.cos(th), np.zeros_like(th)], axis=1),
           np.tile([0.0, 0.0, 1.0], (th.size, 1))]
    return np.ascontiguousarray(np.concatenate(fam[:nFn], axis=1))


def cep_slab(nx: int = 135, ny: int = 135, nz: int = 27, nsteps: int = 5000,
             A: float = -52.0, ode: int = 0, Diso: float = 0.1, nFn: int = 0,
             Dani=(0.4, 0.05, 0.02)) -> Problem:
    """Config: monodomain electrophysiology (Aliev-Panfilov) on a 10x10x2
    slab (135x135x27 hexes -> 2,952,450 tets at full size), isotropic
    diffusivity 0.1, stimulus amplitude A for 2 ms from t = 0 on the nodes
    of the 1x1x2 corner block x <= 1, y <= 1, dt = 0.01, CG + diagonal
    preconditioner.  The reference applies a stimulus per domain; here the
    corner block is the explicit stimulated node set.  nFn > 0 adds that
    many fibre families (slab_fibers) with anisotropic diffusivities
    Dani[:nFn] (CEP3D's D = Diso I + sum Dani f f^T)."""
    x, ien = meshgen.kuhn_box(nx, ny, nz, 10.0, 10.0, 2.0)
    rp, cp = meshgen.csr_from_ien(x.shape[0], ien)
    am, af, beta, gam = genalpha(0.2, second_order=False)
    params = dict(am=am, af=af, beta=beta, gam=gam, dt=0.01, Diso=Diso)
    fib = None
    if nFn > 0:
        params["Dani"] = tuple(Dani[:nFn])
        fib = slab_fibers(x, ien, nFn)
    stim = ((x[:, 0] <= 1.0 + 1e-12) & (x[:, 1] <= 1.0 + 1e-12)).astype(np.int32)
    cep = dict(ode=ode, dt_ode=0.01, A=A, Ts=0.0, Td=2.0, CL=1e9, V0=-80.0, X20=1e-3)
    return Problem(name=f"cep_slab_{nx}x{ny}x{nz}" + (f"_fib{nFn}" if nFn else ""), x=x,
                   ien=ien, rowPtr=rp, colPtr=cp, phys=PHYS_CEP, dof=1, tDof=1, params=params,
                   LS_type=LS_TYPE_CG, prec=PRECOND_FSILS, minItr=1, maxItr=5, tol=1e-6,
                   nsteps=nsteps, cep=cep, stim=stim, fibers=fib)


VISC_CONST, VISC_CY, VISC_CASSON = 0, 1, 2


def viscosity_params(model: str = "constant", mu: float = 0.04, mu_o: float = 0.0,
                     lam: float = 0.0, a: float = 0.0, n: float = 0.0) -> dict:
    """Equation parameters of a viscosity model as READVISCMODEL reads them
    (F/READFILES.f:2875-2925): "constant" (mu), "carreau-yasuda" (mu = high
    shear-rate limit, mu_o = low shear-rate limit, lam, a, n) or "cassons"
    (mu = asymptotic viscosity parameter, mu_o = yield stress parameter, lam
    = low shear-rate threshold, 0.5 when not given)."""
    m = model.lower()
    if m in ("constant", "const", "newtonian"):
        return dict(viscType=VISC_CONST, mu_f=mu)
    if m in ("carreau-yasuda", "cy"):
        if mu > mu_o:
            raise ValueError("Carreau-Yasuda: the high shear-rate viscosity must not exceed "
                             "the low shear-rate one")
        return dict(viscType=VISC_CY, mu_f=mu, mu_o=mu_o, vlam=lam, va=a, vn=n)
    if m in ("cassons", "cass"):
        return dict(viscType=VISC_CASSON, mu_f=mu, mu_o=mu_o, vlam=lam if lam > 0 else 0.5)
    raise ValueError(f"undefined viscosity model {model!r}")


def fluid_cylinder(h: float = 0.027, nsteps: int = 20, R: float = 0.5, L: float = 5.0,
                   u_max: float = 30.0, rho: float = 1.06, mu: float = 0.04,
                   dt: float = 1e-3, viscosity: dict | None = None) -> Problem:
    """Config: cylinder R=0.5, L=5 (seeded Delaunay cross-section), rho 1.06,
    mu 0.04, parabolic inlet with peak u_max at z=0 (value -u_max along the
    outward normal -z, profile of BCINI), no-slip wall, outlet z = L a
    Neumann face of value 0 (p = 0; BFLUID adds its backflow stabilisation,
    coefficient 0.2, where u.n < 0), dt 1e-3, NS solver with RCS preconditioning and
    Krylov dimension 100 (outer tolerance 1e-2, inner GMRES 1e-2 and Schur CG
    0.2 as LS_CREATE sets them), Newton to 1e-10 (a converged implicit step:
    ~8 iterations).  Fluid starts at rest.  ``viscosity``: the result of
    ``viscosity_params`` (default: constant mu)."""
    x, ien, info = meshgen.cylinder(R, L, h)
    rp, cp = meshgen.csr_from_ien(x.shape[0], ien)
    am, af, beta, gam = genalpha(0.2, second_order=False)
    params = dict(am=am, af=af, beta=beta, gam=gam, dt=dt, rho=rho, mu_f=mu, ctM=1.0, ctC=36.0,
                  fb=(0.0, 0.0, 0.0), bstab=0.2)
    if viscosity:
        params.update(viscosity)
    inlet, wall = info["inlet"], info["wall"]
    perim = np.intersect1d(inlet, wall)
    gx = meshgen.parabolic_profile(x, info["inlet_faces"], inlet, perim)
    nV = np.tile(np.array([0.0, 0.0, -1.0]), (inlet.size, 1))
    return Problem(name=f"fluid_cylinder_h{h:g}", x=x, ien=ien, rowPtr=rp, colPtr=cp,
                   phys=PHYS_FLUID, dof=4, tDof=4, params=params,
                   dirichlet=[DirBC(inlet, -u_max, gx=gx, nV=nV), DirBC(wall, 0.0)],
                   neumann=[NeuBC(meshgen.faces_on_plane(x, ien, 2, L), 0.0)],
                   LS_type=LS_TYPE_NS, prec=PRECOND_RCS, ls_relTol=1e-2, ls_sD=100, minItr=1,
                   maxItr=12, tol=1e-10, nsteps=nsteps)


def heatf_cylinder(h: float = 0.027, nsteps: int = 10, R: float = 0.5, L: float = 5.0,
                   u_max: float = 30.0, cond: float = 0.1, dt: float = 1e-3,
                   T0_linear: bool = False) -> Problem:
    """Heat transported by a prescribed Poiseuille flow (HEATF3D) in the fluid
    cylinder: state (u, v, w, p, T) with the velocity u_z = u_max (1 - r^2/R^2)
    held in components 0..2 and the temperature the equation's unknown
    (component 4); conductivity 0.1, no source, T = 1 on the inlet, T = 0
    initially (T0_linear: T = 1 - z/L), insulated wall and open outlet,
    dt 1e-3, first-order
    generalized-alpha (rho_inf 0.2), GMRES + diagonal preconditioner (the
    reference's default for heatF), Newton to 1e-8."""
    x, ien, info = meshgen.cylinder(R, L, h)
    rp, cp = meshgen.csr_from_ien(x.shape[0], ien)
    am, af, beta, gam = genalpha(0.2, second_order=False)
    params = dict(am=am, af=af, beta=beta, gam=gam, dt=dt, cond=cond, src=0.0)
    Y0 = np.zeros((x.shape[0], 5))
    Y0[:, 2] = u_max * np.clip(1.0 - (x[:, 0] ** 2 + x[:, 1] ** 2) / (R * R), 0.0, None)
    if T0_linear:
        Y0[:, 4] = 1.0 - x[:, 2] / L
    return Problem(name=f"heatf_cylinder_h{h:g}", x=x, ien=ien, rowPtr=rp, colPtr=cp,
                   phys=PHYS_HEATF, dof=1, tDof=5, s=4, params=params,
                   dirichlet=[DirBC(info["inlet"], 1.0)], LS_type=LS_TYPE_GMRES,
                   prec=PRECOND_FSILS, minItr=1, maxItr=10, tol=1e-8, nsteps=nsteps, Y0=Y0)


def make_lhs_arrays(p: Problem):
    """1-based rowPtr/colPtr/gNodes for FSILS_LHS_CREATE."""
    return (np.arange(1, p.nNo + 1, dtype=np.int32), (p.rowPtr + 1).astype(np.int32),
            (p.colPtr + 1).astype(np.int32))


def build_equation(p: Problem, precision=PREC_FP64):
    """LHS + mesh + equation on the GPU for a Problem."""
    from .fsils import Mesh, FSILS_LHS_CREATE
    g, rp1, cp1 = make_lhs_arrays(p)
    lhs = FSILS_LHS_CREATE(p.nNo, p.nNo, p.nnz, g, rp1, cp1, max(1, len(p.dirichlet)))
    mesh = Mesh(lhs, p.ien, p.x)
    return lhs, mesh, equation_on(p, mesh, precision)


def equation_on(p: Problem, mesh, precision=PREC_FP64):
    """A fresh equation of the Problem (parameters, boundary conditions,
    initial state) on an existing mesh; the previous equation on the mesh
    must have been freed (it holds the lhs faces of its Dirichlet sets)."""
    from .fsils import Equation
    prm = p.eq_params()
    eq = Equation(mesh, prm, p.eq_solver(precision))
    if p.eparam is not None:
        eq.set_eparam(p.eparam)
    for d in p.dirichlet:
        eq.add_dirichlet(d.nodes, d.g, d.gx, d.mask, d.nV)
    for t in p.traction:
        eq.add_traction(t.faces, t.h)
    for nf in p.neumann:
        eq.add_neumann(nf.faces, nf.g)
    if p.cep:
        eq.set_cep(p.cep, np.nonzero(p.stim)[0])
    Ao, Yo, Do = p.initial_state()
    eq.set_state(Ao, Yo, Do)
    return eq
