"""Python bridge to the oracle shared library (oracle/build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "build" / "liboracle.so"

c_int_p = C.POINTER(C.c_int)
c_double_p = C.POINTER(C.c_double)

LS_TYPE_CG, LS_TYPE_GMRES, LS_TYPE_NS, LS_TYPE_BICGS = 798, 797, 796, 795
PRECOND_FSILS, PRECOND_RCS = 701, 709


class SubLs(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("suc", "mItr", "sD", "itr", "cM", "cN", "cD", "reserve")] + \
               [(n, C.c_double) for n in ("absTol", "relTol", "iNorm", "fNorm", "dB", "callD")]


class Ls(C.Structure):
    _fields_ = [("foC", C.c_int), ("LS_type", C.c_int), ("Resm", C.c_int), ("Resc", C.c_int),
                ("GM", SubLs), ("CG", SubLs), ("RI", SubLs)]


class EqP(C.Structure):
    _fields_ = [("phys", C.c_int), ("dof", C.c_int), ("tDof", C.c_int), ("s", C.c_int),
                ("am", C.c_double), ("af", C.c_double), ("beta", C.c_double),
                ("gam", C.c_double), ("dt", C.c_double),
                ("rho", C.c_double), ("cond", C.c_double), ("src", C.c_double),
                ("C10", C.c_double), ("Kpen", C.c_double), ("visc", C.c_double),
                ("dmp", C.c_double), ("fb", C.c_double * 3), ("Diso", C.c_double),
                ("mu_f", C.c_double), ("ctM", C.c_double),
                ("ctC", C.c_double), ("eparam", c_double_p), ("elM", C.c_double),
                ("nu", C.c_double), ("viscType", C.c_int), ("mu_o", C.c_double),
                ("vlam", C.c_double), ("va", C.c_double), ("vn", C.c_double),
                ("bstab", C.c_double), ("volType", C.c_int), ("nFn", C.c_int),
                ("Dani", C.c_double * 3), ("fN", c_double_p)]


class DirBC(C.Structure):
    _fields_ = [("nNo", C.c_int), ("nodes", c_int_p), ("gx", c_double_p), ("nV", c_double_p),
                ("g", C.c_double), ("mask", C.c_int)]


class TracBC(C.Structure):
    _fields_ = [("nFel", C.c_int), ("fIEN", c_int_p), ("h", C.c_double * 3)]


class CepP(C.Structure):
    _fields_ = [("ode", C.c_int), ("dt_ode", C.c_double), ("A", C.c_double), ("Ts", C.c_double),
                ("Td", C.c_double), ("CL", C.c_double), ("Ksac", C.c_double)]


class NeuBC(C.Structure):
    _fields_ = [("nFel", C.c_int), ("fIEN", c_int_p), ("g", C.c_double)]


class Eq(C.Structure):
    _fields_ = [("p", EqP), ("nNo", C.c_int), ("nEl", C.c_int), ("IEN", c_int_p),
                ("x", c_double_p), ("rowPtr", c_int_p), ("colPtr", c_int_p), ("nnz", C.c_int),
                ("nDir", C.c_int), ("dir", C.POINTER(DirBC)), ("nTrac", C.c_int),
                ("trac", C.POINTER(TracBC)), ("LS_type", C.c_int), ("prec", C.c_int),
                ("ls_relTol", C.c_double), ("ls_absTol", C.c_double), ("ls_mItr", C.c_int),
                ("ls_sD", C.c_int), ("ls_relTolIn", C.c_double * 2),
                ("ls_absTolIn", C.c_double * 2), ("ls_mItrIn", C.c_int * 2),
                ("minItr", C.c_int), ("maxItr", C.c_int), ("tol", C.c_double),
                ("eqAbsTol", C.c_double),
                ("Ao", c_double_p), ("Yo", c_double_p), ("Do", c_double_p),
                ("An", c_double_p), ("Yn", c_double_p), ("Dn", c_double_p),
                ("eq_iNorm", C.c_double), ("eq_pNorm", C.c_double),
                ("cep", CepP), ("stim", c_int_p), ("Xion", c_double_p), ("time", C.c_double),
                ("cep_ipass_done", C.c_int), ("nNeu", C.c_int), ("neu", C.POINTER(NeuBC)),
                ("ncolor", C.c_int), ("color_off", c_int_p), ("color_order", c_int_p),
                ("Ad", c_double_p)]


class StepInfo(C.Structure):
    _fields_ = [("newton_itr", C.c_int), ("ls_itr_total", C.c_int),
                ("last_iNorm", C.c_double), ("r1_last", C.c_double), ("last_suc", C.c_int)]


_L = None


def build(force: bool = False) -> Path:
    if force or not LIB.exists() or any(p.stat().st_mtime > LIB.stat().st_mtime
                                        for p in list(HERE.glob("*.c")) + list(HERE.glob("*.h"))):
        subprocess.run(["make", "-s", "-C", str(HERE)] + (["-B"] if force else []), check=True)
    return LIB


def load():
    global _L
    if _L is None:
        build()
        L = C.CDLL(str(LIB))
        L.orc_lhs_create.restype = C.c_void_p
        L.orc_lhs_create.argtypes = [C.c_int, C.c_int, c_int_p, c_int_p, C.c_int]
        L.orc_lhs_free.argtypes = [C.c_void_p]
        L.orc_bc_create.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, c_int_p,
                                    c_double_p]
        L.orc_ls_create.argtypes = [C.POINTER(Ls), C.c_int]
        L.orc_solve.argtypes = [C.c_void_p, C.POINTER(Ls), C.c_int, c_double_p, c_double_p,
                                C.c_int, c_int_p, c_double_p]
        L.orc_spar_vv.argtypes = [C.c_void_p, C.c_int, c_double_p, c_double_p, c_double_p]
        L.orc_dotv.restype = C.c_double
        L.orc_dotv.argtypes = [C.c_int, C.c_int, c_double_p, c_double_p]
        L.orc_lhsa.argtypes = [C.c_int, C.c_int, C.c_int, c_int_p, c_int_p, c_int_p, C.c_int]
        L.orc_lhsa_count.argtypes = [C.c_int, C.c_int, C.c_int, c_int_p]
        L.orc_assemble.argtypes = [C.POINTER(EqP), C.c_int, C.c_int, c_int_p, c_double_p,
                                   c_double_p, c_double_p, c_double_p, c_int_p, c_int_p,
                                   c_double_p, c_double_p]
        L.orc_elem_heats.argtypes = [C.POINTER(EqP), c_double_p, c_double_p, c_double_p,
                                     c_double_p, c_double_p]
        L.orc_elem_struct.argtypes = [C.POINTER(EqP), C.c_double, c_double_p, c_double_p,
                                      c_double_p, c_double_p, c_double_p, c_double_p]
        L.orc_elem_fluid.argtypes = [C.POINTER(EqP), c_double_p, c_double_p, c_double_p,
                                     c_double_p, c_double_p]
        L.orc_elem_ustruct.argtypes = [C.POINTER(EqP), c_double_p, c_double_p, c_double_p,
                                       c_double_p, c_double_p, c_double_p, c_double_p]
        L.orc_assemble_ustruct.argtypes = [C.POINTER(EqP), C.c_int, C.c_int, c_int_p,
                                           c_double_p, c_double_p, c_double_p, c_double_p,
                                           c_int_p, c_int_p, c_double_p, c_double_p,
                                           c_double_p]
        L.orc_ge.restype = C.c_int
        L.orc_ge.argtypes = [C.c_int, C.c_int, c_double_p, c_double_p]
        L.orc_pk2cc_nhk.argtypes = [C.c_double, C.c_double, c_double_p, c_double_p, c_double_p]
        L.orc_genalpha.argtypes = [C.c_double, C.c_int, c_double_p, c_double_p, c_double_p,
                                   c_double_p]
        L.orc_eq_step.argtypes = [C.POINTER(Eq), C.POINTER(StepInfo)]
        L.orc_bfluid.argtypes = [C.POINTER(EqP), C.c_int, c_int_p, C.c_double, C.c_int,
                                 c_int_p, c_double_p, c_double_p, c_int_p, c_int_p,
                                 c_double_p, c_double_p]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_color_elements.restype = C.c_int
        L.orc_color_elements.argtypes = [C.c_int, C.c_int, c_int_p, c_int_p, c_int_p]
        _L = L
    return _L


def ip(a):
    return a.ctypes.data_as(c_int_p)


def dp(a):
    return a.ctypes.data_as(c_double_p)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def set_threads(n: int):
    load().orc_set_threads(int(n))


def lhsa(nNo, ien):
    L = load()
    ien = i32(ien)
    nnz = L.orc_lhsa_count(nNo, ien.shape[0], ien.shape[1], ip(ien))
    rp = np.zeros(nNo + 1, np.int32)
    cp = np.zeros(nnz, np.int32)
    rc = L.orc_lhsa(nNo, ien.shape[0], ien.shape[1], ip(ien), ip(rp), ip(cp), nnz)
    assert rc == nnz, rc
    return rp, cp


def eqp_from(problem, eparam=None) -> EqP:
    """The problem's parameters; its CEP fibres (nEl x 3 nFn, original
    element order) are held by the returned structure."""
    p = EqP()
    p.phys, p.dof, p.tDof, p.s = problem.phys, problem.dof, problem.tDof, getattr(problem, "s", 0)
    for k, v in problem.params.items():
        if k in ("fb", "Dani"):
            for i, vi in enumerate(v):
                getattr(p, k)[i] = vi
        else:
            setattr(p, k, v)
    fib = getattr(problem, "fibers", None)
    if fib is not None:
        p._fib = f64(fib)
        p.nFn = p._fib.shape[1] // 3
        p.fN = dp(p._fib)
    return p


def assemble(problem, Ag, Yg, Dg=None, eparam=None):
    L = load()
    p = eqp_from(problem)
    keep = []
    if eparam is not None:
        e = f64(eparam)
        keep.append(e)
        p.eparam = dp(e)
    d = problem.dof
    R = np.zeros((problem.nNo, d))
    Val = np.zeros((problem.nnz, d * d))
    Dg = np.zeros_like(Ag) if Dg is None else Dg
    ien, x, rp, cp = i32(problem.ien), f64(problem.x), i32(problem.rowPtr), i32(problem.colPtr)
    Ag, Yg, Dg = f64(Ag), f64(Yg), f64(Dg)
    rc = L.orc_assemble(C.byref(p), problem.nNo, problem.nEl, ip(ien), dp(x), dp(Ag), dp(Yg),
                        dp(Dg), ip(rp), ip(cp), dp(R), dp(Val))
    assert rc == 0, rc
    return R, Val


def assemble_ustruct(problem, Ag, Yg, Dg):
    """CONSTRUCT_uSOLID + USTRUCT_DOASSEM: (R(nNo,4), Val(nnz,16), Kd(nnz,12))."""
    L = load()
    p = eqp_from(problem)
    R = np.zeros((problem.nNo, 4))
    Val = np.zeros((problem.nnz, 16))
    Kd = np.zeros((problem.nnz, 12))
    ien, x, rp, cp = i32(problem.ien), f64(problem.x), i32(problem.rowPtr), i32(problem.colPtr)
    Ag, Yg, Dg = f64(Ag), f64(Yg), f64(Dg)
    rc = L.orc_assemble_ustruct(C.byref(p), problem.nNo, problem.nEl, ip(ien), dp(x), dp(Ag),
                                dp(Yg), dp(Dg), ip(rp), ip(cp), dp(R), dp(Val), dp(Kd))
    assert rc == 0, rc
    return R, Val, Kd


class OracleSolver:
    """FSILS_LHS_CREATE / BC_CREATE / LS_CREATE / SOLVE on the oracle."""

    def __init__(self, nNo, rowPtr0, colPtr0, nFaces):
        L = load()
        self.rp, self.cp = i32(rowPtr0), i32(colPtr0)
        self.h = L.orc_lhs_create(nNo, self.cp.size, ip(self.rp), ip(self.cp), nFaces)
        self.nNo, self.nFaces = nNo, nFaces

    def bc_create(self, faIn, nodes0, dof, bctype=0, val=None):
        n = i32(nodes0)
        v = None if val is None else f64(val)
        rc = load().orc_bc_create(self.h, faIn, n.size, dof, bctype, ip(n),
                                  dp(v) if v is not None else None)
        assert rc == 0

    def solve(self, ls: Ls, dof, R, Val, prec, incL=None, res=None):
        il = None if incL is None else i32(incL)
        rs = None if res is None else f64(res)
        rc = load().orc_solve(self.h, C.byref(ls), dof, dp(R), dp(Val), prec,
                              ip(il) if il is not None else None,
                              dp(rs) if rs is not None else None)
        assert rc == 0, rc

    def spmv(self, dof, Val, U):
        KU = np.zeros_like(U)
        load().orc_spar_vv(self.h, dof, dp(f64(Val)), dp(f64(U)), dp(KU))
        return KU

    def __del__(self):
        try:
            load().orc_lhs_free(self.h)
        except Exception:
            pass


def ls_create(LS_type, relTol=None, absTol=None, mItr=None, sD=None) -> Ls:
    ls = Ls()
    load().orc_ls_create(C.byref(ls), LS_type)
    if relTol is not None:
        ls.RI.relTol = relTol
    if absTol is not None:
        ls.RI.absTol = absTol
    if mItr is not None:
        ls.RI.mItr = mItr
    if sD is not None:
        ls.RI.sD = sD
        ls.GM.sD = sD
    return ls


def color_elements(nNo, ien):
    """Greedy conflict-free element colouring (orc_color_elements):
    returns (ncolor, color_off[ncolor+1], order[nEl])."""
    ien = i32(ien)
    off = np.zeros(65, np.int32)
    order = np.zeros(max(ien.shape[0], 1), np.int32)
    nc = load().orc_color_elements(nNo, ien.shape[0], ip(ien), ip(off), ip(order))
    assert nc > 0, nc
    return nc, off[:nc + 1].copy(), order[:ien.shape[0]].copy()


class OracleEquation:
    """Time stepping of a Problem on the oracle (orc_eq_step).  colored:
    assemble colour by colour with OpenMP (the multi-core CPU baseline);
    otherwise the serial element loop."""

    def __init__(self, problem, eparam=None, colored=False):
        self.P = problem
        p = problem
        self._keep = []

        def keep(a):
            self._keep.append(a)
            return a

        eq = Eq()
        ep_ = eqp_from(p)
        if hasattr(ep_, "_fib"):
            keep(ep_._fib)  # eq.p is a copy: the fibre array must outlive it
        eq.p = ep_
        ep = eparam if eparam is not None else p.eparam
        if ep is not None:
            eq.p.eparam = dp(keep(f64(ep)))
        eq.nNo, eq.nEl = p.nNo, p.nEl
        eq.IEN = ip(keep(i32(p.ien)))
        eq.x = dp(keep(f64(p.x)))
        eq.rowPtr = ip(keep(i32(p.rowPtr)))
        eq.colPtr = ip(keep(i32(p.colPtr)))
        eq.nnz = p.nnz
        dirs = (DirBC * max(1, len(p.dirichlet)))()
        for k, d in enumerate(p.dirichlet):
            dirs[k].nNo = d.nodes.size
            dirs[k].nodes = ip(keep(i32(d.nodes)))
            dirs[k].gx = dp(keep(f64(d.gx))) if d.gx is not None else None
            nV = getattr(d, "nV", None)
            dirs[k].nV = dp(keep(f64(nV))) if nV is not None else None
            dirs[k].g = d.g
            dirs[k].mask = d.mask
        keep(dirs)
        eq.nDir = len(p.dirichlet)
        eq.dir = C.cast(dirs, C.POINTER(DirBC))
        tr = (TracBC * max(1, len(p.traction)))()
        for k, t in enumerate(p.traction):
            tr[k].nFel = t.faces.shape[0]
            tr[k].fIEN = ip(keep(i32(t.faces)))
            for i in range(3):
                tr[k].h[i] = t.h[i]
        keep(tr)
        eq.nTrac = len(p.traction)
        eq.trac = C.cast(tr, C.POINTER(TracBC))
        neus = getattr(p, "neumann", [])
        nb = (NeuBC * max(1, len(neus)))()
        for k, nf in enumerate(neus):
            nb[k].nFel = nf.faces.shape[0]
            nb[k].fIEN = ip(keep(i32(nf.faces)))
            nb[k].g = nf.g
        keep(nb)
        eq.nNeu = len(neus)
        eq.neu = C.cast(nb, C.POINTER(NeuBC))
        eq.LS_type, eq.prec = p.LS_type, p.prec
        eq.ls_relTol, eq.ls_absTol, eq.ls_mItr, eq.ls_sD = p.ls_relTol, p.ls_absTol, p.ls_mItr, p.ls_sD
        eq.ls_relTolIn[0] = eq.ls_relTolIn[1] = -1.0
        eq.ls_mItrIn[0] = eq.ls_mItrIn[1] = -1
        eq.minItr, eq.maxItr, eq.tol, eq.eqAbsTol = p.minItr, p.maxItr, p.tol, p.absTol
        shp = (p.nNo, p.tDof)
        self.Ao, self.Yo, self.Do = (keep(np.zeros(shp)) for _ in range(3))
        self.An, self.Yn, self.Dn = (keep(np.zeros(shp)) for _ in range(3))
        eq.Ao, eq.Yo, eq.Do = dp(self.Ao), dp(self.Yo), dp(self.Do)
        eq.An, eq.Yn, eq.Dn = dp(self.An), dp(self.Yn), dp(self.Dn)
        self.Xion = keep(np.zeros((p.nNo, 2)))
        if getattr(p, "cep", None):
            c = p.cep
            eq.cep.ode, eq.cep.dt_ode = c["ode"], c["dt_ode"]
            eq.cep.A, eq.cep.Ts, eq.cep.Td, eq.cep.CL = c["A"], c["Ts"], c["Td"], c["CL"]
            eq.cep.Ksac = 0.0
            eq.stim = ip(keep(i32(p.stim)))
            self.Xion[:, 0] = c["V0"]
            self.Xion[:, 1] = c["X20"]
        eq.Xion = dp(self.Xion)
        self.Ad = keep(np.zeros((p.nNo, 3)))
        if p.phys == 7:
            eq.Ad = dp(self.Ad)
        if colored:
            nc, off, order = color_elements(p.nNo, p.ien)
            eq.ncolor = nc
            eq.color_off = ip(keep(off))
            eq.color_order = ip(keep(order))
        self.eq = eq

    def set_state(self, Ao, Yo, Do):
        self.Ao[:] = Ao
        self.Yo[:] = Yo
        self.Do[:] = Do

    def step(self) -> StepInfo:
        info = StepInfo()
        rc = load().orc_eq_step(C.byref(self.eq), C.byref(info))
        assert rc == 0, rc
        return info

    def state(self):
        return self.Ao.copy(), self.Yo.copy(), self.Do.copy()
