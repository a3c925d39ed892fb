"""Python host side mirroring the svFSILS call surface on top of the gsls
C ABI (the names follow Code/Source/svFSILS/FSILS_API.h:51-135).

Arrays are numpy; indices passed to the FSILS_* functions are 1-based as in
the reference.  Every call goes through libgsls.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import (BC_TYPE_DIR, BC_TYPE_NEU, LS_TYPE_BICGS, LS_TYPE_CG, LS_TYPE_GMRES,
                   LS_TYPE_NS, PREC_FP64, PREC_MIXED, PRECOND_FSILS, PRECOND_RCS, EqParams,
                   EqSolver, Ls, StepInfo, check)

__all__ = [
    "FSILS_LHS_CREATE", "FSILS_BC_CREATE", "FSILS_LS_CREATE", "FSILS_SOLVE", "Lhs", "Mesh",
    "Equation", "LS_TYPE_CG", "LS_TYPE_GMRES", "LS_TYPE_NS", "LS_TYPE_BICGS", "PRECOND_FSILS",
    "PRECOND_RCS", "BC_TYPE_DIR", "BC_TYPE_NEU", "PREC_FP64", "PREC_MIXED",
]


def _ip(a: np.ndarray):
    return a.ctypes.data_as(_lib.c_int_p)


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_lib.c_double_p)


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


class Lhs:
    """Handle of FSILS_lhsType (gsls_lhs)."""

    def __init__(self, gnNo, nNo, nnz, gNodes, rowPtr, colPtr, nFaces):
        L = _lib.load()
        self._keep = [_i32(gNodes), _i32(rowPtr), _i32(colPtr)]
        h = C.c_void_p()
        check(L.gsls_lhs_create(C.byref(h), gnNo, nNo, nnz, _ip(self._keep[0]),
                                _ip(self._keep[1]), _ip(self._keep[2]), nFaces),
              "FSILS_LHS_CREATE")
        self.h = h
        self.nNo, self.nnz, self.nFaces = nNo, nnz, nFaces

    def free(self):
        if self.h:
            _lib.load().gsls_lhs_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def FSILS_LHS_CREATE(gnNo, nNo, nnz, gNodes, rowPtr, colPtr, nFaces) -> Lhs:
    """Code/Source/svFSILS/LHS.f:51 -- rowPtr/colPtr/gNodes 1-based."""
    return Lhs(gnNo, nNo, nnz, gNodes, rowPtr, colPtr, nFaces)


def FSILS_BC_CREATE(lhs: Lhs, faIn, nNo, dof, BC_type, gNodes, Val=None):
    """Code/Source/svFSILS/BC.f:50 -- faIn and gNodes 1-based, Val(dof,nNo)."""
    g = _i32(gNodes)
    v = None if Val is None else _f64(Val)
    check(_lib.load().gsls_bc_create(lhs.h, faIn, nNo, dof, BC_type, _ip(g),
                                     _dp(v) if v is not None else None), "FSILS_BC_CREATE")


def FSILS_LS_CREATE(LS_type, relTol=None, absTol=None, maxItr=None, dimKry=None,
                    relTolIn=None, absTolIn=None, maxItrIn=None) -> Ls:
    """Code/Source/svFSILS/LS.f:50 -- optional arguments as in the reference."""
    ls = Ls()

    def d(v):
        return None if v is None else C.byref(C.c_double(v))

    def i(v):
        return None if v is None else C.byref(C.c_int(v))

    def d2(v):
        return None if v is None else (C.c_double * 2)(*v)

    def i2(v):
        return None if v is None else (C.c_int * 2)(*v)

    check(_lib.load().gsls_ls_create(C.byref(ls), LS_type, d(relTol), d(absTol), i(maxItr),
                                     i(dimKry), d2(relTolIn), d2(absTolIn), i2(maxItrIn)),
          "FSILS_LS_CREATE")
    return ls


def FSILS_SOLVE(lhs: Lhs, ls: Ls, dof, Ri: np.ndarray, Val: np.ndarray, prec, incL=None,
                res=None):
    """Code/Source/svFSILS/SOLVE.f:51 -- Ri(dof,nNo) overwritten with the
    solution, Val(dof*dof,nnz) left preconditioned (in place)."""
    assert Ri.dtype == np.float64 and Ri.flags.c_contiguous
    assert Val.dtype == np.float64 and Val.flags.c_contiguous
    il = None if incL is None else _i32(incL)
    rs = None if res is None else _f64(res)
    check(_lib.load().gsls_solve(lhs.h, C.byref(ls), dof, _dp(Ri), _dp(Val), prec,
                                 _ip(il) if il is not None else None,
                                 _dp(rs) if rs is not None else None), "FSILS_SOLVE")


class Mesh:
    """tet4 mesh bound to an Lhs (element -> CSR map + colouring on device)."""

    def __init__(self, lhs: Lhs, ien0: np.ndarray, x: np.ndarray):
        ien1 = _i32(np.asarray(ien0) + 1)
        xx = _f64(x)
        h = C.c_void_p()
        check(_lib.load().gsls_mesh_create(C.byref(h), lhs.h, ien1.shape[0], 4, _ip(ien1), 3,
                                           _dp(xx)), "gsls_mesh_create")
        self.h = h
        self.lhs = lhs
        self.nEl = ien1.shape[0]

    @property
    def ncolors(self) -> int:
        return _lib.load().gsls_mesh_ncolors(self.h)

    def assemble(self, params: EqParams, Ag, Yg, Dg, dof):
        """Host-array assembly: returns (R[nNo,dof], Val[nnz,dof*dof])."""
        nNo, nnz = self.lhs.nNo, self.lhs.nnz
        R = np.zeros((nNo, dof))
        Val = np.zeros((nnz, dof * dof))
        a, y = _f64(Ag), _f64(Yg)
        d = None if Dg is None else _f64(Dg)
        check(_lib.load().gsls_assemble(self.h, C.byref(params), _dp(a), _dp(y),
                                        _dp(d) if d is not None else None, _dp(R), _dp(Val)),
              "gsls_assemble")
        return R, Val

    def free(self):
        if self.h:
            _lib.load().gsls_mesh_free(self.h)
            self.h = None

    def __del__(self):
        # the Lhs outlives this mesh: self.lhs keeps it referenced
        try:
            self.free()
        except Exception:
            pass


class Equation:
    """Device-resident time integrator of one equation (gsls_eq)."""

    def __init__(self, mesh: Mesh, params: EqParams, solver: EqSolver):
        h = C.c_void_p()
        check(_lib.load().gsls_eq_create(C.byref(h), mesh.h, C.byref(params), C.byref(solver)),
              "gsls_eq_create")
        self.h = h
        self.mesh = mesh
        self.params = params
        self.nNo = mesh.lhs.nNo
        self.tDof = params.tDof

    def add_dirichlet(self, nodes0, g, gx=None, mask=0, nV=None):
        n1 = _i32(np.asarray(nodes0) + 1)
        gxa = None if gx is None else _f64(gx)
        nva = None if nV is None else _f64(nV)
        check(_lib.load().gsls_eq_add_dirichlet_nv(self.h, n1.size, _ip(n1),
                                                   _dp(gxa) if gxa is not None else None,
                                                   _dp(nva) if nva is not None else None,
                                                   float(g), int(mask)),
              "gsls_eq_add_dirichlet_nv")

    def add_neumann(self, faces0, g):
        """Neumann BC of value g on tri3 faces (HEATF: BASSEMNEUBC + BHEATF)."""
        f1 = _i32(np.asarray(faces0) + 1)
        check(_lib.load().gsls_eq_add_neumann(self.h, f1.shape[0], _ip(f1), float(g)),
              "gsls_eq_add_neumann")

    def add_traction(self, faces0, h):
        f1 = _i32(np.asarray(faces0) + 1)
        hh = _f64(h)
        check(_lib.load().gsls_eq_add_traction(self.h, f1.shape[0], _ip(f1), _dp(hh)),
              "gsls_eq_add_traction")

    def set_state(self, Ao, Yo, Do=None):
        a, y = _f64(Ao), _f64(Yo)
        d = None if Do is None else _f64(Do)
        check(_lib.load().gsls_eq_set_state(self.h, _dp(a), _dp(y),
                                            _dp(d) if d is not None else None),
              "gsls_eq_set_state")

    def get_state(self, out=None):
        """(Ao, Yo, Do) as (nNo, tDof) FP64 arrays; out: three C-contiguous
        FP64 arrays of that shape to copy into (e.g. pinned host buffers,
        which the device-to-host copy then reaches directly)."""
        shp = (self.nNo, self.tDof)
        if out is None:
            out = (np.zeros(shp), np.zeros(shp), np.zeros(shp))
        for a in out:
            if a.shape != shp or a.dtype != np.float64 or not a.flags.c_contiguous:
                raise ValueError(f"get_state: out arrays must be C-contiguous float64 {shp}")
        Ao, Yo, Do = out
        check(_lib.load().gsls_eq_get_state(self.h, _dp(Ao), _dp(Yo), _dp(Do)),
              "gsls_eq_get_state")
        return Ao, Yo, Do

    def step(self) -> StepInfo:
        info = StepInfo()
        check(_lib.load().gsls_eq_step(self.h, C.byref(info)), "gsls_eq_step")
        return info

    def write_restart(self, path, cTS: int, cpu_time: float = 0.0):
        """Restart record in the reference's layout (WRITERESTART)."""
        check(_lib.load().gsls_eq_write_restart(self.h, str(path).encode(), int(cTS),
                                                float(cpu_time)), "gsls_eq_write_restart")

    def read_restart(self, path):
        """Restore state, time and eq%iNorm (INITFROMBIN); returns (cTS, cpu_time)."""
        c, t = C.c_int(), C.c_double()
        check(_lib.load().gsls_eq_read_restart(self.h, str(path).encode(), C.byref(c), C.byref(t)),
              "gsls_eq_read_restart")
        return c.value, t.value

    def set_cep(self, cep: dict, stim_nodes0):
        """Aliev-Panfilov reaction step (gsls_eq_set_cep); stim_nodes0 0-based."""
        c = _lib.CepParams()
        for k in ("ode", "dt_ode", "A", "Ts", "Td", "CL", "V0", "X20"):
            setattr(c, k, cep[k])
        s1 = _i32(np.asarray(stim_nodes0) + 1)
        check(_lib.load().gsls_eq_set_cep(self.h, C.byref(c), s1.size, _ip(s1)), "gsls_eq_set_cep")

    def get_cep_state(self):
        X = np.zeros((self.nNo, 2))
        check(_lib.load().gsls_eq_get_cep_state(self.h, _dp(X)), "gsls_eq_get_cep_state")
        return X

    def adjoint_forward(self, nsteps, every=5):
        """Take nsteps steps with checkpoints every `every` steps; returns a
        Tape whose backward() gives dJ/dp for the per-element parameter."""
        h = C.c_void_p()
        check(_lib.load().gsls_adjoint_forward(self.h, int(nsteps), int(every), C.byref(h)),
              "gsls_adjoint_forward")
        return Tape(h, self)

    def cep_adjoint_forward(self, nsteps, every=5, vth=-30.0, vw=5.0):
        """CEP: take nsteps steps with checkpoints; returns (T, CepTape) with
        T the smoothed activation time per node (gsls_cep_adjoint_forward)."""
        h = C.c_void_p()
        T = np.zeros(self.nNo)
        check(_lib.load().gsls_cep_adjoint_forward(self.h, int(nsteps), int(every), float(vth),
                                                   float(vw), _dp(T), C.byref(h)),
              "gsls_cep_adjoint_forward")
        return T, CepTape(h, self)

    def set_eparam(self, ep):
        e = None if ep is None else _f64(ep)
        check(_lib.load().gsls_eq_set_eparam(self.h, _dp(e) if e is not None else None),
              "gsls_eq_set_eparam")

    def free(self):
        if self.h:
            _lib.load().gsls_eq_free(self.h)
            self.h = None

    def __del__(self):
        # the Mesh and Lhs outlive this equation: self.mesh keeps them referenced
        try:
            self.free()
        except Exception:
            pass


class Tape:
    """Checkpoints of an adjoint forward run (gsls_tape)."""

    def __init__(self, h, eq: Equation):
        self.h = h
        self.eq = eq

    def backward(self, Abar=None, Ybar=None, Dbar=None):
        """dJ/dp (nEl) from the cotangents of the final state (nNo x tDof each)."""
        nEl = self.eq.mesh.nEl
        g = np.zeros(nEl)
        arrs = [None if a is None else _f64(a) for a in (Abar, Ybar, Dbar)]
        ptrs = [None if a is None else _dp(a) for a in arrs]
        check(_lib.load().gsls_adjoint_backward(self.h, ptrs[0], ptrs[1], ptrs[2], _dp(g)),
              "gsls_adjoint_backward")
        return g

    def free(self):
        if self.h:
            _lib.load().gsls_tape_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class CepTape(Tape):
    """Checkpoints of a CEP activation-time forward run."""

    def backward(self, Tbar):
        """dJ/dDiso (nEl) from dJ/dT (nNo)."""
        g = np.zeros(self.eq.mesh.nEl)
        tb = _f64(Tbar)
        check(_lib.load().gsls_cep_adjoint_backward(self.h, _dp(tb), _dp(g)),
              "gsls_cep_adjoint_backward")
        return g
