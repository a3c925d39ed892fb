"""ctypes declarations of the gsls C ABI (include/gsls.h).

The shared library is built in-tree by ``svfsi_gb300.build``; loading fails
loudly when it is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import build as _build

c_int_p = C.POINTER(C.c_int)
c_double_p = C.POINTER(C.c_double)

GSLS_OK = 0
LS_TYPE_CG, LS_TYPE_GMRES, LS_TYPE_NS, LS_TYPE_BICGS = 798, 797, 796, 795
PRECOND_FSILS, PRECOND_RCS = 701, 709
BC_TYPE_DIR, BC_TYPE_NEU = 0, 1
PREC_FP64, PREC_MIXED = 0, 1
PHYS_HEATS, PHYS_STRUCT, PHYS_CEP, PHYS_FLUID, PHYS_LELAS, PHYS_HEATF = 1, 2, 3, 4, 5, 6
PHYS_USTRUCT = 7


class SubLs(C.Structure):
    """FSILS_subLsType (Code/Source/svFSILS/FSILS_STRUCT.h:162-191)."""
    _fields_ = [(n, C.c_int) for n in ("suc", "mItr", "sD", "itr", "cM", "cN", "cD", "reserve")] + \
               [(n, C.c_double) for n in ("absTol", "relTol", "iNorm", "fNorm", "dB", "callD")]


class Ls(C.Structure):
    """FSILS_lsType (Code/Source/svFSILS/FSILS_STRUCT.h:193-204)."""
    _fields_ = [("foC", C.c_int), ("LS_type", C.c_int), ("Resm", C.c_int), ("Resc", C.c_int),
                ("GM", SubLs), ("CG", SubLs), ("RI", SubLs)]


class EqParams(C.Structure):
    _fields_ = [("phys", C.c_int), ("dof", C.c_int), ("tDof", C.c_int), ("s", C.c_int),
                ("am", C.c_double), ("af", C.c_double), ("beta", C.c_double),
                ("gam", C.c_double), ("dt", C.c_double),
                ("rho", C.c_double), ("cond", C.c_double), ("src", C.c_double),
                ("C10", C.c_double), ("Kpen", C.c_double), ("visc", C.c_double),
                ("dmp", C.c_double), ("fb", C.c_double * 3), ("Diso", C.c_double),
                ("mu_f", C.c_double), ("ctM", C.c_double), ("ctC", C.c_double),
                ("eparam", c_double_p), ("elM", C.c_double), ("nu", C.c_double),
                ("viscType", C.c_int), ("mu_o", C.c_double), ("vlam", C.c_double),
                ("va", C.c_double), ("vn", C.c_double), ("bstab", C.c_double),
                ("volType", C.c_int), ("nFn", C.c_int), ("Dani", C.c_double * 3),
                ("fN", c_double_p)]


class EqSolver(C.Structure):
    _fields_ = [("LS_type", C.c_int), ("prec", C.c_int),
                ("ls_relTol", C.c_double), ("ls_absTol", C.c_double),
                ("ls_mItr", C.c_int), ("ls_sD", C.c_int),
                ("ls_relTolIn", C.c_double * 2), ("ls_mItrIn", C.c_int * 2),
                ("minItr", C.c_int), ("maxItr", C.c_int),
                ("tol", C.c_double), ("absTol", C.c_double), ("precision", C.c_int)]


class CepParams(C.Structure):
    _fields_ = [("ode", C.c_int), ("dt_ode", C.c_double), ("A", C.c_double), ("Ts", C.c_double),
                ("Td", C.c_double), ("CL", C.c_double), ("V0", C.c_double), ("X20", C.c_double)]


class AdjPoint(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("Ao", "Yo", "Do", "An", "Yn", "Dn")]


class StepInfo(C.Structure):
    _fields_ = [("newton_itr", C.c_int), ("ls_itr_total", C.c_int),
                ("last_iNorm", C.c_double), ("r1_last", C.c_double), ("last_suc", C.c_int),
                ("t_assembly_ms", C.c_double), ("t_solve_ms", C.c_double)]


# name -> (restype, argtypes)
SIGNATURES = {
    "gsls_init": (C.c_int, [C.c_int]),
    "gsls_version": (C.c_int, []),
    "gsls_set_wait_limit": (C.c_int, [C.c_uint]),
    "gsls_last_error": (C.c_char_p, []),
    "gsls_lhs_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int, c_int_p,
                                  c_int_p, c_int_p, C.c_int]),
    "gsls_lhs_free": (C.c_int, [C.c_void_p]),
    "gsls_bc_create": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, c_int_p,
                                 c_double_p]),
    "gsls_ls_create": (C.c_int, [C.POINTER(Ls), C.c_int, c_double_p, c_double_p, c_int_p,
                                 c_int_p, c_double_p, c_double_p, c_int_p]),
    "gsls_solve": (C.c_int, [C.c_void_p, C.POINTER(Ls), C.c_int, c_double_p, c_double_p,
                             C.c_int, c_int_p, c_double_p]),
    "gsls_solve_dev": (C.c_int, [C.c_void_p, C.POINTER(Ls), C.c_int, C.c_void_p, C.c_void_p,
                                 C.c_int, C.c_int, c_int_p, c_double_p]),
    "gsls_spmv_dev": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                C.c_void_p]),
    "gsls_dot_dev": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, c_double_p]),
    "gsls_norm_dev": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, c_double_p]),
    "gsls_dot_noalloc": (C.c_int, [C.c_longlong, C.c_void_p, C.c_void_p, c_double_p,
                                   C.c_void_p]),
    "gsls_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gsls_get_stream": (C.c_void_p, [C.c_void_p]),
    "gsls_mesh_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_void_p, C.c_int, C.c_int, c_int_p,
                                   C.c_int, c_double_p]),
    "gsls_mesh_free": (C.c_int, [C.c_void_p]),
    "gsls_mesh_ncolors": (C.c_int, [C.c_void_p]),
    "gsls_assemble_dev": (C.c_int, [C.c_void_p, C.POINTER(EqParams), C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "gsls_assemble_ustruct_dev": (C.c_int, [C.c_void_p, C.POINTER(EqParams), C.c_void_p,
                                            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_int]),
    "gsls_assemble": (C.c_int, [C.c_void_p, C.POINTER(EqParams), c_double_p, c_double_p,
                                c_double_p, c_double_p, c_double_p]),
    "gsls_eq_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_void_p, C.POINTER(EqParams),
                                 C.POINTER(EqSolver)]),
    "gsls_eq_free": (C.c_int, [C.c_void_p]),
    "gsls_eq_add_dirichlet": (C.c_int, [C.c_void_p, C.c_int, c_int_p, c_double_p, C.c_double,
                                        C.c_int]),
    "gsls_eq_add_dirichlet_nv": (C.c_int, [C.c_void_p, C.c_int, c_int_p, c_double_p, c_double_p,
                                           C.c_double, C.c_int]),
    "gsls_eq_add_traction": (C.c_int, [C.c_void_p, C.c_int, c_int_p, c_double_p]),
    "gsls_eq_add_neumann": (C.c_int, [C.c_void_p, C.c_int, c_int_p, C.c_double]),
    "gsls_eq_set_state": (C.c_int, [C.c_void_p, c_double_p, c_double_p, c_double_p]),
    "gsls_eq_get_state": (C.c_int, [C.c_void_p, c_double_p, c_double_p, c_double_p]),
    "gsls_eq_state_dev": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                    C.POINTER(C.c_void_p)]),
    "gsls_eq_step": (C.c_int, [C.c_void_p, C.POINTER(StepInfo)]),
    "gsls_eq_set_cep": (C.c_int, [C.c_void_p, C.POINTER(CepParams), C.c_int, c_int_p]),
    "gsls_eq_get_cep_state": (C.c_int, [C.c_void_p, c_double_p]),
    "gsls_eq_write_restart": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int, C.c_double]),
    "gsls_eq_read_restart": (C.c_int, [C.c_void_p, C.c_char_p, c_int_p, c_double_p]),
    "gsls_eq_set_eparam": (C.c_int, [C.c_void_p, c_double_p]),
    "gsls_adjoint_forward": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "gsls_adjoint_backward": (C.c_int, [C.c_void_p, c_double_p, c_double_p, c_double_p,
                                        c_double_p]),
    "gsls_cep_adjoint_forward": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double,
                                           c_double_p, C.POINTER(C.c_void_p)]),
    "gsls_cep_adjoint_backward": (C.c_int, [C.c_void_p, c_double_p, c_double_p]),
    "gsls_tape_free": (C.c_int, [C.c_void_p]),
    "gsls_adjoint_solve": (C.c_int, [C.c_void_p, C.POINTER(AdjPoint), C.c_void_p, C.c_void_p]),
    "gsls_dRdp": (C.c_int, [C.c_void_p, C.POINTER(AdjPoint), C.c_void_p, C.c_void_p]),
    "gsls_launch_count": (C.c_longlong, []),
    "gsls_profile_enable": (C.c_int, [C.c_int]),
    "gsls_profile_reset": (C.c_int, []),
    "gsls_profile_read": (C.c_int, [C.c_char_p, C.POINTER(C.c_longlong), c_double_p]),
    "gsls_fp64_fma_rate": (C.c_int, [c_double_p]),
    "gsls_l2_read_rate": (C.c_int, [c_double_p]),
}

_LIB = None


def lib_path() -> Path:
    return _build.lib_path()


def load(build_if_missing: bool = False):
    """Load libgsls.so; raise if it is not built (no fallback)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = lib_path()
    if not p.exists():
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError(f"gsls CUDA library not built: {p} (run svfsi_gb300.build.build())")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _LIB = lib
    return lib


class GslsError(RuntimeError):
    pass


def check(rc: int, what: str = ""):
    if rc != GSLS_OK:
        msg = load().gsls_last_error()
        raise GslsError(f"{what} failed with status {rc}: {msg.decode() if msg else ''}")
