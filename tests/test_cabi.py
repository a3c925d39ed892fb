"""The C-ABI library builds for sm_103a, loads without a GPU and exports
every function that include/gsls.h declares; host-only entry points behave
like the reference (CPU only, no kernel launches)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        txt = h.read_text()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(gsls_\w+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def libpath():
    from svfsi_gb300 import build
    return build.build()


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("gsls_lhs_create", "gsls_bc_create", "gsls_ls_create", "gsls_solve",
                 "gsls_assemble", "gsls_eq_step"):
        assert must in names


def test_library_exports_every_declared_symbol(libpath):
    lib = C.CDLL(str(libpath))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_header(libpath):
    from svfsi_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.SIGNATURES), \
        set(declared_functions()) - set(_lib.SIGNATURES)


def test_ls_create_defaults_match_oracle(libpath, orc):
    from svfsi_gb300 import fsils
    for t in (fsils.LS_TYPE_CG, fsils.LS_TYPE_GMRES, fsils.LS_TYPE_NS, fsils.LS_TYPE_BICGS):
        a = fsils.FSILS_LS_CREATE(t)
        b = orc.ls_create(t)
        for sub in ("RI", "GM", "CG"):
            sa, sb = getattr(a, sub), getattr(b, sub)
            for f in ("mItr", "sD", "relTol", "absTol"):
                assert getattr(sa, f) == getattr(sb, f), (t, sub, f)
    ls = fsils.FSILS_LS_CREATE(fsils.LS_TYPE_NS, relTol=0.3, maxItr=7, dimKry=33,
                               relTolIn=(0.05, 0.1), maxItrIn=(3, 99))
    assert (ls.RI.relTol, ls.RI.mItr, ls.RI.sD, ls.GM.sD) == (0.3, 7, 33, 33)
    assert (ls.GM.relTol, ls.CG.relTol, ls.GM.mItr, ls.CG.mItr) == (0.05, 0.1, 3, 99)


def test_ls_create_rejects_unknown_type(libpath):
    from svfsi_gb300 import _lib, fsils
    with pytest.raises(_lib.GslsError):
        fsils.FSILS_LS_CREATE(123)


_MIRRORS = {"EqParams": "gsls_eq_params", "EqSolver": "gsls_eq_solver", "CepParams": "gsls_cep_params",
            "Ls": "gsls_ls", "SubLs": "gsls_sub_ls", "StepInfo": "gsls_step_info",
            "AdjPoint": "gsls_adj_point"}


def test_ctypes_mirrors_match_the_header_layout(tmp_path):
    """Every ctypes structure of the Python mirror has the size and field
    offsets that a C compiler gives the header's struct (a probe compiled
    with gcc against include/gsls.h)."""
    import shutil
    import subprocess
    from svfsi_gb300 import _lib
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "gsls.h"', "int main(void) {"]
    expect = []
    for py, c in _MIRRORS.items():
        cls = getattr(_lib, py)
        lines.append(f'  printf("%zu\\n", sizeof({c}));')
        expect.append((py, "sizeof", C.sizeof(cls)))
        for f, _ in cls._fields_:
            lines.append(f'  printf("%zu\\n", offsetof({c}, {f}));')
            expect.append((py, f, getattr(cls, f).offset))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", str(ROOT / "include"), str(src), "-o", str(exe)],
                   check=True)
    got = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert len(got) == len(expect)
    for (py, f, off), g in zip(expect, got):
        assert off == int(g), (py, f, off, g)
