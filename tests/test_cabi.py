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


def _fortran_bind_c_types(path):
    """(name -> [(field, kind, count)]) of the BIND(C) derived types of a
    free-form Fortran source: kind C_INT / C_DOUBLE / C_PTR or the name of a
    nested type, count the array extent (1 for scalars)."""
    import re
    types, cur = {}, None
    for raw in Path(path).read_text().splitlines():
        line = raw.split("!")[0].strip()
        m = re.match(r"TYPE\s*,\s*BIND\(C\)\s*::\s*(\w+)", line, re.I)
        if m:
            cur = types.setdefault(m.group(1).lower(), [])
            continue
        if cur is not None and re.match(r"END\s*TYPE", line, re.I):
            cur = None
            continue
        if cur is None or "::" not in line:
            continue
        decl, names = line.split("::", 1)
        m = re.match(r"(INTEGER|REAL)\s*\(\s*(C_\w+)\s*\)|TYPE\s*\(\s*(\w+)\s*\)", decl.strip(), re.I)
        assert m, raw
        kind = (m.group(2) or m.group(3)).upper()
        for item in re.sub(r"=\s*[^,]+", "", names).split(","):
            item = item.strip()
            a = re.match(r"(\w+)\s*(?:\((\d+)\))?", item)
            cur.append((a.group(1).lower(), kind, int(a.group(2) or 1)))
    return types


def test_fortran_interop_types_mirror_the_header():
    """The Fortran module's BIND(C) types (svfsi_gb300/fortran/gsls_c.f90)
    declare the header's structs field for field: same order, same
    interoperable kinds and array extents as the ctypes mirror, whose
    offsets the probe above pins to include/gsls.h.  (No Fortran compiler
    here: this reads the declarations.)"""
    from svfsi_gb300 import _lib
    ft = _fortran_bind_c_types(ROOT / "svfsi_gb300" / "fortran" / "gsls_c.f90")
    pairs = {"gsls_sub_ls": _lib.SubLs, "gsls_ls": _lib.Ls, "gsls_eq_params": _lib.EqParams}
    names = {_lib.SubLs: "GSLS_SUB_LS"}
    for fname, cls in pairs.items():
        assert fname in ft, fname
        want = []
        for f, t in cls._fields_:
            if t is C.c_int:
                want.append((f.lower(), "C_INT", 1))
            elif t is C.c_double:
                want.append((f.lower(), "C_DOUBLE", 1))
            elif isinstance(t, type) and issubclass(t, C.Array) and t._type_ is C.c_double:
                want.append((f.lower(), "C_DOUBLE", t._length_))
            elif isinstance(t, type) and issubclass(t, C._Pointer):
                want.append((f.lower(), "C_PTR", 1))
            else:
                want.append((f.lower(), names[t], 1))
        assert ft[fname] == want, (fname, ft[fname], want)


def test_fortran_bindings_name_exported_symbols(libpath):
    """Every C entry point the Fortran module binds (BIND(C, NAME=...)) is
    declared in include/gsls.h and exported by the library."""
    import re
    src = (ROOT / "svfsi_gb300" / "fortran" / "gsls_c.f90").read_text()
    bound = sorted(set(re.findall(r'BIND\(C,\s*NAME="(\w+)"\)', src)))
    assert "gsls_solve" in bound and "gsls_assemble" in bound
    declared = set(declared_functions())
    lib = C.CDLL(str(libpath))
    assert [n for n in bound if n not in declared] == []
    assert [n for n in bound if not hasattr(lib, n)] == []
