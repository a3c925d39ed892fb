"""Restart files in the reference's layout (WRITERESTART / INITFROMBIN,
Code/Source/svFSI/OUTPUT.f:132-232, INITIALIZE.f:152-163 and 508-621):

* the record is stamp(7), cTS (int32), time, cpu time, eq%iNorm, Y, A
  [, D] [, Xion] (float64), of exactly the reference's record length
  IKIND*(1+7) + RKIND*(2 + nEq + nX + i*tnNo);
* a run interrupted by write/read continues bit for bit as the
  uninterrupted run (state, time, Newton normalisation and cell state
  restored), in FP64 and in mixed precision (whose solver caches -- the kept
  linear tangent, the first CG batch size -- change no arithmetic);
* a file of another problem is rejected, naming the stamp field.
"""
import numpy as np
import pytest

from svfsi_gb300 import fsils, problems
from svfsi_gb300._lib import GslsError

PRECS = {"fp64": fsils.PREC_FP64, "mixed": fsils.PREC_MIXED}

pytestmark = pytest.mark.gpu


def _parse(path, nNo, tDof, dFlag, nxion=0):
    raw = open(path, "rb").read()
    ints = np.frombuffer(raw[:32], dtype=np.int32)
    f = np.frombuffer(raw[32:], dtype=np.float64)
    n = nNo * tDof
    out = {"stamp": ints[:7].tolist(), "cTS": int(ints[7]), "time": f[0], "cpu": f[1],
           "iNorm": f[2], "Y": f[3:3 + n].reshape(nNo, tDof),
           "A": f[3 + n:3 + 2 * n].reshape(nNo, tDof)}
    k = 3 + 2 * n
    if dFlag:
        out["D"] = f[k:k + n].reshape(nNo, tDof)
        k += n
    if nxion:
        out["Xion"] = f[k:k + nxion * nNo].reshape(nNo, nxion)
        k += nxion * nNo
    assert k == f.size
    i = (3 if dFlag else 2) * tDof + nxion
    assert len(raw) == 4 * (1 + 7) + 8 * (2 + 1 + 0 + i * nNo)  # INITIALIZE.f:156-163
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_struct_restart_layout_and_bitwise_resume(gsls, tmp_path, precision):
    p = problems.struct_beam(8, 2, 2, nsteps=4)
    _, _, ref = problems.build_equation(p, precision=PRECS[precision])
    for _ in range(4):
        ref.step()
    Ar, Yr, Dr = ref.get_state()
    _, _, eq = problems.build_equation(p, precision=PRECS[precision])
    for _ in range(2):
        eq.step()
    f = tmp_path / "stFile_last.bin"
    eq.write_restart(f, 2, 1.5)
    A2, Y2, D2 = eq.get_state()
    rec = _parse(f, p.nNo, 3, True)
    assert rec["stamp"] == [1, 1, 1, p.nNo, 0, 3, 1]
    assert rec["cTS"] == 2 and rec["cpu"] == 1.5
    assert rec["time"] == pytest.approx(2 * p.params["dt"], rel=1e-15)
    assert rec["iNorm"] > 0
    assert np.array_equal(rec["Y"], Y2) and np.array_equal(rec["A"], A2)
    assert np.array_equal(rec["D"], D2)
    _, _, res = problems.build_equation(p, precision=PRECS[precision])
    cts, cpu = res.read_restart(f)
    assert (cts, cpu) == (2, 1.5)
    for _ in range(2):
        res.step()
    A, Y, D = res.get_state()
    assert np.array_equal(A, Ar) and np.array_equal(Y, Yr) and np.array_equal(D, Dr)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cep_restart_carries_the_cell_state(gsls, tmp_path, precision):
    p = problems.cep_slab(6, 6, 2, nsteps=6, A=52.0)
    _, _, ref = problems.build_equation(p, precision=PRECS[precision])
    for _ in range(6):
        ref.step()
    Yr = ref.get_state()[1]
    _, _, eq = problems.build_equation(p, precision=PRECS[precision])
    for _ in range(3):
        eq.step()
    f = tmp_path / "cep.bin"
    eq.write_restart(f, 3)
    rec = _parse(f, p.nNo, 1, False, nxion=2)
    assert rec["stamp"] == [1, 1, 1, p.nNo, 0, 1, 0]
    _, _, res = problems.build_equation(p, precision=PRECS[precision])
    res.read_restart(f)
    for _ in range(3):
        res.step()
    assert np.array_equal(res.get_state()[1], Yr)


def test_restart_of_another_mesh_is_rejected(gsls, tmp_path):
    p = problems.struct_beam(8, 2, 2, nsteps=1)
    _, _, eq = problems.build_equation(p)
    eq.step()
    f = tmp_path / "a.bin"
    eq.write_restart(f, 1)
    q = problems.struct_beam(6, 2, 2, nsteps=1)
    _, _, other = problems.build_equation(q)
    with pytest.raises(GslsError, match="Number of nodes"):
        other.read_restart(f)
