"""Full-size parity: the benchmark meshes stepped by the GPU (FP64 drop-in
and mixed precision) beside the oracle's own FP64 implicit steps from the
same initial state, on all host cores (coloured OpenMP assembly).

* beam, neo-Hookean + ST91: 176x44x44 hexes -> 2,044,416 tet4, 2 steps;
* monodomain slab, Aliev-Panfilov: 135x135x27 hexes -> 2,952,450 tet4,
  stimulus -52 (the configured amplitude), 20 steps;
* cylinder, VMS Navier-Stokes + RCS + NS solver: h 0.027 -> 1,225,440 tet4,
  1 step;
* the beam with linear elasticity (LELAS3D), 2 steps, and the cylinder with
  heat carried by a Poiseuille flow (HEATF3D, 10 Newton iterations per
  step), 2 steps.

Bar: identical Newton counts per step; the FP64 GPU state within 1e-10
relative L2 of the oracle's and the mixed one within 1e-8 (the Newton
iteration on the FP64 residual refines the FP32 tangent and inner Krylov
solve to the FP64 fixed point).  Newton stop rule: F/PIC.f:263-275.
"""
import os

import numpy as np
import pytest

from svfsi_gb300 import fsils, problems

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, float).ravel(), np.asarray(b, float).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _oracle(orc, p, n):
    orc.set_threads(os.cpu_count() or 1)
    try:
        eq = orc.OracleEquation(p, colored=True)
        eq.set_state(*p.initial_state())
        newton = [eq.step().newton_itr for _ in range(n)]
        return eq.state(), newton
    finally:
        orc.set_threads(1)


def _gpu(p, n, precision):
    lhs, mesh, eq = problems.build_equation(p, precision=precision)
    try:
        newton = [eq.step().newton_itr for _ in range(n)]
        return eq.get_state(), newton
    finally:
        eq.free()
        mesh.free()
        lhs.free()


def _check(orc, p, n, field, fp64_tol=1e-10, mixed_tol=1e-8):
    so, no = _oracle(orc, p, n)
    s64, n64 = _gpu(p, n, fsils.PREC_FP64)
    smx, nmx = _gpu(p, n, fsils.PREC_MIXED)
    ref = field(so)
    assert np.linalg.norm(ref) > 0
    e64, emx = rel(field(s64), ref), rel(field(smx), ref)
    print(f"{p.name}: newton oracle {no} fp64 {n64} mixed {nmx}; rel L2 fp64 {e64:.3e} "
          f"mixed {emx:.3e}")
    assert n64 == no and nmx == no
    assert e64 < fp64_tol
    assert emx < mixed_tol


def test_struct_beam_full_size(gsls, orc):
    p = problems.struct_beam(nsteps=2)
    assert (p.nEl, p.nNo, p.nnz) == (2_044_416, 358_425, 5_233_801)
    _check(orc, p, 2, lambda s: s[2])


def test_cep_slab_full_size(gsls, orc):
    p = problems.cep_slab(nsteps=20, A=-52.0)
    assert (p.nEl, p.nNo, p.nnz) == (2_952_450, 517_888, 7_560_622)
    # the potential's departure from rest (the field itself is ~-80 mV
    # almost everywhere)
    v0 = p.cep["V0"]
    _check(orc, p, 20, lambda s: s[1] - v0)


def test_fluid_cylinder_full_size(gsls, orc):
    p = problems.fluid_cylinder(h=0.027, nsteps=1)
    assert p.nEl == 1_225_440
    _check(orc, p, 1, lambda s: s[1])


def test_lelas_beam_full_size(gsls, orc):
    p = problems.lelas_beam(nsteps=2)
    assert (p.nEl, p.nNo, p.nnz) == (2_044_416, 358_425, 5_233_801)
    _check(orc, p, 2, lambda s: s[2])


def test_heatf_cylinder_full_size(gsls, orc):
    p = problems.heatf_cylinder(h=0.027, nsteps=2)
    assert p.nEl == 1_225_440
    # the temperature column (the velocity is prescribed and carried unchanged)
    _check(orc, p, 2, lambda s: s[1][:, 4])
