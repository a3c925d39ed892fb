#!/usr/bin/env python
"""Benchmark: seconds per implicit time step (assembly + Krylov) of the
neo-Hookean elastodynamics workload (4x1x1 beam, 176x44x44 hexes -> 2,044,416
tet4, 358,425 nodes, 5,233,801 3x3 CSR blocks; CG + diagonal preconditioner),
mixed precision (FP32 tangent + FP32 inner CG, FP64 residual/Newton) beside
the plain FP64 GPU path, with the relative L2 distance between the two,
and the HBM roofline of the dominant SpMV on both paths (`roofline` for the
FP32 values of the mixed path, `roofline_fp64` for the FP64 one).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gsls|reference]
                  [--workload struct|fluid|cep|lelas|adjoint]

--workload fluid times the VMS Navier-Stokes workload instead (cylinder
R 0.5, L 5, ~1.2M tet4, 4x4 blocks; RCS + NS block solver), the same line
format with its own roofline kernel (the GMRES block SpMV on the K block);
cep the monodomain slab, lelas linear elastodynamics on the beam mesh,
adjoint the discrete adjoint of the beam with a finite-difference check.

--impl reference times W + K real implicit steps of the CPU restatement of the
reference's algorithm (oracle/, coloured OpenMP assembly and OpenMP Krylov
over all host cores) on the same workload from its initial state.  The
default run also steps the oracle beside the GPU for a few steps (the
cpu_baseline sample) and reports the error of the FP64 and the mixed GPU
solution against the oracle's on the full mesh, with the Newton counts of
all three.  N > 1 runs independent replicas (the path does not shard across
GPUs), one per rank.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "s/implicit step (assembly+Krylov), mixed vs FP64 GPU at <=1e-8 rel L2; HBM GB/s"
WORKLOAD = dict(nx=176, ny=44, nz=44)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gsls", choices=["gsls", "reference"])
    ap.add_argument("--small", action="store_true", help="small mesh (debugging only)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--only", choices=["all", "mixed", "fp64"], default="all",
                    help="time one precision only (profiling runs)")
    ap.add_argument("--workload",
                    choices=["struct", "fluid", "cep", "lelas", "heatf", "ustruct", "heats",
                             "adjoint"],
                    default="struct")
    ap.add_argument("--fd-dirs", type=int, default=4,
                    help="adjoint workload: random directions of the central-FD check")
    ap.add_argument("--fd-h", type=float, default=1e-3,
                    help="adjoint workload: relative step of the central differences")
    ap.add_argument("--fluid-h", type=float, default=0.027,
                    help="cylinder mesh spacing (profiling captures use a coarser mesh)")
    ap.add_argument("--cep-amplitude", type=float, default=-52.0,
                    help="cep workload: stimulus amplitude (the configuration's is -52)")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the other configurations' legs of the default run")
    ap.add_argument("--parity-steps", type=int, default=None,
                    help="implicit steps run by the oracle beside the GPU for the "
                         "cpu_baseline and the error against the oracle (default per workload)")
    return ap.parse_args()


def max_over_ranks_(v: float, world: int, device: str) -> float:
    """Slowest rank's time: every rank ran its own replica of the workload
    (no collective on the data path); the job's step time is the maximum."""
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(seconds_per_step_max: float, world: int) -> float:
    """Whole-job seconds per step of N replicas (N steps complete per
    seconds_per_step_max)."""
    return seconds_per_step_max / world


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


def workload(args):
    from svfsi_gb300 import problems
    if args.workload == "ustruct":
        if args.small:
            return problems.ustruct_beam(24, 6, 6, nsteps=args.steps)
        return problems.ustruct_beam(**WORKLOAD, nsteps=args.steps)
    if args.workload == "fluid":
        return problems.fluid_cylinder(h=0.08 if args.small else args.fluid_h, nsteps=args.steps)
    if args.workload == "cep":
        # the configured stimulus amplitude is -52 (under the Aliev-Panfilov
        # sign convention it hyperpolarises the corner: no upstroke);
        # --cep-amplitude 52 times a propagating front instead
        if args.small:
            return problems.cep_slab(27, 27, 6, nsteps=args.steps, A=args.cep_amplitude)
        return problems.cep_slab(nsteps=args.steps, A=args.cep_amplitude)
    if args.workload == "heatf":
        return problems.heatf_cylinder(h=0.08 if args.small else args.fluid_h, nsteps=args.steps)
    if args.workload == "heats":
        # the heat cube: 20^3 hexes, 48,000 tets
        return problems.heats_cube(8 if args.small else 20, nsteps=args.steps)
    if args.workload == "lelas":
        if args.small:
            return problems.lelas_beam(24, 6, 6, nsteps=args.steps)
        return problems.lelas_beam(**WORKLOAD, nsteps=args.steps)
    if args.small:
        return problems.struct_beam(24, 6, 6, nsteps=args.steps)
    return problems.struct_beam(**WORKLOAD, nsteps=args.steps)


def is_fluid(p):
    from svfsi_gb300 import problems
    return p.phys == problems.PHYS_FLUID


def is_heatf(p):
    from svfsi_gb300 import problems
    return p.phys == problems.PHYS_HEATF


def compared_field(p, state):
    """The unknown compared between runs: D (solids), Y (fluid), the
    potential's departure from rest (CEP) or the temperature column of Y
    (HEATF)."""
    if is_heatf(p):
        return state[1][:, p.s]
    if is_cep(p):
        return state[1] - p.cep["V0"]
    return state[1] if (is_fluid(p) or is_heats(p)) else state[2]


def is_cep(p):
    return bool(getattr(p, "cep", None))


def is_ust(p):
    from svfsi_gb300 import problems
    return p.phys == problems.PHYS_USTRUCT


def is_heats(p):
    from svfsi_gb300 import problems
    return p.phys == problems.PHYS_HEATS


def compared_name(p):
    if is_heatf(p):
        return "Y[:, temperature]"
    return ("Y (velocity, pressure)" if is_fluid(p) else "Y - V_rest (potential)" if is_cep(p)
            else "Y (temperature)" if is_heats(p) else "D")


def l2_note(p):
    """What keeps the timed steps from running out of a warm L2 (129 MB)."""
    v32, v64 = p.nnz * p.dof ** 2 * 4 / 1e6, p.nnz * p.dof ** 2 * 8 / 1e6
    if v32 > 129.0:
        return f"inputs larger than L2 (FP32 Val {v32:.0f} MB, FP64 Val {v64:.0f} MB)"
    per_el = (13 * 8 + 64 + 16) * p.nEl / 1e6  # geometry table, element->CSR map, IEN
    return (f"per-step working set larger than L2: every assembly streams the element geometry, "
            f"element->CSR map and IEN ({per_el:.0f} MB) and the state; FP32 Val {v32:.0f} MB")


def workload_desc(p):
    if is_heatf(p):
        return (f"{p.name}: heat carried by a prescribed Poiseuille flow (HEATF3D, peak 30, "
                f"conductivity 0.1, T = 1 on the inlet), {p.nEl:,} tet4, {p.nNo:,} nodes, nnz "
                f"{p.nnz:,}, GMRES+diag, dt 1e-3, {p.maxItr} Newton iterations per step (the "
                f"discontinuity-capturing fixed point converges linearly)")
    if is_heats(p):
        return (f"{p.name}: HEATS3D, conductivity 1, rho 1, T = 1 at x = 0 and 0 at x = 1, "
                f"{p.nEl:,} tet4, {p.nNo:,} nodes, nnz {p.nnz:,}, CG+diag relTol 1e-10, dt 0.01")
    if is_cep(p):
        return (f"{p.name}: monodomain Aliev-Panfilov (FE reaction step), Diso 0.1, stimulus "
                f"{p.cep['A']:+g} for 2 ms on the 1x1x2 corner block, {p.nEl:,} tet4, {p.nNo:,} "
                f"nodes, nnz {p.nnz:,}, CG+diag, dt 0.01, Newton tol 1e-6")
    if is_fluid(p):
        return (f"{p.name}: VMS incompressible Navier-Stokes (rho 1.06, mu 0.04, parabolic "
                f"inlet peak 30, impulsive start), {p.nEl:,} tet4, {p.nNo:,} nodes, nnz "
                f"{p.nnz:,} 4x4 blocks, RCS + NS solver (sD 100, relTol 1e-2), dt 1e-3, Newton "
                f"tol 1e-10")
    if is_ust(p):
        return (f"{p.name}: USTRUCT velocity-pressure neo-Hookean + ST91 solid (VMS, ctM 1e-3), "
                f"E 1e6, nu 0.45, {p.nEl:,} tet4, {p.nNo:,} nodes, nnz {p.nnz:,} 4x4 blocks, "
                f"GMRES+diag, dt 1e-3, Newton tol 1e-8")
    if p.phys == problems_phys_lelas():
        return (f"{p.name}: linear elastodynamics (LELAS3D, E 1e6, nu 0.45), {p.nEl:,} tet4, "
                f"{p.nNo:,} nodes, nnz {p.nnz:,} 3x3 blocks, CG+diag, dt 1e-3, Newton tol 1e-8")
    return (f"{p.name}: neo-Hookean+ST91 elastodynamics, {p.nEl:,} tet4, {p.nNo:,} nodes, "
            f"nnz {p.nnz:,} 3x3 blocks, CG+diag, dt 1e-3, Newton tol 1e-8")


def problems_phys_lelas():
    from svfsi_gb300 import problems
    return problems.PHYS_LELAS


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, n in enumerate(names):
                if f[5 + k].lower() in ("active", "1"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_from_profiles(kernel_key: str):
    f = ROOT / "profiles" / "traffic.json"
    if f.exists():
        d = json.loads(f.read_text())
        v = d.get(kernel_key)
        if v is not None:
            return float(v)
    return None


# ---------------------------------------------------------------------------
def run_gsls(args):
    import torch
    from svfsi_gb300 import _lib, build, fsils, problems
    rank, local, world = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    build.build()
    L = _lib.load()
    _lib.check(L.gsls_init(local), "gsls_init")
    p = workload(args)
    K, W = args.steps, args.warmup

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    def timed_run(precision, profile=False, nsteps=None, nwarm=None):
        nK = K if nsteps is None else nsteps
        nW = W if nwarm is None else nwarm
        lhs, mesh, eq = problems.build_equation(p, precision=precision)
        stream = torch.cuda.ExternalStream(L.gsls_get_stream(lhs.h))
        infos = []
        for _ in range(nW):
            infos.append(eq.step())
        barrier()
        torch.cuda.synchronize()
        if profile:
            L.gsls_profile_reset()
            L.gsls_profile_enable(1)
        n0 = L.gsls_launch_count()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        timed = []
        for _ in range(nK):
            timed.append(eq.step())
        ev1.record(stream)
        ev1.synchronize()
        barrier()
        torch.cuda.synchronize()
        launches = L.gsls_launch_count() - n0
        ms = ev0.elapsed_time(ev1)
        prof = None
        if profile:
            L.gsls_profile_enable(0)
            cnt, tot = C.c_longlong(), C.c_double()
            key = (b"gm_spmv_d3" if is_fluid(p) else b"gm_spmv" if (is_heatf(p) or is_ust(p))
                   else b"cg_spmv")
            L.gsls_profile_read(key, C.byref(cnt), C.byref(tot))
            acnt, atot = C.c_longlong(), C.c_double()
            L.gsls_profile_read(b"assembly", C.byref(acnt), C.byref(atot))
            prof = {"cg_spmv": (cnt.value, tot.value), "assembly": (acnt.value, atot.value)}
            for extra in (b"cg_update", b"cg_pupdate", b"schur", b"schur_calls", b"gm_orth",
                          b"cg_persistent"):
                ec, et = C.c_longlong(), C.c_double()
                if L.gsls_profile_read(extra, C.byref(ec), C.byref(et)) == 0 and ec.value:
                    prof[extra.decode()] = (ec.value, et.value)
        state = eq.get_state()
        res = dict(ms=ms, launches=launches, prof=prof, state=state,
                   newton=np.mean([i.newton_itr for i in timed]),
                   cg=np.mean([i.ls_itr_total for i in timed]),
                   asm_ms=np.mean([i.t_assembly_ms for i in timed]),
                   suc=all(i.last_suc for i in timed))
        eq.free()
        mesh.free()
        lhs.free()
        return res

    def max_over_ranks(v):
        return max_over_ranks_(v, world, "cuda")

    def gpu_steps(precision, n):
        """n implicit steps from the initial state: (state, [(Newton, Krylov)])."""
        lhs, mesh, eq = problems.build_equation(p, precision=precision)
        counts = []
        for _ in range(n):
            i = eq.step()
            counts.append((int(i.newton_itr), int(i.ls_itr_total)))
        st = eq.get_state()
        eq.free()
        mesh.free()
        lhs.free()
        return st, counts

    if args.only != "all":
        # one precision: the plain step time, then the per-kernel times of a
        # separate profiled run (CUDA events around the kernels)
        prec = fsils.PREC_MIXED if args.only == "mixed" else fsils.PREC_FP64
        r = timed_run(prec)
        rp = timed_run(prec, profile=True)
        if rank == 0:
            print(json.dumps({"only": args.only, "ms_per_step": r["ms"] / K, "newton": r["newton"],
                              "cg": r["cg"], "launches": r["launches"],
                              "profiled_ms_per_step": rp["ms"] / K, "prof": rp["prof"]}))
        return
    clocks = ClockSampler(local)
    clocks.start()
    mixed = timed_run(fsils.PREC_MIXED)
    clk = clocks.stop()
    fp64 = timed_run(fsils.PREC_FP64)
    # kernel-level timing (CUDA events around every CG SpMV) in a separate,
    # shorter run so that the headline numbers carry no event overhead
    profd = timed_run(fsils.PREC_MIXED, profile=True, nsteps=2, nwarm=1)
    profd64 = timed_run(fsils.PREC_FP64, profile=True, nsteps=1, nwarm=1)
    ms_mixed = max_over_ranks(mixed["ms"]) / K
    ms_fp64 = max_over_ranks(fp64["ms"]) / K
    D_m, D_f = compared_field(p, mixed["state"]), compared_field(p, fp64["state"])
    rel_l2 = float(np.linalg.norm(D_m - D_f) / np.linalg.norm(D_f))

    # e2e through the public API with host buffers (pinned), H2D + D2H per step
    lhs, mesh, eq = problems.build_equation(p, precision=fsils.PREC_MIXED)
    shp = (p.nNo, p.tDof)
    host = [torch.zeros(shp, dtype=torch.float64).pin_memory() for _ in range(3)]
    hv = [h.numpy() for h in host]
    for h_, s_ in zip(hv, p.initial_state()):
        h_[:] = s_
    for _ in range(W):
        eq.set_state(*hv)
        eq.step()
        eq.get_state(out=hv)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(K):
        eq.set_state(*hv)
        eq.step()
        eq.get_state(out=hv)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0) / K
    eq.free()
    mesh.free()
    lhs.free()
    state_bytes = 3 * p.nNo * p.tDof * 8

    # roofline of the dominant kernel: the CG SpMV + fused dot (struct) or
    # the GMRES SpMV on the 3x3 K block (fluid); FP32 values on the mixed
    # path, FP64 on the drop-in one
    peak, peak_kind = peaks()

    def roofline(prof, s):
        cnt, tot_ms = prof["cg_spmv"]
        t = "float" if s == 4 else "double"
        if "cg_persistent" in prof:
            # small systems run each CG solve as one cooperative launch: the
            # roof is per CG iteration (SpMV + updates), the operator and
            # vectors L2-resident across iterations
            it, ms = prof["cg_persistent"]
            B = p.algorithmic_bytes(s, s)["cg_iter"]
            it_s = (ms / max(it, 1)) / 1e3
            ach = B / it_s / 1e9 if it else None
            r = C.c_double()
            _lib.check(L.gsls_l2_read_rate(C.byref(r)), "gsls_l2_read_rate")
            l2 = r.value / 1e9
            return {"kernel": f"k_cg_persistent<{p.dof},{t},{t}> (every CG iteration of a solve "
                              "in one cooperative launch, two grid barriers per iteration)",
                    "bound": "l2", "achieved": ach, "peak": l2, "unit": "GB/s",
                    "frac": (ach / l2) if ach else None,
                    "peak_source": "measured L2 read bandwidth (gsls_l2_read_rate)",
                    "hbm_frac": (ach / peak) if ach else None,
                    "bytes_per_launch": B, "avg_launch_us": it_s * 1e6, "launches": it,
                    "note": "per CG iteration: B_cg algorithmic bytes / (launch time / "
                            "iterations of the launch)", "traffic": None}
        if is_fluid(p):
            B = p.nnz * (9 * s + 4) + 8 * p.nNo + 2 * p.nNo * 3 * s
            kname = f"k_gm_spmv<3,{t},{t}> (block-CSR SpMV on the K block of the NS solver)"
            tkey = f"gm_spmv_d3_f{8 * s}_fluid_cylinder"
        elif is_heatf(p):
            B = p.algorithmic_bytes(s, s)["spmv"]
            kname = f"k_gm_spmv<1,{t},{t}> (CSR SpMV of the GMRES Arnoldi step)"
            tkey = f"gm_spmv_d1_f{8 * s}_{p.name}"
        elif is_ust(p):
            B = p.algorithmic_bytes(s, s)["spmv"]
            kname = f"k_gm_spmv<4,{t},{t}> (block-CSR SpMV of the GMRES Arnoldi step, 4x4 blocks)"
            tkey = f"gm_spmv_d4_f{8 * s}_{p.name}"
        elif is_cep(p) or is_heats(p):
            B = p.algorithmic_bytes(s, s)["spmv"]
            kname = f"k_cg_spmv<1,{t},{t}> (CSR SpMV + fused P.KP)"
            tkey = f"cg_spmv_d1_f{8 * s}_{p.name}"
        else:
            B = p.algorithmic_bytes(s, s)["spmv"]
            kname = (f"k_cg_spmv_sell<3,{t},{t},{8 if s == 4 else 4}> (sliced block-ELL SpMV + "
                     "fused P.KP, zig-zag order; the first batch of each solve runs k_cg_spmv "
                     "on the CSR)")
            tkey = f"cg_spmv_sell_d3_f{8 * s}_{p.name}"
        avg_s = (tot_ms / max(cnt, 1)) / 1e3
        achieved = B / avg_s / 1e9 if cnt else None
        return {"kernel": kname,
                "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None,
                "peak_source": f"{peak_kind} hbm_gbs", "bytes_per_launch": B,
                "avg_launch_us": avg_s * 1e6, "launches": cnt,
                "traffic": traffic_from_profiles(tkey)}

    roof = roofline(profd["prof"], 4)
    roof64 = roofline(profd64["prof"], 8)
    l2rate = None
    if is_fluid(p):
        # the NS solver's time is the Schur-complement CG (one persistent
        # launch per call, its operator L2-resident): its roof is the L2
        # read bandwidth, measured live
        r = C.c_double()
        _lib.check(L.gsls_l2_read_rate(C.byref(r)), "gsls_l2_read_rate")
        l2rate = r.value / 1e9

        def schur_roof(prof, s):
            cnt, tot_ms = prof.get("schur", (0, 0.0))
            calls, _ = prof.get("schur_calls", (0, 0.0))
            t = "float" if s == 4 else "double"
            B = p.nnz * (7 * s + 4) + 4 * p.nNo + 16 * p.nNo * s
            it_s = (tot_ms / max(cnt, 1)) / 1e3
            ach = B / it_s / 1e9 if cnt else None
            return {"kernel": f"k_schur_persistent<{t},{t}> (CGRAD_SCHUR: every CG iteration "
                              "of one call in one cooperative launch, 3 grid barriers per "
                              "iteration)",
                    "bound": "l2", "achieved": ach, "peak": l2rate, "unit": "GB/s",
                    "frac": (ach / l2rate) if ach else None,
                    "peak_source": "measured L2 read bandwidth (gsls_l2_read_rate)",
                    "bytes_per_iteration": B, "avg_iteration_us": it_s * 1e6,
                    "iterations": cnt, "launches": calls,
                    "note": "per CG iteration: operator mG, Gt, mL and columns "
                            "(nnz (7 s + 4) B) + 16 vector passes; time = launch time / "
                            "iterations of the call"}

        roof_gm, roof_gm64 = roof, roof64
        roof, roof64 = schur_roof(profd["prof"], 4), schur_roof(profd64["prof"], 8)
    # the FP64 SpMV issues one FP64 FMA per matrix entry; GB300 runs FP64 at
    # ~1/74 of FP32, so its roof is the FP64 pipe when that takes longer
    # than the HBM stream (measured live by the library's probe kernel)
    rate = C.c_double()
    _lib.check(L.gsls_fp64_fma_rate(C.byref(rate)), "gsls_fp64_fma_rate")
    d = 3 if is_fluid(p) else p.dof
    fmas = d * d * p.nnz
    if roof64["achieved"] and not is_fluid(p):
        avg_s = roof64["avg_launch_us"] / 1e6
        t_fma, t_hbm = fmas / rate.value, roof64["bytes_per_launch"] / (peak * 1e9)
        hbm = {k: roof64[k] for k in ("achieved", "peak", "unit", "frac", "peak_source", "traffic")}
        if t_fma > t_hbm:
            roof64.update({"bound": "fp64", "achieved": 2 * fmas / avg_s / 1e12,
                           "peak": 2 * rate.value / 1e12, "unit": "TFLOP/s",
                           "frac": t_fma / avg_s,
                           "peak_source": "measured FP64 FMA rate (gsls_fp64_fma_rate)",
                           "fma_per_launch": fmas, "hbm": hbm})

    out = {
        "metric": METRIC, "value": job_value(ms_mixed / 1e3, world), "unit": "s/step",
        "n_gpus": world, "steps": K, "warmup": W, "ms_per_step": ms_mixed,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 tangent+inner CG / f64 residual,Newton,reductions",
        "data": ("synthetic: seeded Delaunay cylinder mesh, no external data"
                 if (is_fluid(p) or is_heatf(p))
                 else "synthetic: Kuhn-split slab mesh, no external data" if is_cep(p)
                 else "synthetic: Kuhn-split unit-cube mesh, no external data" if is_heats(p)
                 else "synthetic: seeded Kuhn-split beam mesh, no external data"),
        "config": {"workload": workload_desc(p), "precision": "mixed",
                   "l2": l2_note(p),
                   "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"},
        "fp64": {"value": ms_fp64 / 1e3 / world, "ms_per_step": ms_fp64,
                 "newton_itr_per_step": fp64["newton"], "cg_itr_per_step": fp64["cg"],
                 "assembly_ms_per_newton": fp64["asm_ms"] / max(fp64["newton"], 1)},
        "mixed": {"newton_itr_per_step": mixed["newton"], "cg_itr_per_step": mixed["cg"],
                  "assembly_ms_per_newton": mixed["asm_ms"] / max(mixed["newton"], 1),
                  "all_solves_converged": bool(mixed["suc"])},
        "ls_itr_note": ("NS outer iterations per step" if is_fluid(p)
                        else "GMRES iterations per step" if (is_heatf(p) or is_ust(p))
                        else "CG iterations per step"),
        "speedup_mixed_vs_fp64": ms_fp64 / ms_mixed,
        "rel_l2_mixed_vs_fp64": rel_l2,
        "roofline": roof,
        "roofline_fp64": roof64,
        "e2e": {"value": e2e_s / world, "unit": "s/step", "h2d_bytes_per_step": state_bytes,
                "d2h_bytes_per_step": state_bytes},
        "gpu_launches": int(mixed["launches"]),
        "clocks": clk,
    }
    if is_fluid(p):
        out["roofline_gm_spmv"] = roof_gm
        out["roofline_gm_spmv_fp64"] = roof_gm64
    if rank == 0 and world == 1 and not args.no_cpu:
        # the oracle's own implicit steps of the workload (timed: the CPU
        # baseline) and the same steps on the GPU in both precisions: the
        # error of each against the oracle's FP64 solution on the full mesh
        n = args.parity_steps or PARITY_STEPS[args.workload]
        threads = os.cpu_count() or 1
        so, secs, co = oracle_steps(p, n, threads)
        s64, c64 = gpu_steps(fsils.PREC_FP64, n)
        smx, cmx = gpu_steps(fsils.PREC_MIXED, n)
        ref = compared_field(p, so)
        nref = float(np.linalg.norm(ref))
        e64 = float(np.linalg.norm(compared_field(p, s64) - ref)) / nref
        emx = float(np.linalg.norm(compared_field(p, smx) - ref)) / nref
        out["rel_l2_fp64_vs_oracle"] = e64
        out["rel_l2_mixed_vs_oracle"] = emx
        out["parity_vs_oracle"] = {
            "steps": n, "field": compared_name(p), "norm_oracle": nref,
            "newton_oracle": [c[0] for c in co], "newton_fp64": [c[0] for c in c64],
            "newton_mixed": [c[0] for c in cmx],
            "ls_itr_oracle": [c[1] for c in co], "ls_itr_fp64": [c[1] for c in c64],
            "ls_itr_mixed": [c[1] for c in cmx],
            "newton_counts_equal": ([c[0] for c in co] == [c[0] for c in c64] ==
                                    [c[0] for c in cmx])}
        out["cpu_baseline"] = {"value": float(sum(secs) / len(secs)), "unit": "s/step",
                               "cores": threads, "kind": "port",
                               "sample": oracle_sample_desc(p, n, threads, co, 1),
                               "step_s": secs}
    if (rank == 0 and world == 1 and not args.no_cpu and not args.no_configs and not args.small
            and args.workload == "struct"):
        try:
            out["configs"] = config_legs(L, problems, fsils, torch)
        except Exception as e:  # the headline line is printed regardless
            out["configs"] = {"error": f"{type(e).__name__}: {e}"}
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def config_legs(L, problems, fsils, torch):
    """The other benchmark configurations, run briefly beside the headline
    one: the heat cube (20^3 hexes, 48,000 tets), the monodomain slab
    (135x135x27 hexes, 2,952,450 tets, stimulus -52) and the VMS cylinder
    (h 0.027, 1,225,440 tets).  For each, the oracle's first n_par implicit
    steps from the initial state beside the FP64 and mixed GPU steps (error
    of each against the oracle, Newton counts), then n_time more GPU steps
    per precision timed with CUDA events on the library's stream.  The
    cylinder runs its configured 20 steps, the heat cube its 10 steps twice.
    The slab with the configured stimulus -52 runs 250 steps: it
    hyperpolarises the corner below -110 mV, where the Aliev-Panfilov
    recovery term mu1 X2 / (mu2 + X1) has its pole, and on this mesh a node
    lands close enough to the pole near step 257 that the reference's model
    state becomes non-finite (the oracle, FP64 and mixed alike).  The
    configured 5,000 steps are timed with the depolarising stimulus +52 (a
    propagating front)."""
    threads = os.cpu_count() or 1
    legs = [("heats_cube_20", lambda: problems.heats_cube(20, nsteps=20), 10, 10),
            ("cep_slab_135x135x27", lambda: problems.cep_slab(nsteps=250, A=-52.0), 20, 230),
            ("cep_slab_135x135x27_stim+52", lambda: problems.cep_slab(nsteps=5000, A=52.0), 20,
             4980),
            ("fluid_cylinder_h0.027", lambda: problems.fluid_cylinder(h=0.027, nsteps=20), 1, 19)]
    res = {}
    for name, make, n_par, n_time in legs:
        p = make()
        so, secs, co = oracle_steps(p, n_par, threads)
        ref = compared_field(p, so)
        nref = float(np.linalg.norm(ref))
        leg = {"workload": workload_desc(p),
               "oracle": {"s_per_step": float(sum(secs) / len(secs)), "cores": threads,
                          "steps": n_par, "newton": [c[0] for c in co],
                          "ls_itr": [c[1] for c in co], "kind": "port"}}
        fields = {}
        for prec, key in ((fsils.PREC_FP64, "fp64"), (fsils.PREC_MIXED, "mixed")):
            lhs, mesh, eq = problems.build_equation(p, precision=prec)
            stream = torch.cuda.ExternalStream(L.gsls_get_stream(lhs.h))
            newton = [int(eq.step().newton_itr) for _ in range(n_par)]
            st = eq.get_state()
            leg[f"rel_l2_{key}_vs_oracle"] = float(np.linalg.norm(compared_field(p, st) - ref)) / nref
            leg[f"newton_{key}"] = newton
            torch.cuda.synchronize()
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            infos = [eq.step() for _ in range(n_time)]
            ev1.record(stream)
            ev1.synchronize()
            leg[f"{key}_s_per_step"] = ev0.elapsed_time(ev1) / 1e3 / n_time
            leg[f"{key}_newton_per_step"] = float(np.mean([i.newton_itr for i in infos]))
            leg[f"{key}_ls_itr_per_step"] = float(np.mean([i.ls_itr_total for i in infos]))
            leg[f"{key}_assembly_ms_per_newton"] = float(
                np.mean([i.t_assembly_ms for i in infos]) / max(leg[f"{key}_newton_per_step"], 1))
            fields[key] = compared_field(p, eq.get_state())
            eq.free()
            mesh.free()
            lhs.free()
        leg["speedup_mixed_vs_fp64"] = leg["fp64_s_per_step"] / leg["mixed_s_per_step"]
        leg["rel_l2_mixed_vs_fp64"] = float(np.linalg.norm(fields["mixed"] - fields["fp64"]) /
                                            max(np.linalg.norm(fields["fp64"]), 1e-300))
        leg["newton_counts_equal"] = (leg["newton_fp64"] == leg["newton_mixed"] ==
                                      leg["oracle"]["newton"])
        leg["timed"] = (f"steps {n_par + 1}..{n_par + n_time} of the workload per precision "
                        f"(CUDA events); the error columns compare steps 1..{n_par} with the "
                        f"oracle's (field: {compared_name(p)})")
        res[name] = leg
    return res


# ---------------------------------------------------------------------------
# CPU side: real implicit steps of the oracle (the C restatement of the
# reference's algorithm, FP64), assembled colour by colour with OpenMP and
# solved with OpenMP SpMVs and reductions on all host threads.

# implicit steps the oracle runs beside the GPU in the default bench run: the
# cpu_baseline sample and the full-size error against the oracle's solution
PARITY_STEPS = {"struct": 2, "lelas": 2, "fluid": 1, "heatf": 2, "cep": 20, "ustruct": 1,
                "heats": 10}


def oracle_steps(p, nsteps, threads, warm=0):
    """Run warm + nsteps implicit steps of the workload on the oracle from
    its initial state.  Returns the final state (A, Y, D), the seconds of
    each of the last nsteps steps and their (Newton, Krylov) counts."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    O.set_threads(threads)
    eq = O.OracleEquation(p, colored=True)
    eq.set_state(*p.initial_state())
    secs, counts = [], []
    for k in range(warm + nsteps):
        t0 = time.perf_counter()
        info = eq.step()
        dt = time.perf_counter() - t0
        if k >= warm:
            secs.append(dt)
            counts.append((int(info.newton_itr), int(info.ls_itr_total)))
    return eq.state(), secs, counts


def krylov_name(p):
    return "NS outer" if is_fluid(p) else "GMRES" if (is_heatf(p) or is_ust(p)) else "CG"


def oracle_sample_desc(p, n, threads, counts, first):
    newton = [c[0] for c in counts]
    ls = [c[1] for c in counts]
    return (f"{n} implicit steps (steps {first}..{first + n - 1} of the workload) run in full "
            f"by the oracle (C restatement of the reference's algorithm, FP64; coloured OpenMP "
            f"assembly, OpenMP SpMV/reductions) on {threads} host threads: Newton iterations "
            f"per step {newton}, {krylov_name(p)} iterations per step {ls}")


def run_reference(args):
    """The reference arm: the oracle's own implicit steps of the workload on
    the host cores, W untimed then K timed, from the workload's initial
    state (no counts borrowed from the GPU run)."""
    rank, local, world = dist_env()
    if rank != 0:
        return
    p = workload(args)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    _, secs, counts = oracle_steps(p, args.steps, threads, warm=args.warmup)
    wall = time.perf_counter() - t0
    v = float(sum(secs) / len(secs))
    sample = oracle_sample_desc(p, args.steps, threads, counts, args.warmup + 1)
    data = ("synthetic: seeded Delaunay cylinder mesh, no external data"
            if (is_fluid(p) or is_heatf(p))
            else "synthetic: Kuhn-split slab mesh, no external data" if is_cep(p)
            else "synthetic: Kuhn-split unit-cube mesh, no external data" if is_heats(p)
            else "synthetic: seeded Kuhn-split beam mesh, no external data")
    out = {"metric": METRIC, "value": v, "unit": "s/step", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": v * 1e3, "higher_is_better": False,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
           "data": data,
           "config": {"workload": workload_desc(p), "precision": "fp64 (reference CPU)"},
           "cpu_baseline": {"value": v, "unit": "s/step", "cores": threads, "kind": "port",
                            "sample": sample},
           "oracle": {"newton_itr_per_step": float(np.mean([c[0] for c in counts])),
                      "ls_itr_per_step": float(np.mean([c[1] for c in counts])),
                      "ls_itr_note": f"{krylov_name(p)} iterations per step",
                      "timed_s": float(sum(secs)), "wall_s_with_warmup": wall},
           "e2e": {"value": v, "unit": "s/step", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def run_adjoint(args):
    """Adjoint of the elastodynamics workload: per-element shear modulus
    mu_e = 3.45e5 exp(0.2 N(0,1)) (seeded), J = 1/2 |u_tip - u_target|^2 with
    u_target from a seeded perturbed-mu run, checkpoints every 5 steps; times
    the forward (with checkpoints) + backward pass and checks the gradient
    against central finite differences along seeded directions."""
    import torch
    from svfsi_gb300 import _lib, build, fsils, meshgen, problems
    rank, local, world = dist_env()
    torch.cuda.set_device(local)
    build.build()
    L = _lib.load()
    _lib.check(L.gsls_init(local), "gsls_init")
    nsteps = args.steps if args.steps else 10
    if args.small:
        p = problems.struct_beam(24, 6, 6, nsteps=nsteps)
    else:
        p = problems.struct_beam(**WORKLOAD, nsteps=nsteps)
    p.tol, p.maxItr, p.ls_relTol = 1e-12, 25, 1e-8
    rng = np.random.default_rng(20261203)
    mu = 3.45e5 * np.exp(0.2 * rng.standard_normal(p.nEl))
    c10 = 0.5 * mu
    tip = meshgen.nodes_on_plane(p.x, 0, 4.0)

    lhs, mesh, eq = problems.build_equation(p)
    eq.free()

    def forward(e):
        # a fresh equation on the one lhs and mesh (graph, colouring and
        # geometry are built once)
        f = problems.equation_on(p, mesh)
        f.set_eparam(e)
        for _ in range(nsteps):
            f.step()
        D = f.get_state()[2]
        f.free()
        return D

    t_pert = c10 * np.exp(0.05 * rng.standard_normal(p.nEl))
    target = forward(t_pert)[tip]

    def J(D):
        d = D[tip] - target
        return 0.5 * float(np.sum(d * d))

    def adjoint(precision):
        """forward with checkpoints + backward; (gradient w.r.t. mu, J,
        forward s, backward s)"""
        e = problems.equation_on(p, mesh, precision)
        e.set_eparam(c10)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tape = e.adjoint_forward(nsteps, every=5)
        t1 = time.perf_counter()
        DN = e.get_state()[2]
        bar = np.zeros_like(DN)
        bar[tip] = DN[tip] - target
        g_c10 = tape.backward(Dbar=bar)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        tape.free()
        e.free()
        return 0.5 * g_c10, J(DN), t1 - t0, t2 - t1

    g64, J64, f64s, b64s = adjoint(fsils.PREC_FP64)
    gmx, Jmx, fmxs, bmxs = adjoint(fsils.PREC_MIXED)
    h = args.fd_h
    errs, errs_mx, pairs = [], [], []
    for k in range(args.fd_dirs):
        r = rng.standard_normal(p.nEl)
        r /= np.linalg.norm(r)
        dmu = mu * r
        fd = (J(forward(0.5 * (mu + h * dmu))) - J(forward(0.5 * (mu - h * dmu)))) / (2 * h)
        ad, am = float(g64 @ dmu), float(gmx @ dmu)
        errs.append(abs(fd - ad) / abs(ad))
        errs_mx.append(abs(fd - am) / abs(am))
        pairs.append([fd, ad, am])
        print(f"direction {k}: fd {fd:.10e} adjoint fp64 {ad:.10e} mixed {am:.10e} "
              f"rel {errs[-1]:.2e} / {errs_mx[-1]:.2e}", file=sys.stderr, flush=True)
    mesh.free()
    lhs.free()
    rms = float(np.sqrt(np.mean([b * b for _, b, _ in pairs]))) if pairs else None
    out = {"metric": "adjoint s/step (forward with checkpoints + backward), mixed vs FP64",
           "impl": "gsls", "value": (fmxs + bmxs) / nsteps, "unit": "s/step", "n_gpus": 1,
           "steps": nsteps, "higher_is_better": False,
           "dtype": "f32 tangent+inner CG / f64 residual,Newton, refinement of the transpose "
                    "solves",
           "data": "synthetic: seeded Kuhn-split beam",
           "config": {"workload": workload_desc(p) + "; per-element mu log-normal sigma 0.2, "
                      "checkpoint every 5, Newton tol 1e-12", "params": p.nEl},
           "mixed": {"forward_s": fmxs, "backward_s": bmxs, "J": Jmx},
           "fp64": {"value": (f64s + b64s) / nsteps, "forward_s": f64s, "backward_s": b64s,
                    "J": J64},
           "speedup_mixed_vs_fp64": (f64s + b64s) / (fmxs + bmxs),
           "grad_rel_l2_mixed_vs_fp64": float(np.linalg.norm(gmx - g64) / np.linalg.norm(g64)),
           "fd_check": {"directions": args.fd_dirs, "h_rel": h, "fd_ad_fp64_ad_mixed": pairs,
                        "rel_errs_fp64": errs, "rel_errs_mixed": errs_mx,
                        # FD noise is absolute: normalise by the RMS directional derivative
                        "max_err_over_rms_fp64": (max(abs(a - b) for a, b, _ in pairs) / rms)
                        if pairs else None,
                        "max_err_over_rms_mixed": (max(abs(a - c) for a, _, c in pairs) / rms)
                        if pairs else None}}
    print(json.dumps(out))


def main():
    args = parse()
    if args.workload == "adjoint":
        run_adjoint(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gsls(args)


if __name__ == "__main__":
    main()
