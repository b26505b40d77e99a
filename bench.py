#!/usr/bin/env python3
"""Benchmark: Stokes solve time to a 1e-8 coupled relative residual on the 8M-DOF shell.

Workload: level-5 icosahedral shell, 32 layers (1,966,080 curved P2 tets, 7,987,590 velocity
DOF), eta = eta0 exp(-gamma T) with a 1e4 contrast and a 30x jump below 660 km, 12 seeded plate
caps at the surface, free slip at the CMB. One step = one hot-path pass: rebuild the element
operator, Galerkin hierarchy and coarse inverse from the resident inputs and run the Patera / MG-PCG
solve from P = 0 until the coupled FP64 residual is below 1e-8.

Arms:
  default (--impl gb300): FP32 V-cycle with the learned element smoother (one learned sweep per side
      on the two finest levels, weights trained on the 130k-DOF shell; weighted Jacobi below) inside
      FP64 outer CG / Patera on the GPU (libm3sph.so); `value` is its solve time. Beside it, on the
      same GPU: the plain-FP64 path and the Jacobi-smoothed FP32 solve of the same shell; the same
      three solves on the 130k-DOF shell next to the FP64 oracle's full solve of it on the host
      (`c1`); on the 64M-DOF shell (`c5`) one learned and one plain-FP64 solve to 1e-8 and
      device-resident time steps (GPlates surface velocities -> rock_prop -> Stokes -> calculate_dt
      -> semi-Lagrangian advection); semi-Lagrangian rates on the 130k-DOF shell.
  --impl reference: the FP64 CPU oracle (numpy/scipy restatement of the reference algorithm with
      OpenMP sparse products on all host threads): one step = one full solve of the 130k-DOF shell
      (set-up + Patera / MG-PCG to a 1e-8 coupled residual), timed, not extrapolated.

Prints one JSON line. Multi-GPU runs are independent replicas (the solve does not shard).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
import traceback
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Stokes solve time to 1e-8 rel. residual: learned+FP32-MG vs plain FP64 on 1 GPU"
TARGET = 1e-8
# Patera / MG-PCG tolerances: the reference's rtol_U (5e-3) and a pressure tolerance that the
# coupled-residual check tightens (x0.1) until the 1e-8 target is met
SOLVER_KW = dict(rtol_Pat=1e-7, rtol_U=5e-3, itmax_Pat=400, itmax_U=40, target_rel_residual=TARGET)
# accuracy checks: the plain FP64 solution continued from its pressure to a 1e-11 coupled residual,
# the learned FP32-MG path solved from zero to 1e-11 (warm-started from an already converged
# pressure its inner solves can stall); at a 1e-8 residual two solutions of the high-contrast
# shells may still differ by a few 1e-8 in U
TIGHT = 1e-11
TIGHT_KW = dict(rtol_Pat=1e-10, rtol_U=5e-3, itmax_Pat=400, itmax_U=40, target_rel_residual=TIGHT)


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as td
        td.init_process_group("gloo", init_method="env://")
        return rank, ws, td
    return 0, 1, None


def barrier(td):
    if td is not None:
        td.barrier()


def allmax(td, v):
    if td is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, out):
        self.out = out
        self.p = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.out, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p is not None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()
            self.f.close()

    def summary(self, dev=0):
        try:
            rows = [r.split(",") for r in open(self.out).read().strip().splitlines()]
        except OSError:
            return None
        rows = [[c.strip() for c in r] for r in rows if len(r) >= 9 and r[0].strip() == str(dev)]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def clock_csv_path():
    """A private temporary file for the nvidia-smi samples (M3SPH_CLOCKS_CSV overrides it)."""
    import tempfile
    p = os.environ.get("M3SPH_CLOCKS_CSV")
    if p:
        return p
    fd, p = tempfile.mkstemp(prefix="m3sph_clocks_", suffix=".csv")
    os.close(fd)
    return p


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


# DRAM bytes per element of one streamed FP32 apply (both kernels), from the ncu capture of the
# 491,520-element shell: (948.76 + 20.05 + 83.85 + 4.28) MB / 491,520
TRAFFIC_PER_ELEMENT_F32 = (948.76e6 + 20.05e6 + 83.85e6 + 4.28e6) / 491520
# the same for the partially assembled FP32 apply (k_pa_elem_f32 + k_node_gather_f32)
TRAFFIC_PER_ELEMENT_PA = (289.01e6 + 19.20e6 + 83.85e6 + 4.28e6) / 491520
# the same for the double-float outer apply (k_stream_rowlane<RlDF> + k_node_gather_f64)
TRAFFIC_PER_ELEMENT_DF = (1.900e9 + 72.74e6 + 190.52e6 + 10.03e6) / 491520


def algorithmic_apply_bytes(nel, ndof, nvnod, s):
    """Algorithmic bytes of one matrix-free operator application y = K x (the per-unit figure of
    the hot-path scope): x read and y written in the vector precision s, 10 int32 connectivity
    entries and a class byte per element, (theta, phi, r) and log-viscosity of every vertex."""
    return 2 * s * ndof + 40 * nel + nel + (24 + 8) * nvnod


def apply_bytes_df(nel, ndof):
    """Algorithmic bytes of one double-float outer apply: two FP32 packed matrices per element,
    connectivity, x read and y written in FP64."""
    return nel * (2 * 465 * 4 + 40) + 2 * 8 * ndof


def apply_bytes_pa(nel, ndof, nnod):
    """Bytes one partially assembled FP32 apply streams: 14 x 9 FP32 factors, a free-dof word and
    10 int32 connectivity entries per element, 16 B of rotation angles per node, x and y in FP32."""
    return nel * (504 + 4 + 40) + 16 * nnod + 2 * 4 * ndof


def apply_bytes(nel, ndof, s):
    """Algorithmic bytes of one element-by-element operator application: packed element
    matrices (465 values), connectivity (10 int32), x read and y written once."""
    return nel * (465 * s + 40) + 2 * s * ndof


def run_gb300(args, rank, ws, td):
    from m3tet_sph_gb300 import build as B
    B.build()
    from m3tet_sph_gb300 import _lib, stokes, workloads
    import torch
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    t0 = time.time()
    w = workloads.make_workload(args.workload, seed=args.seed)
    t_mesh = time.time() - t0
    lv0 = w["levels"][0]
    nel, ndof = lv0["nel"], 3 * lv0["nnod"]
    nvnod = int(lv0["EL2NOD"][:, :4].max()) + 1
    dm = stokes.DeviceMesh(w["levels"], device=dev)
    dm.set_option("fp32_operator", args.fp32_operator)
    torch.cuda.set_device(dev)
    wfile = ROOT / "m3tet_sph_gb300" / "smoother_c1.npy"
    use_learned = not args.skip_learned

    def setup(prec):
        dm.setup(w["visc"], w["dens"], w["ifix"], w["vfix"], w["phys"], precision=prec)

    # ---- plain FP64 path (same inputs) ----
    plain = None
    if not args.skip_plain:
        setup(0)
        for _ in range(args.plain_warmup):
            dm.step_device(**SOLVER_KW)
        barrier(td)
        torch.cuda.synchronize()
        t = time.perf_counter()
        infos64 = [dm.step_device(**SOLVER_KW) for _ in range(args.plain_steps)]
        torch.cuda.synchronize()
        t_plain = allmax(td, (time.perf_counter() - t) / args.plain_steps)
        plain = dict(s_per_solve=t_plain, info=infos64[-1])
        U64, P64 = dm.solution()
        U64t, P64t, i64t = dm.solve(P0=P64, allow_not_converged=True, **TIGHT_KW)
        fp64_apply_ms = dm.apply_timing(0, 0, 5)
    # ---- the product: FP32 V-cycle with the learned element smoother (one learned sweep per
    # side on the two finest levels) inside FP64 outer CG / Patera; timed region ----
    setup(1)
    if use_learned:
        from m3tet_sph_gb300 import learned as LS
        LS.set_params(dm, np.load(wfile), trained=True)
        dm.set_option("ml_schedule", 1)
    sm = 1 if use_learned else 0
    stream = torch.cuda.ExternalStream(dm.stream())
    timed = make_timed(dm, stream, td, _lib)

    # the same FP32 solve with weighted-Jacobi smoothing (reported beside the product)
    jac = None
    if use_learned and not args.skip_jacobi:
        ms_j, infos_j, _ = timed(0, 1, min(args.steps, args.jacobi_steps))
        lj = infos_j[-1]
        jac = {"s_per_solve": allmax(td, ms_j) / 1e3, "nitU": lj["nitU"], "nitZ": lj["nitZ"], "itPat": lj["itPat"],
               "rel_residual": lj["rel_residual"], "solves_timed": len(infos_j)}
    clk = ClockSampler(clock_csv_path())
    ms, infos, launches = timed(sm, args.warmup, args.steps, clk)
    accuracy = None
    if plain is not None:
        Um, Pm = dm.solution()
        Umt, Pmt, imt = dm.solve(smoother=sm, allow_not_converged=True, **TIGHT_KW)
        accuracy = accuracy_block(Um, Pm, U64, P64, Umt, Pmt, U64t, P64t, imt["rel_residual"], i64t["rel_residual"])
    ms = allmax(td, ms)
    clocks = clk.summary(dev)
    last = infos[-1]
    # ---- operator rooflines: the double-float outer apply (the largest share of the learned solve)
    # and the finest-level FP32 apply, timed with CUDA events on the library's stream ----
    ms_apply32 = dm.apply_timing(0, 1, 10)
    ms_apply_df = dm.apply_timing(0, 2, 10)
    hbm, peak_kind = peaks()
    alg_df = algorithmic_apply_bytes(nel, ndof, nvnod, 8)
    alg_32 = algorithmic_apply_bytes(nel, ndof, nvnod, 4)
    bdf = apply_bytes_df(nel, ndof)
    if args.fp32_operator:
        b32 = apply_bytes_pa(nel, ndof, ndof // 3)
        fp32 = {"kernel": "finest-level FP32 apply, partially assembled: k_pa_elem_f32 + k_node_gather_f32",
                "traffic": TRAFFIC_PER_ELEMENT_PA * nel, "streamed_basis": "per-point geometric factors"}
    else:
        b32 = apply_bytes(nel, ndof, 4)
        fp32 = {"kernel": "finest-level FP32 apply, stored matrices: k_stream_elem_f32 + k_node_gather_f32",
                "traffic": TRAFFIC_PER_ELEMENT_F32 * nel, "streamed_basis": "stored element matrices"}
    fp32.update({"bytes_per_apply": alg_32, "achieved": alg_32 / (ms_apply32 * 1e-3) / 1e9,
                 "ms_per_apply": ms_apply32, "dof_per_s": ndof / (ms_apply32 * 1e-3),
                 "stored_matrix": {"bytes_per_apply": b32, "achieved": b32 / (ms_apply32 * 1e-3) / 1e9}})
    df = {"kernel": "finest-level double-float outer apply: k_stream_rowlane<RlDF> + k_node_gather_f64",
          "bytes_per_apply": alg_df, "achieved": alg_df / (ms_apply_df * 1e-3) / 1e9,
          "traffic": TRAFFIC_PER_ELEMENT_DF * nel, "ms_per_apply": ms_apply_df, "dof_per_s": ndof / (ms_apply_df * 1e-3),
          "stored_matrix": {"bytes_per_apply": bdf, "achieved": bdf / (ms_apply_df * 1e-3) / 1e9}}
    for k in (fp32, df):
        k["frac"] = k["achieved"] / hbm
        k["stored_matrix"]["frac"] = k["stored_matrix"]["achieved"] / hbm
    top, other = (df, fp32) if use_learned else (fp32, df)
    roofline = {"bound": "hbm", **top, "peak": hbm, "unit": "GB/s", "peak_kind": peak_kind,
                "bytes_basis": "algorithmic bytes of a matrix-free apply (x, y, connectivity, class byte, vertex "
                               "coordinates and viscosity); stored_matrix counts everything the kernels stream "
                               "(resident element matrices, or per-point factors for the partially assembled apply)",
                "traffic_source": "ncu dram__bytes_read+write of both kernels on the 491,520-element shell, "
                                  "scaled by element count",
                "other_apply": other,
                "fp64_apply_ms": fp64_apply_ms if plain else None}
    learned = None
    if use_learned:
        learned = {"schedule": "one learned sweep per side on levels 0 and 1 (ml_schedule 1)",
                   "nitU": last["nitU"], "nitZ": last["nitZ"], "itPat": last["itPat"],
                   "smoother_fallbacks": last["smoother_fallbacks"], "fp32_mg_jacobi": jac,
                   "speedup_vs_jacobi": jac["s_per_solve"] / (ms / 1e3) if jac else None,
                   "weights": "trained on the 130,662-DOF shell, 20 viscosity fields (contrast 1e2-1e5), ~2M pairs"}
    # ---- end-to-end through the public API with host buffers ----
    U = np.empty(ndof)
    P = np.zeros(nvnod)
    t_e2e, einfo = None, {"rel_residual": None}
    if not args.skip_e2e:
        te = time.perf_counter()
        for _ in range(max(1, args.e2e_steps)):
            setup(1)
            U, P, einfo = dm.solve(P0=np.zeros_like(P), smoother=sm, **SOLVER_KW)
        t_e2e = allmax(td, (time.perf_counter() - te) / max(1, args.e2e_steps))
    h2d = (w["visc"].nbytes + w["dens"].nbytes + 4 * len(w["ifix"]) + w["vfix"].nbytes + P.nbytes)
    d2h = U.nbytes + P.nbytes
    dm.close()
    out = {
        "metric": METRIC, "value": ms / 1e3, "unit": "s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 outer / f32 V-cycle / bf16 smoother MLP" if use_learned
        else "f64 outer / f32 V-cycle", "data": "synthetic",
        "config": {"workload": f"shell L{w['level']} x {w['nlayer']} layers, {nel} P2 tets, {ndof} velocity DOF, "
                               f"{w['nmg']} MG levels, eta contrast {w.get('contrast', 1e4):.0e} x30 jump, 12 plate caps",
                   "nmg": w["nmg"], "solves_per_s": ws * 1e3 / ms,
                   "smoother": "learned (one sweep per side, levels 0-1) + Jacobi below" if use_learned
                   else "weighted Jacobi",
                   "fp32_operator": "partially assembled (per-point geometric factors)" if args.fp32_operator
                   else "streamed stored element matrices",
                   "l2": f"working set (element matrices {nel * 7440 / 1e9:.0f} GB) > L2; no flush needed",
                   "parallelism": f"replicas x{ws}"},
        "solve": {"itPat": last["itPat"], "nitU": last["nitU"], "nitZ": last["nitZ"], "nvcycle": last["nvcycle"],
                  "rel_residual": last["rel_residual"], "t_setup_ms": last["t_setup_ms"],
                  "t_iter_ms": last["t_iter_ms"]},
        "plain_fp64": None if plain is None else {
            "s_per_solve": plain["s_per_solve"], "rel_residual": plain["info"]["rel_residual"],
            "itPat": plain["info"]["itPat"], "nitU": plain["info"]["nitU"], "nitZ": plain["info"]["nitZ"],
            "t_setup_ms": plain["info"]["t_setup_ms"], "fp64_apply_ms": fp64_apply_ms,
            "speedup_mixed_vs_plain": plain["s_per_solve"] / (ms / 1e3)},
        "roofline": roofline,
        "learned_smoother": learned,
        "accuracy": accuracy,
        "e2e": {"value": t_e2e, "unit": "s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "rel_residual": einfo["rel_residual"]},
        "gpu_launches": int(launches),
        "clocks": clocks,
        "mesh_build_s": t_mesh,
    }
    # ---- the extra legs run once, on rank 0 of a 1-GPU run: with N replicas only the timed solve
    # above is the scaling measurement ----
    extras = rank == 0 and ws == 1
    # ---- the 130k-DOF shell: GPU solves beside the oracle's full CPU solve ----
    if extras and not args.skip_c1:
        out["c1"] = extra_leg(c1_leg, args, wfile)
    out["cpu_baseline"] = None
    if extras and not args.skip_cpu:
        out["cpu_baseline"] = extra_leg(cpu_baseline, args)
        if out.get("c1") and "error" not in out["c1"] and "error" not in out["cpu_baseline"]:
            out["c1"]["cpu_oracle_s"] = out["cpu_baseline"]["value"]
            out["c1"]["cpu_over_gpu_learned"] = out["cpu_baseline"]["value"] / out["c1"]["learned_fp32_s"]
    if extras and not args.skip_sl:
        out["advection"] = extra_leg(sl_rates, args)
    if extras and not args.skip_c5:
        out["c5"] = extra_leg(c5_leg, args, wfile)
    if rank == 0:
        print(json.dumps(out))


def extra_leg(fn, *a):
    """One of the once-only legs beside the timed solve: a failure is reported in the line (and its
    traceback on stderr) rather than losing the measurements already taken."""
    try:
        return fn(*a)
    except Exception as e:  # noqa: BLE001 - any failure of a side measurement is reported, not raised
        traceback.print_exc()
        return {"error": f"{type(e).__name__}: {e}"[:400]}


def make_timed(dm, stream, td, _lib):
    """Solve timer: warm-up solves, then `steps` device-resident solves bracketed by a barrier, a
    synchronize and CUDA events on the library's stream."""
    import torch

    def timed(smoother, warmup, steps, clk=None):
        for _ in range(warmup):
            dm.step_device(smoother=smoother, **SOLVER_KW)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n0 = _lib.launch_count()
        barrier(td)
        torch.cuda.synchronize()
        with (clk if clk is not None else _Null()):
            ev0.record(stream)
            infos = [dm.step_device(smoother=smoother, **SOLVER_KW) for _ in range(steps)]
            ev1.record(stream)
            ev1.synchronize()
        return ev0.elapsed_time(ev1) / steps, infos, _lib.launch_count() - n0
    return timed


def solution_distance(U, P, Uref, Pref):
    """Relative L2 distances of velocity and mean-free pressure, and whether both are within 1e-8."""
    Pc, Pcr = P - P.mean(), Pref - Pref.mean()
    d = {"dU_rel_l2_vs_plain_fp64": float(np.linalg.norm(U - Uref) / np.linalg.norm(Uref)),
         "dP_rel_l2_vs_plain_fp64": float(np.linalg.norm(Pc - Pcr) / np.linalg.norm(Pcr))}
    d["within_1e-8"] = bool(d["dU_rel_l2_vs_plain_fp64"] <= TARGET and d["dP_rel_l2_vs_plain_fp64"] <= TARGET)
    return d


def accuracy_block(Ul, Pl, Up, Pp, Ult, Plt, Upt, Ppt, res_lt=None, res_pt=None):
    """Distances of the learned (l) and plain FP64 (p) solutions at the 1e-8 target and at TIGHT
    (t): the headline pair (learned at 1e-8 against plain FP64 at 1e-8), the learned 1e-8 solution
    against the tight FP64 solution, and the two tight solutions."""
    d = solution_distance(Ul, Pl, Up, Pp)
    a = solution_distance(Ul, Pl, Upt, Ppt)
    b = solution_distance(Ult, Plt, Upt, Ppt)
    c = solution_distance(Up, Pp, Upt, Ppt)
    d["learned_1e-8_vs_plain_1e-11"] = {"dU": a["dU_rel_l2_vs_plain_fp64"], "dP": a["dP_rel_l2_vs_plain_fp64"]}
    d["plain_1e-8_vs_plain_1e-11"] = {"dU": c["dU_rel_l2_vs_plain_fp64"], "dP": c["dP_rel_l2_vs_plain_fp64"]}
    d["learned_1e-11_vs_plain_1e-11"] = {"dU": b["dU_rel_l2_vs_plain_fp64"], "dP": b["dP_rel_l2_vs_plain_fp64"],
                                         "within_1e-8": b["within_1e-8"],
                                         "rel_residuals": [res_lt, res_pt]}
    return d


def c1_leg(args, wfile):
    """The 130,662-DOF shell (level 3 x 8 layers, 3 MG levels), the configuration the reference
    runs on its CPU: learned + FP32-MG, Jacobi FP32-MG and plain FP64 solves to the 1e-8 coupled
    residual, each the mean of 3 device-resident solves after one warm-up."""
    import torch
    from m3tet_sph_gb300 import _lib, learned as LS, stokes, workloads
    w = workloads.make_workload("c1", seed=args.seed)
    dm = stokes.DeviceMesh(w["levels"])
    dm.set_option("fp32_operator", args.fp32_operator)
    out = {"workload": "shell L3 x 8 layers, 30720 P2 tets, 130662 velocity DOF, 3 MG levels, isoviscous, free slip"}
    try:
        stream = torch.cuda.ExternalStream(dm.stream())
        timed = make_timed(dm, stream, None, _lib)
        dm.setup(w["visc"], w["dens"], w["ifix"], w["vfix"], w["phys"], precision=0)
        ms, infos, _ = timed(0, 1, 3)
        U64, P64 = dm.solution()
        U64t, P64t, i64t = dm.solve(P0=P64, allow_not_converged=True, **TIGHT_KW)
        out["plain_fp64_s"] = ms / 1e3
        dm.setup(w["visc"], w["dens"], w["ifix"], w["vfix"], w["phys"], precision=1)
        ms, infos, _ = timed(0, 1, 3)
        out["jacobi_fp32_s"] = ms / 1e3
        LS.set_params(dm, np.load(wfile), trained=True)
        ms, infos, _ = timed(1, 1, 3)
        out["learned_fp32_s"] = ms / 1e3
        out["learned_rel_residual"] = infos[-1]["rel_residual"]
        out["learned_its"] = infos[-1]["nitU"] + infos[-1]["nitZ"]
        Ul, Pl = dm.solution()
        Ult, Plt, ilt = dm.solve(smoother=1, allow_not_converged=True, **TIGHT_KW)
        out["accuracy"] = accuracy_block(Ul, Pl, U64, P64, Ult, Plt, U64t, P64t, ilt["rel_residual"],
                                         i64t["rel_residual"])
    finally:
        dm.close()
    return out


def c5_leg(args, wfile):
    """The 64M-DOF shell (level 6 x 64 layers, 15,728,640 curved P2 tets, 63,406,854 velocity DOF,
    1e6 viscosity contrast x30 below 660 km, 12 plate caps): one learned + FP32-MG solve and one
    plain-FP64 solve to the 1e-8 coupled residual, their distance, then device-resident time steps
    (GPlates surface velocities at the step's model time -> rock_prop -> Stokes at the reference's
    default tolerances -> calculate_dt -> diffusion half step -> PC2 + cubic semi-Lagrangian
    advection of T -> diffusion half step) with each path."""
    from m3tet_sph_gb300 import gplates, learned as LS, stokes, workloads
    t0 = time.time()
    w = workloads.make_workload(args.c5_workload, seed=args.seed)
    f = w["levels"][0]
    dm = stokes.DeviceMesh(w["levels"])
    dm.set_option("fp32_operator", args.fp32_operator)
    t_mesh = time.time() - t0
    nnod = f["nnod"]
    out = {"workload": f"shell L{w['level']} x {w['nlayer']} layers, {f['nel']} P2 tets, {3 * nnod} velocity DOF, "
                       f"{w['nmg']} MG levels, eta contrast 1e6 x30 jump, 12 plate caps",
           "mesh_build_s": t_mesh}
    params = np.load(wfile)
    rock = workloads.rock_params(1e6)
    step_kw = dict(rtol_Pat=1e-4, rtol_U=5e-3, itmax_Pat=120, itmin_Pat=3, itmax_U=20)
    try:
        def setup(prec):
            dm.setup(w["visc"], w["dens"], w["ifix"], w["vfix"], w["phys"], precision=prec)
            if prec == 1:
                LS.set_params(dm, params, trained=True)
                dm.set_option("ml_schedule", 1)
        setup(1)
        il = dm.step_device(smoother=1, **SOLVER_KW)
        Ul, Pl = dm.solution()
        out["learned_fp32"] = {"s": (il["t_setup_ms"] + il["t_iter_ms"]) / 1e3, "its": il["nitU"] + il["nitZ"],
                               "itPat": il["itPat"], "rel_residual": il["rel_residual"],
                               "fallbacks": il["smoother_fallbacks"]}
        if not args.c5_skip_plain:
            setup(0)
            ip = dm.step_device(**SOLVER_KW)
            Up, Pp = dm.solution()
            out["plain_fp64"] = {"s": (ip["t_setup_ms"] + ip["t_iter_ms"]) / 1e3, "its": ip["nitU"] + ip["nitZ"],
                                 "itPat": ip["itPat"], "rel_residual": ip["rel_residual"]}
            out["speedup_learned_vs_plain"] = out["plain_fp64"]["s"] / out["learned_fp32"]["s"]
            # at this size the 1e-11 continuations of both solves would add several minutes; the
            # 8M-DOF and 130k-DOF blocks carry them
            out["accuracy"] = solution_distance(Ul, Pl, Up, Pp)
        # the time steps take their surface velocities from a GPlates series, updated before every
        # step as the reference's loop does (update_vel_bc); the series is seeded (four 1-Myr exports
        # in GPlates' format, written and read back), the reference's own exports not being shipped
        t_rd = time.time()
        with tempfile.TemporaryDirectory() as tmp:
            folder = gplates.write_synthetic_folder(tmp, gplates.synthetic_vel_bcs(f, seed=args.seed))
            V_BCs, t_files = gplates.read_vel_gplates_folder(folder)
        series = gplates.VelBCSeries(V_BCs, t_files, f["PointID"], workloads.R_SURF)
        out["gplates"] = {"files": len(V_BCs), "surface_nodes": int(V_BCs[0]["Uth_Uph"].shape[1]),
                          "write_and_read_s": time.time() - t_rd,
                          "source": "seeded exports in GPlates' five-column format (Euler-pole plates)"}
        steps = {}
        for name, prec, n in (("learned_fp32", 1, args.c5_steps), ("plain_fp64", 0, args.c5_plain_steps)):
            if n <= 0:
                continue
            setup(prec)
            T0 = workloads.DT_K * w["T"]
            fix = np.nonzero(f["PointID"] > 0)[0]
            dm.diffusion_setup(workloads.KAPPA, fix, T0[fix])
            dm.set_temperature(T0)
            infos = [dm.time_step(step_kw, slm=dict(method_BT="PC2", method_interp="cubic"), rock=rock,
                                  smoother=prec, dt_adv_limit=0.005, dtmax=0.1, diffusion=True, vel_bcs=series)
                     for _ in range(n)]
            t_st = sum(i["t_stokes_ms"] for i in infos) / 1e3
            t_ad = sum(i["t_advect_ms"] for i in infos) / 1e3
            steps[name] = {"steps": n, "s_per_step": sum(i["t_total_ms"] for i in infos) / 1e3 / n,
                           "diffusion_s_per_step": sum(i["t_diffusion_ms"] for i in infos) / 1e3 / n,
                           "diffusion_its": [i["diffusion_its"] for i in infos],
                           "stokes_solves_per_s": n / t_st, "departure_points_per_s": n * nnod / t_ad,
                           "its_per_step": [i["stokes"]["nitU"] + i["stokes"]["nitZ"] for i in infos],
                           "dt": [i["dt"] for i in infos], "locate_nties": sum(i["locate"]["nties"] for i in infos),
                           "locate_ngap": sum(i["locate"]["ngap"] for i in infos),
                           "locate_nlost": sum(i["locate"]["nlost"] for i in infos),
                           "vel_bc_update_ms_per_step": sum(i["t_vel_bc_ms"] for i in infos) / n}
        if steps:
            out["time_steps"] = steps
            if "learned_fp32" in steps and "plain_fp64" in steps:
                out["time_steps"]["solves_per_s_learned_over_plain"] = (steps["learned_fp32"]["stokes_solves_per_s"]
                                                                        / steps["plain_fp64"]["stokes_solves_per_s"])
    finally:
        dm.close()
    return out


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def shell_points(n, seed, r0=3480.0, r1=6371.0):
    """(theta, phi, r) of n seeded points: directions uniform on the sphere, r uniform in volume."""
    from m3tet_sph_gb300 import mesh as M
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(3, n))
    v /= np.linalg.norm(v, axis=0)
    r = (r0 ** 3 + rng.uniform(size=n) * (r1 ** 3 - r0 ** 3)) ** (1.0 / 3.0)
    r = np.clip(r, r0 + 1e-9 * (r1 - r0), r1 - 1e-9 * (r1 - r0))
    return M.cart2sph(v * r)


def sl_rates(args):
    """Semi-Lagrangian rates on the 130k-DOF shell (public API, host buffers, copies included): one
    advection step of T (RK4 over 3 substeps, curved-element location, cubic interpolation) in the
    Stokes velocity at the CFL dt, and a seeded point-location sweep inside the shell."""
    from m3tet_sph_gb300 import advection as A, stokes, workloads
    w = workloads.make_workload(args.sl_workload, seed=args.seed)
    f = w["levels"][0]
    dm = stokes.DeviceMesh(w["levels"])
    step = None
    try:
        if not args.sweep_only:
            dm.setup(w["visc"], w["dens"], w["ifix"], w["vfix"], w["phys"], precision=1)
            U, _, _ = dm.solve(**SOLVER_KW)
            Ux, Uy, Uz = U[0::3], U[1::3], U[2::3]
            X, EL = f["GCOORD"], f["EL2NOD"]
            hmin = min(np.linalg.norm(X[:, EL[:, a]] - X[:, EL[:, b]], axis=0).min()
                       for a, b in ((0, 1), (1, 2), (2, 3), (3, 0), (0, 2), (1, 3)))
            umax = np.sqrt(Ux ** 2 + Uy ** 2 + Uz ** 2).max()
            dt = 0.5 * hmin / umax                                     # CFL number 0.5
            MESH = dict(levels=w["levels"], device_mesh=dm, r_cmb=workloads.R_CMB, r_surf=workloads.R_SURF)
            opts = dict(method_BT="RK4", method_interp="cubic")
            A.advect3d_slm_p_sph(MESH, None, Ux, Uy, Uz, w["T"], dt, opts)
            t = time.perf_counter()
            _, WS = A.advect3d_slm_p_sph(MESH, None, Ux, Uy, Uz, w["T"], dt, opts)
            t_sl = time.perf_counter() - t
            n = f["nnod"]
            step = {"workload": f"shell L{w['level']} x {w['nlayer']} layers, {n} P2 nodes", "dt": dt,
                    "method": "RK4 (3 substeps) + cubic", "s": t_sl, "departure_points_per_s": n / t_sl,
                    "locate": WS["locate_info"]}
        pts = shell_points(args.sweep_points, args.seed + 3)
        A.tsearch2_sph(dm, pts[:, :100000])
        t = time.perf_counter()
        _, _, info = A.tsearch2_sph(dm, pts)
        t_loc = time.perf_counter() - t
        ms_dev, _ = A.locate_timing(dm, pts, 5)
    finally:
        dm.close()
    return {"sl_step": step,
            "location_sweep": {"points": args.sweep_points, "s": t_loc, "points_per_s": args.sweep_points / t_loc,
                               "device_s": ms_dev / 1e3, "device_points_per_s": args.sweep_points / (ms_dev * 1e-3),
                               "basis": "s: public API with host arrays (copies and layout changes included); "
                                        "device_s: device-resident location (CUDA events)",
                               "locate": info}}


def run_diffusion_only(args, rank):
    """Thermal-diffusion rates (profiling): set up diffusion3d_p's operator on the workload's mesh
    (P1 split, kappa 1e-6 m^2/s, T prescribed on both boundaries) and time --op-reps half steps of
    50 Myr; one operator application is timed as the mean CG iteration."""
    from m3tet_sph_gb300 import build as B
    B.build()
    from m3tet_sph_gb300 import stokes, workloads
    w = workloads.make_workload(args.workload, seed=args.seed)
    f = w["levels"][0]
    dm = stokes.DeviceMesh(w["levels"])
    try:
        T0 = workloads.DT_K * w["T"]
        fix = np.nonzero(f["PointID"] > 0)[0]
        t = time.perf_counter()
        dm.diffusion_setup(workloads.KAPPA, fix, T0[fix])
        t_setup = time.perf_counter() - t
        T, _ = dm.diffusion(T0, 50.0)
        its, t = 0, time.perf_counter()
        for _ in range(args.op_reps):
            T, nit = dm.diffusion(T, 50.0)
            its += nit
        dt = time.perf_counter() - t
    finally:
        dm.close()
    nsub = 8 * f["nel"]
    if rank == 0:
        print(json.dumps({"workload": args.workload, "split_elements": nsub, "nodes": f["nnod"], "setup_s": t_setup,
                          "s_per_half_step": dt / args.op_reps, "cg_its_per_half_step": its / args.op_reps,
                          "ms_per_cg_iteration": dt / max(its, 1) * 1e3}))


def run_operator_only(args, rank):
    """Operator-only run for profiler captures: set up the mixed-precision operator once, then time
    --op-reps applications of one level operator (precision 0 FP64, 1 FP32, 2 double-float)."""
    from m3tet_sph_gb300 import build as B
    B.build()
    from m3tet_sph_gb300 import stokes, workloads
    w = workloads.make_workload(args.workload, seed=args.seed, nmg=args.nmg)
    lv0 = w["levels"][0]
    dm = stokes.DeviceMesh(w["levels"])
    for kv in args.set_option:
        k, v = kv.split("=")
        dm.set_option(k, int(v))
    t = time.perf_counter()
    dm.setup(w["visc"], w["dens"], w["ifix"], w["vfix"], w["phys"], precision=1)
    t_setup = time.perf_counter() - t
    ms = dm.apply_timing(args.op_level, args.op_precision, args.op_reps)
    nc = dm.ncolors(args.op_level)
    dm.close()
    s = 8 if args.op_precision in (0, 2) else 4
    b = apply_bytes(lv0["nel"], 3 * lv0["nnod"], s) if args.op_level == 0 else None
    if rank == 0:
        print(json.dumps({"workload": args.workload, "options": args.set_option, "nel": lv0["nel"], "colours": nc,
                          "nmg": w["nmg"], "coarse_dofs": 3 * w["levels"][-1]["nnod"], "setup_s": t_setup,
                          "level": args.op_level,
                          "precision": args.op_precision, "ms_per_apply": ms,
                          "gbs": None if b is None else b / (ms * 1e-3) / 1e9}))


def cpu_solve_c1(seed, nthreads):
    """One full solve of the 130,662-DOF shell by the FP64 oracle on the host: element matrices,
    assembly, rotation, Galerkin hierarchy and coarse Cholesky (StokesSystem), then Patera / MG-PCG
    to the 1e-8 coupled residual with the sparse products on `nthreads` host threads. Returns
    (seconds, info)."""
    from oracle import stokes_oracle as O
    from m3tet_sph_gb300 import workloads
    w = workloads.make_workload("c1", seed=seed)
    t = time.perf_counter()
    S = O.StokesSystem(w["levels"], w["visc"], w["dens"], w["ifix"], w["vfix"], w["phys"], nthreads=nthreads)
    S.mg.use_threads(nthreads)
    U, P, info = O.patera(S, target_rel_residual=TARGET, **{k: v for k, v in SOLVER_KW.items()
                                                             if k != "target_rel_residual"})
    t = time.perf_counter() - t
    info = dict(info, rel_residual=float(S.residual(U, P)))
    return t, info


def cpu_baseline(args):
    """The FP64 oracle's full solve of the 130,662-DOF shell, timed on the host threads (not scaled
    or extrapolated)."""
    nth = host_threads()
    t, info = cpu_solve_c1(args.seed, nth)
    return {"value": t, "unit": "s", "cores": nth, "kind": "port",
            "sample": f"one full FP64 oracle solve of the 130,662-DOF shell (set-up + Patera/MG-PCG to a "
                      f"{info['rel_residual']:.1e} coupled residual, {info['nitU'] + info['nitZ']} MG-PCG iterations; "
                      f"sparse products on {nth} OpenMP threads)",
            "workload": "shell L3 x 8 layers, 30720 P2 tets, 130662 velocity DOF, 3 MG levels"}


def host_threads():
    """Host threads this process may run on."""
    try:
        return max(1, len(os.sched_getaffinity(0)))
    except AttributeError:
        return max(1, os.cpu_count() or 1)


def run_reference(args, rank, ws, td):
    """CPU reference arm: the FP64 oracle restating the reference algorithm, on all host threads.
    One step = one full solve of the 130,662-DOF shell (set-up included), timed."""
    if rank != 0:
        return
    nth = host_threads()
    for _ in range(args.warmup):
        cpu_solve_c1(args.seed, nth)
    ts, info = [], None
    for _ in range(args.steps):
        t, info = cpu_solve_c1(args.seed, nth)
        ts.append(t)
    v = float(np.mean(ts))
    sample = (f"one full FP64 oracle solve per step of the 130,662-DOF shell (set-up + Patera/MG-PCG to a "
              f"{info['rel_residual']:.1e} coupled residual, {info['nitU'] + info['nitZ']} MG-PCG iterations; sparse "
              f"products on {nth} OpenMP threads)")
    out = {"metric": METRIC, "value": v, "unit": "s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": "synthetic", "impl": "reference",
           "config": {"workload": "shell L3 x 8 layers, 30720 P2 tets, 130662 velocity DOF, 3 MG levels "
                                  "(the configuration the reference runs on its CPU; the GPU arm reports its own "
                                  "solves of this shell under c1)"},
           "cpu_baseline": {"value": v, "unit": "s", "cores": nth, "kind": "port", "sample": sample},
           "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c2")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--plain-steps", type=int, default=1)
    ap.add_argument("--plain-warmup", type=int, default=1)
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--skip-plain", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-c1", action="store_true", help="skip the GPU solves of the 130k-DOF shell")
    ap.add_argument("--skip-c5", action="store_true", help="skip the 64M-DOF shell")
    ap.add_argument("--c5-skip-plain", action="store_true", help="64M-DOF shell: no plain-FP64 1e-8 solve")
    ap.add_argument("--c5-steps", type=int, default=3, help="64M-DOF time steps with the learned + FP32-MG solve")
    ap.add_argument("--c5-plain-steps", type=int, default=1, help="64M-DOF time steps with the plain FP64 solve")
    ap.add_argument("--c5-workload", default="c5", help="mesh of the time-step leg (a plate workload)")
    ap.add_argument("--jacobi-steps", type=int, default=3, help="timed Jacobi-smoothed comparison solves")
    ap.add_argument("--skip-learned", action="store_true", help="time the Jacobi-smoothed FP32 solve instead")
    ap.add_argument("--skip-jacobi", action="store_true", help="skip the Jacobi-smoothed comparison solve")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--sl-only", action="store_true", help="semi-Lagrangian rates only (profiling)")
    ap.add_argument("--sweep-only", action="store_true", help="with --sl-only: the location sweep alone")
    ap.add_argument("--sl-workload", default="c1", help="mesh of the semi-Lagrangian measurements")
    ap.add_argument("--skip-sl", action="store_true")
    ap.add_argument("--sweep-points", type=int, default=16_000_000)
    ap.add_argument("--fp32-operator", type=int, default=1, choices=[0, 1],
                    help="finest-level FP32 V-cycle operator: 0 streamed stored matrices, 1 partially assembled")
    ap.add_argument("--op-only", action="store_true", help="time one level operator only (profiling)")
    ap.add_argument("--diff-only", action="store_true", help="time thermal-diffusion half steps only (profiling)")
    ap.add_argument("--op-level", type=int, default=0)
    ap.add_argument("--nmg", type=int, default=None, help="multigrid levels of the --op-only workload")
    ap.add_argument("--op-precision", type=int, default=1)
    ap.add_argument("--op-reps", type=int, default=20)
    ap.add_argument("--set-option", action="append", default=[], help="library option name=value (--op-only)")
    args = ap.parse_args()
    rank, ws, td = dist_init()
    if args.sl_only:
        if rank == 0:
            from m3tet_sph_gb300 import build as B
            B.build()
            print(json.dumps(sl_rates(args)))
    elif args.op_only:
        run_operator_only(args, rank)
    elif args.diff_only:
        run_diffusion_only(args, rank)
    elif args.impl == "reference":
        run_reference(args, rank, ws, td)
    else:
        run_gb300(args, rank, ws, td)
    if td is not None:
        td.destroy_process_group()


if __name__ == "__main__":
    main()
