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
      FP64 outer CG / Patera on the GPU (libm3sph.so); `value` is its solve time. The plain-FP64 GPU
      path (FP64 V-cycle) and the same FP32 solve with weighted-Jacobi smoothing are timed on the
      same inputs for the comparison (--skip-learned makes the Jacobi solve the timed one);
      semi-Lagrangian rates are measured on the 130k-DOF shell (RK4 + cubic step, 16M-point
      location sweep).
  --impl reference: the FP64 CPU oracle (numpy/scipy restatement of the reference algorithm) on
      the host cores, on a bounded sample of the same workload, extrapolated to one solve.

Prints one JSON line. Multi-GPU runs are independent replicas (the solve does not shard).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Stokes solve time to 1e-8 rel. residual: learned+FP32-MG vs plain FP64 on 1 GPU"
TARGET = 1e-8
# Patera / MG-PCG tolerances: the reference's rtol_U (5e-3) and a pressure tolerance that the
# coupled-residual check tightens (x0.1) until the 1e-8 target is met
SOLVER_KW = dict(rtol_Pat=1e-7, rtol_U=5e-3, itmax_Pat=400, itmax_U=40, target_rel_residual=TARGET)


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
# the same for the double-float outer apply (k_stream_rowlane<RlDF> + k_node_gather_f64)
TRAFFIC_PER_ELEMENT_DF = (1.900e9 + 72.74e6 + 190.52e6 + 10.03e6) / 491520


def apply_bytes_df(nel, ndof):
    """Algorithmic bytes of one double-float outer apply: two FP32 packed matrices per element,
    connectivity, x read and y written in FP64."""
    return nel * (2 * 465 * 4 + 40) + 2 * 8 * ndof


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
    dm = stokes.DeviceMesh(w["levels"], device=dev)
    torch.cuda.set_device(dev)

    def setup(prec):
        dm.setup(w["visc"], w["dens"], w["ifix"], w["vfix"], w["phys"], precision=prec)

    # ---- plain FP64 path (same inputs) ----
    plain = None
    if not args.skip_plain:
        setup(0)
        for _ in range(args.plain_warmup):
            info64 = dm.step_device(**SOLVER_KW)
        barrier(td)
        torch.cuda.synchronize()
        t = time.perf_counter()
        infos64 = [dm.step_device(**SOLVER_KW) for _ in range(args.plain_steps)]
        torch.cuda.synchronize()
        t_plain = allmax(td, (time.perf_counter() - t) / args.plain_steps)
        plain = dict(s_per_solve=t_plain, info=infos64[-1])
        U64, P64 = dm.solution()
        fp64_apply_ms = dm.apply_timing(0, 0, 5)
    # ---- the product: FP32 V-cycle with the learned element smoother (one learned sweep per
    # side on the two finest levels) inside FP64 outer CG / Patera; timed region ----
    setup(1)
    wfile = ROOT / "m3tet_sph_gb300" / "smoother_c1.npy"
    use_learned = not args.skip_learned
    if use_learned:
        from m3tet_sph_gb300 import learned as LS
        LS.set_params(dm, np.load(wfile), trained=True)
        dm.set_option("ml_schedule", 1)
    sm = 1 if use_learned else 0
    stream = torch.cuda.ExternalStream(dm.stream())

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

    # the same FP32 solve with weighted-Jacobi smoothing (reported beside the product)
    jac = None
    if use_learned and not args.skip_jacobi:
        ms_j, infos_j, _ = timed(0, 1, args.steps)
        lj = infos_j[-1]
        jac = {"s_per_solve": allmax(td, ms_j) / 1e3, "nitU": lj["nitU"], "nitZ": lj["nitZ"], "itPat": lj["itPat"],
               "rel_residual": lj["rel_residual"]}
    clk = ClockSampler(clock_csv_path())
    ms, infos, launches = timed(sm, args.warmup, args.steps, clk)
    accuracy = None
    if plain is not None:
        Um, Pm = dm.solution()
        Pc, Pc64 = Pm - Pm.mean(), P64 - P64.mean()
        accuracy = {"dU_rel_l2_vs_plain_fp64": float(np.linalg.norm(Um - U64) / np.linalg.norm(U64)),
                    "dP_rel_l2_vs_plain_fp64": float(np.linalg.norm(Pc - Pc64) / np.linalg.norm(Pc64))}
    ms = allmax(td, ms)
    clocks = clk.summary(dev)
    last = infos[-1]
    # ---- operator rooflines: the finest-level FP32 apply (phase 1 k_stream_elem_f32 + phase 2
    # k_node_gather_f32) and the double-float outer apply, both timed with CUDA events ----
    ms_apply32 = dm.apply_timing(0, 1, 10)
    ms_apply_df = dm.apply_timing(0, 2, 10)
    hbm, peak_kind = peaks()
    b32 = apply_bytes(nel, ndof, 4)
    achieved = b32 / (ms_apply32 * 1e-3) / 1e9
    # dominant kernel: with the learned smoother (2 finest FP32 applies per iteration) the one
    # double-float outer apply per iteration takes the largest share; with Jacobi (6 FP32 applies
    # per iteration) the FP32 apply does
    bdf = apply_bytes_df(nel, ndof)
    fp32 = {"kernel": "finest-level FP32 apply: k_stream_elem_f32 + k_node_gather_f32",
            "achieved": achieved, "frac": achieved / hbm, "traffic": TRAFFIC_PER_ELEMENT_F32 * nel,
            "bytes_per_apply": b32, "ms_per_apply": ms_apply32, "dof_per_s": ndof / (ms_apply32 * 1e-3)}
    df = {"kernel": "finest-level double-float outer apply: k_stream_rowlane<RlDF> + k_node_gather_f64",
          "achieved": bdf / (ms_apply_df * 1e-3) / 1e9, "traffic": TRAFFIC_PER_ELEMENT_DF * nel,
          "bytes_per_apply": bdf, "ms_per_apply": ms_apply_df, "dof_per_s": ndof / (ms_apply_df * 1e-3)}
    df["frac"] = df["achieved"] / hbm
    top, other = (df, fp32) if use_learned else (fp32, df)
    roofline = {"bound": "hbm", **top, "peak": hbm, "unit": "GB/s", "peak_kind": peak_kind,
                "traffic_source": "ncu dram__bytes_read+write of both kernels on the 491,520-element shell, "
                                  "scaled by element count",
                "other_apply": other,
                "fp64_apply_ms": fp64_apply_ms if plain else None,
                "fp64_apply_gbs": apply_bytes(nel, ndof, 8) / (fp64_apply_ms * 1e-3) / 1e9 if plain else None}
    learned = None
    if use_learned:
        learned = {"schedule": "one learned sweep per side on levels 0 and 1 (ml_schedule 1)",
                   "nitU": last["nitU"], "nitZ": last["nitZ"], "itPat": last["itPat"],
                   "smoother_fallbacks": last["smoother_fallbacks"], "fp32_mg_jacobi": jac,
                   "speedup_vs_jacobi": jac["s_per_solve"] / (ms / 1e3) if jac else None,
                   "weights": "trained on the 130,662-DOF shell, 20 viscosity fields (contrast 1e2-1e5), ~2M pairs"}
    # ---- end-to-end through the public API with host buffers ----
    U = np.empty(ndof)
    P = np.zeros(lv0["EL2NOD"][:, :4].max() + 1)
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
    # ---- CPU baseline (rank 0, N=1): oracle on a bounded sample ----
    cpu = None
    if rank == 0 and ws == 1 and not args.skip_cpu:
        cpu = cpu_baseline(w, plain["info"] if plain else last, args)
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
        "cpu_baseline": cpu,
        "mesh_build_s": t_mesh,
    }
    if rank == 0 and not args.skip_sl:
        out["advection"] = sl_rates(args)
    if rank == 0:
        print(json.dumps(out))


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
    finally:
        dm.close()
    return {"sl_step": step,
            "location_sweep": {"points": args.sweep_points, "s": t_loc, "points_per_s": args.sweep_points / t_loc,
                               "locate": info}}


def run_operator_only(args, rank):
    """Operator-only run for profiler captures: set up the mixed-precision operator once, then time
    --op-reps applications of one level operator (precision 0 FP64, 1 FP32, 2 double-float)."""
    from m3tet_sph_gb300 import build as B
    B.build()
    from m3tet_sph_gb300 import stokes, workloads
    w = workloads.make_workload(args.workload, seed=args.seed)
    lv0 = w["levels"][0]
    dm = stokes.DeviceMesh(w["levels"])
    dm.setup(w["visc"], w["dens"], w["ifix"], w["vfix"], w["phys"], precision=1)
    for kv in args.set_option:
        k, v = kv.split("=")
        dm.set_option(k, int(v))
    ms = dm.apply_timing(args.op_level, args.op_precision, args.op_reps)
    nc = dm.ncolors(args.op_level)
    dm.close()
    s = 8 if args.op_precision in (0, 2) else 4
    b = apply_bytes(lv0["nel"], 3 * lv0["nnod"], s) if args.op_level == 0 else None
    if rank == 0:
        print(json.dumps({"workload": args.workload, "options": args.set_option, "nel": lv0["nel"], "colours": nc,
                          "level": args.op_level,
                          "precision": args.op_precision, "ms_per_apply": ms,
                          "gbs": None if b is None else b / (ms * 1e-3) / 1e9}))


def cpu_baseline(w, gpu_info, args):
    """FP64 oracle timed on the host: element matrices of a contiguous slice of the benchmark mesh
    (scaled to all elements) plus MG-PCG iterations on the 3-level 130k-DOF shell (scaled per DOF
    and by the iteration count the plain-FP64 GPU solve needed on the benchmark mesh)."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import stokes_oracle as O
    from m3tet_sph_gb300 import workloads
    lv0 = w["levels"][0]
    nel = lv0["nel"]
    S = args.cpu_sample_els
    nth = host_threads()
    # element matrices: the sample split into one block per host thread (numpy releases the GIL
    # in its array kernels), like the reference's element blocks over MATLAB's worker threads
    subs = [submesh(lv0, blk) for blk in np.array_split(np.arange(S), nth)]
    with ThreadPoolExecutor(nth) as pool:
        t = time.perf_counter()
        list(pool.map(lambda sb: O.element_matrices(sb, w["visc"][sb["gnodes"]], w["dens"][sb["gnodes"]],
                                                    **w["phys"]), subs))
        t_el = (time.perf_counter() - t) / S
    c1 = workloads.make_workload("c1", seed=args.seed)
    sysm = O.StokesSystem(c1["levels"], c1["visc"], c1["dens"], c1["ifix"], c1["vfix"], c1["phys"])
    # sparse products on threads only where that makes an MG-PCG iteration faster on this host (it
    # depends on whether the installed scipy releases the GIL in its CSR product, and on other
    # threads competing for the cores): time two iterations both ways
    nth_mg, t_ser, t_thr = 1, None, None
    if nth > 1:
        bt = np.random.default_rng(1).standard_normal(len(sysm.ifree))
        its = lambda: sysm.mg.solve(bt, np.zeros_like(bt), rtol=1e-30, itmax=2)
        t_ser = best_time(its, reps=2)
        sysm.mg.use_threads(nth)
        t_thr = best_time(its, reps=2)
        if t_thr < 0.95 * t_ser:
            nth_mg = nth
        else:
            sysm.mg.use_serial()
    rng = np.random.default_rng(0)
    b = rng.standard_normal(len(sysm.ifree))
    t = time.perf_counter()
    _, it, _ = sysm.mg.solve(b, np.zeros_like(b), rtol=1e-30, itmax=args.cpu_iters)
    t_it = (time.perf_counter() - t) / it
    nU1 = 3 * c1["levels"][0]["nnod"]
    nU2 = 3 * lv0["nnod"]
    iters = gpu_info["nitU"] + gpu_info["nitZ"]
    est = t_el * nel + t_it * (nU2 / nU1) * iters
    return {"value": est, "unit": "s", "cores": nth, "kind": "port",
            "sample": f"oracle element matrices of {S} of {nel} elements of this mesh ({t_el * 1e3:.3f} ms/el) + "
                      f"{it} MG-PCG iterations on the 130,662-DOF shell ({t_it:.2f} s/it; sparse products on "
                      f"{nth_mg} thread(s){thr_note(t_ser, t_thr, nth)}) scaled by DOF x {iters} iterations of "
                      f"the plain-FP64 solve"}


def best_time(f, reps=5):
    """Shortest of `reps` timed calls of f (after one untimed call)."""
    f()
    best = float("inf")
    for _ in range(reps):
        t = time.perf_counter()
        f()
        best = min(best, time.perf_counter() - t)
    return best


def thr_note(t_ser, t_thr, nth):
    if t_ser is None:
        return ""
    return f"; two iterations {t_ser:.2f} s on 1 thread, {t_thr:.2f} s on {nth}"


def host_threads():
    """Host threads this process may run on."""
    try:
        return max(1, len(os.sched_getaffinity(0)))
    except AttributeError:
        return max(1, os.cpu_count() or 1)


def submesh(lv, els):
    """Elements `els` of a level with their nodes renumbered (for bounded oracle samples)."""
    from m3tet_sph_gb300 import mesh as M
    EL = lv["EL2NOD"][els]
    g, inv = np.unique(EL, return_inverse=True)
    iso_mask = np.isin(lv["els_iso"], els)
    iso_new = np.searchsorted(els, lv["els_iso"][iso_mask]) if iso_mask.any() else np.zeros(0, np.int64)
    return {"EL2NOD": inv.reshape(EL.shape), "GCOORD": lv["GCOORD"][:, g], "GCOORD_SPH": lv["GCOORD_SPH"][:, g],
            "cls": lv["cls"][els], "els_iso": iso_new, "cubic_sph_rot": lv["cubic_sph_rot"][iso_mask],
            "gnodes": g, "PointID": lv["PointID"][g]}


def run_reference(args, rank, ws, td):
    """CPU reference arm: the FP64 oracle on all host threads it can use, bounded per step."""
    if rank != 0:
        return
    from m3tet_sph_gb300 import workloads
    w = workloads.make_workload(args.workload, seed=args.seed)
    fake_info = {"nitU": args.ref_iters // 2, "nitZ": args.ref_iters - args.ref_iters // 2}
    for _ in range(args.warmup):
        cpu_baseline(w, fake_info, argparse.Namespace(**{**vars(args), "cpu_sample_els": 2000, "cpu_iters": 1}))
    vals = []
    for _ in range(args.steps):
        vals.append(cpu_baseline(w, fake_info, args))
    v = float(np.mean([c["value"] for c in vals]))
    out = {"metric": METRIC, "value": v, "unit": "s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": v * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": "synthetic", "impl": "reference",
           "config": {"workload": f"shell L{w['level']} x {w['nlayer']} layers, {w['levels'][0]['nel']} P2 tets"},
           "cpu_baseline": {"value": v, "unit": "s", "cores": vals[-1]["cores"], "kind": "port",
                            "sample": vals[-1]["sample"]},
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
    ap.add_argument("--cpu-sample-els", type=int, default=20000)
    ap.add_argument("--cpu-iters", type=int, default=3)
    ap.add_argument("--ref-iters", type=int, default=988,
                    help="MG-PCG iterations the reference arm charges per solve (nitU + nitZ of the "
                         "plain-FP64 GPU solve of the 8M-DOF shell)")
    ap.add_argument("--skip-learned", action="store_true", help="time the Jacobi-smoothed FP32 solve instead")
    ap.add_argument("--skip-jacobi", action="store_true", help="skip the Jacobi-smoothed comparison solve")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--sl-only", action="store_true", help="semi-Lagrangian rates only (profiling)")
    ap.add_argument("--sweep-only", action="store_true", help="with --sl-only: the location sweep alone")
    ap.add_argument("--sl-workload", default="c1", help="mesh of the semi-Lagrangian measurements")
    ap.add_argument("--skip-sl", action="store_true")
    ap.add_argument("--sweep-points", type=int, default=16_000_000)
    ap.add_argument("--op-only", action="store_true", help="time one level operator only (profiling)")
    ap.add_argument("--op-level", type=int, default=0)
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
    elif args.impl == "reference":
        run_reference(args, rank, ws, td)
    else:
        run_gb300(args, rank, ws, td)
    if td is not None:
        td.destroy_process_group()


if __name__ == "__main__":
    main()
