"""Training driver for the learned element smoother (no counterpart in the reference).

Training pairs (local residual, local error) come from plain-multigrid solves of the project's own
operator on a shell mesh over seeded viscosity fields; the network is trained on the GPU by the
library's forward / backward kernels (m3sph_ml_train_epoch). Weights are a flat FP32 vector
(m3sph_ml_nparam values) that can be saved with numpy and loaded into any mesh handle.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import _lib as L
from . import workloads


def nparam():
    n = C.c_int32()
    L.check(L.lib().m3sph_ml_nparam(C.byref(n)))
    return n.value


def init_params(seed=0):
    """Xavier-uniform weights, zero biases, zero padding (W1 [128][64], b1, W2 [32][128], b2)."""
    rng = np.random.default_rng(seed)
    W1 = np.zeros((128, 64), np.float32)
    W1[:, :52] = rng.uniform(-1, 1, (128, 52)) * np.sqrt(6.0 / (52 + 128))
    W2 = np.zeros((32, 128), np.float32)
    W2[:30] = rng.uniform(-1, 1, (30, 128)) * np.sqrt(6.0 / (128 + 30))
    p = np.concatenate([W1.ravel(), np.zeros(128, np.float32), W2.ravel(), np.zeros(32, np.float32)])
    assert p.size == nparam()
    return p


def set_params(dm, p, trained=True):
    p = np.ascontiguousarray(p, dtype=np.float32)
    L.check(L.lib().m3sph_ml_set_params(dm.h, L.fptr(p), int(trained)))


def get_params(dm):
    p = np.zeros(nparam(), np.float32)
    L.check(L.lib().m3sph_ml_get_params(dm.h, L.fptr(p)))
    return p


def forward(dm, X):
    X = np.ascontiguousarray(X, dtype=np.float32)
    Y = np.zeros((X.shape[0], 30), np.float32)
    L.check(L.lib().m3sph_ml_forward(dm.h, L.fptr(X), X.shape[0], L.fptr(Y)))
    return Y


def sweep32(dm, level, r, d, kd=None):
    """One learned sweep of `level` in FP32 (m3sph_ml_sweep32): returns d + the gathered corrections."""
    r = np.ascontiguousarray(r, dtype=np.float32)
    out = np.array(d, dtype=np.float32, copy=True)
    kdp = None if kd is None else L.fptr(np.ascontiguousarray(kd, dtype=np.float32))
    L.check(L.lib().m3sph_ml_sweep32(dm.h, int(level), L.fptr(r), kdp, L.fptr(out)))
    return out


def features(dm, level, z):
    """Inputs of the learned smoother on `level` for a Jacobi-scaled residual z (m3sph_ml_features):
    (X [nel][52] in original element order, residual norms s [nel])."""
    z = np.ascontiguousarray(z, dtype=np.float32)
    nel = dm.levels[level]['nel']
    X = np.zeros((nel, 52), np.float32)
    s = np.zeros(nel, np.float32)
    L.check(L.lib().m3sph_ml_features(dm.h, int(level), L.fptr(z), L.fptr(X), L.fptr(s)))
    return X, s


def gradients(dm, X, T):
    X = np.ascontiguousarray(X, dtype=np.float32)
    T = np.ascontiguousarray(T, dtype=np.float32)
    g = np.zeros(nparam(), np.float32)
    loss = C.c_double()
    L.check(L.lib().m3sph_ml_gradients(dm.h, L.fptr(X), L.fptr(T), X.shape[0], L.fptr(g), C.byref(loss)))
    return g, loss.value


def collect(dm, seed, n_iterates=4, stride=1):
    n = C.c_int64()
    L.check(L.lib().m3sph_ml_collect(dm.h, int(seed), int(n_iterates), int(stride), C.byref(n)))
    return n.value


def collect_mg_pairs(dm, seed, n_rhs, n_iterates, stride):
    """(residual, error) pairs of plain multigrid iterates: for seeded right-hand sides b on the
    free dofs, x* from a tight MG-PCG solve, then the iterates x_k after k = 1..n_iterates MG-PCG
    iterations from zero with r_k = b - K x_k and e_k = x* - x_k (the operator and V-cycle of the
    current set-up, Jacobi smoothing)."""
    rng = np.random.default_rng(seed)
    count = C.c_int64()
    for i in range(n_rhs):
        b = rng.standard_normal(dm.ndof)
        x_star, _, _ = dm.mgpcg(b, np.zeros(dm.ndof), 1e-12, is_abs_tol=False, itmax=300)
        for k in range(1, n_iterates + 1):
            x_k, _, _ = dm.mgpcg(b, np.zeros(dm.ndof), 1e-30, is_abs_tol=False, itmax=k)
            r_k = b - dm.apply(x_k)
            e_k = np.ascontiguousarray(x_star - x_k)
            L.check(L.lib().m3sph_ml_add_pairs(dm.h, L.dptr(np.ascontiguousarray(r_k)), L.dptr(e_k), int(stride),
                                                int((seed + i * n_iterates + k) % stride), C.byref(count)))
    return count.value


def train_smoother(dm, w, n_fields=20, contrast_range=(1e2, 1e5), samples=2_000_000, n_iterates=4, epochs=12,
                   batch=4096, lr=2e-3, seed=0, precision=1, log=None, pairs="noise"):
    """Collect pairs over `n_fields` seeded viscosity fields on the mesh of workload `w`, train,
    and leave the trained weights loaded in `dm`. pairs: "noise" -- (K e, e) for white-noise errors
    e; "mg" -- residuals and errors of plain multigrid iterates (collect_mg_pairs). Returns
    (params, history)."""
    rng = np.random.default_rng(seed)
    nel = w['levels'][0]['nel']
    per_field = samples / n_fields
    stride = max(1, int(nel * n_iterates // per_field))
    dm.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=precision)
    L.check(L.lib().m3sph_ml_reserve(dm.h, int(samples) + nel))
    t0 = time.time()
    for i in range(n_fields):
        c = float(np.exp(rng.uniform(np.log(contrast_range[0]), np.log(contrast_range[1]))))
        T = workloads.temperature(w['levels'], seed + 1000 + i)
        visc = workloads.viscosity(w['levels'], T, c, 30.0)
        dm.setup(visc, workloads.density(T), w['ifix'], w['vfix'], w['phys'], precision=precision)
        if pairs == "mg":
            count = collect_mg_pairs(dm, seed * 7919 + i, 1, n_iterates, stride)
        else:
            count = collect(dm, seed * 7919 + i, n_iterates, stride)
        if log:
            log(f"field {i}: contrast {c:.3g}, samples {count}")
    t_collect = time.time() - t0
    set_params(dm, init_params(seed), trained=False)
    hist = []
    t0 = time.time()
    for ep in range(epochs):
        mse = C.c_double()
        lr_ep = lr * (0.5 ** (ep // max(1, epochs // 3)))
        L.check(L.lib().m3sph_ml_train_epoch(dm.h, int(batch), float(lr_ep), int(seed + ep), C.byref(mse)))
        hist.append(mse.value)
        if log:
            log(f"epoch {ep}: mse {mse.value:.5f}")
    t_train = time.time() - t0
    return get_params(dm), dict(mse=hist, t_collect=t_collect, t_train=t_train, stride=stride)


def evaluate(dm, w, params=None, solver_kw=None, repeats=1, schedule=1):
    """Solve once with the Jacobi smoother and once with the learned smoother on the mesh and fields
    of workload `w` (FP32 V-cycle): iteration counts, times and the difference of the answers."""
    kw = dict(rtol_Pat=1e-7, rtol_U=5e-3, itmax_Pat=400, itmax_U=40, target_rel_residual=1e-8)
    kw.update(solver_kw or {})
    dm.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=1)
    if params is not None:
        set_params(dm, params, trained=True)
    dm.set_option("ml_schedule", schedule)
    out, sols = {"schedule": schedule}, {}
    for name, sm in (('jacobi', 0), ('learned', 1)):
        best = None
        for _ in range(repeats):
            info = dm.step_device(smoother=sm, **kw)
            best = info if best is None or info['t_iter_ms'] < best['t_iter_ms'] else best
        sols[name] = dm.solution()[0]
        out[name] = dict(its=best['nitU'] + best['nitZ'], itPat=best['itPat'], t_iter_ms=best['t_iter_ms'],
                         rel_residual=best['rel_residual'], fallbacks=best['smoother_fallbacks'])
    out['dU'] = float(np.linalg.norm(sols['learned'] - sols['jacobi']) / np.linalg.norm(sols['jacobi']))
    return out


def main(argv=None):
    import argparse
    import json
    from . import stokes
    ap = argparse.ArgumentParser(description="train / evaluate the learned element smoother")
    ap.add_argument("cmd", choices=["train", "evaluate"])
    ap.add_argument("--workload", default="c1")
    ap.add_argument("--weights", required=True, help=".npy file written by train, read by evaluate")
    ap.add_argument("--fields", type=int, default=20)
    ap.add_argument("--samples", type=int, default=2_000_000)
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--schedule", type=int, default=1, help="0: learned-Jacobi-learned per side, 1: one learned sweep")
    ap.add_argument("--pairs", default="noise", choices=["noise", "mg"],
                    help="training pairs: white-noise (K e, e) or plain-multigrid iterates")
    a = ap.parse_args(argv)
    w = workloads.make_workload(a.workload, seed=a.seed)
    dm = stokes.DeviceMesh(w['levels'])
    try:
        if a.cmd == "train":
            p, h = train_smoother(dm, w, n_fields=a.fields, samples=a.samples, epochs=a.epochs, seed=a.seed,
                                  log=lambda m: print(m, flush=True), pairs=a.pairs)
            np.save(a.weights, p)
            print(json.dumps({"mse": h["mse"], "t_collect_s": h["t_collect"], "t_train_s": h["t_train"],
                              "stride": h["stride"]}))
        else:
            print(json.dumps({"workload": a.workload, **evaluate(dm, w, np.load(a.weights), schedule=a.schedule)}))
    finally:
        dm.close()


if __name__ == "__main__":
    main()
