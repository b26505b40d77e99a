"""Learned element smoother: forward / gradients against CPU autograd, and its effect on MG-PCG."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def dm_tiny(built_lib, tiny_plates):
    from m3tet_sph_gb300 import stokes
    w = tiny_plates
    dm = stokes.DeviceMesh(w['levels'])
    dm.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=1)
    yield w, dm
    dm.close()


def _torch_reference(p, X, T):
    torch = pytest.importorskip("torch")
    t = torch.tensor
    W1 = t(p[:128 * 64].reshape(128, 64), dtype=torch.float64, requires_grad=True)
    b1 = t(p[8192:8192 + 128], dtype=torch.float64, requires_grad=True)
    W2 = t(p[8320:8320 + 4096].reshape(32, 128), dtype=torch.float64, requires_grad=True)
    b2 = t(p[12416:12448], dtype=torch.float64, requires_grad=True)
    bf = lambda a: a.to(torch.bfloat16).to(torch.float64)
    Xb = bf(t(X, dtype=torch.float64))
    H = Xb @ bf(W1).T + b1
    G = torch.nn.functional.gelu(H)
    Y = bf(G) @ bf(W2).T + b2
    loss = ((Y[:, :30] - t(T[:, :30], dtype=torch.float64)) ** 2).mean()
    loss.backward()
    g = np.concatenate([W1.grad.numpy().ravel(), b1.grad.numpy(), W2.grad.numpy().ravel(), b2.grad.numpy()])
    return Y.detach().numpy()[:, :30], g, loss.item() * X.shape[0] * 30


def test_forward_and_gradients_match_autograd(dm_tiny):
    from m3tet_sph_gb300 import learned
    w, dm = dm_tiny
    rng = np.random.default_rng(0)
    p = learned.init_params(3)
    p[8192:8192 + 128] = rng.normal(0, 0.1, 128)
    p[12416:12416 + 30] = rng.normal(0, 0.1, 30)
    learned.set_params(dm, p, trained=False)
    n = 256
    X = np.zeros((n, 64), np.float32)
    X[:, :52] = rng.normal(size=(n, 52))
    T = np.zeros((n, 32), np.float32)
    T[:, :30] = rng.normal(size=(n, 30))
    Y = learned.forward(dm, X)
    g, loss = learned.gradients(dm, X, T)
    Yr, gr, lossr = _torch_reference(p, X, T)
    assert np.abs(Y - Yr).max() < 2e-2 * np.abs(Yr).max()
    assert abs(loss - lossr) < 1e-2 * lossr
    # bf16 rounding of dY, G and dH in the backward GEMMs: agreement to ~1e-2 of the gradient scale
    for a, b, name in ((0, 8192, 'W1'), (8192, 8320, 'b1'), (8320, 12416, 'W2'), (12416, 12448, 'b2')):
        err = np.linalg.norm(g[a:b] - gr[a:b]) / np.linalg.norm(gr[a:b])
        assert err < 3e-2, (name, err)


def test_training_reduces_loss(dm_tiny):
    from m3tet_sph_gb300 import learned
    w, dm = dm_tiny
    p, hist = learned.train_smoother(dm, w, n_fields=3, samples=60000, n_iterates=3, epochs=6, batch=1024,
                                     lr=2e-3, seed=1)
    assert hist['mse'][-1] < 0.8 * hist['mse'][0], hist
    assert np.isfinite(p).all()


def test_learned_smoother_solution_and_fallback(dm_tiny):
    """With the learned smoother the converged answer is the same (outer FP64 CG judges it);
    the iteration counts with / without it are reported."""
    from m3tet_sph_gb300 import learned
    w, dm = dm_tiny
    dm.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=1)
    kw = dict(rtol_Pat=1e-8, rtol_U=5e-3, itmax_Pat=200, itmax_U=40, target_rel_residual=1e-8)
    U0, P0, i0 = dm.solve(smoother=0, **kw)
    U1, P1, i1 = dm.solve(smoother=1, **kw)
    assert i1['rel_residual'] < 1e-8 and i0['rel_residual'] < 1e-8
    assert np.linalg.norm(U1 - U0) < 1e-6 * np.linalg.norm(U0)
    print(f"jacobi: {i0['nitU'] + i0['nitZ']} its, learned: {i1['nitU'] + i1['nitZ']} its, "
          f"fallbacks {i1['smoother_fallbacks']}")


def _sweep_both(dm, level, r, d0, kd):
    from m3tet_sph_gb300 import learned
    y1 = learned.sweep32(dm, level, r, d0, kd)
    y1b = learned.sweep32(dm, level, r, d0, kd)
    try:
        dm.set_option("ml_infer", 0)
        y0 = learned.sweep32(dm, level, r, d0, kd)
    finally:
        dm.set_option("ml_infer", 1)
    return y1, y1b, y0


@pytest.mark.parametrize("mesh", ["tiny", "shell491k"])
def test_fused_tcgen05_sweep_matches_wmma_kernel(built_lib, tiny_plates, mesh):
    """The fused tcgen05 sweep (default) against the WMMA tile kernel on the same residuals and
    the trained weights: the same features, FP32 accumulation in either order, BF16 hidden
    activations (a rounding flip moves an output by ~1e-3 of its size), the same node sums. The
    491,520-element shell gives each persistent CTA several tiles."""
    from pathlib import Path
    from m3tet_sph_gb300 import learned, stokes, workloads
    w = tiny_plates if mesh == "tiny" else workloads.make_workload('prof')
    dm = stokes.DeviceMesh(w['levels'])
    try:
        dm.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=1)
        p = np.load(Path(learned.__file__).with_name('smoother_c1.npy'))
        learned.set_params(dm, p, trained=True)
        rng = np.random.default_rng(21)
        for level in (0, 1):
            n = 3 * w['levels'][level]['nnod']
            # d0 = 0: the sweep's output is the correction itself (added to a nonzero d0, corrections
            # below half an ulp of d0 would vanish and look like fixed dofs)
            r, kd = (rng.standard_normal(n).astype(np.float32) for _ in range(2))
            d0 = np.zeros(n, np.float32)
            for k in (kd, None):
                y1, y1b, y0 = _sweep_both(dm, level, r, d0, k)
                assert np.array_equal(y1, y1b)                     # deterministic
                c1, c0 = y1, y0
                assert np.all(np.isfinite(c1)) and np.linalg.norm(c0) > 0
                assert np.linalg.norm(c1 - c0) < 1e-2 * np.linalg.norm(c0), (level, k is None)
                fixed = c0 == 0
                assert np.all(c1[fixed] == 0)                      # fixed dofs untouched
    finally:
        dm.close()


@pytest.mark.parametrize("level", [0, 1])
def test_features_match_cpu_restatement(built_lib, tiny_plates, level):
    """The 52 inputs the fused sweep builds per element (Jacobi-scaled local residual over its norm,
    standardised log-viscosities, scale-free geometry) against the CPU restatement in the oracle."""
    from pathlib import Path
    from oracle import ml_oracle as MO
    from m3tet_sph_gb300 import learned, stokes
    w = tiny_plates
    dm = stokes.DeviceMesh(w['levels'])
    try:
        dm.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=1)
        learned.set_params(dm, np.load(Path(learned.__file__).with_name('smoother_c1.npy')), trained=True)
        n = 3 * w['levels'][level]['nnod']
        z = np.random.default_rng(5).standard_normal(n).astype(np.float32)
        X, s = learned.features(dm, level, z)
    finally:
        dm.close()
    r = w['levels'][0]['GCOORD_SPH'][2]
    Xr, sr = MO.features(w['levels'], level, w['visc'], z, float(r.min()), float(r.max()))
    assert np.allclose(s, sr, rtol=1e-5, atol=0)
    assert np.max(np.abs(X[:, :30] - Xr[:, :30])) < 1e-5        # unit-norm residual part
    assert np.max(np.abs(X[:, 30:40] - Xr[:, 30:40])) < 1e-4    # standardised log-viscosities
    assert np.max(np.abs(X[:, 40:] - Xr[:, 40:])) < 1e-5        # geometry factors


def test_trained_network_gain_per_sweep(built_lib):
    """What the trained network gains over the method without it, per sweep, on the 130,662-DOF
    shell: for white-noise errors e (r = K e), the K-norm of the error left by one learned sweep is
    well below that left by one weighted-Jacobi sweep (the plain smoother's first finest-level sweep,
    weight 0.9) and far below that of the same network with untrained (initial) weights."""
    from pathlib import Path
    from m3tet_sph_gb300 import learned, stokes, workloads
    w = workloads.make_workload('c1')
    dm = stokes.DeviceMesh(w['levels'])
    try:
        dm.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=1)
        n = 3 * w['levels'][0]['nnod']
        dinv = dm.level_inverse_diag32(0)                 # 0 on fixed dofs
        free = dinv != 0
        rng = np.random.default_rng(17)

        def knorm(e):
            e = e.astype(np.float32)
            return float(np.sqrt(np.dot(e.astype(np.float64), dm.level_apply32(0, e).astype(np.float64))))

        trained = np.load(Path(learned.__file__).with_name('smoother_c1.npy'))
        ratios = {"learned": [], "untrained": [], "jacobi": []}
        for k in range(3):
            e = np.where(free, rng.standard_normal(n), 0.0).astype(np.float32)
            r = dm.level_apply32(0, e)
            e0 = knorm(e)
            for name, p in (("learned", trained), ("untrained", learned.init_params(0))):
                learned.set_params(dm, p, trained=True)
                d = learned.sweep32(dm, 0, r, np.zeros(n, np.float32))
                ratios[name].append(knorm(e - d) / e0)
            dj = (0.9 * r * dinv).astype(np.float32)
            ratios["jacobi"].append(knorm(e - dj) / e0)
    finally:
        dm.close()
    m = {k: float(np.mean(v)) for k, v in ratios.items()}
    print("error left in the K-norm after one sweep:", m)
    assert m["learned"] < 0.9 * m["jacobi"]
    assert m["learned"] < 0.5 * m["untrained"]
