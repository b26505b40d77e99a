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
