"""Failure visibility of the Stokes solve, through the C ABI: a Patera iteration that runs out of
iterations is reported as M3SPH_ERR_NOT_CONVERGED (with the last iterate still delivered), and a
learned smoother that stops contracting is switched off by the outer FP64 CG without changing the
converged answer."""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def dm_plates(built_lib, tiny_plates):
    from m3tet_sph_gb300 import stokes
    w = tiny_plates
    dm = stokes.DeviceMesh(w['levels'])
    yield w, dm
    dm.close()


def test_itmax_pat_exhausted_is_not_converged(dm_plates):
    from m3tet_sph_gb300 import _lib as L
    w, dm = dm_plates
    dm.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=0)
    kw = dict(rtol_Pat=1e-12, rtol_U=1e-3, itmax_Pat=2, itmin_Pat=1, itmax_U=20)
    with pytest.raises(L.M3SphError) as ei:
        dm.solve(**kw)
    assert ei.value.code == L.ERR_NOT_CONVERGED
    assert 'not converged' in str(ei.value)
    U, P, info = ei.value.result
    assert info['status'] == L.ERR_NOT_CONVERGED and info['itPat'] == 2
    assert np.isfinite(U).all() and np.isfinite(P).all() and np.linalg.norm(U) > 0
    # the same call with the status accepted returns the same iterate
    U2, P2, info2 = dm.solve(allow_not_converged=True, **kw)
    assert info2['status'] == L.ERR_NOT_CONVERGED
    assert np.array_equal(U, U2) and np.array_equal(P, P2)
    # the device-resident step reports it too
    with pytest.raises(L.M3SphError) as ei:
        dm.step_device(**kw)
    assert ei.value.code == L.ERR_NOT_CONVERGED


def test_unreachable_target_is_not_converged(dm_plates):
    from m3tet_sph_gb300 import _lib as L
    w, dm = dm_plates
    dm.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=1)
    U, P, info = dm.solve(rtol_Pat=1e-6, itmax_Pat=6, target_rel_residual=1e-30, allow_not_converged=True)
    assert info['status'] == L.ERR_NOT_CONVERGED and info['rel_residual'] > 1e-30
    # a reachable target converges with status 0
    U, P, info = dm.solve(rtol_Pat=1e-6, itmax_Pat=200, target_rel_residual=1e-8)
    assert info['status'] == 0 and info['rel_residual'] <= 1e-8


def test_learned_smoother_fallback_is_forced_and_harmless(dm_plates):
    """A smoother that amplifies the error (the trained network's correction negated and scaled by
    3) makes the MG-PCG residual grow; the rate check must switch it off (smoother_fallbacks >= 1)
    and the solve must reach the same answer as the Jacobi-smoothed one."""
    from m3tet_sph_gb300 import learned
    w, dm = dm_plates
    dm.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=1)
    p = np.load(Path(learned.__file__).with_name('smoother_c1.npy')).astype(np.float32)
    bad = p.copy()
    bad[8320:] *= -1.0                      # W2 and b2 negated: the correction points the wrong way
    learned.set_params(dm, bad, trained=True)
    dm.set_option("ml_omega_pct", 300)
    kw = dict(rtol_Pat=1e-8, rtol_U=5e-3, itmax_Pat=200, itmax_U=40, target_rel_residual=1e-8)
    try:
        U0, P0, i0 = dm.solve(smoother=0, **kw)
        U1, P1, i1 = dm.solve(smoother=1, **kw)
    finally:
        dm.set_option("ml_omega_pct", 100)
        learned.set_params(dm, p, trained=True)
    assert i1['smoother_fallbacks'] >= 1, i1
    assert i0['smoother_fallbacks'] == 0
    assert i1['rel_residual'] <= 1e-8 and i0['rel_residual'] <= 1e-8
    assert np.linalg.norm(U1 - U0) < 1e-6 * np.linalg.norm(U0)
    Pc0, Pc1 = P0 - P0.mean(), P1 - P1.mean()
    assert np.linalg.norm(Pc1 - Pc0) < 1e-6 * np.linalg.norm(Pc0)


def test_calculate_dt_matches_oracle(dm_plates):
    """Device max-reduction CFL step (calculate_dt.m:40-52) on the resident velocity: bit-identical
    to the oracle's on the same velocity (a max is exact; one division and one multiply)."""
    from oracle import stokes_oracle as O
    w, dm = dm_plates
    dm.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=1)
    dm.solve(rtol_Pat=1e-6, itmax_Pat=200)
    U, _ = dm.solution()
    X = w['levels'][0]['GCOORD']
    for limit, dtmax in ((0.005, 0.1), (0.005, 1e-30), (1.0, 1e30)):
        dt, adv = dm.calculate_dt(limit, dtmax)
        dt_r, adv_r = O.calculate_dt(X, U[0::3], U[1::3], U[2::3], limit, dtmax)
        assert dt == dt_r and adv == adv_r, (limit, dtmax, dt, dt_r)
