"""rock_prop and the device-resident time step (rock_prop -> Stokes -> calculate_dt -> SL advection,
M3TET_SPH_SOUTH_ATLANTIC_PLUME.m:213-296), through the C ABI, against the oracle and against the
same calls made one by one."""
import numpy as np
import pytest

from oracle import slm_oracle as SO
from oracle import stokes_oracle as O

pytestmark = pytest.mark.gpu

R_CMB, R_SURF = 3480.0, 6371.0


@pytest.fixture(scope='module')
def plates(built_lib, tiny_plates):
    return tiny_plates


@pytest.mark.parametrize("variant", ["full", "no_arrhenius", "no_pressure", "no_cutoffs"])
def test_rock_prop_matches_oracle(plates, variant):
    from m3tet_sph_gb300 import stokes, workloads
    w = plates
    p = workloads.rock_params(1e6)
    if variant == "no_arrhenius":
        p['Ea'] = 0.0
    elif variant == "no_pressure":
        p['Va'], p['a_UM2LM'] = 0.0, 0.0
    elif variant == "no_cutoffs":
        p.update(minVisc=None, maxVisc=None, minDens=None, maxDens=None)
    else:
        p.update(minDens=3200.0, maxDens=3400.0)
    T = 2500.0 * w['T']
    dm = stokes.DeviceMesh(w['levels'])
    try:
        V, D = dm.rock_prop(T, p)
    finally:
        dm.close()
    Vr, Dr = O.rock_prop(T, w['levels'][0]['GCOORD'], **p)
    # exp() of the device and of the host may differ in the last bit
    assert np.max(np.abs(V - Vr) / np.abs(Vr)) < 1e-13
    assert np.max(np.abs(D - Dr) / np.abs(Dr)) < 1e-15


def test_rock_prop_rejects_kj_per_mol(plates):
    from m3tet_sph_gb300 import _lib as L, stokes, workloads
    w = plates
    p = workloads.rock_params()
    p['Ea'] = 250.0
    dm = stokes.DeviceMesh(w['levels'])
    try:
        with pytest.raises(L.M3SphError, match='kJ/mol'):
            dm.rock_prop(w['T'], p)
    finally:
        dm.close()


def _setup(dm, w, visc, dens, precision):
    dm.setup(visc, dens, w['ifix'], w['vfix'], w['phys'], precision=precision)


def test_time_step_equals_the_calls_one_by_one(plates):
    """Two device-resident steps give the temperature, time step and velocity of the same hot-path
    calls made one by one through the C ABI with host arrays (rock_prop, stokes_setup + stokes_solve
    from the previous pressure, calculate_dt, advect_slm with the WS_SLM guesses). They agree to
    rounding rather than bit for bit: the element set-up sums the right-hand side of the nonzero
    prescribed velocities with shared-memory atomics, whose order varies between set-ups."""
    from m3tet_sph_gb300 import advection as A, stokes, workloads
    w = plates
    rock = workloads.rock_params(1e3)
    kw = dict(rtol_Pat=1e-6, rtol_U=5e-3, itmax_Pat=200, itmax_U=40, target_rel_residual=1e-8)
    T0 = 2500.0 * w['T']
    dm, dm2 = stokes.DeviceMesh(w['levels']), stokes.DeviceMesh(w['levels'])
    try:
        _setup(dm, w, w['visc'], w['dens'], 1)
        dm.set_temperature(T0)
        steps = [dm.time_step(kw, rock=rock, dt_adv_limit=0.01, dtmax=50.0) for _ in range(2)]
        T_dev = dm.get_temperature()
        U_dev, P_dev = dm.solution()
        T = T0.copy()
        P = None
        WS = None
        MESH = dict(levels=w['levels'], device_mesh=dm2, r_cmb=R_CMB, r_surf=R_SURF)
        for k in range(2):
            V, D = dm2.rock_prop(T, rock)
            _setup(dm2, w, V, D, 1)
            U, P, info = dm2.solve(P0=P, **kw)
            dt, adv = dm2.calculate_dt(0.01, 50.0)
            assert dt == pytest.approx(steps[k]['dt'], rel=1e-12)
            assert adv == pytest.approx(steps[k]['dt_adv'], rel=1e-12)
            T, WS = A.advect3d_slm_p_sph(MESH, None, U[0::3], U[1::3], U[2::3], T, dt,
                                         dict(method_BT='PC2', method_interp='cubic'), WS)
            assert np.array_equal(WS['els_INTERP'] > 0, np.ones(len(T), bool))
        assert np.linalg.norm(U - U_dev) <= 1e-12 * np.linalg.norm(U)
        assert np.linalg.norm((P - P.mean()) - (P_dev - P_dev.mean())) <= 1e-12 * np.linalg.norm(P - P.mean())
        assert np.max(np.abs(T - T_dev)) <= 1e-12 * np.max(np.abs(T0))
        assert steps[1]['time'] == steps[0]['dt'] + steps[1]['dt']
        for st in steps:
            assert st['status'] == 0 and st['locate']['nlost'] == 0 and st['dt'] > 0
    finally:
        dm.close()
        dm2.close()


def test_time_step_matches_oracle(plates):
    """One step against the oracle's rock_prop -> Patera (tight) -> calculate_dt -> PC2 + cubic
    advection: the same time step and the same advected temperature to the accuracy of the solves."""
    from m3tet_sph_gb300 import stokes, workloads
    w = plates
    f = w['levels'][0]
    rock = workloads.rock_params(1e3)
    T0 = 2500.0 * w['T']
    dm = stokes.DeviceMesh(w['levels'])
    try:
        _setup(dm, w, w['visc'], w['dens'], 0)
        dm.set_temperature(T0)
        st = dm.time_step(dict(rtol_Pat=1e-9, rtol_U=1e-4, itmax_Pat=300, itmax_U=40, target_rel_residual=1e-11),
                          rock=rock, dt_adv_limit=0.01, dtmax=50.0)
        T_dev = dm.get_temperature()
    finally:
        dm.close()
    V, D = O.rock_prop(T0, f['GCOORD'], **rock)
    S = O.StokesSystem(w['levels'], V, D, w['ifix'], w['vfix'], w['phys'])
    Ur, Pr, _ = O.patera(S, rtol_Pat=1e-11, rtol_U=1e-4, itmax_Pat=400, itmax_U=60)
    Uxyz = (S.RR @ Ur).reshape(-1, 3)
    dt, adv = O.calculate_dt(f['GCOORD'], Uxyz[:, 0], Uxyz[:, 1], Uxyz[:, 2], 0.01, 50.0)
    assert abs(st['dt'] - dt) < 1e-8 * dt
    Tr, Pd, e1, e2 = SO.advect_pc2(f, Uxyz, T0, dt, R_CMB, R_SURF, method_interp='cubic')
    assert np.max(np.abs(T_dev - Tr)) < 1e-7 * np.max(np.abs(T0))


def test_time_steps_with_learned_smoother_c1(built_lib):
    """Three steps on the 130,662-DOF shell with the learned smoother and RK4 backtracking: every
    solve converges to its target, every departure point is located, the step grows the model time,
    and the cubic monotone interpolation keeps T inside its initial range."""
    from pathlib import Path
    from m3tet_sph_gb300 import learned, stokes, workloads
    w = workloads.make_workload('c1')
    T0 = 2500.0 * w['T']
    dm = stokes.DeviceMesh(w['levels'])
    try:
        _setup(dm, w, w['visc'], w['dens'], 1)
        learned.set_params(dm, np.load(Path(learned.__file__).with_name('smoother_c1.npy')), trained=True)
        dm.set_temperature(T0)
        t = 0.0
        for k in range(3):
            st = dm.time_step(dict(rtol_Pat=1e-7, itmax_Pat=400, itmax_U=40, target_rel_residual=1e-8),
                              slm=dict(method_BT='RK4'), rock=workloads.rock_params(1e4), smoother=1,
                              dt_adv_limit=0.005, dtmax=100.0)
            assert st['status'] == 0 and st['stokes']['rel_residual'] <= 1e-8
            assert st['locate']['nlost'] == 0 and st['dt'] > 0
            t += st['dt']
            assert st['time'] == pytest.approx(t)
        T = dm.get_temperature()
        assert np.all(np.isfinite(T))
        assert T.min() >= T0.min() - 1e-9 and T.max() <= T0.max() + 1e-9
    finally:
        dm.close()


def test_restart_file_resumes_the_time_series(plates, tmp_path):
    """Two steps in one handle; the same series written to a restart file after step 1 and resumed
    in a fresh handle gives the same step 2 (write_restart_file.m / load_restart_data.m)."""
    from m3tet_sph_gb300 import restart as R, stokes, workloads
    w = plates
    rock = workloads.rock_params(1e3)
    kw = dict(rtol_Pat=1e-6, rtol_U=5e-3, itmax_Pat=200, itmax_U=40, target_rel_residual=1e-8)
    T0 = 2500.0 * w['T']
    dm, dm2 = stokes.DeviceMesh(w['levels']), stokes.DeviceMesh(w['levels'])
    try:
        _setup(dm, w, w['visc'], w['dens'], 1)
        dm.set_temperature(T0)
        s1 = dm.time_step(kw, rock=rock, dt_adv_limit=0.01, dtmax=50.0)
        path = R.write_restart_file({'outdir': str(tmp_path)}, R.var_from_device(dm), None, 2, 1, s1['time'],
                                    s1['dt'], 1)
        s2 = dm.time_step(kw, rock=rock, dt_adv_limit=0.01, dtmax=50.0)
        T2 = dm.get_temperature()
        VAR, time, istep, iplot = R.load_restart_file(path)
        assert time == s1['time'] and istep == 2
        _setup(dm2, w, VAR['Visc'], VAR['Dens'], 1)
        R.restore_device(dm2, VAR, time)
        r2 = dm2.time_step(kw, rock=rock, dt_adv_limit=0.01, dtmax=50.0)
        assert r2['time'] == pytest.approx(s2['time'], rel=1e-12)
        assert np.max(np.abs(dm2.get_temperature() - T2)) <= 1e-12 * np.max(np.abs(T0))
    finally:
        dm.close()
        dm2.close()
