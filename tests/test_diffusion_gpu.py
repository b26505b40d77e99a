"""Thermal diffusion half step (diffusion3d_p.m with the default options) through the C ABI, against
the FP64 oracle (oracle/thermal_oracle.py) on the same 4-node split of the P2 mesh."""
import numpy as np
import pytest

from oracle import thermal_oracle as TO

pytestmark = pytest.mark.gpu

KAPPA = 31.6          # 1e-6 m^2/s in km^2/Myr (model_parameters_sph_south_atlantic_plume.m:483-487)


def _split(f):
    from m3tet_sph_gb300 import mesh as M
    return M.split_p2(f['GCOORD'], f['EL2NOD'])[0]


@pytest.fixture(scope='module', params=['tiny_plates', 'c1'])
def case(request, built_lib):
    from m3tet_sph_gb300 import stokes, workloads
    w = workloads.make_workload('c1') if request.param == 'c1' else request.getfixturevalue('tiny_plates')
    dm = stokes.DeviceMesh(w['levels'])
    yield w, dm
    dm.close()


@pytest.mark.parametrize("theta,dt", [(1.0, 50.0), (0.5, 200.0), (1.0, 0.05)])
def test_diffusion_matches_oracle(case, theta, dt):
    w, dm = case
    f = w['levels'][0]
    T0 = 2500.0 * w['T']
    fix = np.nonzero(f['PointID'] > 0)[0]
    dm.diffusion_setup(KAPPA, fix, T0[fix], theta=theta)
    T, nit = dm.diffusion(T0, dt)
    D = TO.Diffusion(f['GCOORD'], f['GCOORD_SPH'], _split(f), KAPPA, fix, theta=theta)
    Tr, nitr = D.step(T0, dt, T0[fix])
    print(f"theta {theta} dt {dt}: {nit} CG iterations (oracle {nitr}), max change {np.abs(T - T0).max():.3g}")
    assert nit == nitr
    assert np.max(np.abs(T - Tr)) <= 1e-10 * np.max(np.abs(T0))
    assert np.array_equal(T[fix], T0[fix])


def test_diffusion_keeps_a_constant_field(case):
    w, dm = case
    f = w['levels'][0]
    fix = np.nonzero(f['PointID'] > 0)[0]
    T0 = np.full(f['nnod'], 1300.0)
    dm.diffusion_setup(KAPPA, fix, T0[fix])
    T, nit = dm.diffusion(T0, 100.0)
    assert np.max(np.abs(T - 1300.0)) < 1e-9 * 1300.0


def test_time_step_with_diffusion_half_steps(built_lib, tiny_plates):
    """thermal_advdiff_3d_p inside the device time step: diffusion(dt/2) -> advection ->
    diffusion(dt/2) gives the temperature of the same three calls made one by one."""
    from m3tet_sph_gb300 import advection as A, stokes, workloads
    w = tiny_plates
    f = w['levels'][0]
    T0 = 2500.0 * w['T']
    fix = np.nonzero(f['PointID'] > 0)[0]
    kw = dict(rtol_Pat=1e-6, rtol_U=5e-3, itmax_Pat=200, itmax_U=40, target_rel_residual=1e-8)
    dm, dm2 = stokes.DeviceMesh(w['levels']), stokes.DeviceMesh(w['levels'])
    try:
        for d in (dm, dm2):
            d.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=1)
            d.diffusion_setup(KAPPA, fix, T0[fix])
        dm.set_temperature(T0)
        st = dm.time_step(kw, dt_adv_limit=0.01, dtmax=50.0, diffusion=True)
        T_dev = dm.get_temperature()
        U, P, info = dm2.solve(**kw)
        dt, _ = dm2.calculate_dt(0.01, 50.0)
        assert dt == pytest.approx(st['dt'], rel=1e-12)
        T, n1 = dm2.diffusion(T0, 0.5 * dt)
        MESH = dict(levels=w['levels'], device_mesh=dm2, r_cmb=3480.0, r_surf=6371.0)
        T, _ = A.advect3d_slm_p_sph(MESH, None, U[0::3], U[1::3], U[2::3], T, dt, dict(method_interp='cubic'))
        T, n2 = dm2.diffusion(T, 0.5 * dt)
        assert st['diffusion_its'] == n1 + n2
        assert np.max(np.abs(T - T_dev)) <= 1e-12 * np.max(np.abs(T0))
    finally:
        dm.close()
        dm2.close()
