"""GPlates-driven surface velocities on the device (m3sph_stokes_set_vel_bc): between solves, and in
the device-resident time loop, where update_vel_bc runs before every flow3d_patera_sph
(M3TET_SPH_SOUTH_ATLANTIC_PLUME.m:236-241). Seeded series in the GPlates export format stand in for
the reference's files."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KW = dict(rtol_Pat=1e-9, rtol_U=1e-4, itmax_Pat=300, itmax_U=40, target_rel_residual=1e-10)


@pytest.fixture(scope='module')
def series(built_lib, tiny_plates, tmp_path_factory):
    from m3tet_sph_gb300 import gplates as G
    f = tiny_plates['levels'][0]
    folder = G.write_synthetic_folder(tmp_path_factory.mktemp('vel_bcs'), G.synthetic_vel_bcs(f, seed=5))
    V, t = G.read_vel_gplates_folder(folder)
    return G.VelBCSeries(V, t, f['PointID'], 6371.0)


@pytest.mark.parametrize('precision', [0, 1])
def test_set_vel_bc_equals_a_fresh_setup(tiny_plates, series, precision):
    """New values pushed into a set-up handle give the solve of a handle set up with them, to
    rounding (the element set-up sums the prescribed-velocity right-hand side with shared-memory
    atomics, whose order varies between set-ups)."""
    from m3tet_sph_gb300 import stokes
    w = tiny_plates
    UBC, _ = series.at(1.3)
    a, b = stokes.DeviceMesh(w['levels']), stokes.DeviceMesh(w['levels'])
    try:
        a.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=precision)
        U0, _, _ = a.solve(**KW)
        a.set_vel_bc(UBC['ifix'] - 1, UBC['vfix'])
        U1, P1, _ = a.solve(**KW)
        b.setup(w['visc'], w['dens'], UBC['ifix'] - 1, UBC['vfix'], w['phys'], precision=precision)
        U2, P2, _ = b.solve(**KW)
    finally:
        a.close()
        b.close()
    assert np.linalg.norm(U1 - U2) <= 1e-11 * np.linalg.norm(U2)
    dP1, dP2 = P1 - P1.mean(), P2 - P2.mean()
    assert np.linalg.norm(dP1 - dP2) <= 1e-11 * np.linalg.norm(dP2)
    # the new plate velocities did change the flow
    assert np.linalg.norm(U1 - U0) > 1e-2 * np.linalg.norm(U0)


def test_set_vel_bc_rejects_another_dof_set(tiny_plates):
    from m3tet_sph_gb300 import _lib as L, stokes
    w = tiny_plates
    dm = stokes.DeviceMesh(w['levels'])
    try:
        dm.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=1)
        with pytest.raises(L.M3SphError, match='differ'):
            dm.set_vel_bc(w['ifix'][:-1], w['vfix'][:-1])
        moved = w['ifix'].copy()
        moved[-1] = np.setdiff1d(np.arange(3 * dm.nnod), w['ifix'])[0]
        with pytest.raises(L.M3SphError, match='differ'):
            dm.set_vel_bc(moved, w['vfix'])
    finally:
        dm.close()


def test_time_steps_follow_the_gplates_series(tiny_plates, series):
    """Three device-resident steps with the series: each step's solve carries, on every fixed dof,
    the series' values at the model time the step starts from (0, then the growing model time,
    crossing the 103 / 102 / 101 Ma files), and the step reports VAR.Plate."""
    from m3tet_sph_gb300 import mesh as M, stokes, workloads
    w = tiny_plates
    f = w['levels'][0]
    R = M.rotation_blocks(f['GCOORD'])
    dm = stokes.DeviceMesh(w['levels'])
    try:
        dm.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=1)
        dm.set_temperature(2500.0 * w['T'])
        starts = []
        for _ in range(3):
            t0 = dm.model_time
            st = dm.time_step(dict(rtol_Pat=1e-6, rtol_U=5e-3, itmax_Pat=200, itmax_U=40, target_rel_residual=1e-8),
                              rock=workloads.rock_params(1e3), dt_adv_limit=0.01, dtmax=0.6, vel_bcs=series)
            U, _ = dm.solution()
            UBC, Plate = series.at(t0)
            Ul = np.einsum('nji,nj->ni', R, U.reshape(-1, 3)).ravel()
            assert np.max(np.abs(Ul[UBC['ifix'] - 1] - UBC['vfix'])) <= 1e-11 * np.max(np.abs(UBC['vfix']))
            assert np.array_equal(st['Plate'], Plate)
            assert st['status'] == 0 and st['locate']['nlost'] == 0 and st['time'] > t0
            starts.append(t0)
    finally:
        dm.close()
    assert starts[0] == 0.0 and 0.0 < starts[1] < starts[2]
