"""GPlates velocity files and update_vel_bc (readVelGPlates.m, SAVE_GPLATES_VEL_BCS_TO_MAT_FILE.m,
update_vel_bc.m) against the oracle's record-by-record restatement, on seeded files in GPlates'
format (the reference's own exports are not distributed)."""
import numpy as np
import pytest

from oracle import bc_oracle as BO


def _rot(axis, ang):
    a = np.asarray(axis, dtype=np.float64)
    a /= np.linalg.norm(a)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(ang) * K + (1 - np.cos(ang)) * K @ K


RR1 = _rot([0.3, -0.5, 0.8], 0.7)
RR2 = _rot([1.0, 0.2, -0.1], -1.1)


@pytest.fixture(scope='module')
def shell():
    from m3tet_sph_gb300 import mesh as M
    return M.build_hierarchy(2, 4, 1)[0]


@pytest.fixture(scope='module', params=['identity', 'rotated'])
def series(request, shell, tmp_path_factory):
    from m3tet_sph_gb300 import gplates as G
    rr = (None, None) if request.param == 'identity' else (RR1, RR2)
    ser = G.synthetic_vel_bcs(shell, seed=3, RR1=rr[0], RR2=rr[1])
    folder = G.write_synthetic_folder(tmp_path_factory.mktemp('vel_bcs_' + request.param), ser)
    V, t = G.read_vel_gplates_folder(folder)
    return dict(folder=folder, V=V, t=t, RR1=rr[0], RR2=rr[1], raw=ser)


def test_reader_known_answer(tmp_path):
    from m3tet_sph_gb300 import gplates as G
    text = ("10.5 -20.25 201 1.5 -2.0\n"
            "11.0 -21.00 0 0.5 0.25\n"
            "12.0 -22.00 701 -1.0 3.0\n"
            "13.0 -23.00 901 2.0 -0.5\n")
    U, ll, pid, names = G.parse_vel_gplates(text)
    assert np.array_equal(ll, [[10.5, 11.0, 12.0, 13.0], [-20.25, -21.0, -22.0, -23.0]])
    assert np.array_equal(U, [[15.0, 5.0, -10.0, 20.0], [-20.0, 2.5, 30.0, -5.0]])
    # the unassigned record takes the previous record's plate (201 = SAM, the 4th row of the table)
    assert np.array_equal(pid, [4.0, 4.0, 9.0, 12.0])
    assert names[3] == dict(plate_id=201, index=4, plate_abr='SAM') and len(names) == 15
    with pytest.raises(ValueError, match='need to be updated'):
        G.parse_vel_gplates("1 2 555 0 0\n")
    with pytest.raises(ValueError, match='first or last'):
        G.parse_vel_gplates("1 2 0 0 0\n3 4 201 0 0\n")
    # a run of unassigned records: each takes its (already reassigned) predecessor's plate
    _, _, pid, _ = G.parse_vel_gplates("1 2 701 0 0\n1 2 0 0 0\n1 2 0 0 0\n5 6 201 0 0\n")
    assert np.array_equal(pid, [9.0, 9.0, 9.0, 4.0])


def test_reader_matches_oracle(series):
    for v in series['V']:
        text = (series['folder'] / f"{int(v['time'])}Ma.txt").read_text()
        U, ll, pid = BO.read_records(text)
        assert np.array_equal(U, v['Uth_Uph']) and np.array_equal(ll, v['latlon'])
        assert np.array_equal(pid, v['PlateID'])
    # oldest file first, 1 Myr apart, as the reference's loader numbers them
    assert np.array_equal(series['t'], [103.0, 102.0, 101.0, 100.0])


def test_folder_of_xy_exports(series, tmp_path):
    """GPlates writes .xy files; the folder reader takes them as the reference does after renaming."""
    from m3tet_sph_gb300 import gplates as G
    for p in series['folder'].glob('*.txt'):
        (tmp_path / (p.stem + '.xy')).write_text(p.read_text())
    V, t = G.read_vel_gplates_folder(tmp_path)
    assert np.array_equal(t, series['t'])
    assert all(np.array_equal(a['Uth_Uph'], b['Uth_Uph']) for a, b in zip(V, series['V']))
    with pytest.raises(ValueError, match='no GPlates'):
        G.read_vel_gplates_folder(tmp_path / 'missing')


def test_mat_round_trip(series, tmp_path):
    from m3tet_sph_gb300 import gplates as G
    p = tmp_path / 'Vel_BCs_test.mat'
    G.save_vel_bcs(p, series['V'], series['t'])
    V, t = G.load_vel_bcs(p)
    assert np.array_equal(t, series['t'])
    for a, b in zip(V, series['V']):
        assert a['time'] == b['time']
        for k in ('Uth_Uph', 'latlon', 'PlateID'):
            assert np.array_equal(a[k], b[k])
        assert a['plateid2name'] == b['plateid2name']


@pytest.mark.parametrize('model_time', [-0.5, 0.0, 0.25, 1.0, 1.75, 3.0, 3.5])
def test_interpolation_matches_oracle(series, model_time):
    from m3tet_sph_gb300 import gplates as G
    U, i0 = G.interpolate_velocities(series['V'], series['t'], model_time)
    Ur, ir = BO.velocities_at(series['V'], series['t'], model_time)
    assert i0 == ir and np.array_equal(U, Ur)


def test_interpolation_weights(series):
    from m3tet_sph_gb300 import gplates as G
    V, t = series['V'], series['t']
    U, _ = G.interpolate_velocities(V, t, 1.0)          # exactly the 102 Ma file
    assert np.array_equal(U, V[1]['Uth_Uph'])
    U, _ = G.interpolate_velocities(V, t, 1.25)         # a quarter of the way from 102 Ma to 101 Ma
    assert np.allclose(U, 0.75 * V[1]['Uth_Uph'] + 0.25 * V[2]['Uth_Uph'], rtol=1e-14, atol=1e-14)
    with pytest.raises(ValueError, match='outside'):
        G.interpolate_velocities(V, t, 4.5)


@pytest.mark.parametrize('model_time', [0.0, 0.6, 2.0, 2.9])
def test_update_vel_bc_matches_oracle(series, shell, model_time):
    from m3tet_sph_gb300 import gplates as G
    UBC, Plate = G.update_vel_bc(shell['PointID'], series['V'], series['t'], model_time, 6371.0,
                                 series['RR1'], series['RR2'])
    ifix, vfix, Plate_r = BO.update_vel_bc(shell['PointID'], series['V'], series['t'], model_time, 6371.0,
                                           series['RR1'], series['RR2'])
    assert np.array_equal(UBC['ifix'], ifix) and UBC['nfix'] == ifix.size
    scale = np.max(np.abs(vfix))
    # (theta, phi) components in the frame of the rotated point: on the polar axis that frame's phi
    # follows the rounding of the rotated position, so there only the tangential speed is defined
    polar = _polar_dofs(shell, ifix)
    assert np.max(np.abs(UBC['vfix'] - vfix)[~polar]) <= 1e-13 * scale
    sp = lambda v: np.hypot(v[polar][0::2], v[polar][1::2])
    assert np.max(np.abs(sp(UBC['vfix']) - sp(vfix))) <= 1e-13 * scale
    assert np.array_equal(Plate, Plate_r)


def _polar_dofs(shell, ifix):
    """theta / phi dofs of surface nodes on the z axis (sin theta < 1e-9)."""
    from m3tet_sph_gb300 import mesh as M
    node = (np.asarray(ifix) - 1) // 3
    th = M.cart2sph(shell['GCOORD'][:, node])[0]
    return (np.sin(th) < 1e-9) & ((np.asarray(ifix) - 1) % 3 != 2) & (shell['PointID'][node] == 306)


def test_update_vel_bc_recovers_the_mesh_frame_plates(series, shell):
    """The files hold Earth-frame positions and velocities (the mesh frame rotated by RR2 RR1);
    update_vel_bc's (RR2 RR1)^T brings them back onto the mesh's surface nodes, so the prescribed
    (theta, phi) values are the file's plate rotation seen in the mesh frame, and every surface
    node gets the plate index of its record."""
    from m3tet_sph_gb300 import gplates as G, mesh as M
    UBC, Plate = G.update_vel_bc(shell['PointID'], series['V'], series['t'], 0.0, 6371.0,
                                 series['RR1'], series['RR2'])
    surf = np.nonzero(shell['PointID'] == G.PID_SURF)[0]
    RR = (np.eye(3) if series['RR2'] is None else series['RR2']) @ (np.eye(3) if series['RR1'] is None else series['RR1'])
    # velocities of file 0 in the Earth frame, Cartesian, mm/yr
    V0 = series['V'][0]
    xe = RR @ shell['GCOORD'][:, surf]
    Fe = M.rotation_blocks(xe)
    ve = np.einsum('nij,jn->ni', Fe, np.vstack([V0['Uth_Uph'], np.zeros((1, surf.size))]))
    vm = ve @ RR                                        # (RR^T v) per node, mesh frame
    Fm = M.rotation_blocks(shell['GCOORD'][:, surf])
    vl = np.einsum('nji,nj->ni', Fm, vm)
    th = UBC['vfix'][np.isin(UBC['ifix'], 3 * (surf + 1) - 2)]
    ph = UBC['vfix'][np.isin(UBC['ifix'], 3 * (surf + 1) - 1)]
    # the files keep 10 decimals of a degree: positions agree to ~1e-8 relative; on the polar axis
    # the (theta, phi) frame is undefined and only the speed is compared
    ok = np.sin(M.cart2sph(shell['GCOORD'][:, surf])[0]) > 1e-9
    assert np.max(np.abs(th - vl[:, 0])[ok]) < 1e-6 * np.max(np.abs(vl))
    assert np.max(np.abs(ph - vl[:, 1])[ok]) < 1e-6 * np.max(np.abs(vl))
    assert np.max(np.abs(np.hypot(th, ph) - np.hypot(vl[:, 0], vl[:, 1]))) < 1e-6 * np.max(np.abs(vl))
    assert np.array_equal(Plate[surf], V0['PlateID']) and np.all(Plate[surf] >= 1)


def test_update_vel_bc_dof_set_is_the_plate_workloads(series, shell):
    """Free slip on the core-mantle boundary and all three dofs of every surface node: the fixed
    dof set of the seeded plate workloads, so a device set up with those takes the GPlates values
    through m3sph_stokes_set_vel_bc."""
    from m3tet_sph_gb300 import gplates as G, workloads as W
    UBC, _ = G.update_vel_bc(shell['PointID'], series['V'], series['t'], 1.5, 6371.0, series['RR1'], series['RR2'])
    ifix0, _ = W.boundary_conditions(shell, 'plates')
    assert np.array_equal(np.sort(UBC['ifix'] - 1), ifix0)
    # node-major order of the reference's loop: r dof of each CMB node; theta, phi, r of each surface node
    assert np.all(np.diff(UBC['ifix']) > 0)
    r_dofs = UBC['vfix'][UBC['ifix'] % 3 == 0]
    assert np.all(r_dofs == 0.0)


def test_update_vel_bc_appends_plume_and_checks_boundaries(series, shell):
    from m3tet_sph_gb300 import gplates as G
    plume = dict(iUbc_plume=2, iUfix_plume=[4, 5], vUfix_plume=[1.5, -2.5])
    UBC, _ = G.update_vel_bc(shell['PointID'], series['V'], series['t'], 0.0, 6371.0, series['RR1'],
                             series['RR2'], UBC=dict(PLUME=plume))
    assert np.array_equal(UBC['ifix'][-2:], [4, 5]) and np.array_equal(UBC['vfix'][-2:], [1.5, -2.5])
    pid = shell['PointID'].copy()
    pid[pid == G.PID_SURF] = 0
    with pytest.raises(ValueError, match='306'):
        G.update_vel_bc(pid, series['V'], series['t'], 0.0, 6371.0)
    pid = shell['PointID'].copy()
    pid[np.nonzero(pid == 0)[0][:3]] = 999
    with pytest.warns(UserWarning, match='999'):
        G.boundary_nodes(pid)


@pytest.mark.parametrize('model_time', [0.0, 0.6, 2.0, 3.2])
def test_series_equals_update_vel_bc(series, shell, model_time):
    """The time-loop form (layout and frame change formed once) gives update_vel_bc's lists."""
    from m3tet_sph_gb300 import gplates as G
    plume = dict(iUbc_plume=2, iUfix_plume=[4, 5], vUfix_plume=[1.5, -2.5])
    S = G.VelBCSeries(series['V'], series['t'], shell['PointID'], 6371.0, series['RR1'], series['RR2'],
                      UBC=dict(PLUME=plume))
    UBC, Plate = S.at(model_time)
    ref, Plate_r = G.update_vel_bc(shell['PointID'], series['V'], series['t'], model_time, 6371.0,
                                   series['RR1'], series['RR2'], UBC=dict(PLUME=plume))
    assert np.array_equal(UBC['ifix'], ref['ifix']) and UBC['nfix'] == ref['nfix']
    assert np.max(np.abs(UBC['vfix'] - ref['vfix'])) <= 1e-13 * np.max(np.abs(ref['vfix']))
    assert np.array_equal(Plate, Plate_r) and np.array_equal(UBC['PlateInfo'], ref['PlateInfo'])


# ---- the reference's shipped embedded mesh (SETUP_TEST/MESHES/EarthShell_n37k.mat) and its frame ----

@pytest.fixture(scope='module')
def ref_mesh():
    import json
    from pathlib import Path
    g = Path(__file__).resolve().parent / 'golden'
    d = np.load(g / 'earthshell_n37k.npz')
    fr = json.loads((g / 'earthshell_n37k_frame.json').read_text())
    f = dict(GCOORD=d['GCOORD'].T.copy(), PointID=d['PointID'].astype(np.int64))
    return f, fr, float(d['r_surf'])


def test_reference_frame_puts_the_refined_region_at_the_mesh_centre(ref_mesh):
    """Pinned against the reference's mesh file: (RR2 RR1)^T takes the refined region's centre given
    in the GPlates frame (theta_center, phi_center = 128, 353 degrees: the South Atlantic) onto the
    mesh frame's (theta0, phi0) = (90, 90), the convention update_vel_bc.m:71-77 states."""
    from m3tet_sph_gb300 import gplates as G, mesh as M
    f, fr, r_surf = ref_mesh
    lat, lon = 90.0 - fr['theta_center'], fr['phi_center']
    p = G.earth_to_mesh_points(np.array([[lat], [lon]]), r_surf, fr['RR1_center'], fr['RR2_center'])
    th, ph, r = M.cart2sph(p)[:, 0]
    assert abs(np.rad2deg(th) - fr['theta0']) < 1e-12 and abs(np.rad2deg(ph) - fr['phi0']) < 1e-12
    assert abs(r - r_surf) < 1e-9


def test_update_vel_bc_on_the_reference_mesh(ref_mesh, tmp_path):
    """A seeded series on the reference mesh's 3,954 surface nodes, written in the Earth frame of its
    own RR1/RR2: update_vel_bc matches the oracle, brings every record back onto its surface node,
    and leaves free slip on its 162 core-mantle-boundary nodes."""
    from m3tet_sph_gb300 import gplates as G
    f, fr, r_surf = ref_mesh
    RR1, RR2 = np.array(fr['RR1_center']), np.array(fr['RR2_center'])
    folder = G.write_synthetic_folder(tmp_path, G.synthetic_vel_bcs(f, seed=7, RR1=RR1, RR2=RR2))
    V, t = G.read_vel_gplates_folder(folder)
    surf = np.nonzero(f['PointID'] == G.PID_SURF)[0]
    assert V[0]['Uth_Uph'].shape == (2, surf.size) == (2, 3954)
    # the records sit on the mesh's surface nodes once rotated (10 decimals of a degree in the files)
    p = G.earth_to_mesh_points(V[0]['latlon'], r_surf, RR1, RR2)
    assert np.max(np.linalg.norm(p - f['GCOORD'][:, surf], axis=0)) < 1e-5
    for mt in (0.0, 1.4):
        UBC, Plate = G.update_vel_bc(f['PointID'], V, t, mt, r_surf, RR1, RR2)
        ifix, vfix, Plate_r = BO.update_vel_bc(f['PointID'], V, t, mt, r_surf, RR1, RR2)
        assert np.array_equal(UBC['ifix'], ifix) and np.array_equal(Plate, Plate_r)
        assert np.max(np.abs(UBC['vfix'] - vfix)) <= 1e-13 * np.max(np.abs(vfix))
        S = G.VelBCSeries(V, t, f['PointID'], r_surf, RR1, RR2)
        U2, _ = S.at(mt)
        assert np.max(np.abs(U2['vfix'] - vfix)) <= 1e-13 * np.max(np.abs(vfix))
    assert UBC['nfix'] == 162 + 3 * 3954
