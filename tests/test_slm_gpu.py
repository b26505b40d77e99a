"""GPU parity of semi-Lagrangian advection: point location, interpolation, PC2 backtracking."""
import numpy as np
import pytest

from oracle import slm_oracle as SO

pytestmark = pytest.mark.gpu

R_CMB, R_SURF = 3480.0, 6371.0


def random_shell_points(n, seed):
    """Directions uniform on S^2, r = (r0^3 + u (r1^3 - r0^3))^(1/3) (uniform in volume)."""
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(3, n))
    v /= np.linalg.norm(v, axis=0)
    u = rng.uniform(size=n)
    r = (R_CMB ** 3 + u * (R_SURF ** 3 - R_CMB ** 3)) ** (1.0 / 3.0)
    r = np.clip(r, R_CMB + 1e-9 * (R_SURF - R_CMB), R_SURF - 1e-9 * (R_SURF - R_CMB))
    return SO.cart2sph(v * r)


@pytest.fixture(scope='module', params=['tiny', 'c1'])
def mesh_case(request, built_lib):
    from m3tet_sph_gb300 import stokes, workloads
    w = workloads.make_workload(request.param) if request.param == 'c1' else request.getfixturevalue('tiny')
    dm = stokes.DeviceMesh(w['levels'])
    yield w, dm, SO.Locator(w['levels'][0])
    dm.close()


def _check_location(w, dm, loc, P):
    """GPU ids equal the oracle's on every point; local coordinates agree to rounding; the tie /
    gap / ambiguity counts are the same."""
    from m3tet_sph_gb300 import advection as A
    els, lc, info = A.tsearch2_sph(dm, P)
    e_ref, lc_ref, rinfo = loc.locate(P, return_info=True)
    assert info['nlost'] == 0 and rinfo['nlost'] == 0
    bad = np.nonzero(els - 1 != e_ref)[0]
    assert len(bad) == 0, (len(bad), bad[:10], els[bad[:10]] - 1, e_ref[bad[:10]], rinfo['kind'][bad[:10]])
    assert np.abs(lc - lc_ref).max() < 1e-10
    for k in ('nties', 'ngap', 'nambig'):
        assert info[k] == rinfo[k], (k, info, rinfo)
    return info


def test_tsearch_bit_exact_random_points(mesh_case):
    w, dm, loc = mesh_case
    info = _check_location(w, dm, loc, random_shell_points(20000, seed=11))
    print(f"random points: {info}")


def test_tsearch_bit_exact_on_ties(mesh_case):
    """Points that several elements contain: mesh nodes (vertices and edge nodes, shared by up to
    ~40 elements, across frames at the cone boundary and the 2 pi seam), the same points moved by
    1e-13 of the shell thickness, and vertex-face centroids."""
    w, dm, loc = mesh_case
    f = w['levels'][0]
    S = f['GCOORD_SPH']
    n = min(S.shape[1], 20000)
    rng = np.random.default_rng(4)
    nodes = S[:, :n]
    moved = nodes + np.array([[1e-13], [1e-13], [1e-13 * (R_SURF - R_CMB)]]) * rng.uniform(-1, 1, size=(3, n))
    moved[2] = np.clip(moved[2], R_CMB, R_SURF)
    EL = f['EL2NOD']
    X = f['GCOORD']
    # chord centroids of faces lie below curved faces; those of CMB faces fall outside the shell,
    # so they are moved radially inside as the semi-Lagrangian path does (find_pts_outside_domain_sph)
    fc = SO.clamp_radius(SO.cart2sph(X[:, EL[:min(len(EL), 5000), :3]].mean(axis=2)), R_CMB, R_SURF)
    info = _check_location(w, dm, loc, np.hstack([nodes, moved, fc]))
    assert info['nties'] > 0.5 * n
    print(f"tie points: {info}")


def test_tsearch_known_elements(mesh_case):
    """Points mapped from interior local coordinates of given elements are found there."""
    from m3tet_sph_gb300 import advection as A
    w, dm, loc = mesh_case
    f = w['levels'][0]
    rng = np.random.default_rng(3)
    els0 = rng.choice(f['nel'], min(5000, f['nel']), replace=False)
    lc0 = rng.dirichlet([3, 3, 3, 3], size=len(els0)).T[:3]
    N, _ = SO.sf10(*lc0)
    X = np.einsum('in,kni->kn', N, f['GCOORD'][:, f['EL2NOD'][els0]])
    P = SO.cart2sph(X)
    _check_location(w, dm, loc, P)
    els, _, _ = A.tsearch2_sph(dm, P)
    assert np.mean(els - 1 == els0) > 0.99


def test_interpolation_parity(mesh_case):
    from m3tet_sph_gb300 import advection as A
    w, dm, loc = mesh_case
    f = w['levels'][0]
    P = random_shell_points(5000, seed=5)
    els, lc, _ = A.tsearch2_sph(dm, P)
    e0 = els - 1
    lc_adj = SO.adjust_local_coords(lc.copy())
    T = w['T']
    V = np.stack([T, np.sin(T), T ** 2], 1)
    gv = A.interp3d_tet(dm, els, lc_adj, V, monotonic=True)
    rv = SO.interp3d_tet(f['EL2NOD'], e0, lc_adj, V, monotonic=True)
    assert np.abs(gv - rv).max() < 1e-13 * np.abs(rv).max()
    gc = A.interp3d_cubic_p(dm, els, lc_adj, T, monotonic=True)
    rc = SO.interp3d_cubic(f['GCOORD'], f['EL2NOD'], e0, lc_adj, T, monotonic=True)
    assert np.abs(gc - rc).max() < 1e-12 * np.abs(rc).max()
    gcn = A.interp3d_cubic_p(dm, els, lc_adj, T, monotonic=False, method_wght='ones')
    rcn = SO.interp3d_cubic(f['GCOORD'], f['EL2NOD'], e0, lc_adj, T, monotonic=False, method_wght='ones')
    assert np.abs(gcn - rcn).max() < 1e-12 * np.abs(rcn).max()


def test_cubic_interpolation_reproduces_linear_fields(mesh_case):
    """Quasi-cubic interpolation is exact for fields linear in Cartesian coordinates."""
    from m3tet_sph_gb300 import advection as A
    w, dm, loc = mesh_case
    f = w['levels'][0]
    X = f['GCOORD']
    B = 0.3 * X[0] - 0.2 * X[1] + 0.1 * X[2] + 5.0
    rng = np.random.default_rng(2)
    els0 = rng.choice(f['nel'], 2000, replace=False)
    lc0 = rng.dirichlet([2, 2, 2, 2], size=len(els0)).T[:3]
    # Cartesian point of the straight (vertex) tet at lc0 -> exact linear value there
    V4 = X[:, f['EL2NOD'][els0, :4]]
    lam = np.vstack([lc0, 1 - lc0.sum(0)])
    xp = np.einsum('kni,in->kn', V4, lam)
    exact = 0.3 * xp[0] - 0.2 * xp[1] + 0.1 * xp[2] + 5.0
    got = A.interp3d_cubic_p(dm, els0.astype(np.int32) + 1, lc0, B, monotonic=False)
    assert np.abs(got - exact).max() < 1e-9 * np.abs(exact).max()


def _velocity(X):
    """A smooth velocity field: rigid rotation + a radial/tangential perturbation (km/Myr)."""
    om = np.array([0.2, -0.1, 0.35]) * 1e-3
    return np.cross(om[None, :], X.T).T + 0.5 * np.array([np.sin(X[1] / 1500), np.cos(X[2] / 1700),
                                                          np.sin(X[0] / 1900)])


def test_pc2_advection_parity(mesh_case):
    """PC2: predictor and departure elements equal the oracle's on every node; T agrees on every
    node to the rounding carried through two locations and interpolations."""
    from m3tet_sph_gb300 import advection as A
    w, dm, loc = mesh_case
    f = w['levels'][0]
    U = _velocity(f['GCOORD'])
    dt = 20.0
    T = w['T']
    for method in ('quadratic', 'cubic'):
        MESH = dict(levels=w['levels'], device_mesh=dm, r_cmb=R_CMB, r_surf=R_SURF)
        Tg, WS = A.advect3d_slm_p_sph(MESH, None, U[0], U[1], U[2], T, dt, dict(method_interp=method))
        Tr, Pd, e1, e2 = SO.advect_pc2(f, U.T, T, dt, R_CMB, R_SURF, method_interp=method)
        assert WS['locate_info']['nlost'] == 0
        assert np.array_equal(WS['els_BT'] - 1, e1)
        assert np.array_equal(WS['els_INTERP'] - 1, e2)
        assert np.abs(Tg - Tr).max() < 1e-10, method
        print(f"PC2 {method}: {WS['locate_info']}")


def test_rk4_advection_parity(mesh_case):
    """RK4 over 3 substeps (builder-defined; the reference's RK4 is an error stub): departure
    elements equal on every node, T agrees on every node."""
    from m3tet_sph_gb300 import advection as A
    w, dm, loc = mesh_case
    f = w['levels'][0]
    U = _velocity(f['GCOORD'])
    dt = 20.0
    MESH = dict(levels=w['levels'], device_mesh=dm, r_cmb=R_CMB, r_surf=R_SURF)
    Tg, WS = A.advect3d_slm_p_sph(MESH, None, U[0], U[1], U[2], w['T'], dt, dict(method_BT='RK4', method_interp='cubic'))
    Tr, Pd, e2 = SO.advect_rk4(f, U.T, w['T'], dt, R_CMB, R_SURF, method_interp='cubic')
    assert WS['locate_info']['nlost'] == 0
    assert np.array_equal(WS['els_INTERP'] - 1, e2)
    assert np.abs(Tg - Tr).max() < 1e-10
    print(f"RK4: {WS['locate_info']}")


def test_advection_with_zero_velocity_regions(mesh_case):
    """Departure points of nodes where the velocity vanishes are the nodes themselves -- points on
    vertices and edges shared by many elements, across frames -- and must still match."""
    from m3tet_sph_gb300 import advection as A
    w, dm, loc = mesh_case
    f = w['levels'][0]
    X = f['GCOORD']
    U = _velocity(X)
    U[:, X[2] > 0] = 0.0                       # northern hemisphere at rest (the cone around +z)
    MESH = dict(levels=w['levels'], device_mesh=dm, r_cmb=R_CMB, r_surf=R_SURF)
    Tg, WS = A.advect3d_slm_p_sph(MESH, None, U[0], U[1], U[2], w['T'], 20.0, dict(method_interp='cubic'))
    Tr, Pd, e1, e2 = SO.advect_pc2(f, U.T, w['T'], 20.0, R_CMB, R_SURF, method_interp='cubic')
    assert np.array_equal(WS['els_BT'] - 1, e1)
    assert np.array_equal(WS['els_INTERP'] - 1, e2)
    assert WS['locate_info']['nties'] > 0
    assert np.abs(Tg - Tr).max() < 1e-10


def test_empty_inputs_and_element_id_range(tiny):
    """No points is a no-op for location and both interpolations; interpolation ids outside 1..nel
    are rejected on the host (the reference's own indexing error) before anything runs."""
    from m3tet_sph_gb300 import _lib as L, advection as A, stokes
    f = tiny['levels'][0]
    dm = stokes.DeviceMesh(tiny['levels'])
    try:
        els, lc, info = A.tsearch2_sph(dm, np.zeros((3, 0)))
        assert els.shape == (0,) and lc.shape == (3, 0) and info['npt'] == 0
        T = np.linspace(0.0, 1.0, f['nnod'])
        assert A.interp3d_tet(dm, np.zeros(0, np.int32), np.zeros((3, 0)), T).shape == (0,)
        assert A.interp3d_cubic_p(dm, np.zeros(0, np.int32), np.zeros((3, 0)), T).shape == (0,)
        lc1 = np.full((3, 2), 0.25)
        for bad in ([1, f['nel'] + 1], [0, 1], [-3, 1]):
            with pytest.raises(L.M3SphError, match='outside 1'):
                A.interp3d_tet(dm, np.array(bad, np.int32), lc1, T)
            with pytest.raises(L.M3SphError, match='outside 1'):
                A.interp3d_cubic_p(dm, np.array(bad, np.int32), lc1, T)
        # the first and the last element are valid ids; P2 weights at the centroid sum to one
        v = A.interp3d_tet(dm, np.array([1, f['nel']], np.int32), lc1, np.ones(f['nnod']))
        assert np.allclose(v, 1.0, rtol=0, atol=1e-14)
    finally:
        dm.close()
