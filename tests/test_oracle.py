"""The oracle itself: documented quadrature constants, shape functions, operator identities."""
import json
from pathlib import Path

import numpy as np

from oracle import stokes_oracle as O

GOLD = Path(__file__).resolve().parent / 'golden'


def test_quadrature_matches_documented_values():
    vals = json.loads((GOLD / 'quadrature_14.json').read_text())
    ipx, ipw = O.ip_tetrahedron14()
    a, b, c, d, e, f = ipx[0, 0], ipx[0, 1], ipx[0, 4], ipx[0, 5], ipx[0, 8], ipx[0, 11]
    got = dict(a=a, b=b, c=c, d=d, e=e, f=f, p=ipw[0] * 6, q=ipw[4] * 6, r=ipw[8] * 6)
    for k, v in vals.items():
        assert abs(got[k] - v) < 5e-16 * 10, (k, got[k], v)
    assert abs(ipw.sum() - 1.0 / 6.0) < 1e-15
    # degree-5 exactness on a monomial: int r^2 s t over the unit tet = 2!1!1!/(2+1+1+3)! = 2/5040
    r, s, t = ipx
    assert abs((ipw * r ** 2 * s * t).sum() - 2.0 / 5040.0) < 1e-17


def test_four_point_rule_matches_documented_values():
    """The diffusion operator's 4-point rule against the values ip_tetrahedron.m:41-42 documents
    (eight decimals): point k has coordinate a in direction k and b in the others, weights 1/4."""
    from oracle import thermal_oracle as TO
    vals = json.loads((GOLD / 'quadrature_4.json').read_text())
    assert abs(TO.IPX[0, 0] - vals['a']) < 5e-9 and abs(TO.IPX[1, 0] - vals['b']) < 5e-9
    assert np.array_equal(TO.IPX, [[TO._A, TO._B, TO._B, TO._B], [TO._B, TO._A, TO._B, TO._B],
                                   [TO._B, TO._B, TO._A, TO._B]])
    assert np.array_equal(TO.IPW, [0.25] * 4)
    # degree-2 exactness: the mean of r^2 over the unit tet is 2!/(2+3)! * 6 = 1/10
    assert abs((TO.IPW * TO.IPX[0] ** 2).sum() - 0.1) < 1e-15


def test_workload_units_are_the_reference_mantle_scaling():
    """The seeded workloads' units are numerical_eq_scaling('mantle') (values read from the
    reference source): L0 = 1 km, t0 = 1 Myr, Visc0 = 2e18 Pa s, Dens0 = 3300, and the derived
    U0 = L0/t0 and Bscale = L0^2/(Visc0 U0) of numerical_eq_scaling.m:51-64."""
    from m3tet_sph_gb300 import workloads as W
    sc = json.loads((GOLD / 'scaling_mantle.json').read_text())
    for k in ('L0', 't0', 'Visc0', 'Dens0'):
        assert W.SCALE[k] == sc[k], k
    U0 = sc['L0'] / sc['t0']
    assert W.SCALE['U0'] == U0 and W.SCALE['Bscale'] == sc['L0'] ** 2 / (sc['Visc0'] * U0)
    assert W.physics()['Bscale'] == W.SCALE['Bscale'] and W.physics()['Dens0'] == sc['Dens0']


def test_solver_and_location_constants_are_the_reference_values():
    """Constants read from the reference source (tests/golden/reference_constants.json): the V-cycle's
    Jacobi weights, the Patera defaults of the oracle and of the library's Python mirror, and the
    location's gap tolerance growth and curved Newton iteration."""
    import inspect
    import scipy.sparse as sp
    from oracle import slm_oracle as SO
    from m3tet_sph_gb300 import stokes
    c = json.loads((GOLD / 'reference_constants.json').read_text())
    w = c['mgpcg_weights']
    eye = sp.identity(3, format='csr')
    mg = O.MGPCG(eye, [np.ones(3), eye, eye], [eye, eye], 3)
    assert mg.wd == [w['finest_down'], w['other_down']]
    assert mg.wu == [w['finest_up'], w['other_down'][::-1]]
    pat = c['patera']
    assert pat['rtol_restart'] == '0.8*rtol_Pat'
    for fn in (O.patera, stokes.DeviceMesh.solve, stokes.DeviceMesh.step_device):
        par = inspect.signature(fn).parameters
        for k in ('rtol_Pat', 'rtol_U', 'itmax_Pat', 'itmin_Pat', 'itmax_U'):
            assert par[k].default == pat[k], (fn.__name__, k)
    loc = c['location']
    assert SO.GAP_STEP == loc['gap_step'] and abs(SO.GAP_QMAX * SO.GAP_STEP - loc['gap_max']) < 1e-15
    assert (SO.NEWTON_STEPS, SO.NEWTON_TOL) == (loc['newton_steps'], loc['newton_tol'])
    # rock_prop's gas constant; the time steps' diffusivity K / (rho Cp) of the plume model in model units
    from m3tet_sph_gb300 import workloads as W
    assert O.ROCK_R == c['rock_prop']['R']
    pm = c['plume_model']
    kappa_si = pm['K'] / (pm['Dens'] * pm['Cp'])
    assert abs(W.KAPPA - kappa_si / (W.SCALE['L0'] ** 2 / W.SCALE['t0'])) < 1e-12 * W.KAPPA


def test_shape_function_derivatives_fd():
    rng = np.random.default_rng(0)
    for fn, n in ((O.sf10, 10), (O.sf20, 20)):
        for _ in range(5):
            x = rng.uniform(0.05, 0.3, 3)
            N, dN = fn(*x)
            assert abs(N.sum() - 1.0) < 1e-13
            h = 1e-6
            for j in range(3):
                xp, xm = x.copy(), x.copy()
                xp[j] += h
                xm[j] -= h
                fd = (fn(*xp)[0] - fn(*xm)[0]) / (2 * h)
                assert np.abs(fd - dN[:, j]).max() < 1e-7


def test_element_operator_identities(tiny):
    f = tiny['levels'][0]
    K, G, Mm, Fb = O.element_matrices(f, tiny['visc'], tiny['dens'], **tiny['phys'])
    scale = np.abs(K).max()
    assert np.abs(K - K.transpose(0, 2, 1)).max() <= 1e-14 * scale
    for comp in range(3):
        tr = np.zeros(30)
        tr[comp::3] = 1.0
        assert np.abs(K @ tr).max() < 1e-13 * scale
        assert np.abs(np.einsum('eqp,q->ep', G, tr)).max() < 1e-13 * np.abs(G).max()
    ev = np.linalg.eigvalsh(K[:200])
    assert ev.min() > -1e-13 * ev.max()


def test_transfer_matches_host_setup(tiny):
    """Oracle intermesh_transfer_matrix (barycentric solve + rounding) equals the library's
    combinatorial set-up rows built in m3tet_sph_gb300.mesh."""
    lv = tiny['levels']
    Xs_c = O.p2_straight(lv[1]['GCOORD'], lv[1]['EL2NOD'])
    Xs_f = O.straight_coords(Xs_c, lv[0]['EL2NOD'])
    Ic2f = O.intermesh_transfer_matrix(Xs_f, lv[0]['EL2NOD'], Xs_c, lv[1]['EL2NOD']).toarray()
    cols, W = lv[0]['transfer_cols'], lv[0]['transfer_w']
    dense = np.zeros_like(Ic2f)
    np.add.at(dense, (np.repeat(np.arange(len(cols)), 10), cols.ravel()), W.ravel())
    assert np.abs(dense - Ic2f).max() < 1e-12


def test_threaded_sparse_products_match_serial(tiny):
    """The CPU baseline's threaded mode: row-block products equal the serial CSR product to rounding
    (bit for bit where the host compiler does not fuse scipy's multiply-adds), and MG-PCG iterates
    agree with the serial solver to rounding."""
    w = tiny
    s1 = O.StokesSystem(w['levels'], w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'])
    s4 = O.StokesSystem(w['levels'], w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'])
    s4.mg.use_threads(4)
    x = np.random.default_rng(3).standard_normal(s1.mg.K1.shape[0])
    y1 = s1.mg.K1 @ x
    assert np.max(np.abs(s4.mg.K1 @ x - y1)) <= 1e-14 * np.max(np.abs(y1))
    b = np.random.default_rng(4).standard_normal(len(s1.ifree))
    x1, it1, _ = s1.mg.solve(b, np.zeros_like(b), rtol=1e-30, itmax=4)
    x4, it4, _ = s4.mg.solve(b, np.zeros_like(b), rtol=1e-30, itmax=4)
    assert it1 == it4
    assert np.linalg.norm(x4 - x1) <= 1e-12 * np.linalg.norm(x1)


def test_tie_rule_follows_the_reference_preferences():
    """tsearch2_sph.m:374-404 as restated: iso dropped when a non-iso candidate exists, the first
    frame kept at a shared vertex, then the largest id; cross-frame face ties are flagged."""
    from oracle.slm_oracle import tie_rule
    # one iso + two non-iso on a face: iso dropped, largest remaining id
    assert tie_rule([7, 3, 5], [True, False, False], [0, 0, 1], [False] * 3) == (5, False)
    # all at a shared vertex, frames X-90 (0) and original (1): X-90 kept, then largest id
    assert tie_rule([9, 4, 6], [False] * 3, [1, 0, 0], [True] * 3) == (6, False)
    # cross-frame face tie without iso: the reference's error('no good') -> largest id, flagged
    assert tie_rule([2, 8], [False, False], [1, 2], [False, False]) == (8, True)
    # same-frame face tie: largest id, not flagged
    assert tie_rule([2, 8], [False, False], [1, 1], [False, False]) == (8, False)
    # two iso elements only: largest id
    assert tie_rule([11, 12], [True, True], [0, 0], [False, False]) == (12, False)


def test_gap_rule_follows_the_reference_preferences():
    """locate_points_in_neighboring_element.m: smallest tolerance step; iso dropped if a non-iso
    element remains (then the smallest id); all iso -> the smallest Newton step."""
    from oracle.slm_oracle import gap_rule
    assert gap_rule([5, 3, 9], [False, False, False], [4, 4, 7], [0, 0, 0]) == 3
    assert gap_rule([5, 3, 9], [True, False, True], [4, 4, 4], [0, 0, 0]) == 3
    assert gap_rule([5, 3, 9], [True, True, False], [4, 4, 9], [0.2, 0.1, 0]) == 3
    assert gap_rule([5, 3], [True, True], [4, 4], [0.1, 0.1]) == 3


def test_locator_independent_of_batch_and_neighbour_count():
    """The located element of a point depends on the point alone: not on the other points of the
    call (per-point Newton) nor on how many centroid neighbours seed the search."""
    import numpy as np
    from m3tet_sph_gb300 import workloads
    from oracle import slm_oracle as SO
    w = workloads.make_workload('tiny')
    f = w['levels'][0]
    rng = np.random.default_rng(0)
    v = rng.normal(size=(3, 3000))
    v /= np.linalg.norm(v, axis=0)
    r = (3480.0 ** 3 + rng.uniform(size=3000) * (6371.0 ** 3 - 3480.0 ** 3)) ** (1 / 3)
    P = np.hstack([SO.cart2sph(v * r), f['GCOORD_SPH'][:, :1500]])
    L1, L2 = SO.Locator(f, k=16), SO.Locator(f, k=48)
    e1, lc1, i1 = L1.locate(P, return_info=True)
    e2, lc2 = L2.locate(P)
    assert np.array_equal(e1, e2) and np.array_equal(lc1, lc2)
    e3 = np.concatenate([L1.locate(P[:, :1000])[0], L1.locate(P[:, 1000:])[0]])
    assert np.array_equal(e1, e3)
    assert i1['nlost'] == 0 and i1['nties'] >= 1000


def test_diffusion_oracle_identities(tiny):
    """Conductivity rows sum to zero (constants do not diffuse); the capacities add up to the shell
    volume times 6 (ip_tetrahedron's weights sum to 1, not to the reference tetrahedron's 1/6, in
    both matrices alike); the implicit step keeps a constant field."""
    import numpy as np
    from m3tet_sph_gb300 import mesh as M
    from oracle import thermal_oracle as TO
    f = tiny['levels'][0]
    EL1 = M.split_p2(f['GCOORD'], f['EL2NOD'])[0]
    fix = np.nonzero(f['PointID'] > 0)[0]
    D = TO.Diffusion(f['GCOORD'], f['GCOORD_SPH'], EL1, 31.6, fix)
    assert np.abs(np.asarray(D.C.sum(axis=1))).max() < 1e-12 * np.abs(D.C).max()
    vol = 4.0 / 3.0 * np.pi * (6371.0 ** 3 - 3480.0 ** 3)
    assert abs(D.ML.sum() / (6 * vol) - 1) < 2e-2
    T, nit = D.step(np.full(f['nnod'], 5.0), 100.0, np.full(len(fix), 5.0))
    assert np.abs(T - 5.0).max() < 1e-12


def test_gelu_erf_approximation_bound():
    """The fused inference sweep's GELU uses Abramowitz & Stegun 7.1.26 for erf (|error| <= 1.5e-7);
    the same formula and constants, evaluated in FP64 here, stay within that bound of erf and
    within 1.5e-7 |x| / 2 of the exact GELU."""
    import numpy as np
    from scipy.special import erf
    x = np.linspace(-12.0, 12.0, 200001)
    z = np.abs(x) / np.sqrt(2.0)
    t = 1.0 / (1.0 + 0.3275911 * z)
    poly = t * (0.254829592 + t * (-0.284496736 + t * (1.421413741 + t * (-1.453152027 + t * 1.061405429))))
    erf_as = 1.0 - poly * np.exp(-z * z)
    assert np.max(np.abs(erf_as - erf(z))) <= 1.5e-7
    q = 0.5 * x * poly * np.exp(-0.5 * x * x)
    gelu_as = np.where(x >= 0, x - q, q)
    gelu = 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))
    assert np.all(np.abs(gelu_as - gelu) <= 0.5 * 1.5e-7 * np.abs(x) + 1e-15)
