"""GPU parity of the Stokes hot path against the FP64 oracle (called through the C ABI)."""
import numpy as np
import pytest

from oracle import stokes_oracle as O

pytestmark = pytest.mark.gpu


def _rot_blocks(X):
    S = O.cart2sph(X)
    th, ph = S[0], S[1]
    n = X.shape[1]
    R = np.zeros((n, 3, 3))
    R[:, 0] = np.stack([np.cos(ph) * np.cos(th), -np.sin(ph), np.cos(ph) * np.sin(th)], 1)
    R[:, 1] = np.stack([np.sin(ph) * np.cos(th), np.cos(ph), np.sin(ph) * np.sin(th)], 1)
    R[:, 2] = np.stack([-np.sin(th), np.zeros(n), np.cos(th)], 1)
    return R


@pytest.fixture(scope='module', params=['tiny', 'tiny_plates'])
def case(request, built_lib):
    from m3tet_sph_gb300 import stokes
    w = request.getfixturevalue(request.param)
    S = O.StokesSystem(w['levels'], w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'])
    dm = stokes.DeviceMesh(w['levels'])
    dm.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=0)
    yield w, S, dm
    dm.close()


def _free(S):
    m = np.zeros(S.nU, bool)
    m[S.ifree] = True
    return m


def test_element_matrices_parity(case):
    w, S, dm = case
    f = w['levels'][0]
    K, G, Mm, Fb = O.element_matrices(f, w['visc'], w['dens'], **w['phys'])
    R = _rot_blocks(f['GCOORD'])
    EL = f['EL2NOD']
    Q = np.zeros((len(EL), 30, 30))
    for n in range(10):
        Q[:, 3 * n:3 * n + 3, 3 * n:3 * n + 3] = R[EL[:, n]]
    Kl = np.einsum('eji,ejk,ekl->eil', Q, K, Q)
    mask = _free(S)[O.el2dof(EL)]
    Kl = Kl * mask[:, :, None] * mask[:, None, :]
    Gl = np.einsum('eji,ejp->eip', Q, G)
    Kg, Gg, Mg = dm.element_matrices()
    scale = np.abs(Kl).max(axis=(1, 2), keepdims=True)
    assert (np.abs(Kg - Kl) / scale).max() < 1e-12
    assert np.abs(Gg - Gl).max() < 1e-12 * np.abs(Gl).max()
    assert np.abs(Mg - Mm).max() < 1e-12 * np.abs(Mm).max()


@pytest.mark.parametrize("split", [1, 0])
def test_operator_apply_parity(case, split):
    w, S, dm = case
    dm.set_option("split_apply", split)
    rng = np.random.default_rng(1)
    x = rng.standard_normal(S.nU)
    m = _free(S)
    x[~m] = 0
    y_ref = np.zeros(S.nU)
    y_ref[S.ifree] = S.K1 @ x[S.ifree]
    y = dm.apply(x)
    assert np.linalg.norm(y - y_ref) < 1e-13 * np.linalg.norm(y_ref)
    # fixed entries of the input are ignored (K1 acts on free dofs only)
    x2 = x.copy()
    x2[~m] = 1e3
    assert np.linalg.norm(dm.apply(x2) - y) < 1e-13 * np.linalg.norm(y_ref)
    dm.set_option("split_apply", 1)


def test_grad_div_force_parity(case):
    w, S, dm = case
    rng = np.random.default_rng(2)
    q = rng.standard_normal(S.nP)
    assert np.linalg.norm(dm.grad(q) - S.GG @ q) < 1e-13 * np.linalg.norm(S.GG @ q)
    z = rng.standard_normal(S.nU)
    assert np.linalg.norm(dm.div(z) - S.GG.T @ z) < 1e-13 * np.linalg.norm(S.GG.T @ z)
    assert np.linalg.norm(dm.force() - S.Fb) < 1e-13 * np.linalg.norm(S.Fb)


def test_galerkin_and_transfer_parity(case):
    w, S, dm = case
    rng = np.random.default_rng(3)
    nUc = S.Ps[0].shape[1]
    ifree_c = S.ifree[S.ifree < 3 * w['levels'][1]['nnod']]
    assert nUc == len(ifree_c)
    xc = np.zeros(3 * w['levels'][1]['nnod'])
    xc[ifree_c] = rng.standard_normal(nUc)
    yref = np.zeros_like(xc)
    yref[ifree_c] = S.KK[1] @ xc[ifree_c]
    y = dm.level_apply(1, xc)
    assert np.linalg.norm(y - yref) < 1e-12 * np.linalg.norm(yref)
    # prolongation / restriction on free dofs
    pf = np.zeros(S.nU)
    pf[S.ifree] = S.Ps[0] @ xc[ifree_c]
    assert np.linalg.norm(dm.prolong(0, xc) - pf) < 1e-14 * np.linalg.norm(pf)
    rf = np.zeros(S.nU)
    rf[S.ifree] = rng.standard_normal(len(S.ifree))
    rc = np.zeros_like(xc)
    rc[ifree_c] = S.Ps[0].T @ rf[S.ifree]
    assert np.linalg.norm(dm.restrict(0, rf) - rc) < 1e-14 * np.linalg.norm(rc)


def test_vcycle_parity_fp64(case):
    w, S, dm = case
    rng = np.random.default_rng(4)
    r = np.zeros(S.nU)
    r[S.ifree] = rng.standard_normal(len(S.ifree))
    dref = np.zeros(S.nU)
    dref[S.ifree] = S.mg.vcycle(r[S.ifree])
    d = dm.vcycle(r)
    assert np.linalg.norm(d - dref) < 1e-10 * np.linalg.norm(dref)


def test_mgpcg_parity(case):
    w, S, dm = case
    rng = np.random.default_rng(5)
    b = np.zeros(S.nU)
    b[S.ifree] = rng.standard_normal(len(S.ifree))
    x, it, rr = dm.mgpcg(b, np.zeros(S.nU), 1e-6, is_abs_tol=False, itmax=30)
    xr, itr, hist = S.mg.solve(b[S.ifree], np.zeros(len(S.ifree)), rtol=1e-6, itmax=30)
    assert it == itr
    assert np.linalg.norm(x[S.ifree] - xr) < 1e-8 * np.linalg.norm(xr)


def test_patera_solution_parity(case):
    """Both solves converged tightly: velocity and pressure agree to 1e-8 relative L2."""
    w, S, dm = case
    kw = dict(rtol_Pat=1e-10, rtol_U=1e-4, itmax_Pat=200, itmax_U=40)
    U, P, info = dm.solve(**kw)
    Ur, Pr, infor = O.patera(S, **kw)
    Uxyz_ref = S.RR @ Ur
    Pm, Prm = P - P.mean(), Pr - Pr.mean()
    eU = np.linalg.norm(U - Uxyz_ref) / np.linalg.norm(Uxyz_ref)
    eP = np.linalg.norm(Pm - Prm) / np.linalg.norm(Prm)
    assert info['rel_residual'] < 1e-8, info
    assert eU < 1e-8 and eP < 1e-8, (eU, eP, info, infor)


def test_mixed_precision_solution(case):
    """FP32 V-cycle inside the FP64 outer iterations reaches the same converged answer."""
    w, S, dm = case
    from m3tet_sph_gb300 import stokes
    dm2 = stokes.DeviceMesh(w['levels'])
    try:
        dm2.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=1)
        kw = dict(rtol_Pat=1e-10, rtol_U=1e-4, itmax_Pat=200, itmax_U=40)
        U, P, info = dm2.solve(**kw)
        Ur, Pr, _ = O.patera(S, **kw)
        Uxyz_ref = S.RR @ Ur
        eU = np.linalg.norm(U - Uxyz_ref) / np.linalg.norm(Uxyz_ref)
        eP = np.linalg.norm((P - P.mean()) - (Pr - Pr.mean())) / np.linalg.norm(Pr - Pr.mean())
        assert info['rel_residual'] < 1e-8, info
        assert eU < 1e-8 and eP < 1e-8, (eU, eP, info)
    finally:
        dm2.close()


def test_mixed_operators_parity(case):
    """Mixed-precision set-up: the double-float outer operator keeps FP64 accuracy; the FP32
    coarse block operator matches the FP64 Galerkin operator to FP32 rounding."""
    w, S, dm = case
    from m3tet_sph_gb300 import stokes
    dm2 = stokes.DeviceMesh(w['levels'])
    try:
        dm2.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=1)
        rng = np.random.default_rng(7)
        x = np.zeros(S.nU)
        x[S.ifree] = rng.standard_normal(len(S.ifree))
        y_ref = np.zeros(S.nU)
        y_ref[S.ifree] = S.K1 @ x[S.ifree]
        for split in (1, 0):
            dm2.set_option("split_apply", split)
            y = dm2.apply(x)
            assert np.linalg.norm(y - y_ref) < 1e-12 * np.linalg.norm(y_ref)
        dm2.set_option("split_apply", 1)
        ifree_c = S.ifree[S.ifree < 3 * w['levels'][1]['nnod']]
        xc = np.zeros(3 * w['levels'][1]['nnod'])
        xc[ifree_c] = rng.standard_normal(len(ifree_c))
        yc_ref = np.zeros_like(xc)
        yc_ref[ifree_c] = S.KK[1] @ xc[ifree_c]
        yc = dm2.level_apply(1, xc)
        assert np.linalg.norm(yc - yc_ref) < 1e-5 * np.linalg.norm(yc_ref)
    finally:
        dm2.close()


def _stream_vs_split(dm2, x):
    """(streamed apply twice, per-colour split apply) of the FP32 finest-level operator."""
    try:
        ys = [dm2.level_apply32(0, x) for _ in range(2)]
        dm2.set_option("stream_apply", 0)
        y_split = dm2.level_apply32(0, x)
    finally:
        dm2.set_option("stream_apply", 1)
    return ys, y_split


def test_streamed_fp32_apply(case):
    """The streamed finest-level FP32 apply (TMA ring + fixed-order node sums) is deterministic and
    matches the per-colour split kernel and the FP64 operator to FP32 rounding."""
    w, S, dm = case
    from m3tet_sph_gb300 import stokes
    dm2 = stokes.DeviceMesh(w['levels'])
    try:
        dm2.set_option("fp32_operator", 0)      # the streamed stored matrices
        dm2.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=1)
        rng = np.random.default_rng(11)
        x = np.zeros(S.nU, np.float32)
        x[S.ifree] = rng.standard_normal(len(S.ifree))
        y_ref = np.zeros(S.nU)
        y_ref[S.ifree] = S.K1 @ x[S.ifree].astype(np.float64)
        ys, y_split = _stream_vs_split(dm2, x)
        assert np.array_equal(ys[0], ys[1])
        assert np.linalg.norm(ys[0] - y_split) < 1e-6 * np.linalg.norm(y_split)
        assert np.linalg.norm(ys[0] - y_ref) < 1e-5 * np.linalg.norm(y_ref)
    finally:
        dm2.set_option("fp32_operator", 1)
        dm2.close()


def test_streamed_fp32_apply_many_chunks(built_lib):
    """Same checks on the 15,360-element shell (several chunks per CTA)."""
    from m3tet_sph_gb300 import stokes, workloads
    w = workloads.make_workload('c1')
    dm2 = stokes.DeviceMesh(w['levels'])
    try:
        dm2.set_option("fp32_operator", 0)      # the streamed stored matrices
        dm2.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=1)
        rng = np.random.default_rng(12)
        x = rng.standard_normal(3 * w['levels'][0]['nnod']).astype(np.float32)
        y64s = dm2.level_apply(0, x.astype(np.float64))
        assert np.array_equal(y64s, dm2.level_apply(0, x.astype(np.float64)))
        ydfs = dm2.apply(x.astype(np.float64))
        assert np.array_equal(ydfs, dm2.apply(x.astype(np.float64)))
        try:
            dm2.set_option("stream_outer", 0)
            y64 = dm2.level_apply(0, x.astype(np.float64))
            ydf = dm2.apply(x.astype(np.float64))
        finally:
            dm2.set_option("stream_outer", 1)
        assert np.linalg.norm(y64s - y64) < 1e-14 * np.linalg.norm(y64)
        assert np.linalg.norm(ydfs - ydf) < 1e-14 * np.linalg.norm(ydf)
        assert np.linalg.norm(ydf - y64) < 1e-13 * np.linalg.norm(y64)
        ys, y_split = _stream_vs_split(dm2, x)
        assert np.array_equal(ys[0], ys[1])
        assert np.linalg.norm(ys[0] - y_split) < 1e-6 * np.linalg.norm(y_split)
        assert np.linalg.norm(ys[0] - y64) < 1e-5 * np.linalg.norm(y64)
    finally:
        dm2.set_option("fp32_operator", 1)
        dm2.close()


def test_streamed_fp32_variants_bit_identical(built_lib):
    """Every slot-ring depth / gather-warp count of the streamed FP32 kernel (stream_f32_variant 0..3)
    runs the same arithmetic in the same order: outputs are bit-identical to the default's."""
    from m3tet_sph_gb300 import stokes, workloads
    w = workloads.make_workload('c1')
    dm2 = stokes.DeviceMesh(w['levels'])
    try:
        dm2.set_option("fp32_operator", 0)      # the streamed stored matrices
        dm2.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=1)
        x = np.random.default_rng(13).standard_normal(3 * w['levels'][0]['nnod']).astype(np.float32)
        y0 = dm2.level_apply32(0, x)
        try:
            for v in (1, 2, 3):
                dm2.set_option("stream_f32_variant", v)
                assert np.array_equal(dm2.level_apply32(0, x), y0), v
        finally:
            dm2.set_option("stream_f32_variant", 0)
    finally:
        dm2.set_option("fp32_operator", 1)
        dm2.close()


def test_transfer_matrix_equals_oracle(case):
    """m3sph_transfer_matrix returns intermesh_transfer_matrix's Ic2f (intermesh_transfer_matrix.m:
    1-62) as the oracle builds it from the straight-edged coordinates of both levels."""
    w, S, dm = case
    lv = w['levels']
    Xs_c = O.p2_straight(lv[1]['GCOORD'], lv[1]['EL2NOD'])
    Xs_f = O.straight_coords(Xs_c, lv[0]['EL2NOD'])
    ref = O.intermesh_transfer_matrix(Xs_f, lv[0]['EL2NOD'], Xs_c, lv[1]['EL2NOD'])
    got = dm.transfer_matrix(0)
    assert got.shape == ref.shape
    assert abs(got - ref).max() < 1e-15
