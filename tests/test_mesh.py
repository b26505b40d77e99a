"""Mesh promotion / hierarchy (host set-up), pinned against the reference's shipped mesh."""
from pathlib import Path

import numpy as np
import pytest

from m3tet_sph_gb300 import mesh as M

GOLD = Path(__file__).resolve().parent / 'golden'


def test_promotion_matches_reference_mesh():
    """tetmesh_p1_to_p2_sph on the P1 part of EarthShell_n37k reproduces its EL2NOD exactly and
    its curved midside nodes to rounding (all four element classes present)."""
    g = np.load(GOLD / 'earthshell_n37k.npz')
    E = g['EL2NOD'].astype(np.int64)
    X = g['GCOORD'].T
    nV = E[:, :4].max() + 1
    pid = g['PointID'][:nV]
    out = M.promote_p2_sph(X[:, :nV], M.cart2sph(X[:, :nV]), E[:, :4], pid, float(g['r_cmb']), float(g['r_surf']))
    assert np.array_equal(out['EL2NOD'], E)
    assert np.abs(out['GCOORD'] - X).max() < 1e-9
    assert np.array_equal(out['PointID'], g['PointID'])
    assert np.bincount(out['cls'], minlength=4).tolist() == [25790, 41, 298, 231]


@pytest.mark.parametrize("L,n,nmg", [(2, 4, 2), (3, 8, 3)])
def test_hierarchy_counts(L, n, nmg):
    levels = M.build_hierarchy(L, n, nmg)
    for k, lv in enumerate(levels):
        c = M.mesh_counts(L - k, n // 2 ** k)
        assert lv['nel'] == c['nel'] and lv['nnod'] == c['nnod']
        assert int(lv['EL2NOD'][:, :4].max()) + 1 == c['nP']
    # coarse nodes are the leading nodes of the next finer level
    for k in range(nmg - 1):
        f, c = levels[k], levels[k + 1]
        nc = c['nnod']
        # children of coarse element p are fine elements 8p..8p+7 and use only its nodes as vertices
        ch = f['EL2NOD'][:, :4].reshape(-1, 8, 4)
        for p in range(0, c['nel'], max(1, c['nel'] // 50)):
            assert set(ch[p].ravel()) <= set(c['EL2NOD'][p])
        assert f['EL2NOD'][:, :4].max() + 1 == nc


def test_transfer_rows_partition_of_unity():
    levels = M.build_hierarchy(2, 4, 2)
    W = levels[0]['transfer_w']
    assert np.allclose(W.sum(1), 1.0, atol=1e-14)
    # weights are exact multiples of 1/8
    assert np.allclose(W * 8, np.round(W * 8), atol=1e-12)


def test_positive_orientation_and_classes():
    lv = M.build_hierarchy(3, 8, 3)[0]
    E = lv['EL2NOD']
    X = lv['GCOORD']
    a = X[:, E[:, 0]] - X[:, E[:, 3]]
    b = X[:, E[:, 1]] - X[:, E[:, 3]]
    c = X[:, E[:, 2]] - X[:, E[:, 3]]
    det = np.einsum('ij,ij->j', a, np.cross(b.T, c.T).T)
    assert (det > 0).all()
    assert set(np.unique(lv['cls'])) == {0, 1, 2, 3}
