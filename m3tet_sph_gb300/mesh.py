"""Curved P2 spherical-shell meshes and their geometric multigrid hierarchy (host-side set-up).

This module builds the ``MESH`` data that the reference's ``init_mesh_curved_p`` produces
(mfiles_SPH/init_mesh_curved_p.m:182-217) for synthetic icosahedral shells:

* the coarsest level is an icosahedral surface of level ``L - (nmg-1)`` extruded into
  ``nlayer / 2**(nmg-1)`` radial layers, each prism split into three tetrahedra;
* every finer level is made the reference's way: split each P2 tetrahedron into 8 children
  along its shortest interior diagonal (mfiles_M3TET/tetmesh_p2_to_p1.m) and promote the
  children to curved P2 with spherical midside nodes (mfiles_SPH/tetmesh_p1_to_p2_sph.m);
* element classes follow ``check_els_in_cone`` (mfiles_SPH/check_els_in_cone.m:59-76) and
  ``check_phi`` (mfiles_SPH/check_phi.m:59-71);
* in-cone isoparametric elements get the 20-node cubic geometry of
  ``cubic_els_in_cone_iso`` (mfiles_SPH/cubic_els_in_cone_iso.m).

Node numbering follows the reference: vertices first, then one node per unique edge in
first-occurrence order over the element edge list (edges 1-2, 2-3, 3-4, 4-1, 1-3, 4-2;
tetmesh_p1_to_p2_sph.m:516-550). All indices here are 0-based.
"""
from __future__ import annotations

import numpy as np

# element classes (stored as uint8 per element)
CLS_OUT_NO_CROSS = 0   # els_out_cone_no_cross_2pi
CLS_OUT_CROSS = 1      # els_out_cone_cross_2pi
CLS_IN_NO_ISO = 2      # els_in_cone_no_iso
CLS_IN_ISO = 3         # els_in_cone_iso (20-node cubic geometry)

PID_CMB = 301
PID_SURF = 306

# local edge list of a 10-node tetrahedron (nodes 5..10)
EDGES = np.array([[0, 1], [1, 2], [2, 3], [3, 0], [0, 2], [3, 1]], dtype=np.int64)

# reference rotation matrices (tetmesh_p1_to_p2_sph.m, cubic_els_in_cone_iso.m)
RR_X_90_CCW = np.array([[1.0, 0.0, 0.0], [0.0, 0.0, -1.0], [0.0, 1.0, 0.0]])
RR_X_90_CW = RR_X_90_CCW.T.copy()
RR_Z_180 = np.array([[-1.0, 0.0, 0.0], [0.0, -1.0, 0.0], [0.0, 0.0, 1.0]])

# children of a P2 tetrahedron for the three diagonal choices (tetmesh_p2_to_p1.m, 1-based)
_EL2CHILD = [
    [1, 5, 9, 8, 5, 2, 6, 10, 9, 6, 3, 7, 8, 10, 7, 4, 10, 8, 7, 5, 6, 9, 5, 7, 8, 7, 5, 9, 10, 5, 7, 6],
    [1, 5, 9, 8, 5, 2, 6, 10, 9, 6, 3, 7, 8, 10, 7, 4, 5, 9, 8, 6, 10, 7, 6, 8, 9, 8, 6, 7, 5, 6, 8, 10],
    [1, 5, 9, 8, 5, 2, 6, 10, 9, 6, 3, 7, 8, 10, 7, 4, 8, 5, 9, 10, 7, 6, 10, 9, 5, 9, 10, 6, 8, 10, 9, 7],
]
EL2CHILD = np.array(_EL2CHILD, dtype=np.int64).reshape(3, 8, 4) - 1
# interior diagonals (node pairs) tested by tetmesh_p2_to_p1: [5 7; 6 8; 9 10]
DIAG2NOD = np.array([[4, 6], [5, 7], [8, 9]], dtype=np.int64)

# barycentric lattice coordinates (r, s, t) of the 10 P2 nodes (sf_dsf_tet.m:821-840)
P2_NODE_LC = np.array([
    [1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 0, 0],
    [.5, .5, 0], [0, .5, .5], [0, 0, .5], [.5, 0, 0], [.5, 0, .5], [0, .5, 0]])


def cart2sph(X):
    """(3,n) Cartesian -> (3,n) (theta, phi, r); phi in [0, 2pi) (cartesian2spherical.m)."""
    x, y, z = X
    r = np.sqrt(x * x + y * y + z * z)
    th = np.arctan2(np.sqrt(x * x + y * y), z)
    ph = np.arctan2(y, x)
    ph = np.where(ph < 0, ph + 2 * np.pi, ph)
    return np.array([th, ph, r])


def sph2cart(S):
    """(3,n) (theta, phi, r) -> Cartesian (spherical2cartesian.m)."""
    th, ph, r = S
    return np.array([r * np.sin(th) * np.cos(ph), r * np.sin(th) * np.sin(ph), r * np.cos(th)])


def sf10(lc):
    """P2 shape-function values at local coords lc (3,n) -> (10,n) (sf_dsf_tet10)."""
    r, s, t = lc
    u = 1.0 - r - s - t
    return np.array([r * (2 * r - 1), s * (2 * s - 1), t * (2 * t - 1), u * (2 * u - 1),
                     4 * r * s, 4 * s * t, 4 * t * u, 4 * r * u, 4 * r * t, 4 * s * u])


# --------------------------------------------------------------------------------------
# icosahedral P1 shell
# --------------------------------------------------------------------------------------
def icosphere(level):
    """Unit icosahedron (one vertex on the +z pole) subdivided ``level`` times."""
    p = (1 + 5 ** 0.5) / 2
    V = np.array([[-1, p, 0], [1, p, 0], [-1, -p, 0], [1, -p, 0], [0, -1, p], [0, 1, p],
                  [0, -1, -p], [0, 1, -p], [p, 0, -1], [p, 0, 1], [-p, 0, -1], [-p, 0, 1]], float)
    F = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                  [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                  [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    # rotate so that vertex 0 sits on the +z axis
    a = V[0]
    z = np.array([0.0, 0.0, 1.0])
    v = np.cross(a, z)
    c = float(a @ z)
    vx = np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])
    R = np.eye(3) + vx + vx @ vx / (1 + c)
    V = V @ R.T
    for _ in range(level):
        e = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
        key = np.minimum(e[:, 0], e[:, 1]) * len(V) + np.maximum(e[:, 0], e[:, 1])
        uk, inv = np.unique(key, return_inverse=True)
        a0, a1 = uk // len(V), uk % len(V)
        M = V[a0] + V[a1]
        M /= np.linalg.norm(M, axis=1, keepdims=True)
        mid = inv.reshape(3, -1) + len(V)
        m01, m12, m20 = mid
        V = np.concatenate([V, M])
        F = np.concatenate([
            np.stack([F[:, 0], m01, m20], 1), np.stack([F[:, 1], m12, m01], 1),
            np.stack([F[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)])
    return V, F


def orient_tets(X, T):
    """Reorder vertices so that det[X1-X4, X2-X4, X3-X4] > 0 (positive Jacobian)."""
    a = X[:, T[:, 0]] - X[:, T[:, 3]]
    b = X[:, T[:, 1]] - X[:, T[:, 3]]
    c = X[:, T[:, 2]] - X[:, T[:, 3]]
    det = np.einsum('ij,ij->j', a, np.cross(b.T, c.T).T)
    neg = det < 0
    T = T.copy()
    T[neg, 0], T[neg, 1] = T[neg, 1].copy(), T[neg, 0].copy()
    return T


def shell_p1(level, nlayer, r_cmb, r_surf):
    """Icosahedral surface extruded into ``nlayer`` equal radial layers, prisms split into 3 tets.

    Each prism (a<b<c bottom, a'<b'<c' top) is split as (a,b,c,c'), (a,b,b',c'), (a,a',b',c'):
    every quad face is cut from its lower-index bottom vertex to the higher-index top vertex,
    which is consistent between neighbouring prisms. Returns Cartesian (3,nV), tets (nel,4),
    PointID (nV,).
    """
    V, F = icosphere(level)
    nv = len(V)
    radii = r_cmb + (r_surf - r_cmb) * np.arange(nlayer + 1) / nlayer
    radii[-1] = r_surf
    X = np.concatenate([V.T * r for r in radii], axis=1)
    Fs = np.sort(F, axis=1)
    tets = []
    for k in range(nlayer):
        a, b, c = (Fs[:, 0] + k * nv, Fs[:, 1] + k * nv, Fs[:, 2] + k * nv)
        a2, b2, c2 = a + nv, b + nv, c + nv
        tets.append(np.stack([a, b, c, c2], 1))
        tets.append(np.stack([a, b, b2, c2], 1))
        tets.append(np.stack([a, a2, b2, c2], 1))
    # interleave so that the three tets of a prism are neighbours in memory
    T = np.stack([np.concatenate(tets[3 * k:3 * k + 3]) for k in range(nlayer)])
    T = np.concatenate([T[k].reshape(3, -1, 4).transpose(1, 0, 2).reshape(-1, 4) for k in range(nlayer)])
    T = orient_tets(X, T)
    pid = np.zeros(X.shape[1], np.int32)
    pid[:nv] = PID_CMB
    pid[nlayer * nv:] = PID_SURF
    return X, T, pid


# --------------------------------------------------------------------------------------
# P1 -> curved P2 promotion (tetmesh_p1_to_p2_sph)
# --------------------------------------------------------------------------------------
def classify(S4, T4, theta_cone_deg):
    """Element classes from vertex (theta, phi): check_els_in_cone + check_phi."""
    tc = np.deg2rad(theta_cone_deg)
    th = S4[0][T4]                      # (nel,4)
    nin = np.sum((th <= tc) | (th >= np.pi - tc), axis=1)
    ph = S4[1][T4]
    pairs = [(0, 1), (1, 2), (2, 0), (0, 3), (1, 3), (2, 3)]
    cross = np.zeros(len(T4), bool)
    for i, j in pairs:
        cross |= np.abs(ph[:, i] - ph[:, j]) > np.pi
    cls = np.full(len(T4), CLS_OUT_NO_CROSS, np.uint8)
    cls[(nin == 0) & cross] = CLS_OUT_CROSS
    cls[nin > 0] = CLS_IN_NO_ISO
    cls[(nin > 0) & (nin < 3)] = CLS_IN_ISO
    return cls


def unique_bars(T4):
    """Unique element edges in first-occurrence order (find_unique_bars).

    Returns bars (nbar,2) in the orientation of their first occurrence and EL2BAR (nel,6).
    """
    e = T4[:, EDGES].reshape(-1, 2)
    n = int(T4.max()) + 1
    key = np.minimum(e[:, 0], e[:, 1]) * n + np.maximum(e[:, 0], e[:, 1])
    perm = np.argsort(key, kind='stable')
    ks = key[perm]
    new = np.empty(ks.size, bool)
    new[0] = True
    np.not_equal(ks[1:], ks[:-1], out=new[1:])
    first = perm[new]                            # first occurrence of each edge (stable sort)
    is_first = np.zeros(key.size, bool)
    is_first[first] = True
    bar_at = np.cumsum(is_first) - 1             # bar id of a first occurrence, in occurrence order
    grp = np.empty(key.size, np.int64)
    grp[perm] = np.cumsum(new) - 1               # edge group of every occurrence
    el2bar = bar_at[first][grp].reshape(-1, 6)
    bars = e[is_first]
    return bars, el2bar


def _marked(ids, n, drop=None):
    """Sorted distinct values of non-negative ids below n (np.unique's result), minus ``drop``
    (np.setdiff1d's), by marking instead of sorting."""
    m = np.zeros(n, bool)
    m[ids] = True
    if drop is not None:
        m[drop] = False
    return np.nonzero(m)[0]


def _mid_in_frame(Xc, bars, R):
    """Spherical midpoints of bars computed in the frame rotated by R (no phi unwrap)."""
    Sr = cart2sph(R @ Xc)
    mid = 0.5 * (Sr[:, bars[:, 0]] + Sr[:, bars[:, 1]])
    return cart2sph(R.T @ sph2cart(mid))


def _bar_rows(bars_sub, bars_all, n):
    key_all = np.minimum(bars_all[:, 0], bars_all[:, 1]) * n + np.maximum(bars_all[:, 0], bars_all[:, 1])
    key_sub = np.minimum(bars_sub[:, 0], bars_sub[:, 1]) * n + np.maximum(bars_sub[:, 0], bars_sub[:, 1])
    srt = np.argsort(key_all)
    pos = np.searchsorted(key_all[srt], key_sub)
    return srt[pos]


def promote_p2_sph(Xc, Sc, T4, pid_c, r_cmb, r_surf, theta_cone_deg=45.0):
    """Curved P2 promotion of a P1 tet mesh (tetmesh_p1_to_p2_sph.m:1-230).

    Xc: (3,nV) Cartesian vertices, Sc: (3,nV) their (theta,phi,r), T4: (nel,4).
    Returns dict with EL2NOD (nel,10), GCOORD, GCOORD_SPH, PointID, cls, and the
    20-node cubic geometry of in-cone isoparametric elements.
    """
    nV = Xc.shape[1]
    cls = classify(Sc, T4, theta_cone_deg)
    bars, el2bar = unique_bars(T4)
    nbar = len(bars)
    # default: midpoint in the original frame with phi unwrap (check_ang_dist_phi)
    th_e = Sc[0][bars]
    ph_e = Sc[1][bars].copy()
    r_e = Sc[2][bars]
    wrap = np.abs(ph_e[:, 0] - ph_e[:, 1]) > np.pi
    ph_w = ph_e[wrap]
    ph_w[ph_w < np.pi] += 2 * np.pi
    ph_e[wrap] = ph_w
    mid = np.array([th_e.mean(1), ph_e.mean(1), r_e.mean(1)])
    # cone bars: bars of in-cone elements minus iso-element bars with both ends outside the cone
    tc = np.deg2rad(theta_cone_deg)
    in_cone = cls >= CLS_IN_NO_ISO
    if in_cone.any():
        iso = cls == CLS_IN_ISO
        drop = None
        if iso.any():
            iso_bars = _marked(el2bar[iso].ravel(), nbar)
            thb = Sc[0][bars[iso_bars]]
            out2 = np.sum((thb > tc) & (thb < np.pi - tc), axis=1) == 2
            drop = iso_bars[out2]
        cone_bars = _marked(el2bar[in_cone].ravel(), nbar, drop)
        mid[:, cone_bars] = _mid_in_frame(Xc, bars[cone_bars], RR_X_90_CCW)
    cross = cls == CLS_OUT_CROSS
    if cross.any():
        cb = _marked(el2bar[cross].ravel(), nbar)
        mid[:, cb] = _mid_in_frame(Xc, bars[cb], RR_Z_180)
    EL2NOD = np.concatenate([T4, nV + el2bar], axis=1).astype(np.int64)
    S = np.concatenate([Sc, mid], axis=1)
    X = sph2cart(S)
    # PointID: vertices keep theirs; edge nodes inherit a boundary id shared by both ends
    pid = np.zeros(nV + nbar, np.int32)
    pid[:nV] = pid_c
    pa, pb = pid_c[bars[:, 0]], pid_c[bars[:, 1]]
    pid[nV:] = np.where((pa == pb) & (pa > 0), pa, 0)
    S[2, pid == PID_CMB] = r_cmb
    S[2, pid == PID_SURF] = r_surf
    out = dict(EL2NOD=EL2NOD, GCOORD=X, GCOORD_SPH=S, PointID=pid, cls=cls, nVnod=nV,
               bars=bars)
    iso_idx = np.nonzero(cls == CLS_IN_ISO)[0]
    out['els_iso'] = iso_idx
    out['cubic_sph_rot'] = cubic_geometry(Xc, Sc, T4[iso_idx], theta_cone_deg) if len(iso_idx) else \
        np.zeros((0, 3, 20))
    return out


# --------------------------------------------------------------------------------------
# 20-node cubic geometry of in-cone isoparametric elements (cubic_els_in_cone_iso.m)
# --------------------------------------------------------------------------------------
# the 9 nodes of each face (face k is opposite vertex k), cubic_els_in_cone_iso.m
FACES20 = np.array([[2, 3, 4, 7, 8, 9, 10, 15, 16], [1, 3, 4, 13, 14, 9, 10, 11, 12],
                    [1, 2, 4, 5, 6, 16, 15, 11, 12], [1, 2, 3, 5, 6, 7, 8, 14, 13]]) - 1


def cubic_geometry(Xc, Sc, T4iso, theta_cone_deg):
    """(theta,phi,r) of the 20 cubic nodes of each iso element in the X-90 rotated frame.

    Edge third-points are straight in the original spherical frame (phi unwrapped) for edges
    with both ends outside the cone, and straight in the X-90 frame otherwise; slot 2k-1 of
    edge k = (a,b) is the point one third of the way from a. Face nodes are the mean of the
    face's 9 nodes in the X-90 frame for faces touching the cone, the spherical centroid of the
    3 vertices (Z-180 frame) for out-of-cone faces crossing phi=2pi, and the mean of the 9
    nodes in the original frame otherwise.
    """
    tc = np.deg2rad(theta_cone_deg)
    nel = len(T4iso)
    S_rotX = cart2sph(RR_X_90_CCW @ Xc)
    P = np.zeros((nel, 3, 20))          # Cartesian coordinates of the 20 nodes
    P[:, :, :4] = Xc[:, T4iso].transpose(1, 0, 2)
    out = (Sc[0] > tc) & (Sc[0] < np.pi - tc)
    for k, (i, j) in enumerate(EDGES):
        a, b = T4iso[:, i], T4iso[:, j]
        both_out = out[a] & out[b]
        # original frame, unwrapped phi
        pa, pb = Sc[1][a].copy(), Sc[1][b].copy()
        w = np.abs(pa - pb) > np.pi
        pa = np.where(w & (pa < np.pi), pa + 2 * np.pi, pa)
        pb = np.where(w & (pb < np.pi), pb + 2 * np.pi, pb)
        for m, f in enumerate((1.0 / 3.0, 2.0 / 3.0)):
            so = np.array([Sc[0][a] + f * (Sc[0][b] - Sc[0][a]), pa + f * (pb - pa),
                           Sc[2][a] + f * (Sc[2][b] - Sc[2][a])])
            sr = S_rotX[:, a] + f * (S_rotX[:, b] - S_rotX[:, a])
            xo = sph2cart(so)
            xr = RR_X_90_CW @ sph2cart(sr)
            P[:, :, 4 + 2 * k + m] = np.where(both_out[None, :], xo, xr).T
    # face nodes
    Srot = _cart2sph_nodes(P, RR_X_90_CCW)
    Sorig = _cart2sph_nodes(P, None)
    for f in range(4):
        nodes = FACES20[f]
        verts = nodes[:3]
        vglob = T4iso[:, verts]
        all_out = np.all(out[vglob], axis=1)
        # default: mean of the 9 nodes in the original frame (third points may be unwrapped:
        # recompute their original-frame phi consistently with the unwrapped edge param)
        m_orig = Sorig[:, :, nodes].mean(axis=2)
        # out-of-cone faces crossing 2pi: centroid of 3 vertices in the Z-180 frame
        phv = Sc[1][vglob]
        cross = np.zeros(nel, bool)
        for (i, j) in [(0, 1), (1, 2), (2, 0)]:
            cross |= np.abs(phv[:, i] - phv[:, j]) > np.pi
        S180 = cart2sph(RR_Z_180 @ Xc[:, vglob.ravel()]).reshape(3, nel, 3).mean(axis=2)
        x180 = (RR_Z_180.T @ sph2cart(S180)).T
        m_rot = Srot[:, :, nodes].mean(axis=2)
        x_rot = (RR_X_90_CW @ sph2cart(m_rot.T)).T
        x_orig = sph2cart(_unwrap_face_mean(Sorig[:, :, nodes]).T).T
        xf = np.where((all_out & cross)[:, None], x180, np.where(all_out[:, None], x_orig, x_rot))
        P[:, :, 16 + f] = xf
        del m_orig
    return _cart2sph_nodes(P, RR_X_90_CCW)


def _cart2sph_nodes(P, R):
    """(theta,phi,r) of the nodes P (nel,3,k), rotated by R first if given: (nel,3,k). The rotations
    used here are signed permutations, so applying them to all nodes at once gives the values of
    the per-element products exactly."""
    nel, _, k = P.shape
    if nel == 0:
        return np.zeros((0, 3, k))
    X = P.transpose(1, 0, 2).reshape(3, nel * k)
    if R is not None:
        X = R @ X
    return cart2sph(X).reshape(3, nel, k).transpose(1, 0, 2)


def _unwrap_face_mean(Sn):
    """Mean (theta,phi,r) of face nodes (nel,3,9) with phi unwrapped around the first node."""
    Sn = Sn.copy()
    ph = Sn[:, 1, :]
    ref = ph[:, :1]
    ph = np.where(ph - ref > np.pi, ph - 2 * np.pi, ph)
    ph = np.where(ph - ref < -np.pi, ph + 2 * np.pi, ph)
    Sn[:, 1, :] = ph
    return Sn.mean(axis=2)


# --------------------------------------------------------------------------------------
# refinement (tetmesh_refine_sph) and multigrid transfer (intermesh_transfer_matrix)
# --------------------------------------------------------------------------------------
def split_p2(X, EL2NOD):
    """8 children per P2 tet along the shortest interior diagonal (tetmesh_p2_to_p1.m).

    Child k of parent p is element 8p+k. Returns (8*nel,4) vertex lists and isplit (nel,).
    """
    L = np.stack([np.linalg.norm(X[:, EL2NOD[:, a]] - X[:, EL2NOD[:, b]], axis=0)
                  for a, b in DIAG2NOD])
    isplit = np.argmin(L, axis=0)
    ch = EL2NOD[np.arange(len(EL2NOD))[:, None, None], EL2CHILD[isplit]]   # (nel,8,4)
    return ch.reshape(-1, 4), isplit


def child_lattice(isplit):
    """Lattice (r,s,t) of the 10 nodes of each child in its parent: (3 splits, 8, 10, 3)."""
    lat = np.zeros((3, 8, 10, 3))
    for s in range(3):
        for k in range(8):
            v = P2_NODE_LC[EL2CHILD[s, k]]
            lat[s, k, :4] = v
            for e, (i, j) in enumerate(EDGES):
                lat[s, k, 4 + e] = 0.5 * (v[i] + v[j])
    return lat


CHILD_LATTICE = child_lattice(None)
# per-(split, child) prolongation weights: W[s,k,i,j] = N_j(parent) at child node i
CHILD_PROLONG = np.stack([np.stack([sf10(CHILD_LATTICE[s, k].T).T for k in range(8)]) for s in range(3)])


def transfer_rows(EL2NOD_f, isplit_c, EL2NOD_c):
    """Per fine node: coarse parent nodes (nnod_f,10) and weights (nnod_f,10).

    The parent of a fine node is the parent of the first fine element that lists it
    (column-major first occurrence, intermesh_transfer_matrix.m:19-23); the weights are the
    parent's P2 shape functions at the node's lattice position.
    """
    nel_f = len(EL2NOD_f)
    nnod_f = int(EL2NOD_f.max()) + 1
    flat = EL2NOD_f.ravel()                  # element-major: first occurrence = lowest element
    first = np.full(nnod_f, flat.size, dtype=np.int64)
    np.minimum.at(first, flat, np.arange(flat.size, dtype=np.int64))
    el = first // 10
    loc = first % 10
    par = el // 8
    k = el % 8
    s = isplit_c[par]
    W = CHILD_PROLONG[s, k, loc]             # (nnod_f,10)
    cols = EL2NOD_c[par]                     # (nnod_f,10)
    W = np.where(np.abs(W) < 1e-14, 0.0, W)
    assert np.all(first < flat.size), "fine nodes without an element"
    return cols, W


def build_hierarchy(level, nlayer, nmg, r_cmb=3480.0, r_surf=6371.0, theta_cone=45.0,
                    jitter=0.01, seed=0):
    """MG hierarchy: list of levels, finest first (reference EL2NOD{1} = finest).

    Each level dict holds EL2NOD (nel,10), GCOORD, GCOORD_SPH, PointID, cls, cubic geometry;
    level l (l < nmg-1) also holds ``isplit`` of its coarse parent level and the transfer rows
    from level l+1. Finest interior vertices are jittered by U(-jitter, jitter) x local edge
    length per component, then the finest midside nodes are recomputed.
    """
    L0 = level - (nmg - 1)
    n0 = nlayer // 2 ** (nmg - 1)
    if L0 < 0 or n0 * 2 ** (nmg - 1) != nlayer:
        raise ValueError("level/nlayer not compatible with nmg")
    X, T4, pid = shell_p1(L0, n0, r_cmb, r_surf)
    S = cart2sph(X)
    lev = promote_p2_sph(X, S, T4, pid, r_cmb, r_surf, theta_cone)
    levels = [lev]
    for img in range(nmg - 1):
        c = levels[-1]
        ch, isplit = split_p2(c['GCOORD'], c['EL2NOD'])
        c['isplit'] = isplit
        Xv, Sv, pv = c['GCOORD'], c['GCOORD_SPH'], c['PointID']
        finest = img == nmg - 2
        if finest and jitter > 0:
            Xv, Sv = _jitter(Xv, Sv, ch, pv, jitter, seed)
        f = promote_p2_sph(Xv, Sv, ch, pv, r_cmb, r_surf, theta_cone)
        f['transfer_cols'], f['transfer_w'] = transfer_rows(f['EL2NOD'], isplit, c['EL2NOD'])
        levels.append(f)
    levels = levels[::-1]
    for lv in levels:
        lv['nel'] = len(lv['EL2NOD'])
        lv['nnod'] = lv['GCOORD'].shape[1]
    return levels


def _jitter(X, S, T4, pid, amp, seed):
    rng = np.random.default_rng(seed)
    e = T4[:, EDGES].reshape(-1, 2)
    ln = np.linalg.norm(X[:, e[:, 0]] - X[:, e[:, 1]], axis=0)
    n = X.shape[1]
    hsum = np.bincount(e.ravel(), weights=np.repeat(ln, 2), minlength=n)
    cnt = np.bincount(e.ravel(), minlength=n)
    h = hsum / np.maximum(cnt, 1)
    d = rng.uniform(-amp, amp, size=X.shape) * h[None, :]
    d[:, pid > 0] = 0.0
    X2 = X + d
    S2 = cart2sph(X2)
    keep = pid > 0
    S2[:, keep] = S[:, keep]
    return X2, S2


def rotation_blocks(X):
    """Per-node 3x3 (theta,phi,r)->(x,y,z) rotation (make_rotation_matrix.m:69-112), (n,3,3)."""
    S = cart2sph(X)
    th, ph = S[0], S[1]
    R = np.zeros((X.shape[1], 3, 3))
    R[:, 0, 0] = np.cos(ph) * np.cos(th)
    R[:, 0, 1] = -np.sin(ph)
    R[:, 0, 2] = np.cos(ph) * np.sin(th)
    R[:, 1, 0] = np.sin(ph) * np.cos(th)
    R[:, 1, 1] = np.cos(ph)
    R[:, 1, 2] = np.sin(ph) * np.sin(th)
    R[:, 2, 0] = -np.sin(th)
    R[:, 2, 2] = np.cos(th)
    return R


def mesh_counts(level, nlayer):
    """Closed-form P1 tet / P2 node counts of an icosahedral shell."""
    V, F, E = 10 * 4 ** level + 2, 20 * 4 ** level, 30 * 4 ** level
    return dict(nel=3 * F * nlayer, nnod=V * (nlayer + 1) + E * (nlayer + 1) + V * nlayer + E * nlayer,
                nP=V * (nlayer + 1))
