"""ORACLE (test infrastructure only): CPU FP64 restatement of the semi-Lagrangian advection path.

Checker for the CUDA point-location / interpolation / backtracking kernels and the timed CPU
baseline of that path. Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU leg use it.

Restated reference behaviour (paths inside the reference project):
* mfiles_SPH/advect3d_slm_p_sph.m:165-242 (PC2), :298-410 (predictor), :412-440 (corrector)
* mfiles_SPH/find_pts_outside_domain_sph.m:27-98 (radial clamp)
* mfiles_SPH/local_coords_3d_sph.m:28-147 (per-class frames, barycentric determinant ratios)
* mfiles_SPH/local_coords_curved_3d_sph.m:36-168 (6 Newton steps on the 10-node map, tol 1e-8)
* mfiles_SPH/locate_points_interp_vars_3d_sph.m:34-207 (guess, check, search, adjust_local_coords)
* mfiles_M3TET/locate_points_in_neighboring_element.m:1-158 (tolerance growth 1e-6 .. 15e-3)
* mfiles_M3TET/interp3d_tet.m:39-69 (P2 interpolation, monotone clamp)
* mfiles_M3TET/interp3d_cubic_p.m:80-382 (quasi-cubic interpolation, 'dist' weighted gradients)

Point location (one explicit rule, shared with the CUDA walk). The reference's ``tsearch2_sph``
runs MUTILS ``tsearch2`` (not vendored, not runnable here) in up to five rotated frames, keeps at most
one element per frame pass and then resolves points that several passes placed. Here every element
is tested in its own frame (class 0: original, class 1: Z-180, classes 2-3: X-90), with
need(e) = max(-min barycentric, max barycentric - 1):

1. C = {e : need(e) <= TIE_BAND}. If C is not empty (tsearch2_sph.m:374-404):
   a. if C holds a non-isoparametric element, the isoparametric ones are dropped (:380-382);
   b. if the point is at a vertex of every remaining element (max barycentric >= 1 - TIE_BAND),
      only those of the first frame in the reference's pass order are kept -- X-90 (cone classes),
      then original, then Z-180 (:383-386 keeps the first candidate column);
   c. the largest id is taken (:404).
   Ties (|C| >= 2) are counted; so are the ties where neither (a) nor (b) applies and the remaining
   elements lie in more than one frame -- the reference raises error('no good') there (:387-392).
2. Otherwise the tolerance grows in 1e-6 steps up to 15e-3
   (locate_points_in_neighboring_element.m:1-158): q(e) = ceil(need/1e-6 - 1e-9) <= 15000, and among
   the elements of the smallest q: if all are isoparametric, the one with the smallest last Newton
   step (:52-58), otherwise the non-isoparametric one of the smallest id (the reference takes the
   first of the remaining list, :60-66). These points are counted as gaps.
3. Otherwise the point is not located (the reference raises 'some nodes have not been located').

The Newton iteration for isoparametric elements stops per point (local_coords_curved_3d_sph.m stops
when the largest error of the whole batch is below 1e-8, which makes a point's coordinates depend
on the batch it is processed with). MUTILS's own choice among tied elements is unpinned.
"""
from __future__ import annotations

import numpy as np
from scipy.spatial import cKDTree

RX90 = np.array([[1.0, 0, 0], [0, 0, -1.0], [0, 1.0, 0]])
RZ180 = np.diag([-1.0, -1.0, 1.0])


def cart2sph(X):
    x, y, z = X
    r = np.sqrt(x * x + y * y + z * z)
    th = np.arctan2(np.sqrt(x * x + y * y), z)
    ph = np.arctan2(y, x)
    ph = np.where(ph < 0, ph + 2 * np.pi, ph)
    return np.array([th, ph, r])


def sph2cart(S):
    th, ph, r = S
    return np.array([r * np.sin(th) * np.cos(ph), r * np.sin(th) * np.sin(ph), r * np.cos(th)])


class Frames:
    """Node coordinates in the three spherical frames used by local_coords_3d_sph."""

    def __init__(self, mesh):
        self.mesh = mesh
        self.S0 = mesh['GCOORD_SPH']
        self.SZ = cart2sph(RZ180 @ mesh['GCOORD'])
        self.SX = cart2sph(RX90 @ mesh['GCOORD'])
        self.EL = mesh['EL2NOD']
        self.cls = mesh['cls']

    def point_frames(self, P):
        X = sph2cart(P)
        return P, cart2sph(RZ180 @ X), cart2sph(RX90 @ X)


def compute_lc(V, p):
    """Barycentric (r,s,t) of points p (3,n) in straight tets with vertex coords V (n,3,4)
    (determinant ratios of local_coords_3d_sph.m:94-147)."""
    th, ph, r = V[:, 0, :].T, V[:, 1, :].T, V[:, 2, :].T   # (4,n)
    thp, php, rp = p

    def D(a, b, c, d, ta, pa, ra):
        # det of [x_b - x_a; x_c - x_a; x_d - x_a] style expression used in the reference
        return ((th[b] - ta) * (ph[c] - pa) * (r[d] - ra) + (th[c] - ta) * (ph[d] - pa) * (r[b] - ra)
                + (th[d] - ta) * (ph[b] - pa) * (r[c] - ra) - (r[b] - ra) * (ph[c] - pa) * (th[d] - ta)
                - (r[c] - ra) * (ph[d] - pa) * (th[b] - ta) - (r[d] - ra) * (ph[b] - pa) * (th[c] - ta))
    l1 = D(0, 1, 2, 3, thp, php, rp) / D(0, 1, 2, 3, th[0], ph[0], r[0])
    l2 = D(1, 0, 2, 3, thp, php, rp) / D(1, 0, 2, 3, th[1], ph[1], r[1])
    l3 = D(2, 0, 1, 3, thp, php, rp) / D(2, 0, 1, 3, th[2], ph[2], r[2])
    return np.array([l1, l2, l3])


def sf10(r, s, t):
    u = 1 - r - s - t
    N = np.array([r * (2 * r - 1), s * (2 * s - 1), t * (2 * t - 1), u * (2 * u - 1),
                  4 * r * s, 4 * s * t, 4 * t * u, 4 * r * u, 4 * r * t, 4 * s * u])
    z = np.zeros_like(r)
    dN = np.array([
        [4 * r - 1, z, z], [z, 4 * s - 1, z], [z, z, 4 * t - 1], [1 - 4 * u, 1 - 4 * u, 1 - 4 * u],
        [4 * s, 4 * r, z], [z, 4 * t, 4 * s], [-4 * t, -4 * t, 4 * (u - t)], [4 * (u - r), -4 * r, -4 * r],
        [4 * t, z, 4 * r], [-4 * s, 4 * (u - s), -4 * s]])
    return N, dN


NEWTON_STEPS, NEWTON_TOL = 6, 1e-8      # local_coords_curved_3d_sph.m: nimprove, delTH_tol


def local_coords_curved(SX, EL, els, pX):
    """local_coords_curved_3d_sph: linear guess + up to 6 Newton steps on the 10-node map in the
    X-90 frame; a point stops once its own error is below 1e-8. Returns lc and the sum of |delS| of
    each point's last Newton step (0 if it took none)."""
    V = SX[:, EL[els, :4]].transpose(1, 0, 2)
    lc = compute_lc(V, pX)
    G = SX[:, EL[els]]                      # (3,n,10)
    step = np.zeros(lc.shape[1])
    active = np.ones(lc.shape[1], bool)
    for _ in range(NEWTON_STEPS):
        N, dN = sf10(*lc)                   # N (10,n), dN (10,3,n)
        TH0 = np.einsum('kni,in->kn', G, N)
        dTH = pX - TH0
        err = np.sqrt((dTH * dTH).sum(0))
        active &= ~(err < NEWTON_TOL)
        if not active.any():
            break
        a = np.nonzero(active)[0]
        J = np.einsum('kni,ijn->nkj', G[:, a], dN[:, :, a])    # (n,3,3): d TH_k / d s_j
        delS = np.linalg.solve(J, dTH[:, a].T[:, :, None])[:, :, 0].T
        lc[:, a] = lc[:, a] + delS
        step[a] = np.abs(delS).sum(0)
    return lc, step


def local_coords(F, els, P, return_step=False):
    """Own-frame local coordinates (3,n) of points P (3,n, original (theta,phi,r)) in elements els
    (and the last Newton step of isoparametric elements, 0 elsewhere)."""
    els = np.asarray(els, dtype=np.int64)
    P0, PZ, PX = F.point_frames(P)
    lc = np.zeros((3, len(els)))
    step = np.zeros(len(els))
    cls = F.cls[els]
    EL = F.EL
    for c, S, Pp in ((0, F.S0, P0), (1, F.SZ, PZ), (2, F.SX, PX)):
        m = cls == c
        if m.any():
            V = S[:, EL[els[m], :4]].transpose(1, 0, 2)
            lc[:, m] = compute_lc(V, Pp[:, m])
    m = cls == 3
    if m.any():
        lc[:, m], step[m] = local_coords_curved(F.SX, EL, els[m], PX[:, m])
    return (lc, step) if return_step else lc


def inside(lc, tol=0.0):
    l4 = 1 - lc.sum(0)
    return (lc.min(0) >= -tol) & (lc.max(0) <= 1 + tol) & (l4 >= -tol) & (l4 <= 1 + tol)


TIE_BAND = 1e-10          # containment test: every barycentric within [-TIE_BAND, 1 + TIE_BAND]
TIE_TRIGGER = 1e-7        # an element placing the point this close to its boundary may tie with another
IFACE_TRIGGER = 15e-3     # the same next to another frame or to isoparametric elements (overlaps)
GAP_STEP, GAP_QMAX = 1e-6, 15000
FRAME_RANK = np.array([1, 2, 0, 0])     # pass order of each class's frame: X-90 0, original 1, Z-180 2


def tie_rule(ids, iso, frame, atvtx):
    """Rule 1 of the module docstring for candidates `ids` (all within TIE_BAND): returns
    (element, ambiguous)."""
    ids, iso, frame, atvtx = map(np.asarray, (ids, iso, frame, atvtx))
    keep = np.ones(len(ids), bool)
    dropped_iso = (~iso).any() and iso.any()
    if dropped_iso:
        keep &= ~iso
    all_vtx = bool(atvtx[keep].all())
    if all_vtx and keep.sum() >= 2:
        keep &= frame == frame[keep].min()
    ambiguous = len(ids) >= 2 and not dropped_iso and not all_vtx and len(np.unique(frame[keep])) > 1
    return int(ids[keep].max()), bool(ambiguous)


def gap_rule(ids, iso, q, step):
    """Rule 2 of the module docstring for elements `ids` with quantised tolerances q <= GAP_QMAX."""
    ids, iso, q, step = map(np.asarray, (ids, iso, q, step))
    g = q == q.min()
    if iso[g].all():
        s = step[g]
        return int(ids[g][s == s.min()].min())
    return int(ids[g & ~iso].min())


class Locator:
    """Point location by the explicit rule of the module docstring. Candidate elements come from
    the k nearest element centroids; an element that places the point near its boundary (within
    TIE_TRIGGER, or within IFACE_TRIGGER of a face that borders another frame or an isoparametric
    element, where own-frame shapes overlap) has its vertex neighbours added (every other element
    within the tie band shares a vertex with it),
    and a point outside all of them is tested against every element whose centroid lies within
    1.5 circumradii."""

    def __init__(self, mesh, k=48):
        self.F = Frames(mesh)
        X = mesh['GCOORD']
        EL = mesh['EL2NOD']
        EL4 = EL[:, :4]
        nel = len(EL)
        cls = mesh['cls']
        self.iso = cls == 3
        self.frame = FRAME_RANK[cls]
        nv = int(EL4.max()) + 1
        order = np.argsort(EL4.ravel(), kind='stable')
        self.v2e = order // 4
        self.v2e_ptr = np.searchsorted(EL4.ravel()[order], np.arange(nv + 1))
        self.EL4 = EL4
        key = self.frame * 2 + self.iso
        kmin = np.full(nv, 99)
        kmax = np.full(nv, -1)
        np.minimum.at(kmin, EL4.ravel(), np.repeat(key, 4))
        np.maximum.at(kmax, EL4.ravel(), np.repeat(key, 4))
        multi = (kmin != kmax)[EL4]                            # (nel,4): vertex shared across frames / iso-ness
        # face k (opposite vertex k) borders another frame or iso-ness if one of its vertices does
        self.iface_face = np.stack([multi[:, [i for i in range(4) if i != k]].any(1) for k in range(4)], 1)
        V = X[:, EL4]                                           # (3,nel,4)
        self.cent = V.mean(axis=2).T
        self.rad = np.sqrt(((V - self.cent.T[:, :, None]) ** 2).sum(0)).max()
        self.tree = cKDTree(self.cent)
        self.k = min(k, nel)

    def ring1(self, e):
        return np.unique(np.concatenate([self.v2e[self.v2e_ptr[v]:self.v2e_ptr[v + 1]] for v in self.EL4[e]]))

    def _eval(self, els, P):
        lc, step = local_coords(self.F, els, P, return_step=True)
        l4 = 1 - lc.sum(0)
        mn = np.minimum(lc.min(0), l4)
        mx = np.maximum(lc.max(0), l4)
        return lc, step, mn, mx, np.maximum(-mn, mx - 1.0)

    def _resolve_many(self, lists, P):
        """Rules 1-3 for points P (3,m), point i over candidate elements lists[i]: (els, lc, kind)."""
        m = len(lists)
        R = max(len(l) for l in lists)
        ring = np.full((m, R), -1, np.int64)
        for i, l in enumerate(lists):
            ring[i, :len(l)] = l
        valid = ring >= 0
        rows, cols = np.nonzero(valid)
        lc_v, step_v, mn_v, mx_v, need_v = self._eval(ring[rows, cols], P[:, rows])
        need = np.full((m, R), np.inf)
        mx = np.zeros((m, R))
        step = np.zeros((m, R))
        need[rows, cols], mx[rows, cols], step[rows, cols] = need_v, mx_v, step_v
        idx = np.full((m, R), -1)
        idx[rows, cols] = np.arange(len(rows))
        iso = self.iso[np.maximum(ring, 0)] & valid
        frame = self.frame[np.maximum(ring, 0)]
        # rule 1
        cand = need <= TIE_BAND
        drop = (cand & ~iso).any(1) & (cand & iso).any(1)
        keep = cand & ~(drop[:, None] & iso)
        atv = mx >= 1 - TIE_BAND
        all_vtx = (~keep | atv).all(1)
        vdrop = all_vtx & (keep.sum(1) >= 2)
        rmin = np.where(keep, frame, 9).min(1)
        rmax = np.where(keep, frame, -1).max(1)
        keep2 = keep & (~vdrop[:, None] | (frame == rmin[:, None]))
        tie_e = np.where(keep2, ring, -1).max(1)
        ncand = cand.sum(1)
        amb = (ncand >= 2) & ~drop & ~all_vtx & (rmax > rmin)
        # rule 2
        q = np.where(valid & ~cand, np.ceil(need / GAP_STEP - 1e-9), np.inf)
        q[q > GAP_QMAX] = np.inf
        qmin = q.min(1)
        G = np.isfinite(q) & (q == qmin[:, None])
        all_iso = (~G | iso).all(1)
        non_e = np.where(G & ~iso, ring, np.iinfo(np.int64).max).min(1)
        smin = np.where(G & iso, step, np.inf).min(1)
        iso_e = np.where(G & iso & (step == smin[:, None]), ring, np.iinfo(np.int64).max).min(1)
        gap_e = np.where(all_iso, iso_e, non_e)
        has_tie = ncand > 0
        has_gap = ~has_tie & np.isfinite(qmin)
        els = np.where(has_tie, tie_e, np.where(has_gap, gap_e, -1))
        kind = np.where(has_tie, 1 | np.where(ncand >= 2, 2, 0) | np.where(amb, 32, 0), np.where(has_gap, 4, 8))
        lcs = np.zeros((3, m))
        ok = els >= 0
        j = np.argmax(ring == els[:, None], axis=1)
        lcs[:, ok] = lc_v[:, idx[np.nonzero(ok)[0], j[ok]]]
        return els, lcs, kind.astype(np.int32)

    def locate(self, P, return_info=False):
        """Element ids (0-based, -1 if not located) and own-frame lc (3,n) of points P (3,n,
        (theta,phi,r)). info: per-point kind bits (1 placed, 2 tie, 4 gap, 8 not located,
        32 ambiguous for the reference) and counts."""
        n = P.shape[1]
        Xp = sph2cart(P).T
        _, nb = self.tree.query(Xp, k=self.k)
        nb = nb.reshape(n, self.k)
        lc, _, mn, mx, need = self._eval(nb.ravel(), np.repeat(P, self.k, axis=1))
        lc, mn, mx, need = lc.reshape(3, n, self.k), mn.reshape(n, -1), mx.reshape(n, -1), need.reshape(n, -1)
        j = np.argmin(need, axis=1)
        r = np.arange(n)
        best = nb[r, j]
        els = best.copy()
        lcs = lc[:, r, j].copy()
        kind = np.ones(n, np.int32)
        found = need[r, j] <= TIE_BAND
        lb = lcs
        bary = np.vstack([lb, 1 - lb.sum(0)]).T                  # (n,4): barycentric k <-> face k
        trig = found & ((bary < TIE_TRIGGER) | (bary > 1 - TIE_TRIGGER)
                        | (self.iface_face[best] & (bary < IFACE_TRIGGER))).any(1)
        for sel, lists in ((np.nonzero(trig)[0], None), (np.nonzero(~found)[0], None)):
            if len(sel) == 0:
                continue
            if sel is not None and found[sel[0]]:
                lists = [self.ring1(best[i]) for i in sel]
            else:
                lists = [np.array(sorted(self.tree.query_ball_point(Xp[i], 1.5 * self.rad)), dtype=np.int64)
                         for i in sel]
            for c in range(0, len(sel), 4096):
                ss = sel[c:c + 4096]
                e, l, k = self._resolve_many(lists[c:c + 4096], P[:, ss])
                els[ss], lcs[:, ss], kind[ss] = e, l, k
        if return_info:
            info = dict(kind=kind, npt=n, nties=int(((kind & 2) > 0).sum()), ngap=int(((kind & 4) > 0).sum()),
                        nambig=int(((kind & 32) > 0).sum()), nlost=int(((kind & 8) > 0).sum()))
            return els, lcs, info
        return els, lcs


def adjust_local_coords(lc):
    lc = np.clip(lc, 0.0, 1.0)
    s = lc.sum(0)
    bad = s > 1
    lc[:, bad] = lc[:, bad] / s[bad]
    return lc


def interp3d_tet(EL, els, lc, V, monotonic=False):
    """P2 interpolation of nodal V (nnod,) or (nnod,nvar) (interp3d_tet.m:39-69)."""
    N, _ = sf10(*lc)
    V2 = V[:, None] if V.ndim == 1 else V
    out = np.einsum('in,nik->nk', N, V2[EL[els]])
    if monotonic:
        vals = V2[EL[els]]                       # (n,10,nvar)
        out = np.clip(out, vals.min(1), vals.max(1))
    return out[:, 0] if V.ndim == 1 else out


def calc_derivatives(GCOORD, EL4, B, method_wght='dist'):
    """Nodal gradients of vertex values B from P1 element gradients (interp3d_cubic_p.m:244-375)."""
    nnod = GCOORD.shape[1]
    X = GCOORD[:, EL4]                           # (3,nel,4)
    Mx, My, Mz = X[0], X[1], X[2]
    if method_wght == 'dist':
        C = X.mean(axis=2, keepdims=True)
        w = 1.0 / np.sqrt(((X - C) ** 2).sum(0))
    else:
        w = np.ones_like(Mx)
    A = np.stack([np.ones_like(Mx), Mx, My, Mz], axis=2)   # (nel,4,4): rows = vertices
    Bv = B[EL4]
    coef = np.linalg.solve(A, Bv[:, :, None])[:, :, 0]      # [c0, dB/dx, dB/dy, dB/dz]
    grad_el = coef[:, 1:]
    num = np.zeros((nnod, 3))
    den = np.zeros(nnod)
    for k in range(3):
        num[:, k] = np.bincount(EL4.ravel(), weights=(w * grad_el[:, k:k + 1]).ravel(), minlength=nnod)
    den = np.bincount(EL4.ravel(), weights=w.ravel(), minlength=nnod)
    return num, grad_el, den


def interp3d_cubic(GCOORD, EL, els, lc, B, monotonic=True, method_wght='dist'):
    """Quasi-cubic interpolation of vertex values of B (interp3d_cubic_p.m:80-226)."""
    EL4 = EL[:, :4]
    num, gel, den = calc_derivatives(GCOORD, EL4, B, method_wght)
    with np.errstate(invalid='ignore', divide='ignore'):
        gn = num / den[:, None]
    r, s, t = lc
    u = 1 - r - s - t
    q2 = np.sqrt(2.0)
    N = np.array([r, s, t, u, q2 * r * s, q2 * s * t, t * u, r * u, q2 * r * t, s * u,
                  q2 * s * r * (s - r), q2 * s * t * (t - s), t * u * (u - t), r * u * (u - r),
                  q2 * r * t * (t - r), s * u * (u - s)])
    v = EL4[els]                                 # (n,4)
    X = GCOORD[:, v]                             # (3,n,4)
    dB = gn[v] - gel[els][:, None, :]            # (n,4,3)
    e_r = X[:, :, 0] - X[:, :, 3]
    e_s = X[:, :, 1] - X[:, :, 3]
    e_t = X[:, :, 2] - X[:, :, 3]
    sr = np.einsum('kn,njk->jn', e_r, dB)         # slopeDev_r(node j)
    ss = np.einsum('kn,njk->jn', e_s, dB)
    st = np.einsum('kn,njk->jn', e_t, dB)
    h = np.sqrt(0.5)
    q1n2, q1n1 = h * sr[1] - h * ss[1], h * sr[0] - h * ss[0]
    q2n3, q2n2 = h * ss[2] - h * st[2], h * ss[1] - h * st[1]
    q5n3, q5n1 = h * sr[2] - h * st[2], h * sr[0] - h * st[0]
    info = np.array([(q1n2 - q1n1) / 2, (q2n3 - q2n2) / 2, (st[3] - st[2]) / 2, (sr[3] - sr[0]) / 2,
                     (q5n3 - q5n1) / 2, (ss[3] - ss[1]) / 2, (q1n2 + q1n1) / 2, (q2n3 + q2n2) / 2,
                     (st[3] + st[2]) / 2, (sr[3] + sr[0]) / 2, (q5n3 + q5n1) / 2, (ss[3] + ss[1]) / 2])
    Bi = (N[:4] * B[v].T).sum(0) + (N[4:] * info).sum(0)
    if monotonic:
        Bv = B[v]
        Bi = np.clip(Bi, Bv.min(1), Bv.max(1))
    return Bi


def clamp_radius(P, r_cmb, r_surf):
    """find_pts_outside_domain_sph: move points outside [r_cmb, r_surf] just inside."""
    P = P.copy()
    r_tol = 1e-12 * (r_surf - r_cmb)
    P[2] = np.where(P[2] <= r_cmb + r_tol, r_cmb + r_tol, P[2])
    P[2] = np.where(P[2] >= r_surf - r_tol, r_surf - r_tol, P[2])
    return P


def predictor(X, S, U, dt):
    """predictor_step_with_projections (advect3d_slm_p_sph.m:298-410); U (3,n) Cartesian."""
    rr = S[2]
    ru = X / rr
    upar = (U * ru).sum(0) * ru / (np.sqrt((ru ** 2).sum(0)) ** 2)
    uperp = U - upar
    nperp = np.sqrt((uperp ** 2).sum(0))
    with np.errstate(invalid='ignore', divide='ignore'):
        upu = uperp / nperp
    upu = np.where(np.isnan(upu), 0.0, upu)
    lpar = np.sqrt((upar ** 2).sum(0)) * 0.5 * dt
    lperp = nperp * 0.5 * dt
    lprime = rr * np.tan(lperp / rr)
    rp = X - upu * lprime
    rbu = rp / np.sqrt((rp ** 2).sum(0))
    xyz = rbu * np.abs(rr - lpar)
    return cart2sph(xyz), upu, rbu


def corrector(X, S, U, upu, rpu, dt):
    """corrector_step_with_projections (advect3d_slm_p_sph.m:412-440)."""
    rr = S[2]
    upar = (U * rpu).sum(0) * rpu / (np.sqrt((rpu ** 2).sum(0)) ** 2)
    uperp = U - upar
    lpar = np.sqrt((upar ** 2).sum(0)) * dt
    lperp = np.sqrt((uperp ** 2).sum(0)) * dt
    lprime = rr * np.tan(lperp / rr)
    rp = X - upu * lprime
    rbu = rp / np.sqrt((rp ** 2).sum(0))
    xyz = rbu * np.abs(rr - lpar)
    return cart2sph(xyz)


def advect_pc2(mesh, U, T, dt, r_cmb, r_surf, method_interp='quadratic', monotonic=True, k=48):
    """advect3d_slm_p_sph with PC2 backtracking; U (nnod,3) Cartesian; returns new T, departure
    points (3,nnod), element ids of the predictor and departure points."""
    X = mesh['GCOORD']
    S = mesh['GCOORD_SPH']
    loc = Locator(mesh, k)
    Pp, upu, rpu = predictor(X, S, U.T, dt)
    Pp = clamp_radius(Pp, r_cmb, r_surf)
    e1, lc1 = loc.locate(Pp)
    lc1 = adjust_local_coords(lc1)
    Ubt = interp3d_tet(mesh['EL2NOD'], e1, lc1, U, monotonic=False)
    Pd = corrector(X, S, Ubt.T, upu, rpu, dt)
    Pd = clamp_radius(Pd, r_cmb, r_surf)
    e2, lc2 = loc.locate(Pd)
    lc2 = adjust_local_coords(lc2)
    if method_interp == 'cubic':
        Tn = interp3d_cubic(X, mesh['EL2NOD'], e2, lc2, T, monotonic)
    else:
        Tn = interp3d_tet(mesh['EL2NOD'], e2, lc2, T, monotonic)
    return Tn, Pd, e1, e2


def advect_rk4(mesh, U, T, dt, r_cmb, r_surf, nsub=3, method_interp='quadratic', monotonic=True, k=48):
    """Builder-defined RK4 backtracking over `nsub` substeps (the reference's RK4 is an error stub,
    advect3d_slm_p_sph.m:103-104): classical RK4 on dx/dt = U(x) backwards in Cartesian
    coordinates, every stage point moved radially into [r_cmb + tol, r_surf - tol], U by P2
    interpolation at located points; T interpolated at the departure points."""
    X = mesh['GCOORD']
    loc = Locator(mesh, k)
    r_tol = 1e-12 * (r_surf - r_cmb)

    def U_at(Xp):
        P = clamp_radius(cart2sph(Xp), r_cmb, r_surf)
        e, lc = loc.locate(P)
        return interp3d_tet(mesh['EL2NOD'], e, adjust_local_coords(lc), U).T

    h = dt / nsub
    Xc = X.copy()
    for sub in range(nsub):
        k1 = U.T if sub == 0 else U_at(Xc)
        k2 = U_at(Xc - 0.5 * h * k1)
        k3 = U_at(Xc - 0.5 * h * k2)
        k4 = U_at(Xc - h * k3)
        Xc = Xc - h / 6.0 * (k1 + 2 * k2 + 2 * k3 + k4)
        r = np.sqrt((Xc ** 2).sum(0))
        Xc = Xc * (np.clip(r, r_cmb + r_tol, r_surf - r_tol) / r)
    Pd = cart2sph(Xc)
    e2, lc2 = loc.locate(Pd)
    lc2 = adjust_local_coords(lc2)
    if method_interp == 'cubic':
        Tn = interp3d_cubic(X, mesh['EL2NOD'], e2, lc2, T, monotonic)
    else:
        Tn = interp3d_tet(mesh['EL2NOD'], e2, lc2, T, monotonic)
    return Tn, Pd, e2
