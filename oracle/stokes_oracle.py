"""ORACLE (test infrastructure only): CPU FP64 restatement of the reference's Stokes hot path.

This module checks the CUDA library's results and is the timed CPU baseline. Only tests,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import it. It shares no code
with the product kernels: the element operator, assembly, rotation, boundary conditions,
Galerkin restriction, coarse Cholesky, MG-PCG and Patera pressure CG are restated here in
numpy/scipy, vectorised over element blocks like the reference's MILAMIN code.

Parity status: the reference is MATLAB and needs un-vendored MUTILS/SuiteSparse MEX files, so
it cannot run here and ships no golden vectors for the operator or the solvers. This oracle's
element operator, solver and transfer operators are therefore "parity unpinned" against the
reference's outputs; what IS pinned is (a) the mesh promotion, checked bit-for-bit against the
reference's shipped curved mesh ``SETUP_TEST/MESHES/EarthShell_n37k.mat`` (tests/golden), and
(b) the quadrature constants, checked against the numeric values documented in
``mfiles_M3TET/ip_tetrahedron.m:109-117``.

Reference files restated (paths inside the reference project):
* mfiles_M3TET/ip_tetrahedron.m:100-123 and :193 (14-point Gellert-Harbord rule, weights / 6)
* mfiles_M3TET/sf_dsf_tet.m:821-907 (10-node), :909-946 (4-node), :247-496 (20-node)
* mfiles_SPH/assembly_stokes_els_out_cone_no_cross_2pi_opt.m:93-356 (element matrices)
* mfiles_SPH/assembly_stokes_els_out_cone_cross_2pi_opt.m:96-101, :385-429 (Z-180 frame)
* mfiles_SPH/assembly_stokes_els_in_cone_no_iso_opt.m:93-106, :390-496 (X-90 frame)
* mfiles_SPH/assembly_stokes_els_in_cone_iso_20_nodes_opt.m:97-157 (20-node Jacobian)
* mfiles_M3TET/calc_element_visc.m:5-7,43-48, calc_element_dens.m:5-7
* mfiles_SPH/make_rotation_matrix.m:69-112; mfiles_M3TET/flow3d_patera_mg_sph_p.m
* mfiles_M3TET/mgpcg_solver_p.m; mfiles_M3TET/restrict_stiffmat.m:79-142
* mfiles_M3TET/intermesh_transfer_matrix.m:1-62; mfiles_M3TET/cholesky_factorization.m
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp

# ----------------------------------------------------------------------------------------
# quadrature and shape functions
# ----------------------------------------------------------------------------------------


def ip_tetrahedron14():
    """14-point degree-5 rule (ip_tetrahedron.m:100-123), weights divided by 6 (:193)."""
    g = 1.0 / (46.0 * np.sqrt(46.0))
    h = np.arccos(g) + (2.0 / 3.0) * np.arcsin(g)
    k = (104.0 + 8.0 * np.sqrt(46.0) * np.cos(h)) / 3.0
    s = np.sqrt(49.0 - k)
    b = (7.0 + s) / k
    a = 1.0 - 3.0 * b
    d = (7.0 - s) / k
    c = 1.0 - 3.0 * d
    p = (98.0 - k - 14.0 * s) / (1680.0 * s * (b - a) ** 3)
    q = (98.0 - k + 14.0 * s) / (1680.0 * s * (c - d) ** 3)
    r = (1.0 - 4.0 * (p + q)) / 6.0
    e = (1.0 + (2.0 / (105.0 * r)) ** 0.25) / 4.0
    f = (1.0 - 2.0 * e) / 2.0
    ipx = np.array([[a, b, b, b, c, d, d, d, e, e, e, f, f, f],
                    [b, a, b, b, d, c, d, d, e, f, f, e, e, f],
                    [b, b, a, b, d, d, c, d, f, e, f, e, f, e]])
    ipw = np.array([p] * 4 + [q] * 4 + [r] * 6) / 6.0
    return ipx, ipw


def sf4(r, s, t):
    u = 1.0 - r - s - t
    N = np.array([r, s, t, u])
    dN = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [-1, -1, -1]], float)
    return N, dN


def sf10(r, s, t):
    u = 1.0 - r - s - t
    N = np.array([r * (2 * r - 1), s * (2 * s - 1), t * (2 * t - 1), u * (2 * u - 1),
                  4 * r * s, 4 * s * t, 4 * t * u, 4 * r * u, 4 * r * t, 4 * s * u])
    dN = np.array([
        [4 * r - 1, 0, 0], [0, 4 * s - 1, 0], [0, 0, 4 * t - 1],
        [1 - 4 * u, 1 - 4 * u, 1 - 4 * u],
        [4 * s, 4 * r, 0], [0, 4 * t, 4 * s], [-4 * t, -4 * t, 4 * (u - t)],
        [4 * (u - r), -4 * r, -4 * r], [4 * t, 0, 4 * r], [-4 * s, 4 * (u - s), -4 * s]])
    return N, dN


def sf20(r, s, t):
    """Cubic 20-node Lagrange tetrahedron in the reference's node order (sf_dsf_tet20).

    Nodes 1-4 vertices (r,s,t,u); 5-16 edge third-points (5,6 on r-s; 7,8 s-t; 9,10 t-u;
    11,12 u-r; 13,14 r-t; 15,16 u-s; the first of each pair nearer the first vertex named);
    17-20 face centres opposite vertices 1-4.
    """
    u = 1.0 - r - s - t
    L = [r, s, t, u]
    gL = [np.array([1.0, 0, 0]), np.array([0, 1.0, 0]), np.array([0, 0, 1.0]), np.array([-1.0, -1, -1])]
    N = np.zeros(20)
    dN = np.zeros((20, 3))
    for i in range(4):
        Li = L[i]
        N[i] = 0.5 * Li * (3 * Li - 1) * (3 * Li - 2)
        dN[i] = 0.5 * (27 * Li * Li - 18 * Li + 2) * gL[i]
    pairs = [(0, 1), (1, 0), (1, 2), (2, 1), (2, 3), (3, 2), (3, 0), (0, 3), (0, 2), (2, 0), (3, 1), (1, 3)]
    for m, (a, b) in enumerate(pairs):
        La, Lb = L[a], L[b]
        N[4 + m] = 4.5 * La * Lb * (3 * La - 1)
        dN[4 + m] = 4.5 * (Lb * (6 * La - 1) * gL[a] + La * (3 * La - 1) * gL[b])
    faces = [(1, 2, 3), (0, 2, 3), (0, 1, 3), (0, 1, 2)]
    for m, (a, b, c) in enumerate(faces):
        N[16 + m] = 27 * L[a] * L[b] * L[c]
        dN[16 + m] = 27 * (L[b] * L[c] * gL[a] + L[a] * L[c] * gL[b] + L[a] * L[b] * gL[c])
    return N, dN


def cart2sph(X):
    x, y, z = X
    r = np.sqrt(x * x + y * y + z * z)
    th = np.arctan2(np.sqrt(x * x + y * y), z)
    ph = np.arctan2(y, x)
    ph = np.where(ph < 0, ph + 2 * np.pi, ph)
    return np.array([th, ph, r])


RX90 = np.array([[1.0, 0, 0], [0, 0, -1.0], [0, 1.0, 0]])   # v_rot = RX90 @ v
RZ180 = np.diag([-1.0, -1.0, 1.0])


# ----------------------------------------------------------------------------------------
# element matrices (all four classes)
# ----------------------------------------------------------------------------------------
def element_matrices(mesh, visc, dens, g=-9.81, Bscale=1.0, Dens0=0.0, minVisc=None, maxVisc=None):
    """Element K (nel,30,30), G (nel,30,4), M (nel,4,4), Fb (nel,30) in Cartesian frame.

    Dof order inside an element is node-major (3*node + component), as in the reference.
    ``G[e, 3n+c, p] = sum_ip w * NP_p * dN_n/dx_c``; the global Stokes system reads
    K U - G P = Fb, G^T U = 0 (flow3d_patera_mg_sph_p.m:269-298).
    """
    EL = mesh['EL2NOD']
    nel = len(EL)
    cls = mesh['cls']
    S = mesh['GCOORD_SPH']
    X = mesh['GCOORD']
    ipx, ipw = ip_tetrahedron14()
    K = np.zeros((nel, 30, 30))
    G = np.zeros((nel, 30, 4))
    Mm = np.zeros((nel, 4, 4))
    Fb = np.zeros((nel, 30))
    # '23rd' D-matrix (C1 = 4/3, C2 = -2/3, _opt.m:201-208): for dof (i,a), (j,b)
    # K = w*visc*(d_ab gradNi.gradNj + d_b Ni d_a Nj - 2/3 d_a Ni d_b Nj); on a = b this is
    # C1 d_aNi d_aNj + sum_{c!=a} d_cNi d_cNj as written in _opt.m:263-316.
    C2 = -2.0 / 3.0
    v4 = EL[:, :4]
    # vertex coordinates in each element's frame
    VC = np.zeros((nel, 3, 4))
    VC[:] = S[:, v4].transpose(1, 0, 2)
    c1 = cls == 1
    ph = VC[c1, 1, :] + np.pi
    ph = np.where(ph > 2 * np.pi, ph - 2 * np.pi, ph)
    VC[c1, 1, :] = ph
    c23 = (cls == 2) | (cls == 3)
    if c23.any():
        Xr = RX90 @ X[:, v4[c23].ravel()]
        VC[c23] = cart2sph(Xr).reshape(3, -1, 4).transpose(1, 0, 2)
    iso = np.nonzero(cls == 3)[0]
    EC20 = mesh['cubic_sph_rot']            # (niso,3,20) in X-90 frame
    iso_pos = {e: i for i, e in enumerate(mesh['els_iso'])}
    iso_rows = np.array([iso_pos[e] for e in iso], dtype=np.int64)
    _, dN4 = sf4(0.25, 0.25, 0.25)
    # straight (classes 0-2) J_SL: rows = d(sph)/d(loc)
    J_SL = np.einsum('eki,ij->ejk', VC, dN4)            # (nel,3 loc,3 sph)
    for ip in range(14):
        r_, s_, t_ = ipx[:, ip]
        NU, dNU = sf10(r_, s_, t_)
        NP, _ = sf4(r_, s_, t_)
        Js = J_SL.copy()
        sph_ip = np.einsum('eki,i->ek', VC, NP)         # th, ph, r at IP
        if len(iso):
            N20, dN20 = sf20(r_, s_, t_)
            E = EC20[iso_rows]
            Js[iso] = np.einsum('eki,ij->ejk', E, dN20)
            sph_ip[iso] = np.einsum('eki,i->ek', E, N20)
        detSL = np.linalg.det(Js)
        if np.any(detSL < 0):
            raise ValueError('negative Jacobi')
        J_LS = np.linalg.inv(Js)                        # d(loc)/d(sph) transposed convention
        th, phi, rr = sph_ip[:, 0], sph_ip[:, 1], sph_ip[:, 2]
        st, ct, sph_, cph = np.sin(th), np.cos(th), np.sin(phi), np.cos(phi)
        detCS = rr ** 2 * st
        J_SC = np.zeros((nel, 3, 3))                    # J_SC[k, j] = d sph_j / d cart_k
        J_SC[:, 0] = np.stack([rr * st * ct * cph, -rr * sph_, rr ** 2 * st ** 2 * cph], 1) / detCS[:, None]
        J_SC[:, 1] = np.stack([rr * st * ct * sph_, rr * cph, rr ** 2 * st ** 2 * sph_], 1) / detCS[:, None]
        J_SC[:, 2] = np.stack([-rr * st ** 2, np.zeros(nel), rr ** 2 * st * ct], 1) / detCS[:, None]
        Jdbl = J_SC @ J_LS                               # d loc_j / d cart_k
        dNdx = np.einsum('ekj,nj->enk', Jdbl, dNU)      # (nel,10,3)
        w = detCS * detSL * ipw[ip]
        visc_ip = visc[v4] @ NP
        if minVisc is not None:
            visc_ip = np.maximum(visc_ip, minVisc)
        if maxVisc is not None:
            visc_ip = np.minimum(visc_ip, maxVisc)
        dens_ip = dens[v4] @ NP
        Fg = g * Bscale * (dens_ip - Dens0)
        w2 = visc_ip * w
        lap = np.einsum('eik,ejk->eij', dNdx, dNdx)     # grad Ni . grad Nj
        B = np.einsum('eib,eja->eiajb', dNdx, dNdx)     # d_b N_i d_a N_j
        A = np.einsum('eia,ejb->eiajb', dNdx, dNdx)     # d_a N_i d_b N_j
        Ke = B + C2 * A
        for a in range(3):
            Ke[:, :, a, :, a] += lap
        K += w2[:, None, None] * Ke.reshape(nel, 30, 30)
        G += (w[:, None, None, None] * dNdx[:, :, :, None] * NP[None, None, None, :]).reshape(nel, 30, 4)
        Mm += (w / visc_ip)[:, None, None] * np.outer(NP, NP)[None]
        dirv = np.stack([st * cph, st * sph_, ct], 1)   # radial unit vector in the element frame
        Fb += ((w * Fg)[:, None, None] * NU[None, :, None] * dirv[:, None, :]).reshape(nel, 30)
    # un-rotate frames: K = R^T K_rot R per node block, G = R^T G_rot, Fb = R^T Fb_rot
    for cl, R in ((1, RZ180), (2, RX90), (3, RX90)):
        idx = np.nonzero(cls == cl)[0]
        if len(idx) == 0:
            continue
        Rb = np.kron(np.eye(10), R)                      # (30,30): v_rot = Rb v
        K[idx] = Rb.T @ K[idx] @ Rb
        G[idx] = Rb.T @ G[idx]
        Fb[idx] = Fb[idx] @ Rb
    return K, G, Mm, Fb


def element_matrices_threaded(mesh, visc, dens, nthreads, **phys):
    """element_matrices over contiguous blocks of elements on `nthreads` host threads (numpy
    releases the GIL inside its kernels); the same per-element arithmetic as one call."""
    EL = mesh['EL2NOD']
    nel = len(EL)
    if nthreads <= 1 or nel < 4096:
        return element_matrices(mesh, visc, dens, **phys)
    from concurrent.futures import ThreadPoolExecutor
    iso_pos = {e: i for i, e in enumerate(mesh['els_iso'])}
    bounds = np.linspace(0, nel, nthreads + 1).astype(np.int64)

    def block(k):
        lo, hi = int(bounds[k]), int(bounds[k + 1])
        sub = dict(mesh)
        sub['EL2NOD'] = EL[lo:hi]
        sub['cls'] = mesh['cls'][lo:hi]
        els = [e for e in mesh['els_iso'] if lo <= e < hi]
        sub['els_iso'] = np.array([e - lo for e in els], dtype=np.int64)
        sub['cubic_sph_rot'] = mesh['cubic_sph_rot'][[iso_pos[e] for e in els]] if els else \
            mesh['cubic_sph_rot'][:0]
        return element_matrices(sub, visc, dens, **phys)

    with ThreadPoolExecutor(nthreads) as ex:
        parts = list(ex.map(block, range(nthreads)))
    return tuple(np.concatenate([p[i] for p in parts]) for i in range(4))


# ----------------------------------------------------------------------------------------
# assembly, rotation, boundary conditions
# ----------------------------------------------------------------------------------------
def el2dof(EL):
    return (3 * EL[:, :, None] + np.arange(3)[None, None, :]).reshape(len(EL), 30)


def assemble(mesh, K, G, Mm, Fb):
    EL = mesh['EL2NOD']
    nnod = mesh['GCOORD'].shape[1]
    nP = int(EL[:, :4].max()) + 1
    nU = 3 * nnod
    D = el2dof(EL)
    rows = np.repeat(D, 30, axis=1).ravel()
    cols = np.tile(D, (1, 30)).ravel()
    KK = sp.csr_matrix((K.reshape(len(EL), -1).ravel(), (rows, cols)), shape=(nU, nU))
    P4 = EL[:, :4]
    GG = sp.csr_matrix((G.reshape(len(EL), -1).ravel(),
                        (np.repeat(D, 4, axis=1).ravel(), np.tile(P4, (1, 30)).ravel())), shape=(nU, nP))
    MM = sp.csr_matrix((Mm.reshape(len(EL), -1).ravel(),
                        (np.repeat(P4, 4, axis=1).ravel(), np.tile(P4, (1, 4)).ravel())), shape=(nP, nP))
    FF = np.bincount(D.ravel(), weights=Fb.ravel(), minlength=nU)
    return KK, GG, MM, FF


def rotation_matrix(X):
    """Sparse RR: U_xyz = RR @ U_local, local = (theta, phi, r) components per node."""
    S = cart2sph(X)
    th, ph = S[0], S[1]
    n = X.shape[1]
    blocks = np.zeros((n, 3, 3))
    blocks[:, 0] = np.stack([np.cos(ph) * np.cos(th), -np.sin(ph), np.cos(ph) * np.sin(th)], 1)
    blocks[:, 1] = np.stack([np.sin(ph) * np.cos(th), np.cos(ph), np.sin(ph) * np.sin(th)], 1)
    blocks[:, 2] = np.stack([-np.sin(th), np.zeros(n), np.cos(th)], 1)
    return sp.block_diag(list(blocks), format='csr') if n < 2000 else _bd(blocks)


def _bd(blocks):
    n = len(blocks)
    r = (3 * np.arange(n)[:, None, None] + np.arange(3)[None, :, None]).repeat(3, axis=2)
    c = (3 * np.arange(n)[:, None, None] + np.arange(3)[None, None, :]).repeat(3, axis=1)
    return sp.csr_matrix((blocks.ravel(), (r.ravel(), c.ravel())), shape=(3 * n, 3 * n))


# ----------------------------------------------------------------------------------------
# multigrid transfer (intermesh_transfer_matrix) and Galerkin restriction
# ----------------------------------------------------------------------------------------
def straight_coords(mesh_c_straight_p2, EL2NOD_f):
    """Straight coordinates of fine nodes: coarse P2 nodes keep theirs, fine edge nodes are
    Cartesian midpoints of their fine edge (tetmesh_refine -> tetmesh_p1_to_p2)."""
    Xc = mesh_c_straight_p2
    nc = Xc.shape[1]
    nf = int(EL2NOD_f.max()) + 1
    Xf = np.zeros((3, nf))
    Xf[:, :nc] = Xc
    ed = [(0, 1), (1, 2), (2, 3), (3, 0), (0, 2), (3, 1)]
    for k, (a, b) in enumerate(ed):
        Xf[:, EL2NOD_f[:, 4 + k]] = 0.5 * (Xf[:, EL2NOD_f[:, a]] + Xf[:, EL2NOD_f[:, b]])
    return Xf


def p2_straight(X4, EL2NOD):
    """Straight P2 coordinates: vertices as given, edge nodes at Cartesian midpoints."""
    nn = int(EL2NOD.max()) + 1
    Xs = np.zeros((3, nn))
    nv = X4.shape[1]
    Xs[:, :nv] = X4[:, :nv]
    ed = [(0, 1), (1, 2), (2, 3), (3, 0), (0, 2), (3, 1)]
    for k, (a, b) in enumerate(ed):
        Xs[:, EL2NOD[:, 4 + k]] = 0.5 * (Xs[:, EL2NOD[:, a]] + Xs[:, EL2NOD[:, b]])
    return Xs


def local_coords_3d(Xc, EL4, els, pts):
    """Barycentric (r,s,t) of points in straight tets (local_coords_3d)."""
    x4 = Xc[:, EL4[els, 3]]
    A = np.stack([Xc[:, EL4[els, 0]] - x4, Xc[:, EL4[els, 1]] - x4, Xc[:, EL4[els, 2]] - x4], axis=2)
    b = (pts - x4).T[:, :, None]
    return np.linalg.solve(np.moveaxis(A, 1, 0), b)[:, :, 0].T


def intermesh_transfer_matrix(Xs_f, EL_f, Xs_c, EL_c):
    """Ic2f (scalar, nnod_f x nnod_c) following intermesh_transfer_matrix.m:1-62."""
    flat = EL_f.ravel()
    nod_f, first = np.unique(flat, return_index=True)
    els = first // 10
    els_c = els // 8
    lc = local_coords_3d(Xs_c, EL_c, els_c, Xs_f[:, nod_f])
    tol = 1e-5
    if lc.min() < -tol or lc.max() > 1 + tol or lc.sum(0).max() > 1 + tol:
        raise ValueError('Calculation of interpolation matrix failed.')
    lc = np.clip(lc, 0.0, 1.0)
    lc = np.round(1000 * lc) / 1000
    r, s, t = lc
    u = 1 - r - s - t
    N = np.array([r * (2 * r - 1), s * (2 * s - 1), t * (2 * t - 1), u * (2 * u - 1),
                  4 * r * s, 4 * s * t, 4 * t * u, 4 * r * u, 4 * r * t, 4 * s * u]).T
    ii = np.repeat(nod_f, 10)
    jj = EL_c[els_c].ravel()
    nf = len(nod_f)
    nc = int(EL_c.max()) + 1
    return sp.csr_matrix((N.ravel(), (ii, jj)), shape=(nf, nc))


def expand3(P):
    return sp.kron(P, sp.identity(3), format='csr')


# ----------------------------------------------------------------------------------------
# solvers
# ----------------------------------------------------------------------------------------
def normdf(x):
    return np.linalg.norm(x) / np.sqrt(len(x))


class CoarseChol:
    """Sparse factorisation of the coarsest operator with a minimum-degree ordering, no pivoting
    (cholesky_factorization.m:227-237: AMD + sparse L L^T; cholesky_solve.m:265-281: two
    triangular solves). SuperLU in symmetric mode with the diagonal pivots forced factors the SPD
    matrix as L D L^T-equivalent L U."""

    def __init__(self, K):
        import scipy.sparse.linalg as spla
        K = sp.csc_matrix(K)
        self.lu = spla.splu(K, permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.0,
                            options=dict(SymmetricMode=True))

    def solve(self, r):
        return self.lu.solve(np.asarray(r, dtype=np.float64))


class OmpCSR:
    """y = A @ x on `nthreads` host threads through the oracle's OpenMP product (oracle/csr_omp.c).
    The reference's own product (mgpcg_solver_p.m:728-733, MUTILS spmv) is multi-threaded too. Each
    row is summed in the same order with separate multiply and add, so the result equals scipy's
    ``A @ x`` to rounding (bit for bit where scipy's multiply-adds are not fused)."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            import ctypes as C
            from oracle import build_oracle
            L = C.CDLL(str(build_oracle.build()))
            L.csr_matvec.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
            L.csr_matvec.restype = None
            cls._lib = L
        return cls._lib

    def __init__(self, A, nthreads):
        A = A.tocsr()
        A.sort_indices()
        self.shape = A.shape
        self.ptr = np.ascontiguousarray(A.indptr, dtype=np.int64)
        self.col = np.ascontiguousarray(A.indices, dtype=np.int32)
        self.val = np.ascontiguousarray(A.data, dtype=np.float64)
        self.nthreads = int(nthreads)
        self.lib()

    def __matmul__(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.shape[0])
        self._lib.csr_matvec(self.shape[0], self.ptr.ctypes.data, self.col.ctypes.data, self.val.ctypes.data,
                             x.ctypes.data, y.ctypes.data, self.nthreads)
        return y


class MGPCG:
    """mgpcg_solver_p (flexible Polak-Ribiere PCG, V-cycle v2, Jacobi weights 'Setup 3')."""

    def __init__(self, K1, KK, Ic2f, nmg):
        self.K1 = K1
        self.KK = KK
        self.P = Ic2f
        self.nmesh = len(KK)
        self.KDi = [1.0 / KK[0]] + [1.0 / KK[j].diagonal() for j in range(1, self.nmesh)]
        self.coarse = CoarseChol(KK[-1])
        self.wd = [[0.9, 0.4, 0.25]] + [[0.25, 0.4, 0.9]] * (self.nmesh - 2)
        self.wu = [[0.25, 0.4, 0.9]] + [[0.9, 0.4, 0.25]] * (self.nmesh - 2)
        self.napply = 0
        self.PT = [None] * len(Ic2f)

    def use_threads(self, nthreads):
        """Run the sparse products on `nthreads` host threads (the CPU baseline's timing mode)."""
        if not hasattr(self, "_serial"):
            self._serial = (self.K1, list(self.KK), list(self.P), list(self.PT))
        K1, KK, P = self._serial[0], self._serial[1], self._serial[2]
        self.K1 = OmpCSR(K1, nthreads)
        self.KK = [KK[0]] + [OmpCSR(K, nthreads) for K in KK[1:]]
        self.PT = [OmpCSR(p.T, nthreads) for p in P]
        self.P = [OmpCSR(p, nthreads) for p in P]

    def use_serial(self):
        """Back to the serial products after use_threads."""
        if hasattr(self, "_serial"):
            self.K1, self.KK, self.P, self.PT = self._serial[0], list(self._serial[1]), list(self._serial[2]), \
                list(self._serial[3])

    def _K(self, j, x):
        self.napply += 1
        return self.K1 @ x if j == 0 else self.KK[j] @ x

    def vcycle(self, r):
        r0 = r
        dd, rr = [], []
        for j in range(self.nmesh - 1):
            rr.append(r0)
            r1 = r0
            d1 = np.zeros_like(r0)
            for w in self.wd[j]:
                d1 = d1 + w * r1 * self.KDi[j]
                r1 = r0 - self._K(j, d1)
            dd.append(d1)
            r0 = (self.P[j].T if self.PT[j] is None else self.PT[j]) @ r1
        d = self.coarse.solve(r0)
        for j in range(self.nmesh - 2, -1, -1):
            d = dd[j] + self.P[j] @ d
            for w in self.wu[j]:
                r1 = rr[j] - self._K(j, d)
                d = d + w * r1 * self.KDi[j]
        return d

    def solve(self, b, x, tol=None, rtol=None, itmax=20):
        r = b - self.K1 @ x
        rrms = normdf(r)
        if tol is None:
            tol = rtol * rrms
        hist = [rrms]
        it = 0
        rd = None
        q = None
        rlast = None
        for it in range(1, itmax + 1):
            d = self.vcycle(r)
            if it == 1:
                q = d
            else:
                rdlast = rd
                beta = np.dot(r - rlast, d) / rdlast
                q = d + beta * q
            rd = np.dot(r, d)
            Kq = self.K1 @ q
            qKq = np.dot(q, Kq)
            rlast = r
            alpha = rd / qKq
            x = x + alpha * q
            r = r - alpha * Kq
            rrms = normdf(r)
            hist.append(rrms)
            if rrms < tol:
                break
        return x, it, hist


def rm0space(a):
    return a - a.mean()


class StokesSystem:
    """Rotated, BC-reduced Stokes system + MG hierarchy (flow3d_patera_mg_sph_p.m:182-384)."""

    def __init__(self, levels, visc, dens, ifix, vfix, phys=None, nthreads=1):
        phys = phys or {}
        f = levels[0]
        K, G, Mm, Fb = element_matrices_threaded(f, visc, dens, nthreads, **phys)
        KK, GG, MM, FF = assemble(f, K, G, Mm, Fb)
        RR = rotation_matrix(f['GCOORD'])
        K1 = (RR.T @ KK @ RR).tocsr()
        self.GG = (RR.T @ GG).tocsr()
        self.Fb = RR.T @ FF
        self.RR = RR
        nU = K1.shape[0]
        self.nU = nU
        self.nP = GG.shape[1]
        self.ifix = np.asarray(ifix, dtype=np.int64)
        self.vfix = np.asarray(vfix, dtype=float)
        free = np.ones(nU, bool)
        free[self.ifix] = False
        self.ifree = np.nonzero(free)[0]
        Ufix = np.zeros(nU)
        Ufix[self.ifix] = self.vfix
        self.bc_rhs = K1 @ Ufix
        self.Ufix = Ufix
        self.Kfull = K1
        self.K1 = K1[self.ifree][:, self.ifree].tocsr()
        # Galerkin hierarchy (restrict_stiffmat.m:79-142)
        KKl = [self.K1.diagonal()]
        Ps = []
        Xs_c = p2_straight(levels[-1]['GCOORD'], levels[-1]['EL2NOD'])
        straight = [None] * len(levels)
        straight[-1] = Xs_c
        for j in range(len(levels) - 2, -1, -1):
            straight[j] = straight_coords(straight[j + 1], levels[j]['EL2NOD'])
        ifree_l = self.ifree
        Kprev = self.K1
        for j in range(len(levels) - 1):
            Ic2f = intermesh_transfer_matrix(straight[j], levels[j]['EL2NOD'], straight[j + 1],
                                             levels[j + 1]['EL2NOD'])
            P3 = expand3(Ic2f)
            nUc = P3.shape[1]
            ifree_c = ifree_l[ifree_l < nUc]
            PU = P3[ifree_l][:, ifree_c].tocsr()
            Kc = (PU.T @ Kprev @ PU).tocsr()
            KKl.append(Kc)
            Ps.append(PU)
            Kprev = Kc
            ifree_l = ifree_c
        self.KK = KKl
        self.Ps = Ps
        self.mg = MGPCG(self.K1, KKl, Ps, len(levels))
        MMf = MM
        self.MM = MMf
        self.LMM = np.asarray(MMf.sum(axis=1)).ravel()
        self.LiMM = 1.0 / self.LMM

    def precondition_P(self, r):
        d = r * self.LiMM
        Md = self.MM @ d
        return d + 1.0 * self.LiMM * (r - Md)

    def residual(self, U, P):
        """Coupled FP64 relative residual on free dofs, pressure mean removed."""
        fu = (self.Fb - self.bc_rhs)[self.ifree]
        ru = fu - (self.K1 @ U[self.ifree] - (self.GG @ P)[self.ifree])
        rp = -(self.GG.T @ U)
        rp = rm0space(rp)
        return np.sqrt(np.dot(ru, ru) + np.dot(rp, rp)) / np.sqrt(np.dot(fu, fu))


def patera(sysm, P0=None, rtol_Pat=1e-4, rtol_U=5e-3, itmax_Pat=120, itmax_U=20, itmin_Pat=3,
           verbose=False, target_rel_residual=0.0):
    """Patera pressure CG around MG-PCG (flow3d_patera_mg_sph_p.m:386-632). With a target coupled
    residual (the library's extension): when the pressure tolerance is met but the coupled FP64
    residual is above the target, both tolerances are cut by 10, the velocity is solved for the
    current pressure, the pressure residual is replaced by the true -G'U and CG restarts."""
    s = sysm
    ifree = s.ifree
    nU = s.nU
    U = s.Ufix.copy()
    P = np.zeros(s.nP) if P0 is None else P0.copy()
    rtol_restart = 0.8 * rtol_Pat
    Rhs = (s.Fb + s.GG @ P - s.bc_rhs)[ifree]
    info = dict(nitU=0, nitZ=0)
    U[ifree], nit, _ = s.mg.solve(Rhs, U[ifree], rtol=rtol_U * rtol_restart, itmax=itmax_U)
    info['nitU'] += nit
    r = -(s.GG.T @ U)
    r = rm0space(r)
    norm_rP = normdf(r)
    tol_Pat = rtol_Pat * norm_rP
    U[ifree], nit, _ = s.mg.solve(Rhs, U[ifree], tol=rtol_U * rtol_restart * norm_rP, itmax=itmax_U)
    info['nitU'] += nit
    tol_U_restart = rtol_U * tol_Pat
    restart = True
    conv_problem = False
    q = None
    rd = None
    rlast = None
    norm_rP0 = norm_rP
    itPat = 0
    tol_Z = None
    for itPat in range(1, itmax_Pat + 1):
        d = s.precondition_P(r)
        if restart:
            q = d
            restart = False
            norm_rP0 = norm_rP
            tol_Z = rtol_U * max(rtol_restart * norm_rP0, tol_Pat)
        else:
            rdlast = rd
            beta = np.dot(r - rlast, d) / rdlast
            q = d + beta * q
        q = rm0space(q)
        rd = np.dot(r, d)
        y = s.GG @ q
        z = np.zeros(nU)
        z[ifree], nit, _ = s.mg.solve(y[ifree], z[ifree], tol=tol_Z, itmax=itmax_U)
        info['nitZ'] += nit
        Sq = s.GG.T @ z
        qSq = np.dot(q, Sq)
        rlast = r
        alpha = rd / qSq
        P = P + alpha * q
        U = U + alpha * z
        r = r - alpha * Sq
        r = rm0space(r)
        norm_rP_last = norm_rP
        norm_rP = normdf(r)
        norm_rP_min = min(norm_rP_last, norm_rP)
        if verbose:
            print(itPat, norm_rP, nit)
        if norm_rP < tol_Pat and itPat >= itmin_Pat:
            if target_rel_residual > 0 and s.residual(U, P) > target_rel_residual:
                tol_Pat *= 0.1
                rtol_U *= 0.1
                tol_U_restart = rtol_U * tol_Pat
                Rhs = (s.Fb + s.GG @ P - s.bc_rhs)[ifree]
                U[ifree], nit, _ = s.mg.solve(Rhs, U[ifree], tol=tol_U_restart, itmax=itmax_U)
                info['nitU'] += nit
                r = rm0space(-(s.GG.T @ U))
                norm_rP = normdf(r)
                restart = True
                continue
            break
        if norm_rP < rtol_restart * norm_rP0 or norm_rP > 10 * norm_rP0:
            Rhs = (s.Fb + s.GG @ P - s.bc_rhs)[ifree]
            U[ifree], nit, _ = s.mg.solve(Rhs, U[ifree], tol=tol_U_restart, itmax=itmax_U)
            info['nitU'] += nit
            r = -(s.GG.T @ U)
            norm_rP_true = normdf(r)
            if norm_rP_true > 1.1 * norm_rP:
                rtol_U = rtol_U * 0.75 * (norm_rP / norm_rP_true)
                tol_U_restart = rtol_U * tol_Pat
            if norm_rP > 10 * norm_rP0 or norm_rP > 1.2 * norm_rP_min:
                if conv_problem:
                    break
                rtol_U = 0.1 * rtol_U
                tol_U_restart = rtol_U * tol_Pat
                conv_problem = True
            restart = True
    Rhs = (s.Fb + s.GG @ P - s.bc_rhs)[ifree]
    U[ifree], nit, _ = s.mg.solve(Rhs, U[ifree], tol=tol_U_restart, itmax=itmax_U)
    info['nitU'] += nit
    info['itPat'] = itPat
    info['norm_rP'] = norm_rP
    return U, P, info


def calculate_dt(GCOORD, Ux, Uy, Uz, dt_adv_limit, dtmax):
    """CFL time step (calculate_dt.m:40-52): dt_adv = dt_adv_limit * min(Lx/max|Ux|, Ly/max|Uy|,
    Lz/max|Uz|) with Lx = max(x) - min(x) of the mesh (init_mesh_curved_p.m:264-272), dt = min(dtmax,
    dt_adv); an all-zero velocity gives (dtmax, 0). Returns (dt, dt_adv)."""
    mx = [float(np.max(np.abs(u))) for u in (Ux, Uy, Uz)]
    if mx[0] == 0 and mx[1] == 0 and mx[2] == 0:
        return float(dtmax), 0.0
    Lxyz = GCOORD.max(axis=1) - GCOORD.min(axis=1)
    with np.errstate(divide='ignore'):
        adv = dt_adv_limit * min(float(np.float64(Lxyz[k]) / np.float64(mx[k])) for k in range(3))
    return min(float(dtmax), adv), adv


ROCK_R = 8.314472            # J/(mol K), rock_prop.m


def rock_prop(T, GCOORD, Visc0, Dens0, T_ref, alpha, Ea, Va, g, L0, a_UM2LM=0.0, minDens=None, maxDens=None,
              minVisc=None, maxVisc=None):
    """Nodal density and viscosity from temperature (rock_prop.m:5-66): thermal expansion about
    T_ref with cut-offs; Arrhenius factor exp(Ea/(R T0_K) (T0_K/T_K - 1)) clamped to [1e-8, 1e8];
    activation-volume factor exp(P Va / (R T0_K)) with lithostatic P = |g Dens0 L0 depth|, depth
    below the outermost node; the lower-mantle factor a_UM2LM; their minimum (so the two do not
    compound) times Visc0, with cut-offs. Returns (Visc, Dens)."""
    T = np.asarray(T, dtype=np.float64)
    radius = np.sqrt((GCOORD ** 2).sum(0))
    depth = radius.max() - radius
    Dens = Dens0 * (1 - alpha * (T - T_ref))
    if maxDens is not None:
        Dens = np.minimum(Dens, maxDens)
    if minDens is not None:
        Dens = np.maximum(Dens, minDens)
    v = np.ones_like(T)
    T0_K = T_ref + 273
    if Ea > 0:
        if Ea < 1000:
            raise ValueError(" Activation energy PHYSICS.Ea seems to be in kJ/mol. Convert to J/mol.")
        T_K = T + 273
        eta = Ea / (ROCK_R * T0_K)
        v = v * np.exp(eta * ((T0_K / T_K) - 1))
        v = np.minimum(v, 1e8)
        v = np.maximum(v, 1e-8)
    v2 = v.copy()
    if Va > 0:
        P = np.abs(g * Dens0 * L0 * depth)
        v2 = v2 * np.exp(P * Va / (ROCK_R * T0_K))
    v3 = v.copy()
    if a_UM2LM > 0:
        v3 = v3 * a_UM2LM
    Visc = np.minimum(v2, v3) * Visc0
    if maxVisc is not None:
        Visc = np.minimum(Visc, maxVisc)
    if minVisc is not None:
        Visc = np.maximum(Visc, minVisc)
    return Visc, Dens
