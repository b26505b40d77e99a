"""ORACLE (test infrastructure only): CPU FP64 restatement of the thermal-diffusion half step.

Checker for the CUDA diffusion kernels and the CPU side of their timing. Only tests,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU leg use it.

Restated reference behaviour (paths inside the reference project), for the default options
(mfiles_M3TET/default_numerics_M3TET.m:94-121: eltype 'linear', lumping 'yes', nip 4, theta 1,
solver 'pcg', pc 'diag', tol 1e-8 relative, itmax 500):
* mfiles_M3TET/diffusion3d_p.m:1-121: the P2 mesh is split into 4-node tetrahedra (tetmesh_p2_to_p1),
  capacity lumped to its row sums, rhs = M T - dt (1 - theta) C T, A = dt theta C + M, prescribed
  temperatures moved to the rhs, A(ifree, ifree) T(ifree) = rhs(ifree) solved by PCG from T(ifree);
* mfiles_SPH/assembly_diffusion_3d_double_jacobian.m:78-200: the split elements are classified
  again (check_els_in_cone.m, check_phi.m) and integrated class by class;
* mfiles_SPH/assembly_diffusion_els_*_opt.m: per element and integration point the double
  Jacobian -- J_SL from the 4 vertices' (theta, phi, r) in the element's frame (original; phi + pi
  for elements crossing phi = 2 pi; the X-90-rotated frame for elements in the cone), J_CS at the
  point, detJ_CS = r^2 sin(theta) -- giving C_ij = sum kappa w grad Ni . grad Nj and
  M_ij = sum w Ni Nj;
* mfiles_M3TET/pcg_solver_p.m: Jacobi-preconditioned Polak-Ribiere CG, tolerance relative to the
  initial residual's normdf, stop when normdf(r) < tol.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

RX90 = np.array([[1.0, 0, 0], [0, 0, -1.0], [0, 1.0, 0]])
_A = (5 + 3 * np.sqrt(5)) / 20
_B = (5 - np.sqrt(5)) / 20
IPX = np.array([[_A, _B, _B, _B], [_B, _A, _B, _B], [_B, _B, _A, _B]])   # ip_tetrahedron.m, nip = 4
IPW = np.full(4, 0.25)
DN4 = np.array([[1.0, 0, 0], [0, 1.0, 0], [0, 0, 1.0], [-1.0, -1.0, -1.0]])   # sf_dsf_tet4


def cart2sph(X):
    x, y, z = X
    r = np.sqrt(x * x + y * y + z * z)
    th = np.arctan2(np.sqrt(x * x + y * y), z)
    ph = np.arctan2(y, x)
    ph = np.where(ph < 0, ph + 2 * np.pi, ph)
    return np.array([th, ph, r])


def classes(GCOORD_SPH, EL1, theta_cone=45.0):
    """Classes of 4-node elements (check_els_in_cone.m, check_phi.m): 0 outside the cone and not
    crossing phi = 2 pi, 1 outside and crossing, 2 in the cone with 3-4 vertices inside, 3 in the
    cone with 1-2 vertices inside."""
    tc = np.deg2rad(theta_cone)
    th = GCOORD_SPH[0][EL1]
    nin = ((th <= tc) | (th >= np.pi - tc)).sum(1)
    ph = GCOORD_SPH[1][EL1]
    cross = np.zeros(len(EL1), bool)
    for a, b in ((0, 1), (1, 2), (2, 0), (0, 3), (1, 3), (2, 3)):
        cross |= np.abs(ph[:, a] - ph[:, b]) > np.pi
    cls = np.where(nin == 0, np.where(cross, 1, 0), np.where(nin < 3, 3, 2))
    return cls.astype(np.uint8)


def frame_coords(GCOORD, GCOORD_SPH, EL1, cls):
    """(nsub,3,4) vertex (theta, phi, r) in each element's frame."""
    VC = GCOORD_SPH[:, EL1].transpose(1, 0, 2).copy()
    c1 = cls == 1
    ph = VC[c1, 1, :] + np.pi
    VC[c1, 1, :] = np.where(ph > 2 * np.pi, ph - 2 * np.pi, ph)
    c23 = cls >= 2
    if c23.any():
        VC[c23] = cart2sph(RX90 @ GCOORD[:, EL1[c23].ravel()]).reshape(3, -1, 4).transpose(1, 0, 2)
    return VC


def element_matrices(GCOORD, GCOORD_SPH, EL1, kappa, cls=None):
    """Conductivity C (nsub,4,4) and consistent capacity M (nsub,4,4) of the 4-node elements."""
    if cls is None:
        cls = classes(GCOORD_SPH, EL1)
    VC = frame_coords(GCOORD, GCOORD_SPH, EL1, cls)
    n = len(EL1)
    J_SL = np.einsum('eki,ij->ejk', VC, DN4)           # (n, loc, sph)
    detSL = np.linalg.det(J_SL)
    if np.any(detSL < 0):
        raise ValueError('negative Jacobi')
    J_LS = np.linalg.inv(J_SL)
    C = np.zeros((n, 4, 4))
    M = np.zeros((n, 4, 4))
    for ip in range(4):
        r_, s_, t_ = IPX[:, ip]
        N = np.array([r_, s_, t_, 1 - r_ - s_ - t_])
        th, ph, rr = np.einsum('eki,i->ke', VC, N)
        st, ct, sp_, cp = np.sin(th), np.cos(th), np.sin(ph), np.cos(ph)
        detCS = rr ** 2 * st
        J_SC = np.zeros((n, 3, 3))
        J_SC[:, 0] = np.stack([rr * st * ct * cp, -rr * sp_, rr ** 2 * st ** 2 * cp], 1) / detCS[:, None]
        J_SC[:, 1] = np.stack([rr * st * ct * sp_, rr * cp, rr ** 2 * st ** 2 * sp_], 1) / detCS[:, None]
        J_SC[:, 2] = np.stack([-rr * st ** 2, np.zeros(n), rr ** 2 * st * ct], 1) / detCS[:, None]
        Jdbl = J_SC @ J_LS                                # d loc_j / d cart_k
        dNdx = np.einsum('ekj,nj->enk', Jdbl, DN4)        # (n,4,3)
        w = detCS * detSL * IPW[ip]
        C += kappa * w[:, None, None] * np.einsum('eik,ejk->eij', dNdx, dNdx)
        M += w[:, None, None] * np.outer(N, N)[None]
    return C, M


def assemble(EL1, E, nnod):
    i = np.repeat(EL1, 4, axis=1).ravel()
    j = np.tile(EL1, (1, 4)).ravel()
    return sp.csr_matrix((E.reshape(len(EL1), 16).ravel(), (i, j)), shape=(nnod, nnod))


def pcg_diag(A, b, x, tol=1e-8, itmax=500):
    """pcg_solver_p with pc 'diag' and a relative tolerance: returns (x, iterations)."""
    ADi = 1.0 / A.diagonal()
    r = b - A @ x
    normdf = lambda v: np.linalg.norm(v) / np.sqrt(len(v))
    tol = tol * normdf(r)
    if normdf(r) < tol or normdf(r) == 0.0:
        # zero initial residual: converged (pcg_solver_p.m would go on to alpha = 0/0)
        return x, 0
    rd = q = rlast = None
    it = 0
    for it in range(1, itmax + 1):
        d = r * ADi
        if it == 1:
            q = d
        else:
            rdlast = rd
            beta = np.dot(r - rlast, d) / rdlast
            q = d + beta * q
        rd = np.dot(r, d)
        Aq = A @ q
        alpha = rd / np.dot(q, Aq)
        rlast = r
        x = x + alpha * q
        r = r - alpha * Aq
        if normdf(r) < tol:
            break
    return x, it


class Diffusion:
    """diffusion3d_p(T, kappa, MESH, COMM, SETTINGS, TBC, dt) with the default options, on the
    4-node split EL1 (nsub,4) of the P2 mesh."""

    def __init__(self, GCOORD, GCOORD_SPH, EL1, kappa, ifix, theta=1.0):
        nnod = GCOORD.shape[1]
        C, M = element_matrices(GCOORD, GCOORD_SPH, EL1, kappa)
        self.C = assemble(EL1, C, nnod)
        self.ML = np.asarray(assemble(EL1, M, nnod).sum(axis=1)).ravel()   # lumping 'yes'
        self.theta = theta
        self.ifix = np.asarray(ifix, dtype=np.int64)
        free = np.ones(nnod, bool)
        free[self.ifix] = False
        self.ifree = np.nonzero(free)[0]

    def step(self, T, dt, vfix, tol=1e-8, itmax=500):
        T = np.asarray(T, dtype=np.float64).copy()
        rhs = self.ML * T - dt * (1 - self.theta) * (self.C @ T)
        A = (dt * self.theta * self.C + sp.diags(self.ML)).tocsr()
        T[self.ifix] = vfix
        rhs = rhs - A[:, self.ifix] @ np.asarray(vfix, dtype=np.float64)
        Aff = A[self.ifree][:, self.ifree].tocsr()
        T[self.ifree], nit = pcg_diag(Aff, rhs[self.ifree], T[self.ifree], tol, itmax)
        return T, nit
