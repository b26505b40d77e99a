"""Seeded synthetic spherical-shell workloads (mesh, fields, boundary conditions).

The reference's GPlates plate-velocity files are not shipped, so plates are seeded
spherical-Voronoi caps with random Euler poles. Units follow the reference's 'mantle' scaling
(mfiles_M3TET/numerical_eq_scaling.m: L0 = 1 km, t0 = 1 Myr, Visc0 = 2e18 Pa s, Dens0 = 3300).

* ``shell_c1``: level-3 icosahedral surface, 8 layers, 3 MG levels; isoviscous 1e21 Pa s;
  T = linear conductive profile + 0.05 Re Y_4^3 + U(-1e-3, 1e-3); free slip at both boundaries
  with the rigid-rotation pins of the reference's commented-out recipe (SETUP_TEST/bc_sph.m:569-594).
* ``shell_c2``: level-5 surface, 32 layers, 4 MG levels (coarsest 17,334 DOF); eta = eta0 exp(-gamma T)
  (contrast 1e4) x 30 below 660 km depth; 12 seeded plate caps (|v| <= 10 cm/yr) at the surface,
  free slip at the CMB.
* ``shell_c5``: level-6 surface, 64 layers, 5 MG levels (coarsest 17,334 DOF), contrast 1e6.
"""
from __future__ import annotations

import numpy as np

from . import mesh as M

MYR = 1e6 * 365.25 * 24 * 3600.0
SCALE = dict(L0=1000.0, t0=MYR, Visc0=2e18, Dens0=3300.0)
SCALE['U0'] = SCALE['L0'] / SCALE['t0']
SCALE['Bscale'] = SCALE['L0'] ** 2 / (SCALE['Visc0'] * SCALE['U0'])
R_CMB, R_SURF = 3480.0, 6371.0
ALPHA, DT_K = 3e-5, 2500.0
# thermal diffusivity 1e-6 m^2/s in km^2/Myr (model_parameters_sph_south_atlantic_plume.m:483-487)
KAPPA = 1e-6 / (SCALE['L0'] ** 2 / SCALE['t0'])


def physics():
    return dict(g=-9.81, Bscale=SCALE['Bscale'], Dens0=SCALE['Dens0'], minVisc=None, maxVisc=None)


def temperature(levels, seed):
    """Nodal T on the finest level: conductive profile + 0.05 Re Y_4^3 + U(-1e-3,1e-3)."""
    f = levels[0]
    S = M.cart2sph(f['GCOORD'])
    th, ph, r = S
    xi = np.clip((r - R_CMB) / (R_SURF - R_CMB), 0.0, 1.0)
    y43 = np.sin(th) ** 3 * np.cos(th) * np.cos(3 * ph)
    y43 /= np.abs(y43).max() if np.abs(y43).max() > 0 else 1.0
    rng = np.random.default_rng(seed + 101)
    T = (1.0 - xi) + 0.05 * y43 * np.sin(np.pi * xi) + rng.uniform(-1e-3, 1e-3, size=xi.shape)
    pid = f['PointID']
    T[pid == M.PID_CMB] = 1.0
    T[pid == M.PID_SURF] = 0.0
    return T


def density(T):
    return SCALE['Dens0'] * (1.0 - ALPHA * DT_K * (T - 0.5))


def free_slip_dofs(f, which=(M.PID_CMB, M.PID_SURF)):
    pid = f['PointID']
    nodes = np.nonzero(np.isin(pid, which))[0]
    return 3 * nodes + 2


def rigid_rotation_pins(f):
    """theta,phi dofs of a north-pole surface node and the phi dof of an equator node at
    phi ~ 180-195 deg (bc_sph.m:569-594). Falls back to the nearest surface node."""
    S = np.rad2deg(M.cart2sph(f['GCOORD']))
    surf = np.nonzero(f['PointID'] == M.PID_SURF)[0]
    n1 = surf[S[0, surf] < 5]
    n1 = n1[0] if len(n1) else surf[np.argmin(S[0, surf])]
    sel = surf[(S[0, surf] > 85) & (S[0, surf] < 95) & (S[1, surf] > 185) & (S[1, surf] < 195)]
    if len(sel):
        n2 = sel[0]
    else:
        d = (S[0, surf] - 90) ** 2 + (S[1, surf] - 190) ** 2
        n2 = surf[np.argmin(d)]
    return np.array([3 * n1, 3 * n1 + 1, 3 * n2 + 1])


def plate_velocities(f, nplates, vmax_cm_yr, seed):
    """Surface-node (v_theta, v_phi) from seeded spherical-Voronoi caps with Euler poles."""
    rng = np.random.default_rng(seed + 7)
    X = f['GCOORD']
    surf = np.nonzero(f['PointID'] == M.PID_SURF)[0]
    c = rng.normal(size=(nplates, 3))
    c /= np.linalg.norm(c, axis=1, keepdims=True)
    xs = X[:, surf].T
    xn = xs / np.linalg.norm(xs, axis=1, keepdims=True)
    plate = np.argmax(xn @ c.T, axis=1)
    poles = rng.normal(size=(nplates, 3))
    poles /= np.linalg.norm(poles, axis=1, keepdims=True)
    speed = rng.uniform(0.3, 1.0, size=nplates) * vmax_cm_yr
    vmax_units = 1e-2 * 1e6 / SCALE['L0']                   # 1 cm/yr in L0 per Myr
    omega = poles * (speed * vmax_units / R_SURF)[:, None]   # |omega x r| <= speed
    v = np.cross(omega[plate], xs)
    R = M.rotation_blocks(X[:, surf])
    vl = np.einsum('nji,nj->ni', R, v)                        # local (theta, phi, r)
    return surf, vl


def boundary_conditions(f, kind, seed=0):
    """(ifix, vfix), 0-based rotated-frame dofs, sorted and unique."""
    if kind == 'free_slip':
        ifix = np.concatenate([free_slip_dofs(f), rigid_rotation_pins(f)])
        vfix = np.zeros(len(ifix))
    elif kind == 'plates':
        surf, vl = plate_velocities(f, 12, 10.0, seed)
        cmb = free_slip_dofs(f, (M.PID_CMB,))
        ifix = np.concatenate([cmb, 3 * surf, 3 * surf + 1, 3 * surf + 2])
        vfix = np.concatenate([np.zeros(len(cmb)), vl[:, 0], vl[:, 1], np.zeros(len(surf))])
    elif kind == 'no_slip':
        nodes = np.nonzero(f['PointID'] > 0)[0]
        ifix = np.concatenate([3 * nodes, 3 * nodes + 1, 3 * nodes + 2])
        vfix = np.zeros(len(ifix))
    else:
        raise ValueError(kind)
    order = np.argsort(ifix, kind='stable')
    ifix, vfix = ifix[order], vfix[order]
    keep = np.concatenate([[True], np.diff(ifix) != 0])
    return ifix[keep].astype(np.int64), vfix[keep]


def viscosity(levels, T, contrast, jump=30.0):
    f = levels[0]
    r = M.cart2sph(f['GCOORD'])[2]
    eta0 = 1e21 / SCALE['Visc0']
    if contrast <= 1.0:
        eta = np.full(len(T), eta0)
    else:
        gamma = np.log(contrast)
        eta = eta0 * np.exp(-gamma * (T - 0.5))
    if jump and jump != 1.0:
        eta = np.where(r < R_SURF - 660.0, eta * jump, eta)
    return eta


def make_workload(name, seed=0, nmg=None, level=None, nlayer=None):
    """Returns dict(levels, visc, dens, T, ifix, vfix, phys, name)."""
    if name == 'c1':
        L, n, g, contrast, jump, bc = 3, 8, 3, 1.0, 1.0, 'free_slip'
    elif name == 'c2':
        L, n, g, contrast, jump, bc = 5, 32, 4, 1e4, 30.0, 'plates'
    elif name == 'c5':
        L, n, g, contrast, jump, bc = 6, 64, 5, 1e6, 30.0, 'plates'
    elif name == 'mid':
        # 1/8 of the 8M-DOF shell (level 4, 16 layers): the profiling case (> L2, a few GB on device)
        L, n, g, contrast, jump, bc = 4, 16, 4, 1e4, 30.0, 'plates'
    elif name == 'prof':
        # profiler case: 491,520 elements (about 12k per colour), ~4.5 GB on the device
        L, n, g, contrast, jump, bc = 5, 8, 4, 1e4, 30.0, 'plates'
    elif name == 'tiny':
        L, n, g, contrast, jump, bc = 2, 4, 2, 1.0, 1.0, 'free_slip'
    elif name == 'tiny_plates':
        L, n, g, contrast, jump, bc = 2, 4, 2, 1e2, 30.0, 'plates'
    else:
        raise ValueError(name)
    L = level if level is not None else L
    n = nlayer if nlayer is not None else n
    g = nmg if nmg is not None else g
    levels = M.build_hierarchy(L, n, g, R_CMB, R_SURF, seed=seed)
    T = temperature(levels, seed)
    visc = viscosity(levels, T, contrast, jump)
    dens = density(T)
    ifix, vfix = boundary_conditions(levels[0], bc, seed)
    return dict(name=name, levels=levels, visc=visc, dens=dens, T=T, ifix=ifix, vfix=vfix, phys=physics(),
                level=L, nlayer=n, nmg=g, contrast=contrast)


def rock_params(contrast=1e6):
    """rock_prop parameters (rock_prop.m) for temperatures in degC (T_C = DT_K * T): Arrhenius law
    about 1250 degC, an activation volume whose factor reaches a_UM2LM = 30 at 660 km depth (the
    upper/lower-mantle jump), and viscosity cut-offs giving the requested contrast around 1e21 Pa s."""
    eta0 = 1e21 / SCALE['Visc0']
    T0_K = 1250.0 + 273.0
    P660 = 9.81 * SCALE['Dens0'] * SCALE['L0'] * 660.0
    return dict(Visc0=eta0, Dens0=SCALE['Dens0'], T_ref=1250.0, alpha=ALPHA, Ea=250e3,
                Va=np.log(30.0) * 8.314472 * T0_K / P660, g=-9.81, L0=SCALE['L0'], a_UM2LM=30.0,
                minVisc=eta0 / np.sqrt(contrast), maxVisc=eta0 * np.sqrt(contrast))
