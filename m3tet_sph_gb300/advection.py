"""Host-side mirror of the reference's semi-Lagrangian interface over the C ABI.

``advect3d_slm_p_sph(MESH, COMM, Ux, Uy, Uz, T, dt, OPTS_SLM, WS_SLM)`` keeps the reference's
signature (mfiles_SPH/advect3d_slm_p_sph.m:1) and returns ``(T, WS_SLM)``; ``tsearch2_sph``,
``interp3d_tet`` and ``interp3d_cubic_p`` mirror the location / interpolation helpers. Element
ids are 1-based (0 = not found) as on the MATLAB side.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


def _dm(MESH):
    from .stokes import DeviceMesh
    dm = MESH.get('device_mesh')
    if dm is None:
        dm = DeviceMesh(MESH['levels'])
        MESH['device_mesh'] = dm
    return dm


def tsearch2_sph(dm, gTH_PT, els_guess=None):
    """Locate points (3,npt) given in (theta,phi,r): returns (els 1-based, lc (3,npt), info)."""
    P = np.ascontiguousarray(np.asarray(gTH_PT, dtype=np.float64).T)
    npt = P.shape[0]
    els = np.zeros(npt, np.int32)
    lc = np.zeros((npt, 3))
    info = L.LocateInfo()
    g = None if els_guess is None else np.ascontiguousarray(els_guess, dtype=np.int32)
    L.check(L.lib().m3sph_tsearch_sph(dm.h, L.dptr(P), npt, L.iptr(g) if g is not None else None, L.iptr(els),
                                       L.dptr(lc), C.byref(info)))
    return els, lc.T.copy(), info.as_dict()


def locate_timing(dm, gTH_PT, nrep=5):
    """Device-resident location of points (3,npt) in (theta,phi,r), timed with CUDA events after one
    upload (m3sph_locate_timing): (ms per location, info of the last one)."""
    P = np.ascontiguousarray(np.asarray(gTH_PT, dtype=np.float64).T)
    ms = C.c_double()
    info = L.LocateInfo()
    L.check(L.lib().m3sph_locate_timing(dm.h, L.dptr(P), P.shape[0], int(nrep), C.byref(ms), C.byref(info)))
    return ms.value, info.as_dict()


def interp3d_tet(dm, els, lc, V, monotonic=False):
    V = np.asarray(V, dtype=np.float64)
    V2 = V[:, None] if V.ndim == 1 else V
    npt = len(els)
    out = np.zeros((npt, V2.shape[1]))
    L.check(L.lib().m3sph_interp3d_tet(dm.h, L.iptr(np.ascontiguousarray(els, dtype=np.int32)),
                                        L.dptr(np.ascontiguousarray(np.asarray(lc).T)), npt,
                                        L.dptr(np.ascontiguousarray(V2)), V2.shape[1], int(monotonic), L.dptr(out)))
    return out[:, 0] if V.ndim == 1 else out


def interp3d_cubic_p(dm, els, lc, V, monotonic=True, method_wght='dist'):
    npt = len(els)
    out = np.zeros(npt)
    L.check(L.lib().m3sph_interp3d_cubic(dm.h, L.iptr(np.ascontiguousarray(els, dtype=np.int32)),
                                          L.dptr(np.ascontiguousarray(np.asarray(lc).T)), npt,
                                          L.dptr(np.ascontiguousarray(V, dtype=np.float64)), int(monotonic),
                                          1 if method_wght == 'dist' else 0, L.dptr(out)))
    return out


def advect3d_slm_p_sph(MESH, COMM, Ux, Uy, Uz, T, dt, OPTS_SLM=None, WS_SLM=None):
    """Mirror of advect3d_slm_p_sph.m: PC2 backtracking, locate, interpolate T at departure points."""
    OPTS_SLM = OPTS_SLM or {}
    WS_SLM = dict(WS_SLM or {})
    dm = _dm(MESH)
    n = dm.nnod
    bt = OPTS_SLM.get('method_BT', 'PC2')
    if bt not in ('PC2', 'RK4'):
        raise NotImplementedError("method_BT must be 'PC2' or 'RK4' (3 substeps)")
    o = L.SlmOpts(method_BT=1 if bt == 'PC2' else 2, method_interp=1 if OPTS_SLM.get('method_interp', 'quadratic') == 'cubic' else 0,
                  monotonic=int(OPTS_SLM.get('monotonic', 1)),
                  method_wght=1 if OPTS_SLM.get('method_wght', 'dist') == 'dist' else 0,
                  r_cmb=MESH.get('r_cmb', 3480.0), r_surf=MESH.get('r_surf', 6371.0))
    Tn = np.ascontiguousarray(T, dtype=np.float64).copy()
    elsBT = np.ascontiguousarray(WS_SLM.get('els_BT', np.zeros(n, np.int32)), dtype=np.int32).copy()
    elsIN = np.zeros(n, np.int32)
    info = L.LocateInfo()
    L.check(L.lib().m3sph_advect_slm(dm.h, L.dptr(np.ascontiguousarray(Ux, dtype=np.float64)),
                                      L.dptr(np.ascontiguousarray(Uy, dtype=np.float64)),
                                      L.dptr(np.ascontiguousarray(Uz, dtype=np.float64)), L.dptr(Tn), float(dt),
                                      C.byref(o), L.iptr(elsBT), L.iptr(elsIN), C.byref(info)))
    WS_SLM['els_BT'] = elsBT
    WS_SLM['els_INTERP'] = elsIN
    WS_SLM['locate_info'] = info.as_dict()
    return Tn, WS_SLM
