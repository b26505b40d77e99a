"""Host-side mirror of the reference Stokes interface over the C ABI.

``flow3d_patera_sph(VAR, MESH, COMM, UBC, SETTINGS, PHYSICS, NUMSCALE, dt)`` keeps the reference's
signature (mfiles_M3TET/flow3d_patera_sph.m:1-8) and returns ``(VAR, Uinfo)``; the work is done
by ``m3sph_stokes_setup`` + ``m3sph_stokes_solve`` in libm3sph.so on the GPU.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import _lib as L
from . import mesh as meshmod


class DeviceMesh:
    """Device-resident MESH + multigrid hierarchy (owns an m3sph_mesh handle)."""

    def __init__(self, levels, device=0):
        self.levels = levels
        self.nmg = len(levels)
        self._keep = []
        arr = (L.Level * self.nmg)()
        for i, lv in enumerate(levels):
            el = np.ascontiguousarray(lv['EL2NOD'].astype(np.uint32) + 1)       # 1-based, 10 x nel col-major
            self._keep.append(el)
            a = arr[i]
            a.nel = len(el)
            a.nnod = lv['GCOORD'].shape[1]
            a.nvnod = int(lv['EL2NOD'][:, :4].max()) + 1
            a.EL2NOD = L.u32ptr(el)
            if 'isplit' in lv and i > 0:
                isp = np.ascontiguousarray(lv['isplit'].astype(np.uint8) + 1)
                self._keep.append(isp)
                a.isplit = L.u8ptr(isp)
            if i == 0:
                gc = np.ascontiguousarray(lv['GCOORD'].T)                         # 3 x nnod col-major
                gs = np.ascontiguousarray(lv['GCOORD_SPH'].T)
                cl = np.ascontiguousarray(lv['cls'].astype(np.uint8))
                iso = np.ascontiguousarray(lv['els_iso'].astype(np.uint32) + 1)
                cub = np.ascontiguousarray(lv['cubic_sph_rot'].astype(np.float64))
                self._keep += [gc, gs, cl, iso, cub]
                a.GCOORD = L.dptr(gc)
                a.GCOORD_SPH = L.dptr(gs)
                a.elclass = L.u8ptr(cl)
                a.niso = len(iso)
                a.els_iso = L.u32ptr(iso) if len(iso) else None
                a.cubic_sph_rot = L.dptr(cub) if len(iso) else None
        self._arr = arr
        h = C.c_void_p()
        L.check(L.lib().m3sph_mesh_create(self.nmg, arr, device, C.byref(h)))
        self.h = h
        f = levels[0]
        self.nnod = f['GCOORD'].shape[1]
        self.ndof = 3 * self.nnod
        self.nvnod = int(f['EL2NOD'][:, :4].max()) + 1
        self.precision = None
        self.model_time = 0.0          # model time of the resident time series (set_temperature, time_step)

    def close(self):
        if getattr(self, 'h', None):
            L.lib().m3sph_mesh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def ncolors(self, img=0):
        n = C.c_int32()
        L.check(L.lib().m3sph_mesh_ncolors(self.h, img, C.byref(n)))
        return n.value

    # ---- operator set-up ----
    def setup(self, visc, dens, ifix, vfix, phys=None, precision=0):
        """ifix: 0-based dof ids in the rotated frame; vfix: prescribed values."""
        phys = phys or {}
        ph = L.Physics(g=phys.get('g', -9.81), Bscale=phys.get('Bscale', 1.0), Dens0=phys.get('Dens0', 0.0),
                       minVisc=phys.get('minVisc', 0.0) or 0.0, maxVisc=phys.get('maxVisc', 0.0) or 0.0)
        visc = np.ascontiguousarray(visc, dtype=np.float64)
        dens = np.ascontiguousarray(dens, dtype=np.float64)
        fx = np.ascontiguousarray(np.asarray(ifix, dtype=np.int32) + 1)
        vf = np.ascontiguousarray(vfix, dtype=np.float64)
        L.check(L.lib().m3sph_stokes_setup(self.h, L.dptr(visc), L.dptr(dens), L.iptr(fx), L.dptr(vf),
                                           len(fx), C.byref(ph), int(precision)))
        self.precision = precision

    def set_vel_bc(self, ifix, vfix):
        """New prescribed values on the set-up's fixed dofs (0-based, any order): update_vel_bc's
        UBC between time steps. The next operator rebuild uses them."""
        fx = np.ascontiguousarray(np.asarray(ifix, dtype=np.int32) + 1)
        vf = np.ascontiguousarray(vfix, dtype=np.float64)
        if fx.size != vf.size:
            raise ValueError('ifix and vfix differ in length')
        L.check(L.lib().m3sph_stokes_set_vel_bc(self.h, L.iptr(fx), L.dptr(vf), len(fx)))

    # ---- operators ----
    def apply(self, x):
        y = np.empty(self.ndof)
        L.check(L.lib().m3sph_stokes_apply(self.h, L.dptr(np.ascontiguousarray(x, dtype=np.float64)), L.dptr(y)))
        return y

    def grad(self, q):
        y = np.empty(self.ndof)
        L.check(L.lib().m3sph_grad_apply(self.h, L.dptr(np.ascontiguousarray(q, dtype=np.float64)), L.dptr(y)))
        return y

    def div(self, z):
        s = np.empty(self.nvnod)
        L.check(L.lib().m3sph_div_apply(self.h, L.dptr(np.ascontiguousarray(z, dtype=np.float64)), L.dptr(s)))
        return s

    def force(self):
        f = np.empty(self.ndof)
        L.check(L.lib().m3sph_force_vector(self.h, L.dptr(f)))
        return f

    def element_matrices(self):
        nel = len(self.levels[0]['EL2NOD'])
        K = np.empty((nel, 30, 30))
        G = np.empty((nel, 30, 4))
        M = np.empty((nel, 4, 4))
        L.check(L.lib().m3sph_element_matrices(self.h, L.dptr(K), L.dptr(G), L.dptr(M)))
        return K, G, M

    def level_apply(self, img, x):
        n = 3 * self.levels[img]['GCOORD'].shape[1]
        y = np.empty(n)
        L.check(L.lib().m3sph_level_apply(self.h, img, L.dptr(np.ascontiguousarray(x, dtype=np.float64)), L.dptr(y)))
        return y

    def level_apply32(self, img, x):
        """FP32 level operator (the V-cycle's); x in the level's rotated, dof-interleaved frame."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.empty_like(x)
        L.check(L.lib().m3sph_level_apply32(self.h, img, L.fptr(x), L.fptr(y)))
        return y

    def level_inverse_diag32(self, img):
        """Inverse diagonal of the FP32 level operator (0 on fixed dofs), rotated dof-interleaved."""
        d = np.empty(3 * self.levels[img]['GCOORD'].shape[1], np.float32)
        L.check(L.lib().m3sph_level_inverse_diag32(self.h, img, L.fptr(d)))
        return d

    def transfer_matrix(self, img):
        """intermesh_transfer_matrix of levels img -> img+1 as a scipy CSR matrix (scalar Ic2f)."""
        import scipy.sparse as sp
        nnz = C.c_int64()
        L.check(L.lib().m3sph_transfer_matrix(self.h, img, C.byref(nnz), None, None, None))
        r = np.empty(nnz.value, np.int32)
        c = np.empty(nnz.value, np.int32)
        v = np.empty(nnz.value)
        L.check(L.lib().m3sph_transfer_matrix(self.h, img, C.byref(nnz), L.iptr(r), L.iptr(c), L.dptr(v)))
        return sp.csr_matrix((v, (r - 1, c - 1)), shape=(self.levels[img]['GCOORD'].shape[1],
                                                          self.levels[img + 1]['GCOORD'].shape[1]))

    def prolong(self, img, xc):
        y = np.empty(3 * self.levels[img]['GCOORD'].shape[1])
        L.check(L.lib().m3sph_prolong(self.h, img, L.dptr(np.ascontiguousarray(xc, dtype=np.float64)), L.dptr(y)))
        return y

    def restrict(self, img, rf):
        y = np.empty(3 * self.levels[img + 1]['GCOORD'].shape[1])
        L.check(L.lib().m3sph_restrict(self.h, img, L.dptr(np.ascontiguousarray(rf, dtype=np.float64)), L.dptr(y)))
        return y

    def vcycle(self, r):
        d = np.empty(self.ndof)
        L.check(L.lib().m3sph_vcycle(self.h, L.dptr(np.ascontiguousarray(r, dtype=np.float64)), L.dptr(d)))
        return d

    def mgpcg(self, b, x0, tol, is_abs_tol=True, itmax=20):
        x = np.ascontiguousarray(x0, dtype=np.float64).copy()
        it = C.c_int32()
        rr = C.c_double()
        L.check(L.lib().m3sph_mgpcg(self.h, L.dptr(np.ascontiguousarray(b, dtype=np.float64)), L.dptr(x), tol,
                                    int(is_abs_tol), itmax, C.byref(it), C.byref(rr)))
        return x, it.value, rr.value

    def solve(self, P0=None, rtol_Pat=1e-4, rtol_U=5e-3, itmax_Pat=120, itmin_Pat=3, itmax_U=20,
              target_rel_residual=0.0, smoother=0, allow_not_converged=False):
        """Patera solve from host arrays. A solve that runs out of iterations above its tolerance
        raises M3SphError(ERR_NOT_CONVERGED) whose ``result`` holds (U, P, info); with
        ``allow_not_converged`` the last iterate is returned instead, with info['status'] = 4."""
        U = np.empty(self.ndof)
        P = np.zeros(self.nvnod) if P0 is None else np.ascontiguousarray(P0, dtype=np.float64).copy()
        o = L.Opts(rtol_Pat=rtol_Pat, rtol_U=rtol_U, itmax_Pat=itmax_Pat, itmin_Pat=itmin_Pat, itmax_U=itmax_U,
                   precision=int(self.precision or 0), smoother=smoother, target_rel_residual=target_rel_residual)
        info = L.Info()
        code = L.lib().m3sph_stokes_solve(self.h, L.dptr(U), L.dptr(P), C.byref(o), C.byref(info))
        return self._finish(code, (U, P, info.as_dict()), allow_not_converged)

    def step_device(self, rtol_Pat=1e-4, rtol_U=5e-3, itmax_Pat=120, itmin_Pat=3, itmax_U=20,
                    target_rel_residual=0.0, smoother=0, allow_not_converged=False):
        """Rebuild the operator from resident inputs and solve from P=0; results stay on device."""
        o = L.Opts(rtol_Pat=rtol_Pat, rtol_U=rtol_U, itmax_Pat=itmax_Pat, itmin_Pat=itmin_Pat, itmax_U=itmax_U,
                   precision=int(self.precision or 0), smoother=smoother, target_rel_residual=target_rel_residual)
        info = L.Info()
        code = L.lib().m3sph_stokes_step_device(self.h, C.byref(o), C.byref(info))
        return self._finish(code, info.as_dict(), allow_not_converged)

    @staticmethod
    def _finish(code, result, allow_not_converged):
        if code == L.ERR_NOT_CONVERGED:
            if allow_not_converged:
                return result
            err = L.M3SphError(code, L.lib().m3sph_last_error().decode())
            err.result = result
            raise err
        L.check(code)
        return result

    def solution(self):
        U = np.empty(self.ndof)
        P = np.empty(self.nvnod)
        L.check(L.lib().m3sph_solution(self.h, L.dptr(U), L.dptr(P)))
        return U, P

    def calculate_dt(self, dt_adv_limit, dtmax):
        """calculate_dt.m:40-52 on the device-resident velocity of the last solve: (dt, dt_adv)."""
        dt, adv = C.c_double(), C.c_double()
        L.check(L.lib().m3sph_calculate_dt(self.h, float(dt_adv_limit), float(dtmax), C.byref(dt), C.byref(adv)))
        return dt.value, adv.value

    def rock_prop(self, T, params):
        """rock_prop.m:5-66 on the GPU: (Visc, Dens) of nodal T; params: dict of m3sph_rock_params
        fields (a missing or None cut-off is not applied)."""
        rp = rock_params_struct(params)
        T = np.ascontiguousarray(T, dtype=np.float64)
        V, D = np.empty_like(T), np.empty_like(T)
        L.check(L.lib().m3sph_rock_prop(self.h, C.byref(rp), L.dptr(T), L.dptr(V), L.dptr(D)))
        return V, D

    def properties(self):
        """Resident (Visc, Dens), nnod each."""
        V, D = np.empty(self.nnod), np.empty(self.nnod)
        L.check(L.lib().m3sph_get_properties(self.h, L.dptr(V), L.dptr(D)))
        return V, D

    def set_pressure(self, P):
        L.check(L.lib().m3sph_set_pressure(self.h, L.dptr(np.ascontiguousarray(P, dtype=np.float64))))

    def set_temperature(self, T, time=0.0):
        L.check(L.lib().m3sph_set_temperature(self.h, L.dptr(np.ascontiguousarray(T, dtype=np.float64)), float(time)))
        self.model_time = float(time)

    def get_temperature(self):
        T = np.empty(self.nnod)
        L.check(L.lib().m3sph_get_temperature(self.h, L.dptr(T)))
        return T

    def diffusion_setup(self, kappa, ifix, vfix, theta=1.0, tol=1e-8, itmax=500, theta_cone=45.0):
        """Thermal diffusion state (diffusion3d_p's operator): ifix 0-based node ids of TBC."""
        o = L.DiffusionOpts(kappa=float(kappa), theta=float(theta), tol=float(tol), itmax=int(itmax),
                            theta_cone=float(theta_cone))
        fx = np.ascontiguousarray(np.asarray(ifix, dtype=np.int32) + 1)
        vf = np.ascontiguousarray(vfix, dtype=np.float64)
        L.check(L.lib().m3sph_diffusion_setup(self.h, C.byref(o), L.iptr(fx), L.dptr(vf), len(fx)))

    def diffusion(self, T, dt):
        """diffusion3d_p on the GPU: (T diffused over dt, CG iterations)."""
        T = np.ascontiguousarray(T, dtype=np.float64).copy()
        nit = C.c_int32()
        L.check(L.lib().m3sph_diffusion3d(self.h, L.dptr(T), float(dt), C.byref(nit)))
        return T, nit.value

    def time_step(self, stokes_kw=None, slm=None, rock=None, dt_adv_limit=0.005, dtmax=0.1, smoother=0,
                  r_cmb=3480.0, r_surf=6371.0, diffusion=False, allow_not_converged=False, vel_bcs=None):
        """One device-resident time step (rock_prop if `rock` is given -> Stokes -> calculate_dt ->
        semi-Lagrangian advection of the resident T). Returns the step info as a dict.

        ``vel_bcs`` (a ``gplates.VelBCSeries``): the surface velocities at the model time of the
        step's start are pushed first (update_vel_bc before flow3d_patera_sph,
        M3TET_SPH_SOUTH_ATLANTIC_PLUME.m:236-241); the step info then holds 'Plate' (VAR.Plate) and
        't_vel_bc_ms' (that host update)."""
        plate, t_bc = None, 0.0
        if vel_bcs is not None:
            t0 = time.perf_counter()
            _, plate = vel_bcs.apply(self, self.model_time)
            t_bc = (time.perf_counter() - t0) * 1e3
        kw = dict(rtol_Pat=1e-4, rtol_U=5e-3, itmax_Pat=120, itmin_Pat=3, itmax_U=20, target_rel_residual=0.0)
        kw.update(stokes_kw or {})
        slm = dict(slm or {})
        o = L.StepOpts()
        o.stokes = L.Opts(precision=int(self.precision or 0), smoother=smoother, **kw)
        o.slm = L.SlmOpts(method_BT=1 if slm.get('method_BT', 'PC2') == 'PC2' else 2,
                          method_interp=1 if slm.get('method_interp', 'cubic') == 'cubic' else 0,
                          monotonic=int(slm.get('monotonic', 1)),
                          method_wght=1 if slm.get('method_wght', 'dist') == 'dist' else 0, r_cmb=r_cmb, r_surf=r_surf)
        o.rock_prop = 1 if rock is not None else 0
        if rock is not None:
            o.rock = rock_params_struct(rock)
        o.dt_adv_limit = dt_adv_limit
        o.dtmax = dtmax
        o.diffusion = 1 if diffusion else 0
        info = L.StepInfo()
        code = L.lib().m3sph_time_step(self.h, C.byref(o), C.byref(info))
        d = info.as_dict()
        if code in (L.OK, L.ERR_NOT_CONVERGED):
            self.model_time = d['time']
        if plate is not None:
            d['Plate'] = plate
            d['t_vel_bc_ms'] = t_bc       # host update_vel_bc + upload, before the device step
        return self._finish(code, d, allow_not_converged)

    def set_option(self, name, value):
        L.check(L.lib().m3sph_set_option(self.h, name.encode(), int(value)))

    def apply_timing(self, img=0, precision=1, nrep=10):
        ms = C.c_double()
        L.check(L.lib().m3sph_apply_timing(self.h, img, precision, nrep, C.byref(ms)))
        return ms.value

    def stream(self):
        p = C.c_void_p()
        L.check(L.lib().m3sph_stream(self.h, C.byref(p)))
        return p.value


def flow3d_patera_sph(VAR, MESH, COMM, UBC, SETTINGS, PHYSICS, NUMSCALE, dt):
    """Mirror of flow3d_patera_sph.m:1-8 -> flow3d_patera_mg_sph_p on the GPU.

    VAR: dict with 'Visc', 'Dens' (nnod) and 'P' (nvnod); MESH: dict with 'levels' (finest first)
    and optionally a cached 'device_mesh'; UBC: dict with 'ifix' (1-based rotated-frame dofs) and
    'vfix'. Returns (VAR, Uinfo) with VAR['Ux','Uy','Uz','Uth','Uph','Ur','P'] filled.
    """
    dm = MESH.get('device_mesh')
    if dm is None:
        dm = DeviceMesh(MESH['levels'])
        MESH['device_mesh'] = dm
    prec = 1 if SETTINGS.get('mixed_precision', True) else 0
    phys = dict(g=PHYSICS.get('g', -9.81), Bscale=NUMSCALE.get('Bscale', 1.0), Dens0=NUMSCALE.get('Dens0', 0.0),
                minVisc=PHYSICS.get('minVisc'), maxVisc=PHYSICS.get('maxVisc'))
    t0 = time.perf_counter()
    dm.setup(VAR['Visc'], VAR['Dens'], np.asarray(UBC['ifix']) - 1, UBC['vfix'], phys, precision=prec)
    t1 = time.perf_counter()
    U, P, info = dm.solve(VAR.get('P'), rtol_Pat=SETTINGS.get('rtol_Pat', 1e-4), rtol_U=SETTINGS.get('rtol_U', 5e-3),
                          target_rel_residual=SETTINGS.get('target_rel_residual', 0.0))
    info['t_setup_ms'] = (t1 - t0) * 1e3
    VAR = dict(VAR)
    VAR['Ux'], VAR['Uy'], VAR['Uz'] = U[0::3].copy(), U[1::3].copy(), U[2::3].copy()
    R = meshmod.rotation_blocks(MESH['levels'][0]['GCOORD'])
    Ul = np.einsum('nji,nj->ni', R, U.reshape(-1, 3))
    VAR['Uth'], VAR['Uph'], VAR['Ur'] = Ul[:, 0].copy(), Ul[:, 1].copy(), Ul[:, 2].copy()
    VAR['P'] = P
    return VAR, info


def calculate_dt(MESH, COMM, SETTINGS, NUMSCALE, VAR):
    """Mirror of calculate_dt.m:1-62 for the velocity of the last GPU solve on MESH['device_mesh']
    (the VAR.Ux/Uy/Uz that flow3d_patera_sph returned): dt = min(dtmax, dt_adv_limit * min(L/max|U|))."""
    dt, _ = MESH['device_mesh'].calculate_dt(SETTINGS['dt_adv_limit'], SETTINGS['dtmax'])
    return dt


def rock_params_struct(p):
    """m3sph_rock_params from a dict of PHYSICS / NUMSCALE values; absent cut-offs are NaN."""
    nan = float('nan')
    g = lambda k, d=0.0: d if p.get(k) is None else float(p[k])
    return L.RockParams(Visc0=g('Visc0'), Dens0=g('Dens0'), T_ref=g('T_ref'), alpha=g('alpha'), Ea=g('Ea'),
                        Va=g('Va'), g=g('g'), L0=g('L0', 1.0), a_UM2LM=g('a_UM2LM'), minDens=g('minDens', nan),
                        maxDens=g('maxDens', nan), minVisc=g('minVisc', nan), maxVisc=g('maxVisc', nan))


def rock_prop(VAR, PHYSICS, NUMSCALE, MESH, SETTINGS=None):
    """Mirror of rock_prop.m:1 (VAR = rock_prop(VAR,PHYSICS,NUMSCALE,MESH,SETTINGS)) on the GPU:
    VAR['Visc'] and VAR['Dens'] from VAR['T']."""
    dm = MESH.get('device_mesh')
    if dm is None:
        dm = DeviceMesh(MESH['levels'])
        MESH['device_mesh'] = dm
    p = dict(Visc0=PHYSICS['Visc'], Dens0=PHYSICS['Dens'], T_ref=PHYSICS['T_ref'], alpha=PHYSICS['alpha'],
             Ea=PHYSICS['Ea'], Va=PHYSICS['Va'], g=PHYSICS['g'], L0=NUMSCALE['L0'], a_UM2LM=PHYSICS.get('a_UM2LM'),
             minDens=PHYSICS.get('minDens'), maxDens=PHYSICS.get('maxDens'), minVisc=PHYSICS.get('minVisc'),
             maxVisc=PHYSICS.get('maxVisc'))
    VAR = dict(VAR)
    VAR['Visc'], VAR['Dens'] = dm.rock_prop(VAR['T'], p)
    return VAR


def diffusion3d_p(T, kappa, MESH, COMM, SETTINGS, TBC, dt):
    """Mirror of diffusion3d_p.m:1 (T = diffusion3d_p(T,kappa,MESH,COMM,SETTINGS,TBC,dt)) on the GPU
    with the default element options; TBC: dict with 'ifix' (1-based nodes) and 'vfix'."""
    dm = MESH.get('device_mesh')
    if dm is None:
        dm = DeviceMesh(MESH['levels'])
        MESH['device_mesh'] = dm
    D = (SETTINGS or {}).get('OPTS_D', {})
    dm.diffusion_setup(kappa, np.asarray(TBC['ifix']) - 1, TBC['vfix'], theta=D.get('theta', 1.0),
                       tol=D.get('tol', 1e-8), itmax=D.get('itmax', 500))
    return dm.diffusion(T, dt)[0]
