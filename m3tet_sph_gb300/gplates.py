"""GPlates plate-velocity boundary conditions: the files and ``update_vel_bc``.

* ``read_vel_gplates`` reads one GPlates velocity export (readVelGPlates.m:41-110): five columns
  per surface point (lat, lon, plate id, v_colat, v_lon in cm/yr); points GPlates left without a
  plate (id 0) take the id of the neighbouring record; ids become indices into the plate table of
  readVelGPlates.m:74-75 and velocities mm/yr (= km/Myr, the model's velocity unit).
* ``save_vel_bcs`` / ``load_vel_bcs`` write and read the MAT file that
  PREPROC/SAVE_GPLATES_VEL_BCS_TO_MAT_FILE.m:56-87 makes from a folder of those exports: the struct
  array ``V_BCs`` (time, Uth_Uph, latlon, PlateID, plateid2name) and ``time_VBCs_files``, one file per
  Myr, oldest first.
* ``update_vel_bc`` (mfiles_SPH/update_vel_bc.m:22-150): the velocities at the model time, linearly
  interpolated between the two bracketing files, rotated from the GPlates (Earth) frame into the
  mesh frame by (RR2 RR1)^T, and the UBC lists: free slip (r dof) on the core-mantle boundary (301),
  prescribed (theta, phi) and zero r on the surface (306), in ascending node order; plus the plume
  BCs carried in UBC['PLUME']. As in the reference, the (theta, phi) components are taken in the
  frame of the rotated GPlates point; at a node on the polar axis that frame's phi follows the
  rounding of the rotated position, so only the tangential speed is well defined there.
* ``VelBCSeries`` holds a loaded series for a time loop and pushes each step's values to a
  ``stokes.DeviceMesh`` (``m3sph_stokes_set_vel_bc``) before ``m3sph_time_step``, as the reference
  loop calls update_vel_bc before flow3d_patera_sph (M3TET_SPH_SOUTH_ATLANTIC_PLUME.m:236-241).
* ``synthetic_vel_bcs`` makes a seeded stand-in series in the same format on a mesh's surface nodes
  (the reference's own GPlates exports are not distributed with it).

All of this is host bookkeeping on O(surface nodes) data once per step, as in the reference; the
solve consumes the result on the device.
"""
from __future__ import annotations

import warnings
from pathlib import Path

import numpy as np
import scipy.io as sio

from . import mesh as meshmod

# plate ids and abbreviations that GPlates assigns for 130-100 Ma in the Caltech global
# reconstruction (readVelGPlates.m:74-75); a record's plate index is its 1-based row here
PLATE_IDS = np.array([101, 103, 119, 201, 301, 304, 409, 607, 701, 702, 801, 901, 902, 919, 926])
PLATE_NAMES = ('NAM', 'NSL', 'AAB', 'SAM', 'EUR', 'SPN', 'NES', 'BMP', 'AFR', 'MAD', 'AUS', 'PAC', 'FAR',
               'PHX', 'IZA')
PID_CMB, PID_SURF = meshmod.PID_CMB, meshmod.PID_SURF


def plateid2name():
    return [dict(plate_id=int(p), index=i + 1, plate_abr=n) for i, (p, n) in enumerate(zip(PLATE_IDS, PLATE_NAMES))]


def parse_vel_gplates(text):
    """readVelGPlates.m:41-110 on the text of one export. Returns (Ucolat_Ulon (2,n) mm/yr,
    LatLon (2,n) degrees, PlateID (n,) 1-based plate indices, plateid2name)."""
    tmp = np.array(text.split(), dtype=np.float64)
    if tmp.size % 5:
        raise ValueError('GPlates velocity file: the number of values is not a multiple of 5')
    tmp = tmp.reshape(-1, 5)
    LatLon = tmp[:, 0:2]
    PlateID = tmp[:, 2].copy()
    Ucolat_Ulon = tmp[:, 3:5]
    # a point on a plate boundary has id 0: take the previous record's id, else the next one's
    for i in np.nonzero(PlateID == 0)[0]:
        if i == 0 or i == PlateID.size - 1:
            raise ValueError(f'GPlates velocity file: record {i + 1} (first or last) has no plate id')
        nb = [PlateID[j] for j in (i - 1, i + 1) if PlateID[j] != 0]
        if not nb:
            raise ValueError(f'GPlates velocity file: record {i + 1} and its neighbours have no plate id')
        PlateID[i] = nb[0]
    plates = np.unique(PlateID)
    if not np.all(np.isin(plates, PLATE_IDS)):
        raise ValueError('"plate_ids" and "plate_names" need to be updated with "PlateID"')
    index = np.searchsorted(PLATE_IDS, PlateID.astype(np.int64)) + 1
    return Ucolat_Ulon.T * 10.0, LatLon.T.copy(), index.astype(np.float64), plateid2name()


def read_vel_gplates(path):
    return parse_vel_gplates(Path(path).read_text())


def write_vel_gplates(path, LatLon, PlateID, Ucolat_Ulon_cm_yr):
    """One export in GPlates' five-column layout (lat lon plate_id v_colat v_lon, cm/yr);
    PlateID holds GPlates plate ids (0: no plate)."""
    rows = np.column_stack([LatLon[0], LatLon[1], PlateID, Ucolat_Ulon_cm_yr[0], Ucolat_Ulon_cm_yr[1]])
    with open(path, 'w') as f:
        for r in rows:
            f.write(f'{r[0]:.10f} {r[1]:.10f} {int(r[2]):d} {r[3]:.10f} {r[4]:.10f}\n')


def read_vel_gplates_folder(folder):
    """SAVE_GPLATES_VEL_BCS_TO_MAT_FILE.m:51-81: every ``<t>Ma.txt`` of a folder (or ``<t>Ma.xy``, the
    extension GPlates writes, which the reference renames to .txt first), 1-Myr apart, starting from
    the time in the last file name (three digits) and going down. Returns (V_BCs list of dicts,
    time_VBCs_files)."""
    ext = '.txt'
    files = sorted(Path(folder).glob('*.txt'), key=lambda p: p.name)
    if not files:
        ext = '.xy'
        files = sorted(Path(folder).glob('*.xy'), key=lambda p: p.name)
    if not files:
        raise ValueError('no GPlates velocity files (.txt or .xy) in the folder')
    t = float(files[-1].name[:3])
    V_BCs, times = [], []
    for _ in files:
        U, ll, pid, names = read_vel_gplates(Path(folder) / f'{int(t)}Ma{ext}')
        V_BCs.append(dict(time=t, Uth_Uph=U, latlon=ll, PlateID=pid, plateid2name=names))
        times.append(t)
        t -= 1.0
    return V_BCs, np.array(times)


def save_vel_bcs(path, V_BCs, time_VBCs_files):
    """The MAT file of SAVE_GPLATES_VEL_BCS_TO_MAT_FILE.m:87 (V_BCs, time_VBCs_files)."""
    ndt = np.dtype([('plate_id', object), ('index', object), ('plate_abr', object)])
    dt = np.dtype([('time', object), ('Uth_Uph', object), ('latlon', object), ('PlateID', object),
                   ('plateid2name', object)])
    arr = np.empty((1, len(V_BCs)), dtype=dt)
    for i, v in enumerate(V_BCs):
        names = np.empty((1, len(v['plateid2name'])), dtype=ndt)
        for j, p in enumerate(v['plateid2name']):
            names[0, j] = (float(p['plate_id']), float(p['index']), p['plate_abr'])
        arr[0, i] = (float(v['time']), np.asarray(v['Uth_Uph'], dtype=np.float64),
                     np.asarray(v['latlon'], dtype=np.float64),
                     np.asarray(v['PlateID'], dtype=np.float64).reshape(-1, 1), names)
    sio.savemat(path, {'V_BCs': arr, 'time_VBCs_files': np.asarray(time_VBCs_files, dtype=np.float64).reshape(-1, 1)},
                do_compression=True)


def load_vel_bcs(path):
    """(V_BCs list of dicts, time_VBCs_files) from the MAT file (model_parameters_sph_south_atlantic_
    plume.m:283-287 loads it into PHYSICS.V_BCs / PHYSICS.time_VBCs_files)."""
    m = sio.loadmat(path, squeeze_me=False, struct_as_record=True)
    arr = m['V_BCs'].ravel()
    V_BCs = []
    for rec in arr:
        names = []
        for p in rec['plateid2name'].ravel():
            abr = p['plate_abr']
            abr = str(abr.ravel()[0]) if abr.size else ''
            names.append(dict(plate_id=int(p['plate_id'].ravel()[0]), index=int(p['index'].ravel()[0]), plate_abr=abr))
        V_BCs.append(dict(time=float(rec['time'].ravel()[0]), Uth_Uph=np.asarray(rec['Uth_Uph'], dtype=np.float64),
                          latlon=np.asarray(rec['latlon'], dtype=np.float64),
                          PlateID=np.asarray(rec['PlateID'], dtype=np.float64).ravel(), plateid2name=names))
    return V_BCs, np.asarray(m['time_VBCs_files'], dtype=np.float64).ravel()


def interpolate_velocities(V_BCs, time_VBCs_files, model_time):
    """update_vel_bc.m:26-47: (Uth_Uph (2,n), index of the first bracketing file, 0-based).
    Model time 0 is the oldest file; a file whose time is within 1 Myr of the model time brackets it."""
    times = np.asarray(time_VBCs_files, dtype=np.float64).ravel()
    mt = times.max() - model_time
    i_files = np.nonzero(np.abs(times - mt) < 1)[0]
    nfile = len(V_BCs)
    if i_files.size == 0:
        raise ValueError(f'model time {model_time} lies outside the times of the GPlates files')
    if i_files.size == 1:
        i = int(i_files[0])
        if not (i == 0 or i == nfile - 1):
            w = (mt - times[i]) / (times[i + 1] - times[i])
            a, b = V_BCs[i]['Uth_Uph'], V_BCs[i + 1]['Uth_Uph']
            U = np.vstack([a[0] * (1 - w) + b[0] * w, a[1] * (1 - w) + b[1] * w])
        else:
            U = np.array(V_BCs[i]['Uth_Uph'], dtype=np.float64)
    else:
        i, j = int(i_files[0]), int(i_files[1])
        w = (mt - times[i]) / (times[j] - times[i])
        a, b = V_BCs[i]['Uth_Uph'], V_BCs[j]['Uth_Uph']
        U = np.vstack([a[0] * (1 - w) + b[0] * w, a[1] * (1 - w) + b[1] * w])
    return U, int(i_files[0])


def _frames(X):
    """(n,3,3) per-point (theta, phi, r) -> (x, y, z) blocks of make_rotation_matrix.m:69-112."""
    return meshmod.rotation_blocks(X)


def _earth_points(latlon, r_surf):
    """update_vel_bc.m:66-70: GPlates (lat, lon) in degrees -> Cartesian points at the surface."""
    sph = np.array(latlon, dtype=np.float64)
    sph[0] = 90.0 - sph[0]
    sph = (np.pi / 180.0) * sph
    sph = np.vstack([sph, r_surf * np.ones((1, sph.shape[1]))])
    return meshmod.sph2cart(sph)


def _mesh_rotation(RR1=None, RR2=None):
    """RR2 RR1: mesh frame -> GPlates (Earth) frame; its transpose brings GPlates data onto the mesh
    (MESH.RR1/RR2 of an embedded mesh, load_mesh_sph.m:57-60; identity for a global mesh)."""
    return (np.eye(3) if RR2 is None else np.asarray(RR2)) @ (np.eye(3) if RR1 is None else np.asarray(RR1))


def earth_to_mesh_points(latlon, r_surf, RR1=None, RR2=None):
    """update_vel_bc.m:77: the GPlates points in the mesh frame (3, n)."""
    return _mesh_rotation(RR1, RR2).T @ _earth_points(latlon, r_surf)


def rotate_to_mesh_frame(latlon, Uth_Uph, r_surf, RR1=None, RR2=None):
    """update_vel_bc.m:66-81: (theta, phi) velocities of the GPlates points in the mesh frame."""
    cart = _earth_points(latlon, r_surf)
    u_sph = np.vstack([Uth_Uph, np.zeros((1, Uth_Uph.shape[1]))])
    u_cart = np.einsum('nij,jn->in', _frames(cart), u_sph)
    RR = _mesh_rotation(RR1, RR2)
    u_cart_rot = RR.T @ u_cart
    cart_rot = RR.T @ cart
    u_sph_rot = np.einsum('nji,jn->in', _frames(cart_rot), u_cart_rot)
    return u_sph_rot[:2]


def boundary_nodes(PointID, indx=(PID_CMB, PID_SURF)):
    """prepare_DBnods of update_vel_bc.m:160-190: nodes with a boundary index, ascending; an index
    of ``indx`` with no node is an error, a boundary index outside ``indx`` a warning."""
    PointID = np.asarray(PointID).ravel()
    DBnods = np.nonzero(PointID)[0]
    present = np.unique(PointID[DBnods])
    missing = np.setdiff1d(np.asarray(indx), present)
    if missing.size:
        raise ValueError('The following indices are in setbc but have no associated index in DBnods: '
                         + ' '.join(str(int(m)) for m in missing))
    extra = np.setdiff1d(present, np.asarray(indx))
    if extra.size:
        warnings.warn('Boundaries with the following indices have no boundary condition: '
                      + ' '.join(str(int(m)) for m in extra))
    return DBnods


def update_vel_bc(PointID, V_BCs, time_VBCs_files, model_time, r_surf, RR1=None, RR2=None, UBC=None):
    """update_vel_bc.m:22-150. Returns (UBC, Plate): UBC = dict(nfix, ifix (1-based rotated-frame
    dofs), vfix, PlateInfo, PLUME) and VAR.Plate (nnod, the plate index of each surface node).

    ``PLUME`` (UBC['PLUME'] of bc_sph: iUfix_plume 1-based, vUfix_plume) is appended unchanged."""
    PointID = np.asarray(PointID).ravel()
    Uth_Uph, i0 = interpolate_velocities(V_BCs, time_VBCs_files, model_time)
    DBnods = boundary_nodes(PointID)
    DBindx = PointID[DBnods]
    Uth_Uph = rotate_to_mesh_frame(V_BCs[0]['latlon'], Uth_Uph, r_surf, RR1, RR2)
    surf = DBnods[DBindx == PID_SURF]
    if Uth_Uph.shape[1] != surf.size:
        raise ValueError(f'{Uth_Uph.shape[1]} GPlates points for {surf.size} surface nodes')
    # per boundary node, in ascending node order: CMB -> r dof; surface -> theta, phi, r dofs
    cnt = np.where(DBindx == PID_SURF, 3, np.where(DBindx == PID_CMB, 1, 0))
    start = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    ifix = np.zeros(int(cnt.sum()), dtype=np.int64)
    vfix = np.zeros(int(cnt.sum()))
    c = DBindx == PID_CMB
    ifix[start[c]] = 3 * (DBnods[c] + 1)
    s = DBindx == PID_SURF                     # the k-th surface node takes the k-th record
    ifix[start[s]] = 3 * (DBnods[s] + 1) - 2
    vfix[start[s]] = Uth_Uph[0]
    ifix[start[s] + 1] = 3 * (DBnods[s] + 1) - 1
    vfix[start[s] + 1] = Uth_Uph[1]
    ifix[start[s] + 2] = 3 * (DBnods[s] + 1)
    plume = (UBC or {}).get('PLUME') or None
    if plume:
        ifix = np.concatenate([ifix, np.asarray(plume['iUfix_plume'], dtype=np.int64).ravel()])
        vfix = np.concatenate([vfix, np.asarray(plume['vUfix_plume'], dtype=np.float64).ravel()])
    plate_info = np.asarray(V_BCs[i0]['PlateID'], dtype=np.float64).ravel()
    Plate = np.zeros(PointID.size)
    if plate_info.size != surf.size:
        raise ValueError(f'{plate_info.size} plate ids for {surf.size} surface nodes')
    Plate[PointID == PID_SURF] = plate_info
    return dict(nfix=int(ifix.size), ifix=ifix, vfix=vfix, PlateInfo=plate_info, PLUME=plume), Plate


def rotation_operator(latlon, r_surf, RR1=None, RR2=None):
    """(n,2,2) per-point matrices A with A @ (theta, phi) = rotate_to_mesh_frame's result: the
    frame change of update_vel_bc.m:66-81 is linear in the velocity and depends only on the
    GPlates points, so a time loop forms it once (it agrees with the step-by-step form to rounding)."""
    cart = _earth_points(latlon, r_surf)
    RR = _mesh_rotation(RR1, RR2)
    F, Fr = _frames(cart), _frames(RR.T @ cart)
    return np.einsum('nji,jk,nkl->nil', Fr, RR.T, F)[:, :2, :2]


class VelBCSeries:
    """A loaded GPlates series driving the surface velocities of a device-resident time loop. The
    fixed-dof layout and the frame change are formed once; each step interpolates and applies them."""

    def __init__(self, V_BCs, time_VBCs_files, PointID, r_surf, RR1=None, RR2=None, UBC=None):
        self.V_BCs, self.times = V_BCs, np.asarray(time_VBCs_files, dtype=np.float64).ravel()
        self.PointID, self.r_surf, self.RR1, self.RR2, self.UBC = PointID, r_surf, RR1, RR2, UBC
        # layout and plate lists from one full update_vel_bc at the first file's time
        UBC0, _ = update_vel_bc(PointID, V_BCs, self.times, 0.0, r_surf, RR1, RR2, UBC)
        self._ifix, self._plume = UBC0['ifix'], UBC0['PLUME']
        ifix0 = self._ifix - 1
        pid = np.asarray(PointID).ravel()
        node, comp = ifix0 // 3, ifix0 % 3
        surf_dof = (pid[node] == PID_SURF) & (comp < 2)
        nplume = 0 if not self._plume else len(np.ravel(self._plume['iUfix_plume']))
        surf_dof[self._ifix.size - nplume:] = False
        self._th = np.nonzero(surf_dof & (comp == 0))[0]       # ascending node order = record order
        self._ph = np.nonzero(surf_dof & (comp == 1))[0]
        self._vfix0 = np.zeros(self._ifix.size)
        if nplume:
            self._vfix0[self._ifix.size - nplume:] = np.ravel(self._plume['vUfix_plume'])
        self._A = rotation_operator(V_BCs[0]['latlon'], r_surf, RR1, RR2)
        self._surf = pid == PID_SURF

    @classmethod
    def from_mat(cls, path, PointID, r_surf, **kw):
        V, t = load_vel_bcs(path)
        return cls(V, t, PointID, r_surf, **kw)

    def at(self, model_time):
        """(UBC, Plate) of update_vel_bc at the model time."""
        U, i0 = interpolate_velocities(self.V_BCs, self.times, model_time)
        Ur = np.einsum('nij,jn->in', self._A, U)
        vfix = self._vfix0.copy()
        vfix[self._th] = Ur[0]
        vfix[self._ph] = Ur[1]
        plate_info = np.asarray(self.V_BCs[i0]['PlateID'], dtype=np.float64).ravel()
        Plate = np.zeros(self._surf.size)
        Plate[self._surf] = plate_info
        return dict(nfix=int(self._ifix.size), ifix=self._ifix.copy(), vfix=vfix, PlateInfo=plate_info,
                    PLUME=self._plume), Plate

    def apply(self, dm, model_time):
        """Push the prescribed velocities at ``model_time`` to the device (same fixed dofs as the
        set-up; the next operator rebuild uses them). Returns (UBC, Plate)."""
        UBC, Plate = self.at(model_time)
        dm.set_vel_bc(UBC['ifix'] - 1, UBC['vfix'])
        return UBC, Plate


def synthetic_vel_bcs(f, times=(103.0, 102.0, 101.0, 100.0), nplates=12, vmax_cm_yr=10.0, seed=0, RR1=None,
                      RR2=None, n_unassigned=4):
    """Seeded GPlates-format series on the surface nodes of mesh level ``f`` (ascending node order):
    spherical-Voronoi plates with Euler poles whose axes and rates drift from file to file, positions
    and velocities given in the Earth frame (the mesh frame rotated by RR2 RR1), ``n_unassigned``
    records with plate id 0. Returns a list of (time, LatLon (2,n) deg, GPlates plate ids (n,),
    Ucolat_Ulon (2,n) cm/yr), oldest first."""
    rng = np.random.default_rng(seed + 11)
    X = f['GCOORD']
    surf = np.nonzero(np.asarray(f['PointID']) == PID_SURF)[0]
    xe = _mesh_rotation(RR1, RR2) @ X[:, surf]              # Earth-frame positions
    S = meshmod.cart2sph(xe)
    lat = 90.0 - np.rad2deg(S[0])
    lon = np.rad2deg(S[1])
    lon = np.where(lon > 180.0, lon - 360.0, lon)
    r_surf = float(np.mean(S[2]))
    c = rng.normal(size=(nplates, 3))
    c /= np.linalg.norm(c, axis=1, keepdims=True)
    plate = np.argmax((xe / np.linalg.norm(xe, axis=0)).T @ c.T, axis=1)
    ids = PLATE_IDS[rng.permutation(PLATE_IDS.size)[:nplates]]
    pole0 = rng.normal(size=(nplates, 3))
    drift = 0.05 * rng.normal(size=(nplates, 3))
    rate0 = rng.uniform(0.3, 1.0, size=nplates) * vmax_cm_yr
    unassigned = rng.choice(surf.size, size=min(n_unassigned, surf.size), replace=False)
    unassigned = unassigned[(unassigned > 0) & (unassigned < surf.size - 1)]
    out = []
    for k, t in enumerate(times):
        pole = pole0 + k * drift
        pole /= np.linalg.norm(pole, axis=1, keepdims=True)
        rate = rate0 * (1.0 + 0.02 * k)
        omega = pole * (rate / r_surf)[:, None]             # cm/yr at the surface radius
        v = np.cross(omega[plate], xe.T)                     # Earth-frame Cartesian, cm/yr
        F = meshmod.rotation_blocks(xe)
        vl = np.einsum('nji,nj->in', F, v)
        pid = ids[plate].astype(np.int64)
        pid[unassigned] = 0
        out.append((float(t), np.vstack([lat, lon]), pid, vl[:2].copy()))
    return out


def write_synthetic_folder(folder, series):
    """Write a ``synthetic_vel_bcs`` series as ``<t>Ma.txt`` exports."""
    folder = Path(folder)
    folder.mkdir(parents=True, exist_ok=True)
    for t, ll, pid, u in series:
        write_vel_gplates(folder / f'{int(t)}Ma.txt', ll, pid, u)
    return folder
