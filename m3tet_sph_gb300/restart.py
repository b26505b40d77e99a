"""Output and restart files in the reference's MAT layout, from and to a device-resident time series.

The reference writes with MATLAB's ``save`` (default format: MAT v7, zlib-compressed v5 elements):
* ``write_output_file`` (mfiles_M3TET/write_output_file.m:27-31): ``<outdir>/<prefix>_Data_<iplot,
  4 digits>.mat`` holding ``istep``, ``time``, ``dt``, ``VAR``;
* ``write_restart_file`` (mfiles_M3TET/write_restart_file.m:28-31): ``<outdir>/<prefix>_RestartFile
  <irestart>.mat`` holding ``VAR``, ``dt``, ``time``, ``istep``, ``iplot``;
* ``load_restart_file`` (mfiles_M3TET/load_restart_data.m:296-311) reads either: ``time`` (or
  ``time_yr``), ``istep``, ``VAR`` and ``iplot`` if present.
``<prefix>`` is COMM.prefix, ``Lab<nsd,2 digits>x<myid,2 digits>`` (init_COMM.m:26): ``Lab01x01`` for
the serial curved-mesh code. VAR holds nodal column vectors (Ux Uy Uz Uth Uph Ur T Dens Visc), the
vertex pressure P, and in GPlates runs the surface plate indices Plate. scipy.io writes the same v5
elements with compression, which MATLAB's ``load`` reads.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import scipy.io as sio

from . import mesh as meshmod

# Plate: the plate index of each surface node that update_vel_bc sets in GPlates runs
# (update_vel_bc.m:151-152), written when the caller's VAR holds it
VAR_FIELDS = ('Ux', 'Uy', 'Uz', 'Uth', 'Uph', 'Ur', 'P', 'T', 'Dens', 'Visc', 'Plate')


def prefix(COMM=None):
    COMM = COMM or {}
    if 'prefix' in COMM:
        return COMM['prefix']
    return f"Lab{int(COMM.get('nsd', 1)):02d}x{int(COMM.get('myid', 1)):02d}"


def var_from_device(dm):
    """VAR of the handle's resident state: velocity of the last solve (Cartesian and local spherical
    components), pressure, temperature (if the time series holds one), viscosity and density."""
    U, P = dm.solution()
    V, D = dm.properties()
    Ux, Uy, Uz = U[0::3], U[1::3], U[2::3]
    R = meshmod.rotation_blocks(dm.levels[0]['GCOORD'])
    Ul = np.einsum('nji,nj->ni', R, U.reshape(-1, 3))
    VAR = dict(Ux=Ux, Uy=Uy, Uz=Uz, Uth=Ul[:, 0], Uph=Ul[:, 1], Ur=Ul[:, 2], P=P, Dens=D, Visc=V)
    try:
        VAR['T'] = dm.get_temperature()
    except Exception:
        pass
    return VAR


def _mat_var(VAR):
    return {k: np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(-1, 1))
            for k, v in VAR.items() if k in VAR_FIELDS}


def write_output_file(SETTINGS, VAR, COMM, time, istep, dt, iplot):
    """write_output_file.m:27-31; returns the path."""
    path = Path(SETTINGS['outdir']) / f"{prefix(COMM)}_Data_{int(iplot):04d}.mat"
    sio.savemat(path, {'istep': float(istep), 'time': float(time), 'dt': float(dt), 'VAR': _mat_var(VAR)},
                do_compression=True, oned_as='column')
    return path


def write_restart_file(SETTINGS, VAR, COMM, istep, iplot, time, dt, irestart):
    """write_restart_file.m:28-31; returns the path."""
    path = Path(SETTINGS['outdir']) / f"{prefix(COMM)}_RestartFile{int(irestart)}.mat"
    sio.savemat(path, {'VAR': _mat_var(VAR), 'dt': float(dt), 'time': float(time), 'istep': float(istep),
                       'iplot': float(iplot)}, do_compression=True, oned_as='column')
    return path


def load_restart_file(filename):
    """load_restart_data.m:296-311: (VAR, time, istep, iplot); iplot is None when the file has none."""
    d = sio.loadmat(filename, squeeze_me=True, struct_as_record=False)
    time = float(d['time_yr'] if 'time_yr' in d else d['time'])
    V = d['VAR']
    VAR = {k: np.atleast_1d(np.asarray(getattr(V, k), dtype=np.float64)) for k in V._fieldnames}
    iplot = int(d['iplot']) if 'iplot' in d else None
    return VAR, time, int(d['istep']), iplot


def restore_device(dm, VAR, time):
    """Resume a device-resident time series from a loaded VAR: temperature and model time, and the
    pressure the next step starts from (the operator's set-up stays the caller's)."""
    dm.set_temperature(VAR['T'], time)
    dm.set_pressure(VAR['P'])
