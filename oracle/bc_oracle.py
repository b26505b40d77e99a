"""ORACLE (test infrastructure only): CPU restatement of update_vel_bc and of the GPlates reader.

Checker for ``m3tet_sph_gb300/gplates.py``; only tests use it. It follows the reference's steps one
record and one node at a time, with explicit 3x3 frames, where the product is vectorised:

* ``read_records``: readVelGPlates.m:41-110 (five numbers per record, plate id 0 takes the previous
  record's id, else the next one's; ids to 1-based indices of the plate table; cm/yr x 10);
* ``velocities_at``: update_vel_bc.m:26-47 (files within 1 Myr of the model time, linear weights);
* ``update_vel_bc``: update_vel_bc.m:53-150 (Earth frame -> mesh frame by (RR2 RR1)^T through
  Cartesian components, then the loop over boundary nodes building ifix / vfix).

Parity unpinned against reference outputs: the reference's GPlates exports are not distributed, so
the restatement is checked on seeded files in the same format.
"""
from __future__ import annotations

import math

import numpy as np

PLATE_IDS = [101, 103, 119, 201, 301, 304, 409, 607, 701, 702, 801, 901, 902, 919, 926]


def read_records(text):
    vals = [float(t) for t in text.split()]
    assert len(vals) % 5 == 0
    recs = [vals[i:i + 5] for i in range(0, len(vals), 5)]
    pid = [r[2] for r in recs]
    for i in [k for k, p in enumerate(pid) if p == 0]:
        if i == 0 or i == len(pid) - 1:
            raise ValueError('unassigned first or last record')
        nb = [p for p in (pid[i - 1], pid[i + 1]) if p != 0]
        if not nb:
            raise ValueError('no neighbouring plate id')
        pid[i] = nb[0]
    for p in set(pid):
        if p not in PLATE_IDS:
            raise ValueError('unknown plate id')
    latlon = np.array([[r[0] for r in recs], [r[1] for r in recs]])
    U = np.array([[r[3] * 10 for r in recs], [r[4] * 10 for r in recs]])
    idx = np.array([float(PLATE_IDS.index(p) + 1) for p in pid])
    return U, latlon, idx


def velocities_at(V_BCs, times, model_time):
    times = [float(t) for t in np.ravel(times)]
    mt = max(times) - model_time
    i_files = [i for i, t in enumerate(times) if abs(t - mt) < 1]
    if not i_files:
        raise ValueError('outside the files')
    n = len(V_BCs)
    if len(i_files) == 1:
        i = i_files[0]
        if i == 0 or i == n - 1:
            return np.array(V_BCs[i]['Uth_Uph'], dtype=np.float64), i
        j = i + 1
    else:
        i, j = i_files[0], i_files[1]
    w = (mt - times[i]) / (times[j] - times[i])
    a, b = V_BCs[i]['Uth_Uph'], V_BCs[j]['Uth_Uph']
    U = np.empty((2, a.shape[1]))
    for k in range(a.shape[1]):
        U[0, k] = a[0, k] * (1 - w) + b[0, k] * w
        U[1, k] = a[1, k] * (1 - w) + b[1, k] * w
    return U, i_files[0]


def _frame(x, y, z):
    """make_rotation_matrix.m:69-112 for one point: columns theta, phi, r in Cartesian components."""
    th = math.atan2(math.sqrt(x * x + y * y), z)
    ph = math.atan2(y, x)
    if ph < 0:
        ph += 2 * math.pi
    return np.array([[math.cos(ph) * math.cos(th), -math.sin(ph), math.cos(ph) * math.sin(th)],
                     [math.sin(ph) * math.cos(th), math.cos(ph), math.sin(ph) * math.sin(th)],
                     [-math.sin(th), 0.0, math.cos(th)]])


def update_vel_bc(PointID, V_BCs, times, model_time, r_surf, RR1=None, RR2=None):
    """(ifix 1-based, vfix, Plate) of update_vel_bc at the model time."""
    U, i0 = velocities_at(V_BCs, times, model_time)
    RR = (np.eye(3) if RR2 is None else np.asarray(RR2)) @ (np.eye(3) if RR1 is None else np.asarray(RR1))
    ll = V_BCs[0]['latlon']
    Urot = np.empty_like(U)
    for k in range(ll.shape[1]):
        th = (90.0 - ll[0, k]) * math.pi / 180.0
        ph = ll[1, k] * math.pi / 180.0
        p = np.array([r_surf * math.sin(th) * math.cos(ph), r_surf * math.sin(th) * math.sin(ph), r_surf * math.cos(th)])
        uc = _frame(*p) @ np.array([U[0, k], U[1, k], 0.0])
        ucr = RR.T @ uc
        pr = RR.T @ p
        us = _frame(*pr).T @ ucr
        Urot[0, k], Urot[1, k] = us[0], us[1]
    ifix, vfix = [], []
    ks = 0
    pid = np.ravel(PointID)
    for node in range(pid.size):
        if pid[node] == 301:
            ifix.append(3 * (node + 1))
            vfix.append(0.0)
        elif pid[node] == 306:
            ifix += [3 * (node + 1) - 2, 3 * (node + 1) - 1, 3 * (node + 1)]
            vfix += [Urot[0, ks], Urot[1, ks], 0.0]
            ks += 1
    Plate = np.zeros(pid.size)
    Plate[pid == 306] = np.ravel(V_BCs[i0]['PlateID'])
    return np.array(ifix, dtype=np.int64), np.array(vfix), Plate
