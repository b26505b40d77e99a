"""Regenerate the golden fixtures from the reference project (needs the reference checkout).

* earthshell_n37k.npz: the reference's shipped curved P2 mesh
  (SETUP_TEST/MESHES/EarthShell_n37k.mat, produced by tetmesh_p1_to_p2_sph): vertex
  coordinates, 10-node connectivity (0-based), all node coordinates and PointIDs.
* earthshell_n37k_frame.json: the same file's frame data: RR1_center, RR2_center (the rotations
  between the GPlates (Earth) frame and the mesh frame that update_vel_bc.m:76-77 applies) and the
  refined region's centre in both frames (theta_center, phi_center; theta0, phi0; degrees).
* quadrature_14.json: the numeric values of the 14-point rule documented in
  mfiles_M3TET/ip_tetrahedron.m:109-117 (read from the comments as text).
* quadrature_4.json: the two coordinates of the 4-point rule documented in
  mfiles_M3TET/ip_tetrahedron.m:41-42 (the comments' eight decimals).
* scaling_mantle.json: the 'mantle' units of mfiles_M3TET/numerical_eq_scaling.m:20-27 (L0, t0 = Myr,
  Visc0, Dens0), which the seeded workloads use.
* reference_constants.json: solver and location constants read from the source: the V-cycle's
  Jacobi weights ('Setup 3', mgpcg_solver_p.m:674-682), the Patera defaults
  (flow3d_patera_mg_sph_p.m:70-93), the gap tolerance growth
  (locate_points_in_neighboring_element.m:3,24), the curved Newton iteration
  (local_coords_curved_3d_sph.m:62-64), rock_prop's gas constant (rock_prop.m:67) and the plume
  model's conductivity, heat capacity and density (model_parameters_sph_south_atlantic_plume.m:453,483-484).

Usage: python tests/golden/make_golden.py /path/to/reference
"""
import json
import re
import sys
from pathlib import Path

import numpy as np
import scipy.io as sio

HERE = Path(__file__).resolve().parent


def main(ref):
    ref = Path(ref)
    m = sio.loadmat(ref / 'SETUP_TEST/MESHES/EarthShell_n37k.mat', squeeze_me=True, struct_as_record=False)['MESH']
    el = m.EL2NOD.astype(np.int64).T - 1
    np.savez_compressed(HERE / 'earthshell_n37k.npz', EL2NOD=el.astype(np.int32), GCOORD=m.GCOORD.T.copy(),
                        PointID=m.PointID.astype(np.int32), r_cmb=float(m.r_cmb), r_surf=float(m.r_surf))
    frame = dict(RR1_center=m.RR1_center.tolist(), RR2_center=m.RR2_center.tolist(),
                 theta_center=float(m.theta_center), phi_center=float(m.phi_center),
                 theta0=float(m.theta0), phi0=float(m.phi0))
    (HERE / 'earthshell_n37k_frame.json').write_text(json.dumps(frame, indent=1, sort_keys=True) + '\n')
    txt = (ref / 'mfiles_M3TET/ip_tetrahedron.m').read_text(errors='replace').splitlines()
    vals = {}
    for ln in txt[108:118]:
        mm = re.match(r'\s*([a-z])\s*=.*%\s*=\s*([0-9.]+)', ln)
        if mm:
            vals[mm.group(1)] = float(mm.group(2))
    (HERE / 'quadrature_14.json').write_text(json.dumps(vals, indent=1, sort_keys=True) + '\n')
    vals4 = {}
    for ln in txt[38:48]:
        mm = re.match(r'\s*([ab])\s*=.*%\s*([0-9.]+)', ln)
        if mm:
            vals4[mm.group(1)] = float(mm.group(2))
    (HERE / 'quadrature_4.json').write_text(json.dumps(vals4, indent=1, sort_keys=True) + '\n')
    sc = {}
    src = (ref / 'mfiles_M3TET/numerical_eq_scaling.m').read_text(errors='replace').splitlines()
    blk = src[src.index(next(ln for ln in src if "case 'mantle'" in ln)):]
    blk = blk[:next(i for i, ln in enumerate(blk[1:], 1) if ln.strip().startswith('case'))]
    for ln in blk:
        mm = re.match(r'\s*(Myr|NUMSCALE\.(L0|t0|Visc0|Dens0))\s*=\s*([^;]+);', ln)
        if mm:
            expr = mm.group(3).strip()
            v = sc['Myr'] if expr == 'Myr' else float(np.prod([float(f) for f in expr.split('*')]))
            sc[mm.group(2) or 'Myr'] = v
    (HERE / 'scaling_mantle.json').write_text(json.dumps(sc, indent=1, sort_keys=True) + '\n')
    (HERE / 'reference_constants.json').write_text(json.dumps(reference_constants(ref), indent=1,
                                                              sort_keys=True) + '\n')
    print(sorted(vals.items()), sorted(vals4.items()), sorted(sc.items()))


def _assign(path, name):
    """The right-hand side of the first ``name = value;`` line of a reference file, as text."""
    for ln in path.read_text(errors='replace').splitlines():
        mm = re.match(r'\s*' + re.escape(name) + r'\s*=\s*([^;%]+);', ln)
        if mm:
            return mm.group(1).strip()
    raise KeyError(f'{name} not found in {path}')


def _vec(txt):
    return [float(v) for v in txt.strip('[] ').split()]


def reference_constants(ref):
    mg = ref / 'mfiles_M3TET/mgpcg_solver_p.m'
    pat = ref / 'mfiles_M3TET/flow3d_patera_mg_sph_p.m'
    nb = ref / 'mfiles_M3TET/locate_points_in_neighboring_element.m'
    lcc = ref / 'mfiles_SPH/local_coords_curved_3d_sph.m'
    rock = ref / 'mfiles_M3TET/rock_prop.m'
    mp = ref / 'SETUP_TEST/model_parameters_sph_south_atlantic_plume.m'
    gap_max = re.search(r'while isempty\(iel_ok_nb\) && tol <= ([0-9.e-]+)', nb.read_text()).group(1)
    return {
        'mgpcg_weights': {'finest_down': _vec(_assign(mg, 'Jwght_down{1}')),
                          'finest_up': _vec(_assign(mg, 'Jwght_up{1}')),
                          'other_down': _vec(_assign(mg, 'Jwght_down{jmg}'))},
        'patera': {'rtol_Pat': float(_assign(pat, 'rtol_Pat')), 'itmin_Pat': int(_assign(pat, 'itmin_Pat')),
                   'itmax_Pat': int(_assign(pat, 'itmax_Pat')), 'rtol_U': float(_assign(pat, 'rtol_U')),
                   'itmax_U': int(_assign(pat, 'itmax_U')), 'rtol_restart': _assign(pat, 'rtol_restart')},
        'location': {'gap_step': float(_assign(nb, 'tol_step')), 'gap_max': float(gap_max),
                     'newton_tol': float(_assign(lcc, 'delTH_tol')), 'newton_steps': int(_assign(lcc, 'nimprove'))},
        'rock_prop': {'R': float(_assign(rock, 'R'))},
        'plume_model': {'K': float(_assign(mp, 'PHYSICS.K')), 'Cp': float(_assign(mp, 'PHYSICS.Cp')),
                        'Dens': float(_assign(mp, 'PHYSICS.Dens'))},
    }


if __name__ == '__main__':
    main(sys.argv[1] if len(sys.argv) > 1 else '/root/reference')
