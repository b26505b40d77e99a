"""Stokes solve on the 130,662-DOF shell (level-3 surface x 8 layers, 30,720 curved P2 tets, 3 MG
levels, isoviscous, free slip at both boundaries with the rigid-rotation pins): the plain FP64
path, the FP32 V-cycle with weighted-Jacobi smoothing and the FP32 V-cycle with the learned element
smoother, each against the FP64 oracle's Patera / MG-PCG solve (flow3d_patera_mg_sph_p.m:386-632,
mgpcg_solver_p.m:117-199) converged far below the 1e-8 bar. All GPU solves go through the C ABI."""
from pathlib import Path

import numpy as np
import pytest

from oracle import stokes_oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-8        # relative L2 of U and of the mean-free P against the oracle


@pytest.fixture(scope='module')
def c1_oracle(built_lib):
    from m3tet_sph_gb300 import workloads
    w = workloads.make_workload('c1')
    S = O.StokesSystem(w['levels'], w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'])
    Ur, Pr, info = O.patera(S, rtol_Pat=1e-11, rtol_U=1e-4, itmax_Pat=400, itmax_U=60)
    res = S.residual(Ur, Pr)
    assert res < 1e-10, (res, info)
    return w, S, S.RR @ Ur, Pr - Pr.mean(), res


@pytest.mark.parametrize("path", ["fp64", "fp32_jacobi", "fp32_learned"])
def test_c1_solution_matches_oracle(c1_oracle, path):
    from m3tet_sph_gb300 import learned, stokes
    w, S, Uref, Pref, res = c1_oracle
    dm = stokes.DeviceMesh(w['levels'])
    try:
        dm.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=0 if path == "fp64" else 1)
        smoother = 0
        if path == "fp32_learned":
            learned.set_params(dm, np.load(Path(learned.__file__).with_name('smoother_c1.npy')), trained=True)
            smoother = 1
        U, P, info = dm.solve(rtol_Pat=1e-9, rtol_U=5e-3, itmax_Pat=400, itmax_U=40, target_rel_residual=1e-11,
                              smoother=smoother)
        Pc = P - P.mean()
        eU = np.linalg.norm(U - Uref) / np.linalg.norm(Uref)
        eP = np.linalg.norm(Pc - Pref) / np.linalg.norm(Pref)
        print(f"{path}: eU {eU:.2e} eP {eP:.2e} residual {info['rel_residual']:.2e} "
              f"its {info['nitU'] + info['nitZ']} Patera {info['itPat']} fallbacks {info['smoother_fallbacks']}")
        assert info['status'] == 0 and info['rel_residual'] <= 1e-11
        assert eU < TOL and eP < TOL, (path, eU, eP)
    finally:
        dm.close()

