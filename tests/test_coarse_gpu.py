"""The coarsest-level solve (stands in for cholesky_factorization / cholesky_solve): the blocked
Gauss-Jordan inverse, and on the plain FP64 path for large coarsest levels the FP32 inverse refined
against the FP64 coarsest operator. Through the C ABI."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _vcycles(w, dm, r, f64_direct_max):
    dm.set_option("coarse_f64_direct_max", f64_direct_max)
    try:
        dm.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=0)
        return dm.vcycle(r)
    finally:
        dm.set_option("coarse_f64_direct_max", 6000)


def test_refined_fp64_coarse_solve_equals_the_fp64_inverse(built_lib, tiny_plates):
    """The refined coarse solve (FP32 inverse + 3 refinement steps against the FP64 operator) gives
    the V-cycle of the FP64 inverse to FP64 rounding."""
    from m3tet_sph_gb300 import stokes
    w = tiny_plates
    dm = stokes.DeviceMesh(w['levels'])
    try:
        rng = np.random.default_rng(3)
        r = rng.standard_normal(dm.ndof)
        d_direct = _vcycles(w, dm, r, 6000)
        d_ref = _vcycles(w, dm, r, 0)
        assert np.linalg.norm(d_ref - d_direct) < 1e-12 * np.linalg.norm(d_direct)
    finally:
        dm.close()


def test_17k_coarsest_level(built_lib):
    """The 130,662-DOF shell on 2 levels puts 17,334 dofs on the coarsest level (the size of the
    4-level 8M-DOF and the 5-level 64M-DOF hierarchies). On that problem the plain FP64 path with the
    refined coarse solve and the FP32 V-cycle path (FP32 inverse) both reach the solution of the
    plain FP64 path with the FP64 inverse of the coarsest level."""
    from m3tet_sph_gb300 import stokes, workloads
    kw = dict(rtol_Pat=1e-9, rtol_U=5e-3, itmax_Pat=400, itmax_U=40, target_rel_residual=1e-11)
    w = workloads.make_workload('c1', nmg=2)
    assert 3 * w['levels'][1]['nnod'] == 17334
    sols, its = {}, {}
    dm = stokes.DeviceMesh(w['levels'])
    try:
        for name, prec, direct_max in (("fp64 inverse", 0, 20000), ("fp64 refined", 0, 6000), ("fp32", 1, 6000)):
            dm.set_option("coarse_f64_direct_max", direct_max)
            dm.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=prec)
            U, P, info = dm.solve(**kw)
            assert info['rel_residual'] <= 1e-11, (name, info)
            its[name] = info['nitU'] + info['nitZ']
            print(f"{name}: {its[name]} MG-PCG iterations, set-up {info['t_setup_ms']:.1f} ms")
            sols[name] = (U, P - P.mean())
    finally:
        dm.set_option("coarse_f64_direct_max", 6000)
        dm.close()
    U0, P0 = sols["fp64 inverse"]
    for name in ("fp64 refined", "fp32"):
        U, P = sols[name]
        assert np.linalg.norm(U - U0) < 1e-8 * np.linalg.norm(U0), name
        assert np.linalg.norm(P - P0) < 1e-8 * np.linalg.norm(P0), name
    assert abs(its["fp64 refined"] - its["fp64 inverse"]) <= 2
