"""The partially assembled FP32 operator of the finest level (per integration point the 3x3
geometric factor scaled by sqrt(w eta); the product formed on the fly) against the FP64 element
operator and against the streamed stored FP32 matrices, through the C ABI; and solves that use it
as the V-cycle operator."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(params=['tiny', 'tiny_plates', 'c1'])
def wl(request, built_lib):
    from m3tet_sph_gb300 import workloads
    if request.param == 'c1':
        return workloads.make_workload('c1')
    return request.getfixturevalue(request.param)


def _apply_both(dm, x):
    """(partially assembled apply twice, stored apply) of the FP32 finest-level operator."""
    try:
        dm.set_option("fp32_operator", 1)
        ys = [dm.level_apply32(0, x) for _ in range(2)]
        dm.set_option("fp32_operator", 0)
        yst = dm.level_apply32(0, x)
    finally:
        dm.set_option("fp32_operator", 1)        # the default
    return ys, yst


def test_partially_assembled_apply(wl):
    """Every element class (original, Z-180, X-90 frames; isoparametric cone elements), node
    rotations and free-slip / plate masks: within FP32 accuracy of the FP64 operator,
    deterministic, fixed dofs exactly zero and ignored on input."""
    from m3tet_sph_gb300 import stokes
    w = wl
    dm = stokes.DeviceMesh(w['levels'])
    try:
        dm.set_option("fp32_operator", 1)
        dm.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=1)
        n = 3 * w['levels'][0]['nnod']
        x = np.random.default_rng(31).standard_normal(n).astype(np.float32)
        ys, yst = _apply_both(dm, x)
        y64 = dm.level_apply(0, x.astype(np.float64))
        fixed = np.ones(n, bool)
        fixed[np.nonzero(y64)[0]] = False
        e_pa = np.linalg.norm(ys[0] - y64) / np.linalg.norm(y64)
        e_st = np.linalg.norm(yst - y64) / np.linalg.norm(y64)
        print(f"relative error vs FP64: partially assembled {e_pa:.2e}, stored {e_st:.2e}")
        assert np.array_equal(ys[0], ys[1])
        assert e_pa < 1e-5
        assert np.all(ys[0][fixed] == 0)
        # fixed input components do not contribute
        x2 = x.copy()
        x2[fixed] = 1e3
        ys2, _ = _apply_both(dm, x2)
        assert np.array_equal(ys2[0], ys[0])
    finally:
        dm.close()


@pytest.mark.parametrize("smoother", [0, 1])
def test_solve_with_partially_assembled_vcycle(built_lib, smoother):
    """The 130,662-DOF shell solved to a 1e-10 coupled residual with the partially assembled
    V-cycle operator: the same solution as with the stored FP32 matrices (1e-8) and about the same
    MG-PCG iterations."""
    from pathlib import Path
    from m3tet_sph_gb300 import learned, stokes, workloads
    w = workloads.make_workload('c1')
    kw = dict(rtol_Pat=1e-9, rtol_U=5e-3, itmax_Pat=400, itmax_U=40, target_rel_residual=1e-10, smoother=smoother)
    dm = stokes.DeviceMesh(w['levels'])
    res = {}
    try:
        for op in (0, 1):
            dm.set_option("fp32_operator", op)
            dm.setup(w['visc'], w['dens'], w['ifix'], w['vfix'], w['phys'], precision=1)
            if smoother:
                learned.set_params(dm, np.load(Path(learned.__file__).with_name('smoother_c1.npy')), trained=True)
            U, P, info = dm.solve(**kw)
            res[op] = (U, P - P.mean(), info)
    finally:
        dm.set_option("fp32_operator", 1)
        dm.close()
    (U0, P0, i0), (U1, P1, i1) = res[0], res[1]
    its0, its1 = i0['nitU'] + i0['nitZ'], i1['nitU'] + i1['nitZ']
    print(f"smoother {smoother}: stored {its0} its, partially assembled {its1} its")
    assert i1['status'] == 0 and i1['rel_residual'] <= 1e-10
    assert np.linalg.norm(U1 - U0) < 1e-8 * np.linalg.norm(U0)
    assert np.linalg.norm(P1 - P0) < 1e-8 * np.linalg.norm(P0)
    assert abs(its1 - its0) <= max(3, 0.05 * its0)
