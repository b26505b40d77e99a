"""Allocation-free quasi-cubic interpolation (m3sph_interp3d_cubic_noalloc) against the existing
m3sph_interp3d_cubic entry point. Caller buffers live in device memory owned by torch; the entry
point itself must not allocate. This file is collected last on purpose: it has to pass both in a
fresh process and after every other GPU test of the session."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-13          # relative to max |V|: both entry points run the same FP64 arithmetic


def _points(nel, npt, seed):
    rng = np.random.default_rng(seed)
    els = rng.integers(1, nel + 1, size=npt).astype(np.int32)
    lam = rng.dirichlet(np.ones(4), size=npt)
    return els, np.ascontiguousarray(lam[:, :3])            # (npt, 3): r, s, t


def _noalloc(dm, els_d, lc_d, V_d, out_d, monotonic, wght):
    import torch
    from m3tet_sph_gb300 import _lib as L
    torch.cuda.synchronize()                                 # inputs written by torch's stream
    L.check(L.lib().m3sph_interp3d_cubic_noalloc(dm.h, C.c_void_p(els_d.data_ptr()), C.c_void_p(lc_d.data_ptr()),
                                                 int(els_d.numel()), C.c_void_p(V_d.data_ptr()), int(monotonic),
                                                 int(wght), C.c_void_p(out_d.data_ptr())))
    return out_d.cpu().numpy()


@pytest.fixture(scope='module', params=['tiny_plates', 'c1'])
def case(request, built_lib):
    from m3tet_sph_gb300 import stokes, workloads
    w = workloads.make_workload('c1') if request.param == 'c1' else request.getfixturevalue('tiny_plates')
    dm = stokes.DeviceMesh(w['levels'])
    yield w, dm
    dm.close()


def test_noalloc_matches_existing_entry_point(case):
    import torch
    from m3tet_sph_gb300 import advection as A
    w, dm = case
    f = w['levels'][0]
    nel = f['nel']
    els, lc = _points(nel, 20000, 5)
    rng = np.random.default_rng(9)
    fields = [w['T'], w['T'] + 0.3 * rng.standard_normal(len(w['T']))]
    els_d = torch.from_numpy(els).cuda()
    lc_d = torch.from_numpy(lc).cuda()
    out_d = torch.empty(len(els), dtype=torch.float64, device='cuda')
    # two calls in a row per option set, with different fields: the shared scratch must not carry
    # anything from one call into the next
    for monotonic, wght in ((1, 1), (0, 0)):
        refs = [A.interp3d_cubic_p(dm, els, lc.T, V, monotonic=bool(monotonic), method_wght='dist' if wght else 'ones')
                for V in fields]
        gots = [_noalloc(dm, els_d, lc_d, torch.from_numpy(np.ascontiguousarray(V)).cuda(), out_d, monotonic, wght)
                for V in fields]
        for V, got, ref in zip(fields, gots, refs):
            assert np.all(np.isfinite(got))
            assert np.abs(got - ref).max() <= TOL * np.abs(V).max(), (monotonic, wght)


def _free_bytes():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def test_noalloc_reserves_no_device_memory(built_lib):
    """On a freshly created handle, the first call and the ones after it leave the device's free
    memory unchanged: the scratch array is committed when the handle is created. The device-wide
    free figure can move with other processes, so a change below the 2 MiB granularity of a device
    allocation is tolerated and a mismatch is re-read a few times; torch's own pool must not move."""
    import time
    import torch
    from m3tet_sph_gb300 import stokes, workloads
    w = workloads.make_workload('c1')
    nel = w['levels'][0]['nel']
    els, lc = _points(nel, 4096, 11)
    els_d, lc_d = torch.from_numpy(els).cuda(), torch.from_numpy(lc).cuda()
    V_d = torch.from_numpy(np.ascontiguousarray(w['T'])).cuda()
    out_d = torch.empty(len(els), dtype=torch.float64, device='cuda')
    dm = stokes.DeviceMesh(w['levels'])
    try:
        reserved0 = torch.cuda.memory_reserved()
        free0 = _free_bytes()
        drop = None
        for attempt in range(4):
            for _ in range(3):
                _noalloc(dm, els_d, lc_d, V_d, out_d, 1, 1)
            drop = free0 - _free_bytes()
            if drop < 2 << 20:
                break
            time.sleep(0.5)
            free0 = _free_bytes()
        assert drop < 2 << 20, f"free device memory fell by {drop} bytes across allocation-free calls"
        assert torch.cuda.memory_reserved() == reserved0
    finally:
        dm.close()


def test_noalloc_rejects_meshes_beyond_its_scratch(built_lib):
    """7 values per element + 4 per vertex must fit the fixed 2^20-double scratch."""
    import torch
    from m3tet_sph_gb300 import _lib as L, stokes, workloads
    w = workloads.make_workload('c1', level=5, nlayer=4, nmg=2)    # 245,760 elements
    f = w['levels'][0]
    assert 7 * f['nel'] > 1 << 20
    dm = stokes.DeviceMesh(w['levels'])
    try:
        els_d = torch.ones(8, dtype=torch.int32, device='cuda')
        lc_d = torch.full((8, 3), 0.25, dtype=torch.float64, device='cuda')
        V_d = torch.from_numpy(np.ascontiguousarray(w['T'])).cuda()
        out_d = torch.empty(8, dtype=torch.float64, device='cuda')
        with pytest.raises(L.M3SphError, match='scratch'):
            _noalloc(dm, els_d, lc_d, V_d, out_d, 1, 1)
    finally:
        dm.close()
