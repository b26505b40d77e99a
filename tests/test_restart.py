"""Output / restart files in the reference's MAT layout (write_output_file.m, write_restart_file.m,
load_restart_data.m): names, variables and shapes as MATLAB's save writes them, and a round trip."""
import numpy as np
import scipy.io as sio


def _var(n=7, nv=3, seed=0):
    rng = np.random.default_rng(seed)
    V = {k: rng.standard_normal(n) for k in ('Ux', 'Uy', 'Uz', 'Uth', 'Uph', 'Ur', 'T', 'Dens', 'Visc')}
    V['P'] = rng.standard_normal(nv)
    return V


def test_file_names_and_layout(tmp_path):
    from m3tet_sph_gb300 import restart as R
    VAR = _var()
    S = {'outdir': str(tmp_path)}
    p1 = R.write_output_file(S, VAR, None, 1.25, 7, 0.1, 3)
    p2 = R.write_restart_file(S, VAR, {'nsd': 1, 'myid': 1}, 7, 3, 1.25, 0.1, 2)
    assert p1.name == 'Lab01x01_Data_0003.mat' and p2.name == 'Lab01x01_RestartFile2.mat'
    d = sio.loadmat(p2)
    assert {'VAR', 'dt', 'time', 'istep', 'iplot'} <= set(d)
    assert d['time'].shape == (1, 1) and d['istep'][0, 0] == 7.0
    v = d['VAR'][0, 0]
    assert v['Ux'].shape == (7, 1) and v['P'].shape == (3, 1)            # column vectors
    assert np.array_equal(v['T'][:, 0], VAR['T'])
    o = sio.loadmat(p1)
    assert {'istep', 'time', 'dt', 'VAR'} <= set(o) and 'iplot' not in o


def test_round_trip(tmp_path):
    from m3tet_sph_gb300 import restart as R
    VAR = _var(11, 5, 1)
    p = R.write_restart_file({'outdir': str(tmp_path)}, VAR, None, 4, 2, 3.5, 0.05, 1)
    V2, time, istep, iplot = R.load_restart_file(p)
    assert (time, istep, iplot) == (3.5, 4, 2)
    for k in VAR:
        assert np.array_equal(V2[k], VAR[k]), k
    # an output file restarts too (no iplot), and a time_yr field takes precedence
    q = R.write_output_file({'outdir': str(tmp_path)}, VAR, None, 3.5, 4, 0.05, 9)
    d = sio.loadmat(q)
    d['time_yr'] = 12.0
    sio.savemat(q, d)
    V3, time, istep, iplot = R.load_restart_file(q)
    assert time == 12.0 and iplot is None and np.array_equal(V3['P'], VAR['P'])


def test_plate_field_of_gplates_runs(tmp_path):
    """VAR.Plate (update_vel_bc.m:151-152) is written and read back with the other nodal fields."""
    from m3tet_sph_gb300 import restart as R
    VAR = _var(9, 4, 2)
    VAR['Plate'] = np.array([0, 0, 3, 3, 12, 0, 1, 1, 0], dtype=np.float64)
    p = R.write_output_file({'outdir': str(tmp_path)}, VAR, None, 0.5, 1, 0.1, 1)
    v = sio.loadmat(p)['VAR'][0, 0]
    assert v['Plate'].shape == (9, 1)
    V2, *_ = R.load_restart_file(p)
    assert np.array_equal(V2['Plate'], VAR['Plate'])
