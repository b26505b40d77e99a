"""The bench's host side: its size and byte models against the shell counts and the per-unit figures
they restate (closed-form node / element counts of the three shells; the algorithmic bytes of one
operator apply: x and y in the vector precision, 10 int32 connectivity entries and a class byte per
element, vertex (theta, phi, r) and viscosity), the reporting of failed side legs, and the CPU
reference arm's JSON line."""
import pytest


@pytest.mark.parametrize('level,nlayer,nel,nnod,nP', [
    (3, 8, 30_720, 43_554, 5_778),            # 130,662 velocity DOF
    (5, 32, 1_966_080, 2_662_530, 337_986),   # 7,987,590 velocity DOF
    (6, 64, 15_728_640, 21_135_618, 2_662_530),  # 63,406,854 velocity DOF
])
def test_shell_counts(level, nlayer, nel, nnod, nP):
    from m3tet_sph_gb300 import mesh as M
    c = M.mesh_counts(level, nlayer)
    assert (c['nel'], c['nnod'], c['nP']) == (nel, nnod, nP)


def test_built_shell_matches_the_counts():
    from m3tet_sph_gb300 import mesh as M
    lv = M.build_hierarchy(3, 8, 3)
    for j, (L, n) in enumerate([(3, 8), (2, 4), (1, 2)]):
        c = M.mesh_counts(L, n)
        assert lv[j]['nel'] == c['nel'] and lv[j]['nnod'] == c['nnod']
        assert int(lv[j]['EL2NOD'][:, :4].max()) + 1 == c['nP']


def test_algorithmic_apply_bytes():
    import bench
    from m3tet_sph_gb300 import mesh as M
    c5, c2 = M.mesh_counts(6, 64), M.mesh_counts(5, 32)
    # 64M-DOF shell, FP64: 0.507 + 0.507 + 0.629 + 0.016 + 0.064 + 0.021 GB
    b5 = bench.algorithmic_apply_bytes(c5['nel'], 3 * c5['nnod'], c5['nP'], 8)
    assert b5 == 2 * 8 * 63_406_854 + 41 * 15_728_640 + 32 * 2_662_530
    assert abs(b5 / 1e9 - 1.74) < 0.01
    # 8M-DOF shell: 219 MB in FP64 (the double-float outer apply's roofline), 155 MB in FP32
    b2 = bench.algorithmic_apply_bytes(c2['nel'], 3 * c2['nnod'], c2['nP'], 8)
    assert abs(b2 / 1e6 - 219.2) < 0.1
    b2f = bench.algorithmic_apply_bytes(c2['nel'], 3 * c2['nnod'], c2['nP'], 4)
    assert abs(b2f / 1e6 - 155.3) < 0.1
    # streamed bytes of the partially assembled FP32 apply on the 491,520-element profiling shell
    cp = M.mesh_counts(5, 8)
    assert abs(bench.apply_bytes_pa(cp['nel'], 3 * cp['nnod'], cp['nnod']) / 1e9 - 0.297) < 0.001
    assert abs(bench.apply_bytes(cp['nel'], 3 * cp['nnod'], 4) / 1e9 - 0.951) < 0.001


def test_extra_leg_reports_failures():
    import bench
    assert bench.extra_leg(lambda a, b: {"x": a + b}, 1, 2) == {"x": 3}
    r = bench.extra_leg(lambda: 1 / 0)
    assert r["error"].startswith("ZeroDivisionError")


def test_reference_arm_line():
    """`bench.py --impl reference` (one timed FP64 oracle solve of the 130,662-DOF shell on the host
    threads) prints one JSON line with the contract's keys and a converged solve."""
    import json
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       cwd=root, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "s" and d["higher_is_better"] is False
    assert d["value"] > 0 and d["steps"] == 1 and d["n_gpus"] == 1
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "coupled residual" in d["cpu_baseline"]["sample"]
    res = float(d["cpu_baseline"]["sample"].split("to a ")[1].split(" coupled")[0])
    assert res < 1e-8
