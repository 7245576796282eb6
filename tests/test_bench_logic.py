"""The measurement logic of bench.py, on the host (no GPU): times to a rel-MSE
target (measured, interpolated, bounds and extrapolations labelled as such),
the algorithmic byte counts behind the roofline, the reference log's stage
sums (parse_logs.py:117-154) and the per-stage DRAM traffic from an ncu
launch list."""
import math

import pytest

import bench


def test_time_to_target_measured_interpolated_extrapolated():
    # first point already below the target: that point's time
    assert bench.time_to_target([(2.0, 5e-4), (4.0, 2e-4)], 1e-3) == (2.0, "measured")
    # between two points: log-log interpolation
    t, how = bench.time_to_target([(10.0, 4e-3), (40.0, 1e-3 / 2)], 1e-3)
    f = (math.log(1e-3) - math.log(4e-3)) / (math.log(5e-4) - math.log(4e-3))
    assert how == "interpolated" and t == pytest.approx(math.exp(math.log(10.0) + f * math.log(4.0)))
    # the ladder ends above the target: extrapolated from the last two points
    t, how = bench.time_to_target([(10.0, 4e-3), (20.0, 2e-3)], 1e-3)
    assert how == "extrapolated" and t == pytest.approx(40.0)
    # not decreasing: no estimate
    assert bench.time_to_target([(10.0, 2e-3), (20.0, 2e-3)], 1e-3) == (None, None)
    assert bench.time_to_target([], 1e-3) == (None, None)


def _arm(points, target):
    ladder = [{"spp": 2 ** i, "ms": t, "rel_mse": e} for i, (t, e) in enumerate(points)]
    t, how = bench.time_to_target(points, target)
    return {"ladder": ladder, "ms_to_target": t, "to_target": how}


def test_target_summary_ratio_or_labelled_bound():
    target = 1e-3
    learned = _arm([(10.0, 2e-3), (30.0, 5e-4)], target)
    # both arms reach the target: a measured ratio
    plain = _arm([(20.0, 3e-3), (80.0, 5e-4)], target)
    s = bench.target_summary(plain, learned, target)
    assert "ratio" in s and s["ratio"] == pytest.approx(learned["ms_to_target"] / plain["ms_to_target"], abs=1e-4)
    assert "bound" not in s["how"]
    # plain never reaches it: an upper bound on the ratio from plain's last point,
    # the extrapolation reported apart and labelled
    plain = _arm([(20.0, 4e-3), (60.0, 2e-3)], target)
    s = bench.target_summary(plain, learned, target)
    assert "ratio" not in s
    assert s["plain_ms_lower_bound"] == 60.0
    assert s["ratio_upper_bound"] == pytest.approx(learned["ms_to_target"] / 60.0, abs=1e-4)
    assert "measured bound" in s["how"]
    assert s["ratio_extrapolated"] < s["ratio_upper_bound"]
    # learned never reaches it: no ratio at all
    s = bench.target_summary(plain, _arm([(10.0, 5e-3), (30.0, 5e-3)], target), target)
    assert "ratio" not in s and "ratio_upper_bound" not in s


def test_stage_bytes_formulas():
    D, W, H, L0 = 4, 64, 32, 1000
    passes = [{"L": 1000, "recomputed": 1000, "selected": 400, "splits": 100, "gathered": 1500},
              {"L": 1100, "recomputed": 200, "selected": 500, "splits": 150, "gathered": 1800}]
    b = bench.stage_bytes(D, W, H, L0, passes, 5000, 1250)
    assert b["init"] == L0 * (24 * D + 25)
    err = 4 * 1000 + 1000 * (4 + 16 + 8 * D) + 48 * 1000  # full first pass
    err += 200 * 20 + 12 * (5 * 200 // 2)  # split children: entry + error write, 5 values per pair
    assert b["errors"] == err
    adap = 0
    for p in passes:
        S, P, G, L = p["selected"], p["splits"], p["gathered"], p["L"]
        adap += 13 * L + S * (32 + 12 * D) + 4 * D * G + (S - P) * (17 + 4 * D) + P * (86 + 28 * D)
    assert b["adaptive"] == adap
    assert b["integrate"] == 1250 * (16 + 8 * D) + 12 * 5000 + 32 * W * H


def test_parse_reference_log(tmp_path):
    p = tmp_path / "run.exr.log"
    p.write_text("INITIAL SAMPLES\n4096\nINITIAL SAMPLING TIME\n0.5\nCOMPUTE ERRORS TIME\n1.0\nSAMPLES\n10\n"
                 "ADAPTIVE SAMPLING TIME\n2.0\nCOMPUTE ERRORS TIME\n1.5\nADAPTIVE SAMPLING TIME\n2.5\n"
                 "TOTAL SAMPLES\n5000\nINTEGRATE TIME\n0.25\n")
    t = bench.parse_reference_log(str(p))
    assert t == {"init": 0.5, "errors": 2.5, "adaptive": 4.5, "integrate": 0.25}


def test_ncu_stage_traffic(tmp_path):
    rows = ['"ID","Kernel Name","Metric Name","Metric Unit","Metric Value"']
    launches = [("0", "void mdas_fast::k_adaptive_decide<4, 8, 0>(MdasDeviceGrid, unsigned int, unsigned int)", 10.0, 20.0),
                ("1", "mdas_fast::k_adaptive_scan(MdasDeviceGrid)", 5.0, 0.0),
                ("2", "void mdas_fast::k_adaptive_place<4>(MdasDeviceGrid)", 30.0, 100.0),
                ("3", "void mdas_fast::k_compute_errors<4, 1>(MdasDeviceGrid)", 15.0, 70.0),
                ("4", "void other_kernel(int)", 99.0, 99.0)]
    for i, name, us, mb in launches:
        rows.append(f'"{i}","{name}","gpu__time_duration.sum","usecond","{us}"')
        rows.append(f'"{i}","{name}","dram__bytes_read.sum","Mbyte","{mb * 0.75}"')
        rows.append(f'"{i}","{name}","dram__bytes_write.sum","Mbyte","{mb * 0.25}"')
    p = tmp_path / "launch.csv"
    p.write_text("==PROF== a line before the table\n" + "\n".join(rows) + "\n")
    out = bench.ncu_stage_traffic(str(p))
    assert set(out) == {"adaptive", "errors"}
    assert out["adaptive"]["launches"] == 3
    assert out["adaptive"]["dram_bytes"] == pytest.approx(120e6)
    assert out["adaptive"]["us"] == pytest.approx(45.0)
    assert out["errors"]["dram_mb_per_launch"] == pytest.approx(70.0)
