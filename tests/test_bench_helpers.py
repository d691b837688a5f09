"""Host-side helpers of bench.py that turn measurements into the JSON line's
derived numbers (no GPU)."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def test_profile_traffic_scales_with_the_launch():
    """roofline.traffic = the committed DRAM bytes per extension ray x the
    rays of an average launch."""
    d = json.loads((ROOT / "profiles" / "traffic.json").read_text())
    per_ray = float(d["k_extend"]["bytes_per_unit"])
    t, note, issue = bench.profile_traffic("k_extend", 1.0e6)
    assert t == per_ray * 1.0e6 and note and ".md" not in note
    assert len(issue["threads_per_executed_instruction"]) == len(issue["smsp_issue_active_pct"])
    t2, _, _ = bench.profile_traffic("k_extend", 2.0e6)
    assert t2 == 2 * t
    assert bench.profile_traffic("no_such_kernel", 1.0) == (None, None, None)


def test_relmse_metrics():
    rng = np.random.default_rng(0)
    ref = rng.uniform(0.1, 2.0, (32, 48, 3))
    assert bench.relmse(ref, ref) == 0.0 and bench.relmse_robust(ref, ref) == 0.0
    img = ref * 1.1
    # (0.1 r)^2 / (r^2 + 0.01) averaged over channels and pixels
    expect = np.mean((0.1 * ref) ** 2 / (ref * ref + 1e-2))
    assert abs(bench.relmse(img, ref) - expect) < 1e-12
    # the robust variant leaves out the largest 0.1 % of per-pixel errors
    spiky = img.copy()
    spiky[0, 0] = 1e6
    assert bench.relmse(spiky, ref) > 1e3 * bench.relmse(img, ref)
    assert abs(bench.relmse_robust(spiky, ref) - bench.relmse_robust(img, ref)) < 0.05 * bench.relmse(img, ref)
    # Metrics::calculateRRMSE: RMSE / (sqrt(sum ref^2) + 1e-2)
    r = bench.rrmse_reference_metric(img, ref)
    assert abs(r - np.sqrt(np.mean((0.1 * ref) ** 2)) / (np.sqrt(np.sum(ref ** 2)) + 1e-2)) < 1e-12


def test_measured_peaks_read():
    p = bench.measured_peaks()
    assert p["hbm_gbs"] > 1000 and p["source"] in ("measured", "fallback")


def test_side_measurement_failures_are_recorded():
    """A failing side measurement of the default line is recorded as an
    error in the line instead of ending the run."""
    import bench

    def fails(x):
        raise RuntimeError(f"cannot {x}")

    r = bench.guarded("side", fails, "render")
    assert r == {"error": "RuntimeError: cannot render"}
    assert bench.pick(r, ("a",)) == r
    assert bench.pick({"a": 1, "b": 2}, ("a",)) == {"a": 1}
    assert bench.guarded("side", lambda v: {"v": v}, 3) == {"v": 3}
