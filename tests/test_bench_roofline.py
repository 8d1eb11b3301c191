"""bench.py's roofline arithmetic on CPU, with group times made up here: the
dominant group, its algorithmic bytes (field passes x points x element
size), the achieved bandwidth and fraction, the group shares, and the ncu
traffic attached only to the kernel and precision it was captured for."""
import pytest

import bench
from model_gb300 import configs


def _groups():
    # ms summed over the launches of each group, as ga_profile_get reports
    return {"advect": {"ms": 0.3, "launches": 6}, "div_fft_y": {"ms": 0.09, "launches": 6},
            "thomas": {"ms": 0.18, "launches": 6}, "ifft_y_pi": {"ms": 0.084, "launches": 6},
            "post": {"ms": 0.12, "launches": 8}, "kessler": {"ms": 0.03, "launches": 2}}


def test_roofline_of_the_dominant_group():
    wl = configs.thunderstorm()
    r = bench.roofline(_groups(), wl, 4, 6757.2, "measured", "thunderstorm")
    assert r["kernel"] == "advect"
    nbytes = bench.PASSES_MOIST["advect"] * wl.nx * wl.ny * wl.nz * 4
    assert r["algorithmic_bytes_per_launch"] == nbytes
    assert r["ms_per_launch"] == pytest.approx(0.05)
    assert r["achieved"] == pytest.approx(nbytes / 0.05e-3 / 1e9, abs=0.1)
    assert r["frac"] == pytest.approx(r["achieved"] / 6757.2, abs=1e-4)
    assert sum(g["share"] for g in r["groups"].values()) == pytest.approx(1.0, abs=1e-3)
    assert r["traffic"] == bench.TRAFFIC_NCU["thunderstorm"][2]
    assert "profiles/" in r["traffic_source"] and "not measured by this run" in r["traffic_source"]


def test_roofline_traffic_only_where_it_was_captured():
    wl = configs.thunderstorm()
    # FP64, or another workload: no ncu traffic figure applies
    assert bench.roofline(_groups(), wl, 8, 6757.2, "measured", "thunderstorm")["traffic"] is None
    assert bench.roofline(_groups(), wl, 4, 6757.2, "measured", "squall_line")["traffic"] is None
    # a spectral group dominates: its bytes count the levels 1 .. NZ-2 only
    g = _groups()
    g["thomas"]["ms"] = 1.2
    r = bench.roofline(g, wl, 4, 6757.2, "measured", "thunderstorm")
    assert r["kernel"] == "thomas" and r["traffic"] is None
    assert r["algorithmic_bytes_per_launch"] == bench.PASSES_MOIST["thomas"] * wl.nx * wl.ny * (wl.nz - 2) * 4


def test_replica_value_is_the_whole_job():
    ms, v = bench.replica_result(None, 40.0, 1, 786432, 100, "cpu")
    assert ms == 40.0 and v == pytest.approx(786432 * 100 / 0.04)
