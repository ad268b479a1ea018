"""Host-side pieces of bench.py: the checked-configuration count, the
roofline arithmetic of the distance legs, the per-unit traffic read from the
committed ncu summaries, and the clock sampler's parsing of nvidia-smi lines
(no GPU, no nvidia-smi)."""

import numpy as np
import pytest

import bench


def test_checked_configs_counts_steps_up_to_the_first_hit():
    # a free edge checks all n + 1 steps; an edge that hits at step k checks k + 1
    fh = np.array([-1, 0, 3, -1], np.int32)
    ns = np.array([5, 7, 9, 1], np.int32)
    assert bench.checked_configs(fh, ns) == 6 + 1 + 4 + 2


def test_distance_roofline_uses_oracle_bytes_and_reports_kernel_bytes():
    peak, _ = bench.peaks()
    r = bench._roofline(1.0e6, 2.0e5, 4.0e4, 123.0)
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and r["peak"] == peak
    assert r["achieved"] == pytest.approx(1.0e6 * 2.0e5 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / peak)
    assert r["algorithmic_bytes_per_unit"] == 1.0e6 and r["traffic"] == 123.0
    k = r["kernel_counters"]
    assert k["bytes_per_unit"] == 4.0e4 and k["frac"] == pytest.approx(4.0e4 * 2.0e5 / 1e9 / peak)


def test_kernel_bytes_and_work_per_unit():
    st = {"dist_pairs": 10, "dist_node_pairs": 1000, "dist_tri_pairs": 500, "dist_fp64": 20}
    assert bench._kernel_bytes_per_unit(st, 10, 8.0) == pytest.approx((1000 * 32 + 500 * 72) / 10 + 8.0)
    w = bench._work_per_unit(st, 10)
    assert w == {"link_object_pairs": 1.0, "node_pairs": 100.0, "triangle_pairs": 50.0,
                 "fp64_triangle_pairs": 2.0}


def test_profiled_traffic_lines_exist():
    # the bench reads these per-unit DRAM figures from the committed summaries
    for name, key in (("k_engine_edges.md", "dram_bytes_per_item"),
                      ("k_dist_softmin.md", "dram_bytes_per_waypoint"),
                      ("k_dist_min_distance.md", "dram_bytes_per_terrain_config")):
        v = bench.profiled_traffic(name, key)
        assert v is not None and v > 0, (name, key)
    assert bench.profiled_traffic("k_engine_edges.md", "no_such_key") is None


def test_clock_sampler_parses_samples_inside_the_timed_region():
    cs = bench.ClockSampler(0)
    line = "0, {sm}, 2070, 900.0, 0x0, {hw}, Not Active, Not Active, {pc}"
    cs.lines = [line.format(sm=345, hw="Not Active", pc="Not Active"),   # taken as sampling came up
                line.format(sm=2070, hw="Not Active", pc="Active"),
                line.format(sm=2040, hw="Not Active", pc="Not Active"),
                line.format(sm=2070, hw="Active", pc="Not Active")]
    cs.skip = 1
    cs.proc = _Done()
    out = cs.stop()
    assert out["samples"] == 3 and out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["hw_slowdown", "sw_power_cap"]
    # a region too short for a sample inside it falls back to the last line
    cs2 = bench.ClockSampler(0)
    cs2.lines = [line.format(sm=2070, hw="Not Active", pc="Not Active")]
    cs2.skip = 1
    cs2.proc = _Done()
    assert cs2.stop()["samples"] == 1


class _Done:
    """Stands in for the finished nvidia-smi process."""

    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0

    def kill(self):
        pass
