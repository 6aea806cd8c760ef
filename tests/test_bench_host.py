"""Host-side arithmetic of bench.py's roofline figures (no GPU): algorithmic
bytes per launch, the dominant kernel, the FP64-pipe rate against the nominal
peak at the sampled clock and against a measured FP64 throughput."""
import pytest

import bench


def test_roofline_fractions_and_fp64_pipe():
    cells = 8192 * 4096
    # per-direction launch times (ms): x three launches, z three launches; z dominates
    per = {0: [3.1, 3.1, 3.1], 1: [3.2, 3.2, 3.2]}
    table = {"kx": {"dram_bytes_per_cell": 81.5, "fp64_ops_per_cell": 47.64},
             "kz": {"dram_bytes_per_cell": 82.5, "fp64_ops_per_cell": 49.34}}
    rl = bench.roofline(per, cells, 8, 6793.8, "measured", {0: "kx", 1: "kz"}, table, sm_mhz=2070.0)
    algo = cells * 8 * 32 / 3.0  # 85.33 B per cell per launch on average
    assert rl["algorithmic_bytes_per_launch"] == pytest.approx(algo)
    assert rl["kernel"] == "kz" and rl["other_kernel"]["kernel"] == "kx"
    assert rl["achieved"] == pytest.approx(algo / 3.2e-3 / 1e9, rel=1e-3)
    assert rl["frac"] == pytest.approx(rl["achieved"] / 6793.8, rel=1e-3)
    assert rl["share"] == pytest.approx(3.2 / 6.3, rel=1e-3)
    assert rl["traffic"] == pytest.approx(cells * 82.5)
    fp = rl["fp64_pipe"]
    assert fp["peak_gops"] == pytest.approx(2 * 152 * 2070e6 / 1e9, rel=1e-3)
    assert fp["achieved_gops"] == pytest.approx(49.34 * cells / 3.2e-3 / 1e9, rel=1e-3)
    probe = {"gops": 528.4}
    bench.with_measured_fp64(rl, probe)
    assert fp["frac_of_measured"] == pytest.approx(fp["achieved_gops"] / 528.4, rel=1e-3)
    assert rl["other_kernel"]["fp64_pipe"]["frac_of_measured"] == pytest.approx(
        47.64 * cells / 3.1e-3 / 1e9 / 528.4, rel=1e-3)


def test_roofline_without_operation_counts_has_no_fp64_block():
    rl = bench.roofline({0: [1.0], 1: [2.0]}, 1000, 4, 6793.8, "measured", {0: "a", 1: "b"}, {}, sm_mhz=2070.0)
    assert "fp64_pipe" not in rl and rl["traffic"] is None
    bench.with_measured_fp64(rl, {"gops": 500.0})  # nothing to add
    assert "fp64_pipe" not in rl
