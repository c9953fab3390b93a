"""The bench's roofline `traffic` comes from the committed ncu summary of the psi
sweep: the summary must name the launch shape the bench measures (3 fused
sweeps, 17-row strips on 2049^2) and a DRAM traffic per launch below the
algorithmic bytes of its three node-sweeps and of the order of the bytes a
launch moves once (psi, rhs, link pair, code, three writes; L2 keeps part of
the writes).  No GPU needed."""
import bench


def test_profile_traffic_matches_the_bench_launch_shape():
    t = bench.ncu_traffic("fp32", 3, 17)
    assert t is not None
    n = 2049 * 2049
    once = n * (8 + 8 + 16 + 1 + 3 * 8)          # each input read once, three sweeps written
    algorithmic = 3 * n * 33
    assert 0.5 * once < t < algorithmic
    # another launch shape has no committed capture: the bench reports null, not a stale figure
    assert bench.ncu_traffic("fp32", 3, 12) is None
