"""The bench's roofline `traffic` comes from the committed ncu summary of the psi
sweep: the summary must name the launch shape the bench measures (3 fused
sweeps, 17-row strips on 2049^2) and a DRAM traffic per launch below the
algorithmic bytes of its three node-sweeps and of the order of the bytes a
launch moves once (psi, rhs, link pair, code, three writes; L2 keeps part of
the writes).  The bounded states/s sample of the default line draws its instances
from the field sweep itself.  No GPU needed."""
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


def test_states_sample_instances_are_the_field_sweeps_own():
    """The default line's bounded states/s sample takes instances of the seeded field
    sweep unchanged: instance k of the sample is the k-th sweep instance whose side is
    at most the bound, drawn from the same generator."""
    import numpy as np
    sample = bench.states_instances_bounded(12, 257)
    sweep = [it for it in bench.states_instances(60) if it.n <= 257][:12]
    assert len(sample) == 12 and all(it.n <= 257 for it in sample)
    for a, b in zip(sample, sweep):
        assert a.n == b.n and a.H == b.H and a.kappa == b.kappa
        assert np.array_equal(a.mt, b.mt) and np.array_equal(a.psi0, b.psi0)
