"""Host-side checks of the benchmark's bookkeeping (no GPU)."""
import bench


def test_kernel_counters_match_the_kernel_source():
    """bench.KERNEL_COUNTERS (FP64 instructions and DRAM bytes per environment from an ncu
    capture) describe one version of the fused sweep; when its generated source or device
    headers change, the capture must be redone and KERNEL_SOURCE_SHA256 updated."""
    _, pm = bench.make_model()
    assert bench.kernel_source_digest(pm) == bench.KERNEL_SOURCE_SHA256


def test_algorithmic_flop_counts_are_consistent():
    robot, _ = bench.make_model()
    a = bench.algorithmic_flops(robot)
    assert a == bench.algorithmic_flops(robot)  # deterministic
    parts = a["fk"] + a["jacobian"] + a["crba"] + a["rnea"] + a["aba"]
    assert 0 < a["step"] < parts
    assert a["rnea+aba"] < a["rnea"] + a["aba"]
    assert a["transcendental_calls_per_step"] == 14  # sin and cos of 7 revolute joints


def test_both_arms_name_the_same_workload():
    robot, _ = bench.make_model()
    c = bench.workload_config(bench.N_ENVS, robot.nv, len(robot.link_names))
    assert c["n_envs_per_gpu"] == 16384 and c["nv"] == 9
