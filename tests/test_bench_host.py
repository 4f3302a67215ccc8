"""Host-side pieces of bench.py that need no GPU: the per-launch DRAM traffic
each pair kernel's roofline line takes from its committed ncu summary, the
workload description and the windows the steps walk through."""
import os
import re

import bench


def test_traffic_of_each_pair_kernel_comes_from_its_profile():
    for kernel, name in bench.PROFILE_OF.items():
        path = os.path.join(bench.ROOT, "profiles", name)
        assert os.path.exists(path), path
        t = bench.traffic_from_profiles(kernel)
        assert t is not None and t > 0
        # the number is the summary's read + write bytes of one launch
        text = open(path).read()
        rd = int(re.search(r"dram__bytes_read \| ([\d ]+) B", text).group(1).replace(" ", ""))
        wr = int(re.search(r"dram__bytes_write \| ([\d ]+) B", text).group(1).replace(" ", ""))
        assert t == rd + wr
    assert bench.traffic_from_profiles(2) is None  # the FP64 kernel is not a roofline line


def test_workload_config_names_the_16k_atom_workload():
    cfg = bench.workload_config({"extra": 1})
    assert cfg["natoms"] == 16384 and cfg["nbin"] == 400 and cfg["rmax"] == 12.0
    assert cfg["reset"] == 1800 and cfg["tmax"] == 200 and cfg["skip"] == 4
    assert cfg["extra"] == 1


def test_step_windows_cover_reset_1800():
    starts = sorted({bench.step_window(s) for s in range(bench.STEP_WINDOWS)})
    assert starts == [200 * k for k in range(bench.STEP_WINDOWS)]
    # a step's window of ORIGINS_PER_STEP origins at the workload's skip is 200 frames
    assert bench.ORIGINS_PER_STEP * 4 == 200
