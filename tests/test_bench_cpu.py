"""bench.py without a GPU: the workloads' sizes and the reference arm's JSON line
(the CPU oracle on host cores, run as the benchmark's own subprocess)."""
import json
import subprocess
import sys

import numpy as np

import bench


def test_workload_sizes():
    k, om = bench.workload_points(bench.WORKLOADS["arc_n112"])
    assert k.shape == (201 * 201, 2) and om.shape == (1,)
    k, om = bench.workload_points(bench.WORKLOADS["ss_n40"])
    assert k.shape == (101, 2) and om.shape == (201,)
    k, om = bench.workload_points(bench.WORKLOADS["ss_n264"])
    assert k.shape == (301, 2) and om.shape == (501,)
    assert np.isclose(om[0], -0.5 * bench.EV2HARTREE) and np.isclose(om[-1], 0.5 * bench.EV2HARTREE)
    wl = bench.WORKLOADS["uneven4"]
    assert [nw * np_ for nw, np_ in wl["shapes"]] == [16, 40, 112, 264]
    assert [nw * np_ for nw, np_ in bench.WORKLOADS["serve8"]["shapes"]] == [8, 32, 60, 120, 112,
                                                                            150, 264, 300]


def test_max_rel():
    ref = {n: np.array([1.0, -2.0, 4.0]) for n in bench.NAMES}
    got = {n: v * (1 + np.array([0.0, 1e-6, -2e-6])) for n, v in ref.items()}
    r = bench.max_rel(got, ref)
    assert set(r) == set(bench.NAMES) and all(abs(v - 2e-6) < 1e-12 for v in r.values())


def test_reference_arm_line():
    """`bench.py --impl reference` prints one JSON line with the arm's contract keys."""
    out = subprocess.run([sys.executable, str(bench.ROOT / "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "3", "--ref-per-core", "1"],
                         capture_output=True, text=True, timeout=600, cwd=str(bench.ROOT))
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC
    assert line["unit"] == "solves/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["steps"] == 1 and line["warmup"] == 3
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
