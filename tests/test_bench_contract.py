"""bench.py's JSON line: the keys and units every run must print.

The reference arm (--impl reference: the oracle's OpenMP CPU path) runs here
on the CPU; the library's arm needs the GPU (marked). Small workloads and
short budgets keep each run to seconds.
"""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench(args, env_extra, timeout=600):
    env = dict(os.environ, **env_extra)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=timeout)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    return [json.loads(ln) for ln in lines]


def _common(line, steps_max):
    import bench
    assert line["metric"] == bench.METRIC
    assert line["unit"] == "MLUPS" and line["value"] > 0
    assert line["higher_is_better"] is True and line["scaling"] == "weak"
    assert line["vs_baseline"] is None
    assert line["dtype"] in ("f64", "f32", "f16", "bf16", "int64")
    assert 1 <= line["steps"] <= steps_max and line["warmup"] >= 3
    assert "workload" in line["config"]
    cb = line["cpu_baseline"]
    assert set(cb) >= {"value", "unit", "cores", "kind", "sample"}
    assert cb["kind"] == "port" and cb["unit"] == "MLUPS" and cb["cores"] >= 1
    e2e = line["e2e"]
    assert set(e2e) >= {"value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"}
    assert e2e["unit"] == "MLUPS" and e2e["value"] > 0


def test_reference_arm_line(built):
    sys.path.insert(0, ROOT)
    (line,) = _bench(["--impl", "reference", "--workload", "cylinder_d2q9_1024x512",
                      "--steps", "4", "--warmup", "3"], {"IMEXLB_REF_BUDGET_S": "5"})
    _common(line, 4)
    assert line["impl"] == "reference" and line["n_gpus"] == 1
    # the same label the library arm prints for FP64 storage of this lattice
    import bench
    assert line["config"]["workload"] == "cylinder_d2q9_1024x512_fp64"
    assert line["config"]["workload"] == bench.workload_label("cylinder_d2q9_1024x512", "fp64")
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["e2e"]["value"] == line["value"] == line["cpu_baseline"]["value"]


def test_reference_arm_other_ranks_print_nothing(built):
    out = _bench(["--impl", "reference", "--workload", "cylinder_d2q9_1024x512", "--steps", "2"],
                 {"RANK": "1", "WORLD_SIZE": "2", "IMEXLB_REF_BUDGET_S": "5"})
    assert out == []


@pytest.mark.gpu
@pytest.mark.parametrize("workload,precision", [("sphere_d3q27_128x64x64", "fp64"),
                                                ("cylinder_d2q9_1024x512", "fp16")])
def test_library_arm_line(built, workload, precision):
    sys.path.insert(0, ROOT)
    (line,) = _bench(["--workload", workload, "--precision", precision, "--steps", "6",
                      "--warmup", "3"], {"IMEXLB_CPU_BUDGET_S": "2"})
    _common(line, 6)
    assert "impl" not in line and line["n_gpus"] == 1
    import bench
    assert line["config"]["workload"] == bench.workload_label(workload, precision)
    assert line["ms_per_step"] > 0
    roof = line["roofline"]
    assert set(roof) >= {"bound", "achieved", "peak", "unit", "frac", "traffic"}
    assert roof["bound"] == "hbm" and roof["unit"] == "GB/s"
    assert 0 < roof["frac"] == pytest.approx(roof["achieved"] / roof["peak"], rel=1e-3)
    assert line["e2e"]["h2d_bytes_per_step"] > 0 and line["e2e"]["d2h_bytes_per_step"] > 0
    if not workload.startswith("cylinder"):
        # the link bound beside the upload / download rates
        assert set(line["e2e"]["link_gbs"]) == {"h2d", "d2h"}
        assert min(line["e2e"]["link_gbs"].values()) > 0
        assert min(line["e2e"]["copy_gbs"].values()) > 0
    # one launch per iteration with the boundary copies inside the step kernel
    assert line["gpu_launches"] >= line["steps"]
    assert "clocks" in line
    if workload.startswith("sphere") and precision == "fp64":
        # the fixed-point and FP16 kinds measured beside the bitwise headline
        for v in ("fix64", "fp16"):
            var = line["variants"][v]
            assert var["value"] > 0 and var["e2e"]["value"] > 0 and 0 < var["roofline_frac"]
    l2 = line["config"]["l2"]
    if precision == "fp16" and workload.startswith("cylinder"):
        assert l2.startswith("L2 flushed")
    else:
        assert l2.startswith("inputs larger than L2")
