"""bench.py's roofline accounting on the CPU: the algorithmic bytes per cell
of each pass (the compulsory-traffic model every roofline fraction is taken
against) and the per-kernel DRAM traffic read from the committed ncu
summaries."""
import json
import os
import sys

import pytest

from conftest import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_fp32_bytes_per_cell():
    # FP32: pass A derives face offsets and area from the face vectors
    b = bench.bytes_per_cell(4)
    assert b == {"faces": 16 + 16 + 24 + 48 + 4,           # W, topo, S -> FS, dt
                 "flux": 16 + 24 + 48 + 16,                 # topo, S, FS -> res
                 "smooth": 16 + 16 + 16 + 16,               # topo, src, res -> dst
                 "update": 16 + 16 + 16 + 4 + 4 + 16 + 16}  # topo, src, res, dt, area, W0 -> W
    # one cell-stage with the reference's two smoothing sweeps: one k_smooth
    assert b["faces"] + b["flux"] + b["smooth"] + b["update"] == 364


def test_fp64_bytes_per_cell():
    # FP64 also reads the host face offsets (R) and the area in pass A
    b = bench.bytes_per_cell(8)
    assert b["faces"] == 32 + 16 + 48 + 48 + 8 + 96 + 8
    assert b["flux"] == 16 + 48 + 96 + 32
    assert b["smooth"] == 16 + 3 * 32
    assert b["update"] == 16 + 32 + 32 + 8 + 8 + 32 + 32


@pytest.mark.parametrize("kernel", ["faces", "flux", "update"])
def test_traffic_from_committed_profiles(kernel):
    with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
        t = json.load(f)[f"k_{kernel}"]
    # the per-cell figure is the capture's read + write over its cell count
    assert t["dram_bytes_per_cell"] == pytest.approx((t["read_mb"] + t["write_mb"]) * 1e6 / t["cells"], rel=1e-4)
    assert os.path.exists(os.path.join(ROOT, t["capture"]))
    n = 4194304
    assert bench.traffic_from_profiles(kernel, n) == pytest.approx(t["dram_bytes_per_cell"] * n)
    # DRAM traffic of a launch is at least its compulsory reads (writes may stay in L2)
    assert t["read_mb"] * 1e6 / t["cells"] >= 0.99 * {"faces": 56, "flux": 88, "update": 72}[kernel]


def test_unknown_kernel_has_no_traffic():
    assert bench.traffic_from_profiles("nonexistent", 1000) is None


def test_integral_errors():
    i32 = {"cl": 0.25, "cd": 0.01, "mass": 1000.0, "mass_flux_far": 1e-3, "mass_flux_wall": 0.0}
    i64 = {"cl": 0.2501, "cd": 0.0101, "mass": 1000.0, "mass_flux_far": 2e-3, "mass_flux_wall": 1e-17}
    e = bench.integral_errors(i32, i64)
    assert set(e) == set(i32)
    assert e["cl"]["abs_err"] == pytest.approx(1e-4) and e["mass"]["abs_err"] == 0.0
    assert e["mass_flux_far"] == {"fp32": 1e-3, "fp64": 2e-3, "abs_err": 1e-3}


def test_reference_arm_does_not_load_the_product_library():
    """--impl reference times the oracle's CPU port on the oracle's own
    statement of the mesh; the product package and its library stay
    unloaded in that process."""
    import subprocess
    code = ("import sys, bench\n"
            "sys.argv = ['bench.py', '--impl', 'reference', '--workload', 'transonic', '--steps', '1', '--warmup', '3']\n"
            "bench.main()\n"
            "assert 'gpueularsolver2d_gb300' not in sys.modules\n"
            "maps = open('/proc/self/maps').read()\n"
            "assert 'libeuler2d' not in maps and 'liboracle' in maps\n")
    res = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr[-2000:]
    line = json.loads(res.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["dtype"] == "f64" and line["cpu_baseline"]["cpu_model"]
