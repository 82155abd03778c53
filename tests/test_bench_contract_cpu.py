"""bench.py's output contract, checked without a GPU through the reference
arm (the CPU restatement of the method): one JSON line with the metric,
unit and the keys the reference line must carry."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(*args):
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), *args], capture_output=True, text=True,
                         timeout=600, cwd=REPO)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    return json.loads(lines[0])


def test_reference_arm_line():
    import bench
    d = _run("--impl", "reference", "--workload", "dam_break_16k", "--steps", "1", "--warmup", "0")
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["value"] > 0 and d["higher_is_better"] is True and d["n_gpus"] == 1
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["e2e"]["d2h_bytes_per_step"] == 0
    for k in ("steps", "warmup", "ms_per_step", "scaling", "vs_baseline", "dtype", "data", "config"):
        assert k in d
    assert "workload" in d["config"]


def test_reference_arm_maps_only_the_restatement():
    """The reference arm runs the method through the CPU restatement alone:
    the CUDA library of the product is never mapped into its process."""
    code = ("import sys, bench\n"
            "sys.argv = ['bench.py', '--impl', 'reference', '--workload', 'dam_break_16k', '--steps', '1', "
            "'--warmup', '0', '--settle', '2']\n"
            "bench.main()\n"
            "maps = open('/proc/self/maps').read()\n"
            "assert 'libpbf_oracle' in maps\n"
            "assert 'libpbf_gb300' not in maps, 'product library mapped'\n")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=REPO)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads([l for l in out.stdout.splitlines() if l.startswith("{")][0])
    assert line["config"]["sample"] == "all 16384 particles"
    assert "frame 2" in line["config"]["input_state"]


def test_render_reference_arm_line():
    import bench
    d = _run("--impl", "reference", "--workload", "render_1m_1080p", "--steps", "1", "--warmup", "0")
    assert d["impl"] == "reference" and d["metric"] == bench.RENDER_METRIC
    assert d["unit"] == "ms" and d["higher_is_better"] is False and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port"


def test_voxelize_reference_arm_line():
    import bench
    d = _run("--impl", "reference", "--workload", "voxelize_mesh", "--steps", "1", "--warmup", "0")
    assert d["impl"] == "reference" and d["metric"] == bench.VOXEL_METRIC
    assert d["unit"] == "ms" and d["higher_is_better"] is False and d["value"] > 0
    assert d["config"]["points"] > 10000


def test_neighbor_search_reference_arm_line():
    import bench
    d = _run("--impl", "reference", "--workload", "neighbor_search_16m", "--steps", "1", "--warmup", "0")
    assert d["impl"] == "reference" and d["metric"] == bench.NS_METRIC
    assert d["unit"] == "particles/s" and d["higher_is_better"] is True and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] == 1
