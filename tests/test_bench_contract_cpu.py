"""bench.py's reference arm on the CPU: one step of the reference loop's port on
its bounded sample, printed as the single JSON line the benchmark contract asks
for, with the metric, unit and direction of the GPU arm (so the two lines can
be divided), its CPU-baseline description, and an e2e block with no copies."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    assert line["metric"] == "radiality voxel-volumes/s" and line["unit"] == "voxel-volumes/s"
    assert line["higher_is_better"] is True and line["n_gpus"] == 1
    assert line["steps"] == 1 and line["warmup"] == 0
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert line["config"]["workload"].startswith("mid:")
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_temporal_roofline_block():
    """The bench line's temporal-kernel block: T radiality and T intensity values
    read and one map value written per subvoxel, over the mean launch time,
    against the measured copy bandwidth (absent without timings)."""
    sys.path.insert(0, str(ROOT))
    import bench
    units, T = 512 * 512 * 128 * 100, 100
    r = bench.temporal_roofline([6.0, 7.0], units, T, {"hbm_gbs": 6782.1})
    vox = units // T
    assert r["algorithmic_bytes"] == vox * (2 * T * 4 + 4)
    assert abs(r["kernel_ms"] - 6.5) < 1e-12
    assert abs(r["achieved_gbs"] - r["algorithmic_bytes"] / 6.5e-3 / 1e9) < 1e-6
    assert abs(r["frac"] - r["achieved_gbs"] / 6782.1) < 1e-12
    assert bench.temporal_roofline([], units, T, {}) == {}
    assert bench.temporal_roofline([6.0], units, T, {})["frac"] is None
