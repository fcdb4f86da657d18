"""The benchmark's reference arm and its JSON line (CPU only): `bench.py --impl
reference` times the reference's own CPU render path (or the oracle port where the
reference is not staged) on a bounded sample of the workload and prints one line with
the keys the GPU arm's line carries; ranks other than 0 print nothing. Also the
algorithmic queue-byte count behind the whole-wavefront roofline."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(extra_env=None, *args):
    env = dict(os.environ)
    env.update(extra_env or {})
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2", "--warmup", "1",
           "--grid", "33", "--cpu-sample-res", "32", *args]
    return subprocess.run(cmd, capture_output=True, text=True, env=env, cwd=ROOT, timeout=600)


def test_reference_arm_prints_one_contract_line():
    r = _run()
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    out = json.loads(lines[0])
    assert out["impl"] == "reference"
    assert out["metric"] == "Mpaths/s" and out["unit"] == "Mpaths/s" and out["higher_is_better"] is True
    assert out["value"] > 0 and out["steps"] == 2 and out["warmup"] == 1 and out["n_gpus"] == 1
    assert out["ms_per_step"] > 0
    cb = out["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == out["value"]
    assert out["e2e"] == {"value": out["value"], "unit": "Mpaths/s", "h2d_bytes_per_step": 0,
                          "d2h_bytes_per_step": 0}
    assert "terrain 33x33 grid" in out["config"]["workload"]


def test_reference_arm_other_ranks_exit_without_output():
    r = _run({"RANK": "1", "WORLD_SIZE": "2"}, "--gpus", "2")
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""


def test_wavefront_bytes():
    sys.path.insert(0, ROOT)
    import bench
    # one camera path whose single extension ray ends it: 56 B written by generate,
    # 52 B through traversal, 76 B read by shade, nothing continues
    assert bench.wavefront_bytes(1, 1, 0) == 56 + 52 + 76
    # a second segment adds a continuing 56 B path and another 52 + 76 B; a shadow
    # record is 56 B written and 48 B read
    assert bench.wavefront_bytes(1, 2, 1) == 56 + 2 * (52 + 76) + 56 + 56 + 48
    assert bench.wavefront_bytes(10, 25, 7) == 10 * 56 + 25 * 128 + 15 * 56 + 7 * 104
