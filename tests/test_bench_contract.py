"""bench.py on the CPU: the reference arm's JSON line (it times the
reference's walk, tiny_mc.c:47-49, on the host cores; no GPU), its silence on
ranks other than 0, the clock record's parsing, and the roofline constants'
source hash."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _run(args, env=None):
    e = dict(os.environ)
    e.update(env or {})
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, cwd=ROOT, env=e,
                       capture_output=True, text=True, timeout=240)
    return r


def test_reference_arm_line():
    r = _run(["--impl", "reference", "--steps", "1", "--warmup", "0"])
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config"):
        assert k in line, k
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["value"] > 0 and line["higher_is_better"] is True
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"],
                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert line["config"]["workload"].startswith("plain walk")


def test_reference_arm_other_ranks_exit_quietly():
    r = _run(["--impl", "reference", "--steps", "1", "--warmup", "0"],
             env={"RANK": "1", "WORLD_SIZE": "2"})
    assert r.returncode == 0 and r.stdout.strip() == ""


class _FakeProc:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def test_clock_record_parsing():
    c = bench.ClockSampler(None)
    c.proc = _FakeProc()
    c.lines = [
        "2070, 2070, 510.2, 0x0, Not Active, Not Active, Not Active, Not Active",
        "2055, 2070, 590.6, 0x4, Not Active, Not Active, Not Active, Active",
        "2070, 2070, 575.0, 0x0, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
    ]
    rec = c.stop()
    assert rec["sm_mhz"] == 2070.0 and rec["sm_max_mhz"] == 2070.0
    assert rec["power_w_max"] == 590.6 and rec["samples"] == 3
    assert rec["reasons"] == ["sw_power_cap"]


def test_roofline_constants_match_sources():
    """The ncu figures bench.py reports as this build's are from a capture of
    the current walk sources (otherwise it labels them stale)."""
    assert bench.walk_sources_sha256() == bench.NCU_WALK["sources_sha256"]
    with open(os.path.join(ROOT, bench.NCU_WALK["capture"])) as f:
        assert bench.NCU_WALK["sources_sha256"] in f.read()
