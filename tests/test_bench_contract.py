"""The benchmark's host side on the CPU.  The reference arm, run with a small
volume and a small receiver sample, keeps the keys and units of the
benchmark contract in its JSON line, and under a multi-rank launch only rank
0 prints.  The roofline's pair count is exact, and the kernel summaries the
bench reads its DRAM traffic from carry that figure."""
import json
import re
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(env_extra=None):
    env = dict(os.environ)
    env.update(env_extra or {})
    cmd = [sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "3",
           "--size", "48", "--ref-block", "4"]
    return subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=600, cwd=REPO)


def _json_lines(out):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def test_reference_arm_prints_one_contract_line():
    r = _run()
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    d = lines[0]
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["unit"] == "voxels/s" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["unit"] == d["unit"] and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_reference_arm_runs_on_rank_0_only():
    r = _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert _json_lines(r.stdout) == []


def test_pair_count_is_exact():
    """The roofline's algorithmic work counts in-bounds (receiver, voter)
    pairs exactly: against brute force on small volumes, and on a z-slab."""
    import numpy as np
    import bench
    for dims, hw in [((5, 7, 9), 2), ((3, 4, 20), 5), ((1, 1, 1), 3), ((6, 6, 6), 0)]:
        s0, s1, s2 = dims
        z, y, x = np.meshgrid(np.arange(s0), np.arange(s1), np.arange(s2), indexing="ij")
        brute = 0
        for oz in range(-hw, hw + 1):
            for oy in range(-hw, hw + 1):
                for ox in range(-hw, hw + 1):
                    brute += int(((z + oz >= 0) & (z + oz < s0) & (y + oy >= 0) & (y + oy < s1) &
                                  (x + ox >= 0) & (x + ox < s2)).sum())
        assert bench.pairs_count(dims, hw) == brute
    full = bench.pairs_count((12, 5, 5), 3)
    assert bench.pairs_count((12, 5, 5), 3, (0, 4)) + bench.pairs_count((12, 5, 5), 3, (4, 12)) == full


def test_profiles_carry_the_traffic_the_bench_reads():
    """Every kernel summary the bench takes its DRAM traffic from keeps a
    machine-readable per-launch figure and says where it came from (the
    capture and its date), and the bench line carries that source beside the
    figure."""
    import bench
    for kernel, workload in [("k_vote3_fast", "c2"), ("k_vote3_fast", "c4"), ("k_eig3", "c3"),
                             ("k_vote2_tk", "c1"), ("k_st3", "c2")]:
        t = bench.profiled_traffic(kernel, workload)
        assert t["traffic"] is not None and t["traffic"] > 0, (kernel, workload)
        assert t["traffic_source"].startswith(f"profiles/{kernel}_{workload}.md: "), t
        assert re.search(r"20\d\d-\d\d-\d\d", t["traffic_source"]), t
    assert bench.profiled_traffic("k_none", "c9") == {"traffic": None, "traffic_source": None}
