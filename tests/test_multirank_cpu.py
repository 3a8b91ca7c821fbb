"""bench.py's multi-GPU contract on CPU with gloo, world size 2: every rank
renders its own replica, the job's time is the slowest rank's (a MAX
all-reduce) and the value counts all ranks' units; the reference arm runs
on rank 0 alone."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank r took r + 1 seconds for 3 M units
    v, secs = bench.whole_job_rate(dist, world, 3_000_000, float(rank + 1))
    (Path(out_dir) / f"r{rank}.txt").write_text(f"{v} {secs}")
    dist.barrier()
    dist.destroy_process_group()


def test_whole_job_rate_takes_the_slowest_rank(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    for r in (0, 1):
        v, secs = map(float, (tmp_path / f"r{r}.txt").read_text().split())
        assert secs == 2.0              # the slower rank's time on both ranks
        assert v == pytest.approx(2 * 3.0 / 2.0)  # all ranks' units / that time


def test_single_rank_rate():
    sys.path.insert(0, str(ROOT))
    import bench
    v, secs = bench.whole_job_rate(None, 1, 5_000_000, 2.5)
    assert (v, secs) == (2.0, 2.5)


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun every rank but 0 exits 0 without work or output."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "1"],
                       capture_output=True, text=True, env=env, timeout=120, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_committed_profile_only_for_its_scene_and_layout():
    sys.path.insert(0, str(ROOT))
    import json
    import bench
    d = json.loads((ROOT / "profiles" / "traffic.json").read_text())
    got = bench.committed_profile("k_shadow", d["scene"], d["bvh_width"])
    bpr = got["dram_bytes_per_ray"]
    assert bpr == d["k_shadow"]["dram_bytes_per_ray"] and min(bpr) > 0
    assert all(0 < h <= 100 for h in got["l2_hit_rate_pct"])
    assert all(1 <= t <= 32 for t in got["threads_per_warp_inst"])
    assert bench.committed_profile("k_shadow", "cornell", d["bvh_width"]) is None
    assert bench.committed_profile("k_shadow", d["scene"], 2) is None
    assert bench.committed_profile("k_nothing", d["scene"], d["bvh_width"]) is None
    # each launch takes its bounce's bytes per ray, later ones the last bounce's
    rays = [1000, 100, 10, 10, 1]
    want = (1000 * bpr[0] + 100 * bpr[1] + 10 * bpr[2] + 10 * bpr[2] + bpr[2]) / 5
    assert abs(bench.scaled_traffic(got, rays) - want) < 1e-6 * want
    w = bench.time_weighted(got, "l2_hit_rate_pct")
    assert min(got["l2_hit_rate_pct"]) <= w <= max(got["l2_hit_rate_pct"])


def test_any_hit_total_sums_both_any_hit_kernels():
    """The bench's any-hit summary: algorithmic bytes (node visits x node
    size + triangle tests x 48 B) over device time, for the per-lane kernel,
    the packet launches and both together."""
    sys.path.insert(0, str(ROOT))
    import bench
    log = {"any": [{"ms": 10.0, "rays": 100, "nodes": 1000, "tris": 200},
                   {"ms": 30.0, "rays": 300, "nodes": 3000, "tris": 600}],
           "any_packets": [{"ms": 10.0, "rays": 50, "nodes": 800, "tris": 100}],
           "shade": [{"ms": 99.0, "rays": 0, "nodes": 0, "tris": 0}]}
    got = bench.any_hit_total(log, 128, 1000.0)
    lane = 4000 * 128 + 800 * 48
    assert got["k_shadow"]["rays"] == 400 and got["k_shadow"]["ms"] == 40.0
    assert abs(got["k_shadow"]["achieved_gbs"] - lane / 0.04 / 1e9) < 1e-12
    assert got["together"]["rays"] == 450 and got["together"]["ms"] == 50.0
    both = lane + 800 * 128 + 100 * 48
    assert abs(got["together"]["algorithmic_bytes"] - both) < 1e-6
    assert abs(got["together"]["frac"] - both / 0.05 / 1e9 / 1000.0) < 1e-12
    # no packet launches (packets off): zero rays, no rate
    off = bench.any_hit_total({"any": log["any"]}, 128, 1000.0)
    assert off["k_shadow_packet"] == {"rays": 0, "ms": 0.0, "algorithmic_bytes": 0.0,
                                      "achieved_gbs": None, "frac": None}
