"""CPU tests of bench.py's multi-replica path (one process per GPU under
torchrun): the slowest rank's time is what every rank reports, each replica
reconstructs its own seeded scan, and the reference arm runs on rank 0 only.
The ranks here are gloo processes on the host; no GPU is used."""
import ast
import ctypes as C
import os
import subprocess
import sys

import pytest

from tests.conftest import REPO

torch = pytest.importorskip("torch")
dist = pytest.importorskip("torch.distributed")


def _rank_main(rank, world, port, out_path):
    sys.path.insert(0, REPO)
    import torch.distributed as d

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    d.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = [12.5, 40.25][rank]
    slowest = bench.max_over_ranks(local_ms, d, device="cpu")
    seed = bench.replica_seed(1234, rank)
    gathered = [None] * world
    d.all_gather_object(gathered, seed)
    d.barrier()
    d.destroy_process_group()
    with open("%s.%d" % (out_path, rank), "w") as f:
        f.write("%r %r\n" % (slowest, gathered))


def test_max_over_ranks_and_seeds_with_two_gloo_ranks(tmp_path):
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "rank")
    mp.start_processes(_rank_main, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    for r in range(2):
        slowest, seeds = open("%s.%d" % (out, r)).read().split(" ", 1)
        assert float(slowest) == 40.25
        seeds = ast.literal_eval(seeds.strip())
        assert len(set(seeds)) == 2  # each replica its own scan


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""


def test_served_stream_scans_plan_and_fit(lib):
    """The served-stream workload's scans (bench.serve_spec): every draw plans,
    covers its slices and has a whole-scan footprint under the 150 GB budget."""
    import tempfile

    import numpy as np

    import bench
    from ctbangbang_gb300 import lib as L
    from ctbangbang_gb300 import scans
    rng = np.random.default_rng(1000 * bench.SERVE_CONFIG)
    modes = set()
    for i in range(8):
        spec = bench.serve_spec(rng, i, False)
        assert spec.turns <= 8.5 and 4 <= spec.n_slices <= 120
        modes.add((spec.z_ffs, spec.phi_ffs))
        with tempfile.TemporaryDirectory() as d:
            mr = scans.plan_spec(spec, d)
            need = L.load().ctbb_scan_workspace_bytes(C.byref(mr))
            assert 0 < need < (150 << 30)
            assert mr.ri.n_blocks >= 1
            scans.free_plan(mr)
    assert len(modes) >= 3


def test_reference_arm_line_keeps_the_contract():
    """The reference arm (the reference CPU path as the bit-exact port, on the
    host cores) prints one JSON line with the contract's keys, and never maps
    the reconstruction library: it plans with the oracle and projects its
    input with the test library's CPU projector.  Run on the small no-FFS
    workload to stay quick."""
    import json
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        env.pop(k, None)
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--config', 'config1', "
            "'--steps', '1', '--warmup', '0']; runpy.run_path(%r, run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); "
            "print('MAPPED', 'libctbb_gb300.so' in maps, 'libctbb_oracle.so' in maps)"
            % os.path.join(REPO, "bench.py"))
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=900,
                       cwd=REPO)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "MAPPED False True" in r.stdout, r.stdout[-500:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["metric"] == d["unit"] == "voxel-updates/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["vs_baseline"] is None
    assert d["config"]["workload"].startswith("config1: 672 ch x 16 rows no FFS")
    assert d["config"]["composed_scan_seconds"] > 0 and d["ms_per_step"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "voxel-updates/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
