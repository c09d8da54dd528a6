"""bench.py's reference arm (the FP64 CPU port timed on the host) keeps the
JSON-line contract: one line from rank 0, the same metric and config as the
GPU arm, a cpu_baseline describing the run and an e2e entry without copies;
the process never loads the GPU library.  Runs on a 20,000-node graph so that
it finishes in seconds."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
ARGS = ["--impl", "reference", "--nodes", "20000", "--steps", "1", "--warmup", "1"]


def _lines(out):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def _check(line):
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "e2e",
                "cpu_baseline"):
        assert key in line, key
    assert line["impl"] == "reference"
    assert line["metric"] == "stpm_node_updates_per_s" and line["unit"] == "node-updates/s"
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["config"]["workload"].startswith("mmsb-n200k-k100") and line["config"]["n"] == 20000
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == line["value"] and cb["cores"] >= 1 and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), *ARGS], capture_output=True,
                         text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = _lines(out.stdout)
    assert len(lines) == 1
    _check(lines[0])


def test_reference_arm_does_not_load_the_gpu_library():
    code = ("import runpy, sys; sys.argv = ['bench.py'] + %r; "
            "runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); "
            "print('LOADED', 'libmmsb' in maps, 'mmsb_gb300' in sys.modules)") % (ARGS,)
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                         timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    assert "LOADED False False" in out.stdout
    assert len(_lines(out.stdout)) == 1


def test_reference_arm_under_torchrun_prints_once():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
           "--gpus", "2", *ARGS]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=900, cwd=ROOT, env=env)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = _lines(out.stdout)
    assert len(lines) == 1
    _check(lines[0])
    assert lines[0]["n_gpus"] == 2


def _dist_rank(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE="2", LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    d = bench.Dist(2)
    d.barrier()
    q.put((rank, d.max(1.5 + rank), d.max(-rank)))
    d.close()


def test_dist_barrier_and_max_over_two_gloo_ranks():
    """The replicas' timing is the max over ranks (host-side gloo)."""
    import multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_dist_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2.5, 0.0), (1, 2.5, 0.0)]
