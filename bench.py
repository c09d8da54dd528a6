"""Benchmark of the MMSB tensor-method pipeline on GB300.

Workload (the GPU-at-scale configuration of the reference path): synthetic MMSB
graph with n = 200,000 nodes in four equal random partitions, k = 100,
alpha0 = 0.1, B = 0.05 on the diagonal and 5e-4 off it, int32 CSR; FP32
whitening (Gaussian sketch panels), online STPM for 20 sweeps with minibatch
4,096 and beta_t = 1/(1+t), then unwhitening + normalisation + community sets.

One step = one full pass of the pipeline (whitening, whitened data, 20 STPM
sweeps, unwhitening) over the resident graph.  value = STPM node-updates per
second of the whole job (n_X * sweeps per step / step time).  e2e = the same
through the public C ABI with pinned host buffers: graph upload (H2D), run, Pi
and lambda download (D2H) inside the timed region.

--impl reference times the FP64 CPU restatement of the reference path
(oracle/mmsb_oracle.py) on all host threads, whole pipelines per step, on the
same graph (generated by oracle/mmsb_gen.c without the GPU library).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent

# independent graphs' streams (batched solver) run concurrently only on
# separate hardware work queues; the runtime default is 8 (read when the
# CUDA context is created, so this must precede the first CUDA call)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

WORKLOAD = dict(name="mmsb-n200k-k100-fp32-online", n=200_000, k=100, alpha0=0.1, p_in=0.05,
                p_out=5e-4, sweeps=20, minibatch=4096, seed=0)


# the batching configuration: many independent graphs of uneven size and k
BATCH = dict(name="mmsb-batch256-n2k-200k-k5-64-online", graphs=256, n_lo=2_000, n_hi=200_000,
             k_lo=5, k_hi=64, a0_lo=0.1, a0_hi=2.0, b_lo=0.05, b_hi=0.3, sweeps=5,
             steps_per_sweep=8, degree_cap=30, seed=0)


# the precision configuration: the BF16 form beside the FP32 form, errors of
# both against an FP64 STPM and post-processing
PRECISION = dict(name="mmsb-n2m-k200-bf16-online", n=2_000_000, k=200, alpha0=0.5, p_in=0.02,
                 p_out=1e-5, sweeps=30, minibatch=65536, seed=0)


def load_pkg():
    sys.path.insert(0, str(ROOT))
    import __graft_entry__ as ge
    return ge._package()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Host-side barrier and max-reduction over replicas (gloo, CPU tensors)."""

    def __init__(self, ws):
        self.ws = ws
        self.dist = None
        if ws > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, v):
        if not self.dist:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index, out_path=None):
        self.gpu = gpu_index
        self.out_path = out_path
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        if self.out_path:
            Path(self.out_path).write_text("\n".join(self.lines) + "\n")
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_graph(mm, wl):
    return mm.generate(wl["n"], wl["k"], wl["alpha0"], wl["p_in"], wl["p_out"], wl["seed"])


def peaks():
    """Roofline denominators: the measured copy bandwidth and bf16 GEMM rate
    (sustained: every kernel here is timed inside a long pipeline step)."""
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d.get("hbm_gbs", 6800.0),
                "tflops": d.get("bf16_tflops_sustained", d.get("bf16_tflops", 1700.0)),
                "source": "measured (hbm copy; bf16 GEMM sustained)"}
    return {"hbm_gbs": 6800.0, "tflops": 1700.0, "source": "fallback"}


# DRAM bytes (read + write) per launch of the STPM kernels, from the ncu
# capture summarised in profiles/stpm_kernels_n200k_k100_full.md (this
# workload: k = 100, 4,096-node minibatches)
NCU_TRAFFIC_PER_LAUNCH = {"stpm_step_kernel": 436480, "stpm_contract_kernel": 5017344}


# ---------------------------------------------------------------------------

def oracle_module():
    sys.path.insert(0, str(ROOT / "oracle"))
    import mmsb_oracle as O
    O.FAST_GS = True  # blocked Gram-Schmidt (same result to round-off)
    O.SPMM_THREADS = os.cpu_count() or 1  # sparse products over all host threads
    return O


class CpuPort:
    """The FP64 oracle port of the reference path on the host cores.

    pipeline() runs and times one whole pipeline: whitening (Gaussian sketch
    panels), whitened data, `sweeps` sweeps of minibatch STPM with the per-step
    QR, lambda and unwhitening + normalisation.  Sparse products run row-split
    over all host threads, dense ones in the BLAS threads."""

    def __init__(self, wl, graph):
        self.O, self.wl, self.graph = oracle_module(), wl, graph
        self.blocks = graph.scipy_blocks()
        self.times = []

    def pipeline(self):
        O, wl = self.O, self.wl
        Gxa, Gxb, Gxc, Gba, Gca = self.blocks
        k, a0 = wl["k"], wl["alpha0"]
        rng = np.random.default_rng(wl["seed"])
        nX, nA, nB, nC = self.graph.parts
        t0 = time.perf_counter()
        sk = (rng.standard_normal((nB, 2 * k)), rng.standard_normal((nC, 2 * k)),
              rng.standard_normal((nA, 2 * k)))
        wh = O.second_whiten(Gxa, Gxb, Gxc, k, a0, sk)
        y = O.whitened_data(Gxa, Gxb, Gxc, wh)
        t1 = time.perf_counter()
        phi0 = O.qr_pos(rng.standard_normal((k, k)))
        lam, phi, _ = O.stpm_online(y, a0, phi0, sweeps=wl["sweeps"], minibatch=wl["minibatch"])
        t2 = time.perf_counter()
        O.postprocess(Gxa, Gba, Gca, wh, lam, phi)
        t3 = time.perf_counter()
        self.times.append((t1 - t0, t2 - t1, t3 - t2))
        return t3 - t0

    def sample(self, n):
        w, s_, p = (statistics.median(t[i] for t in self.times[-n:]) for i in range(3))
        return (f"FP64 numpy/scipy port of the reference path on {os.cpu_count()} host threads, "
                f"{n} whole pipeline(s) timed: whitening {w:.2f}s, {self.wl['sweeps']} STPM sweeps "
                f"{s_:.2f}s, unwhitening {p:.2f}s (medians)")


def flush_host_cache():
    """Writes a 256 MiB buffer (larger than the host's last-level cache)."""
    np.ones(1 << 25, dtype=np.float64).sum()


def config_of(wl, nnz_directed, ws):
    return {"workload": wl["name"], "n": wl["n"], "k": wl["k"], "alpha0": wl["alpha0"],
            "p_in": wl["p_in"], "p_out": wl["p_out"], "sweeps": wl["sweeps"],
            "minibatch": wl["minibatch"], "seed": wl["seed"], "nnz_directed": int(nnz_directed),
            "l2": "256 MiB buffer written between timed steps",
            "parallelism": f"replicas{ws}"}


def run_reference(args, wl, ws, rank):
    """The reference path's CPU implementation (the oracle port; the
    reference's own CPU tree is x86-only source that is not present on the GPU
    host) on the same graph as the GPU arm (oracle/mmsb_gen.c restates the
    library's generator bit for bit, so this process never loads the GPU
    library), whole pipelines per step."""
    if rank != 0:
        return
    sys.path.insert(0, str(ROOT / "oracle"))
    import mmsb_gen
    graph = mmsb_gen.generate(wl["n"], wl["k"], wl["alpha0"], wl["p_in"], wl["p_out"], wl["seed"])
    port = CpuPort(wl, graph)
    for _ in range(args.warmup):
        port.pipeline()
    ts = []
    for _ in range(args.steps):
        flush_host_cache()
        ts.append(port.pipeline())
    step = statistics.mean(ts)
    nX = graph.parts[0]
    v = nX * wl["sweeps"] / step
    line = {"impl": "reference", "metric": "stpm_node_updates_per_s", "value": v,
            "unit": "node-updates/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_of(wl, sum(b.nnz for b in graph.blocks[:3]) * 2, ws),
            "cpu_baseline": {"value": v, "unit": "node-updates/s", "cores": os.cpu_count(),
                             "kind": "port", "sample": port.sample(args.steps)},
            "e2e": {"value": v, "unit": "node-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, wl, ws, rank, local):
    mm = load_pkg()
    dist = Dist(ws)
    graph = make_graph(mm, wl)
    nX = graph.parts[0]
    cfg = mm.default_config(k=wl["k"], alpha0=wl["alpha0"], stpm_method=mm.STPM_ONLINE,
                            sweeps=wl["sweeps"], minibatch=wl["minibatch"], seed=wl["seed"],
                            device=local, tau=0.1)
    p = mm.Pipeline(cfg)
    p.upload(graph)
    for _ in range(args.warmup):
        p.run()
    p.synchronize()
    dist.barrier()
    clocks = ClockSampler(local, Path(args.clocks_csv) if args.clocks_csv else None)
    clocks.start()
    dev_ms, spmm_ms, spmm_bytes, spmm_launch, launches = [], 0.0, 0.0, 0, 0
    orth_passes, orth_err, stpm_steps = 0, 0.0, 0
    kern = {"contract_ms": 0.0, "contract_flops": 0.0, "contract_launches": 0,
            "step_ms": 0.0, "step_flops": 0.0, "step_launches": 0}
    stage = {"whiten_ms": 0.0, "stpm_ms": 0.0, "post_ms": 0.0}
    t_host0 = time.perf_counter()
    for _ in range(args.steps):
        p.flush_l2()
        p.synchronize()
        p.run()
        st = p.stats()
        dev_ms.append(st["total_ms"])
        for key in stage:
            stage[key] += st[key]
        spmm_ms += st["spmm_ms"]
        spmm_bytes += st["spmm_bytes"]
        spmm_launch += st["spmm_launches"]
        launches += st["kernel_launches"]
        orth_passes += st["orth_passes"]
        orth_err = max(orth_err, st["orth_err_max"])
        stpm_steps += st["stpm_steps"]
        for key in kern:
            kern[key] += st[key]
    p.synchronize()
    t_host = time.perf_counter() - t_host0
    dist.barrier()
    clk = clocks.stop()
    step_ms = dist.max(sum(dev_ms) / len(dev_ms))
    nu_per_rank = nX * wl["sweeps"] / (step_ms / 1e3)
    value = nu_per_rank * ws

    # e2e: upload from pinned host buffers + run + Pi/lambda download into a
    # pinned buffer, host wall clock (page-locking happens before the clock)
    h2d = sum(b.row_ptr.nbytes + b.col_idx.nbytes for b in graph.blocks)
    d2h = graph.n_nodes * wl["k"] * 4 + wl["k"] * 8
    graph.pin()
    pi_buf = mm.pin_host(np.empty((wl["k"], graph.n_nodes), np.float32, order="F"))
    e2e_ms = []
    for _ in range(max(1, min(args.steps, 3))):
        p.flush_l2()
        p.synchronize()
        dist.barrier()
        t0 = time.perf_counter()
        p.upload(graph)
        p.run()
        pi = p.pi(out=pi_buf)
        lam = p.lam()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    graph.unpin()
    mm.unpin_host(pi_buf)
    e2e_step = dist.max(statistics.median(e2e_ms))
    e2e_value = nX * wl["sweeps"] / (e2e_step / 1e3) * ws

    # BF16 adjoint form on the same graph: y and Phi in BF16 on the tensor
    # cores for all sweeps but the last (FP32 refinement)
    cfg_bf = mm.default_config(k=wl["k"], alpha0=wl["alpha0"], stpm_method=mm.STPM_ADJOINT,
                               sweeps=wl["sweeps"], minibatch=wl["minibatch"], seed=wl["seed"],
                               device=local, tau=0.1, precision=mm.PREC_BF16)
    pb = mm.Pipeline(cfg_bf)
    pb.upload(graph)
    for _ in range(max(1, min(args.warmup, 2))):
        pb.run()
    bf_ms, bf_stage = [], {"whiten_ms": 0.0, "stpm_ms": 0.0, "post_ms": 0.0}
    for _ in range(args.steps):
        pb.flush_l2()
        pb.synchronize()
        pb.run()
        st = pb.stats()
        bf_ms.append(st["total_ms"])
        for key in bf_stage:
            bf_stage[key] += st[key]
    pb.close()
    bf_step = dist.max(sum(bf_ms) / len(bf_ms))
    bf_value = nX * wl["sweeps"] / (bf_step / 1e3) * ws

    pk = peaks()

    def tensor_entry(name, ms, flops, launches):
        if launches == 0 or ms <= 0:
            return None
        per_launch_ms = ms / launches
        achieved = flops / launches / (per_launch_ms / 1e3) / 1e12
        traffic = NCU_TRAFFIC_PER_LAUNCH.get(name.split(" ")[0])
        return {"kernel": name, "bound": "tensor", "achieved": achieved, "peak": pk["tflops"],
                "unit": "TFLOP/s", "frac": achieved / pk["tflops"], "traffic": traffic,
                "launches_per_step": launches / args.steps, "ms_per_step": ms / args.steps,
                "algorithmic_flops_per_launch": flops / launches, "peak_source": pk["source"]}

    step_rf = tensor_entry("stpm_step_kernel (k x k update + Cholesky QR re-orthonormalisation, "
                           "3xTF32 mma.sync on a KP/8-CTA cluster)", kern["step_ms"],
                           kern["step_flops"], kern["step_launches"])
    contract_rf = tensor_entry("stpm_contract_kernel (Z = Phi^T y, alpha0 terms, G += y^T C; "
                               "3xTF32 tcgen05 kind::tf32, accumulators in tensor memory)",
                               kern["contract_ms"], kern["contract_flops"],
                               kern["contract_launches"])
    spmm_achieved = (spmm_bytes / max(spmm_ms, 1e-9) / 1e6) if spmm_ms > 0 else None
    spmm_rf = {"kernel": "spmm_rows_kernel (whitening CSR SpMM)", "bound": "hbm",
               "achieved": spmm_achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
               "frac": (spmm_achieved / pk["hbm_gbs"]) if spmm_achieved else None,
               "traffic": None, "launches_per_step": spmm_launch / args.steps,
               "ms_per_step": spmm_ms / args.steps,
               "algorithmic_bytes_per_step": spmm_bytes / args.steps,
               "note": "algorithmic bytes count one panel-row gather per nonzero; the 2k-wide "
                       "panels (<= 160 MB) stay largely L2-resident, so frac can exceed 1"}
    # post stage: unwhiten + normProb + threshold (unwhiten_normprob_kernel, one
    # launch per partition block); algorithmic bytes = CSR + one k-float panel
    # row gathered per nonzero + the Pi rows and set words written
    k = wl["k"]
    post_blocks = [graph.blocks[0], graph.blocks[3], graph.blocks[4], graph.blocks[3]]  # X, B, C, A
    post_bytes = 0
    for i, b_ in enumerate(post_blocks):
        rows = b_.n_cols if i == 3 else b_.n_rows  # Pi_A runs over the transpose of G_BA
        post_bytes += 8 * (rows + 1) + 4 * b_.nnz + 4 * k * b_.nnz + rows * (4 * k + 4 * ((k + 31) // 32))
    post_ms = stage["post_ms"] / args.steps
    post_gbs = post_bytes / (post_ms / 1e3) / 1e9 if post_ms > 0 else None
    post_rf = {"kernel": "unwhiten_normprob_kernel (post stage: unwhiten, normProb, threshold)",
               "bound": "hbm", "achieved": post_gbs, "peak": pk["hbm_gbs"], "unit": "GB/s",
               "frac": (post_gbs / pk["hbm_gbs"]) if post_gbs else None, "traffic": None,
               "launches_per_step": 4, "ms_per_step": post_ms,
               "algorithmic_bytes_per_step": post_bytes,
               "note": "the k-wide unwhitening panel (n_A x k FP32) stays L2-resident, so the "
                       "per-nonzero row gathers are L2 traffic and frac can exceed 1; the HBM "
                       "part is the CSR and the Pi / set writes"}
    entries = [e for e in (step_rf, contract_rf, spmm_rf, post_rf) if e]
    dominant = max(entries, key=lambda e: e["ms_per_step"])
    line = {
        "metric": "stpm_node_updates_per_s", "value": value, "unit": "node-updates/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": config_of(wl, sum(b.nnz for b in graph.blocks[:3]) * 2, ws),
        "stages_ms_per_step": {k_: v / args.steps for k_, v in stage.items()},
        "host_wall_ms_per_step": t_host * 1e3 / args.steps,
        "cholesky_qr_passes_per_stpm_step": orth_passes / max(stpm_steps, 1),
        "orth_err_before_first_order_pass_max": orth_err,
        "e2e": {"value": e2e_value, "unit": "node-updates/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_step},
        "gpu_launches": launches,
        "roofline": dominant,
        "roofline_kernels": entries,
        "whitening_spmm_gbs": spmm_achieved,
        "bf16_adjoint": {"value": bf_value, "unit": "node-updates/s", "ms_per_step": bf_step,
                         "stages_ms_per_step": {k_: v / args.steps for k_, v in bf_stage.items()},
                         "over_fp32_online": bf_value / value,
                         "schedule": "BF16 y/Phi contraction for sweeps 1..19, FP32 sweep 20"},
        "clocks": clk,
    }
    if rank == 0 and not args.no_cpu_baseline:
        port = CpuPort(wl, graph)
        t = port.pipeline()
        line["cpu_baseline"] = {"value": nX * wl["sweeps"] / t, "unit": "node-updates/s",
                                "cores": os.cpu_count(), "kind": "port", "sample": port.sample(1)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    p.close()
    dist.close()


def make_batch(mm, wb):
    """n log-uniform, k uniform, alpha0 and the diagonal B uniform, off-diagonal
    = diagonal / 100.  The literal diagonal (up to 0.3) would give up to ~1e9
    edges per graph at n = 200,000, so both probabilities are scaled by one
    factor per graph that caps the expected mean degree at degree_cap."""
    rng = np.random.default_rng(wb["seed"])
    G = wb["graphs"]
    ns = np.exp(rng.uniform(np.log(wb["n_lo"]), np.log(wb["n_hi"]), G)).astype(int)
    ks = rng.integers(wb["k_lo"], wb["k_hi"] + 1, G)
    a0s = rng.uniform(wb["a0_lo"], wb["a0_hi"], G)
    bs = rng.uniform(wb["b_lo"], wb["b_hi"], G)
    def gen(i):
        n, k, b = int(ns[i]), int(ks[i]), float(bs[i])
        deg = n * b / k * (1.0 + (k - 1) / 100.0)
        sc = min(1.0, wb["degree_cap"] / deg)
        return mm.generate(n, k, float(a0s[i]), b * sc, b / 100.0 * sc, seed=wb["seed"] + i)

    from concurrent.futures import ThreadPoolExecutor  # the generator releases the GIL
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        graphs = list(ex.map(gen, range(G)))
    mbs = [max(1, -(-g.parts[0] // wb["steps_per_sweep"])) for g in graphs]
    return graphs, ks, a0s, mbs


def run_batch(args, ws, rank, local):
    """graphs/s of the batched solver (whitening queued concurrently, STPM
    rounds of all graphs in shared launches replayed from a CUDA graph)
    against the same graphs solved one after another; per-graph latency
    percentiles of both."""
    mm = load_pkg()
    wb = dict(BATCH)
    t0 = time.perf_counter()
    graphs, ks, a0s, mbs = make_batch(mm, wb)
    t_gen = time.perf_counter() - t0
    b = mm.Batch(ks, a0s, mbs, stpm_method=mm.STPM_ONLINE, sweeps=wb["sweeps"], seed=wb["seed"],
                 device=local, tau=0.1)
    for i, g in enumerate(graphs):
        b.upload(i, g)
    b.run()  # plans, tunes, captures
    runs = []
    for _ in range(max(1, args.steps)):
        b.run()
        runs.append((b.stats(), b.latencies()))
    st = min(runs, key=lambda r: r[0]["total_ms"])
    bat_ms = statistics.median(r[0]["total_ms"] for r in runs)
    b.run_sequential()  # warm-up of the single-graph path
    b.run_sequential()
    seq = b.stats()
    seq_lat = b.latencies()
    b.close()
    G = wb["graphs"]
    line = {
        "metric": "graphs_per_s", "value": G / (bat_ms / 1e3), "unit": "graphs/s", "n_gpus": ws,
        "steps": args.steps, "warmup": 1, "ms_per_step": bat_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": wb["name"], **{k: v for k, v in wb.items() if k != "name"},
                   "nodes_total": int(sum(g.n_nodes for g in graphs)),
                   "nnz_total": int(sum(sum(bk.nnz for bk in g.blocks[:3]) for g in graphs) * 2),
                   "generation_s": t_gen},
        "batched": {"ms": bat_ms, "latency_p50_ms": st[0]["latency_p50_ms"],
                    "latency_p99_ms": st[0]["latency_p99_ms"],
                    "stpm_end_ms": st[0]["stpm_end_ms"], "wall_ms": st[0]["wall_ms"],
                    "rounds": st[0]["rounds"], "batched_launches": st[0]["batched_launches"],
                    "graph_replayed": st[0]["graph_replayed"],
                    "buckets_kp": st[0]["bucket_kp"], "tuned_ctas": st[0]["bucket_ctas"],
                    "graphs_per_bucket": st[0]["bucket_graphs"]},
        "sequential": {"ms": seq["total_ms"], "graphs_per_s": G / (seq["total_ms"] / 1e3),
                       "latency_p50_ms": float(np.percentile(seq_lat, 50)),
                       "latency_p99_ms": float(np.percentile(seq_lat, 99)),
                       "wall_ms": seq["wall_ms"]},
        "speedup_vs_sequential": seq["total_ms"] / bat_ms,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def _match(A, B):
    """Permutation and signs of B's columns best matching A's (greedy on |cos|)."""
    An = A / np.maximum(np.linalg.norm(A, axis=0), 1e-300)
    Bn = B / np.maximum(np.linalg.norm(B, axis=0), 1e-300)
    C = np.abs(An.T @ Bn)
    perm = -np.ones(A.shape[1], dtype=int)
    used = set()
    for i in np.argsort(-C.max(axis=1)):
        for j in np.argsort(-C[i]):
            if j not in used:
                perm[i] = j
                used.add(j)
                break
    sign = np.sign(np.sum(A * B[:, perm], axis=0))
    sign[sign == 0] = 1
    return perm, sign


def run_precision(args, ws, rank, local):
    """The BF16 form (y in BF16, Phi as a BF16 hi/lo pair, FP32 accumulation,
    all sweeps but the last; the last sweep refines in FP32) beside the FP32
    form on the precision configuration, with the error of lambda, Phi and Pi
    of both against the FP64 oracle's STPM and post-processing run from the
    same Phi0 on the device's whitening (an FP64 whitening of the 100M-edge
    graph is beyond the oracle's single-threaded sparse products)."""
    if rank != 0:
        return
    mm = load_pkg()
    sys.path.insert(0, str(ROOT / "oracle"))
    import mmsb_oracle as O
    wl = dict(PRECISION)
    t0 = time.perf_counter()
    graph = make_graph(mm, wl)
    t_gen = time.perf_counter() - t0
    k, a0, nX = wl["k"], wl["alpha0"], graph.parts[0]
    rng = np.random.default_rng(wl["seed"])
    phi0 = O.qr_pos(rng.standard_normal((k, k)))
    forms, res = {}, {}
    y64 = wh = None
    for name, prec in (("fp32", mm.PREC_FP32), ("bf16", mm.PREC_BF16)):
        cfg = mm.default_config(k=k, alpha0=a0, stpm_method=mm.STPM_ONLINE, sweeps=wl["sweeps"],
                                minibatch=wl["minibatch"], seed=wl["seed"], device=local, tau=0.1,
                                precision=prec)
        with mm.Pipeline(cfg) as p:
            p.upload(graph)
            runs = []
            sp_ms = sp_by = 0.0
            for rep in range(1 + max(1, args.steps)):
                p.flush_l2()
                p.synchronize()
                p.whiten()
                w_ms = p.stats()["whiten_ms"]
                if rep > 0:
                    sp_ms += p.stats()["spmm_ms"]
                    sp_by += p.stats()["spmm_bytes"]
                p.stpm(phi0)
                s_ms = p.stats()["stpm_ms"]
                p.postproc()
                st = p.stats()
                if rep > 0:
                    runs.append((w_ms, s_ms, st["post_ms"]))
            step = statistics.median(sum(r) for r in runs)
            forms[name] = {"value": nX * wl["sweeps"] / (step / 1e3), "unit": "node-updates/s",
                           "ms_per_step": step,
                           "stages_ms": {"whiten_ms": statistics.median(r[0] for r in runs),
                                         "stpm_ms": statistics.median(r[1] for r in runs),
                                         "post_ms": statistics.median(r[2] for r in runs)},
                           "whitening_spmm_gbs": sp_by / max(sp_ms, 1e-9) / 1e6}
            res[name] = (np.asarray(p.lam(), np.float64), np.asarray(p.phi(), np.float64), p.pi())
            if y64 is None:
                y64 = {n_: np.asarray(v, dtype=np.float64) for n_, v in p.whitened().items()}
                wh = p.whitening()
    t1 = time.perf_counter()
    Gxa, _, _, Gba, Gca = graph.scipy_blocks()
    lam_o, phi_o, _ = O.stpm_online(y64, a0, phi0, sweeps=wl["sweeps"], minibatch=wl["minibatch"])
    _, pi_o = O.postprocess(Gxa, Gba, Gca, wh, lam_o, phi_o)
    # the oracle's own response to a 1e-6 relative perturbation of y: how far
    # Phi and Pi are determined by the data at this size (near-degenerate
    # eigenvalues let Phi rotate inside their pairs)
    yp = {n_: (v * (1 + 1e-6 * rng.standard_normal(v.shape)) if n_ in ("Da", "Db", "Dc") else v)
          for n_, v in y64.items()}
    lam_p, phi_p, _ = O.stpm_online(yp, a0, phi0, sweeps=wl["sweeps"], minibatch=wl["minibatch"])
    del yp
    _, pi_p = O.postprocess(Gxa, Gba, Gca, wh, lam_p, phi_p)
    t_oracle = time.perf_counter() - t1
    lam_sorted = np.sort(lam_o)

    def residual(lam, phi):
        """max_i |T(I, phi_i, phi_i) - lambda_i phi_i| / max_j lambda_j in FP64 over all of X."""
        G = O.online_grad_terms(phi, y64, np.arange(nX), a0)
        return float(np.linalg.norm(G - phi * lam, axis=0).max() / np.abs(lam).max())

    def compare(lam, phi, pi):
        perm, sign = _match(phi_o, phi)
        e_pi = 0.0
        for c0 in range(0, pi_o.shape[1], 1 << 20):
            sl = slice(c0, c0 + (1 << 20))
            e_pi = max(e_pi, float(np.abs(pi[perm, sl].astype(np.float64) - pi_o[:, sl]).max()))
        return {"lambda_rel": float(np.linalg.norm(lam[perm] - lam_o) / np.linalg.norm(lam_o)),
                "lambda_rel_sorted": float(np.linalg.norm(np.sort(lam) - lam_sorted)
                                           / np.linalg.norm(lam_o)),
                "phi_max": float(np.abs(phi[:, perm] * sign - phi_o).max()),
                "pi_max": e_pi}

    errors = {}
    for name, r in res.items():
        errors[name] = compare(*r)
        errors[name]["eigen_residual"] = residual(r[0], r[1])
    line = {
        "metric": "stpm_node_updates_per_s", "value": forms["bf16"]["value"],
        "unit": "node-updates/s", "n_gpus": 1, "steps": args.steps, "warmup": 1,
        "ms_per_step": forms["bf16"]["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
        "config": {"workload": wl["name"], **{k_: v for k_, v in wl.items() if k_ != "name"},
                   "nnz_directed": int(sum(b.nnz for b in graph.blocks[:3]) * 2),
                   "generation_s": t_gen},
        "forms": forms, "bf16_over_fp32": forms["bf16"]["value"] / forms["fp32"]["value"],
        "errors_vs_fp64": errors,
        "oracle": {"seconds": t_oracle, "eigen_residual": residual(lam_o, phi_o),
                   "sensitivity_to_1e-6_input_noise": compare(lam_p, phi_p, pi_p),
                   "note": "FP64 STPM + post-processing on the device's whitening from the same "
                           "Phi0; eigen_residual = max_i |T(I,phi_i,phi_i) - lambda_i phi_i| / "
                           "max_j lambda_j over all of X"},
    }
    print(json.dumps(line), flush=True)


# the whitening SpMM where its panel cannot stay in L2: n_X = 500,000, 2k = 400
# panel columns (a 400-float row gathered per nonzero from an 800 MB panel)
SPMM = dict(name="mmsb-spmm-n2m-k200", n=2_000_000, k=200, alpha0=0.5, p_in=0.005, p_out=1e-6,
            sweeps=1, minibatch=65536, seed=0)


def run_spmm(args, ws, rank, local):
    """The whitening's CSR SpMM launches (spmm_rows_kernel) on a graph whose
    2k-wide panels are far larger than L2: one untimed whitening, then
    `steps` whitenings; GB/s = the launches' algorithmic bytes (CSR, one
    panel-row gather per nonzero, output) / their CUDA-event time."""
    if rank != 0:
        return
    mm = load_pkg()
    wl = dict(SPMM)
    graph = make_graph(mm, wl)
    cfg = mm.default_config(k=wl["k"], alpha0=wl["alpha0"], stpm_method=mm.STPM_ONLINE,
                            sweeps=wl["sweeps"], minibatch=wl["minibatch"], seed=wl["seed"],
                            device=local)
    ms = by = 0.0
    launches = 0
    with mm.Pipeline(cfg) as p:
        p.upload(graph)
        p.whiten()
        for _ in range(max(1, args.steps)):
            p.flush_l2()
            p.whiten()
            st = p.stats()
            ms += st["spmm_ms"]
            by += st["spmm_bytes"]
            launches += st["spmm_launches"]
    pk = peaks()
    gbs = by / max(ms, 1e-9) / 1e6
    line = {"metric": "whitening_spmm_gbs", "value": gbs, "unit": "GB/s", "n_gpus": 1,
            "steps": max(1, args.steps), "higher_is_better": True, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": wl["name"], **{k_: v for k_, v in wl.items() if k_ != "name"},
                       "nnz_directed": int(sum(b.nnz for b in graph.blocks[:3]) * 2),
                       "panel_columns": 2 * wl["k"]},
            "spmm_launches_per_whitening": launches / max(1, args.steps),
            "spmm_ms_per_whitening": ms / max(1, args.steps),
            "roofline": {"kernel": "spmm_rows_kernel", "bound": "hbm", "achieved": gbs,
                         "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": gbs / pk["hbm_gbs"],
                         "peak_source": pk["source"]}}
    print(json.dumps(line), flush=True)


# the differentiation configuration: the adjoint of the implicit tensor loss
ADJOINT = dict(name="mmsb-n500k-k100-bf16-adjoint", n=500_000, k=100, alpha0=1.0, p_in=0.04,
               p_out=4e-4, sweeps=30, minibatch=8192, seed=0, directions=1000, fd_step=1e-6)


def run_adjoint(args, ws, rank, local):
    """The adjoint form: the device gradient of L(Phi) (mmsb_stpm_loss_bwd, Z
    recomputed per minibatch) against FP64 central differences of the FP64
    loss on the device's whitened data along random unit directions and
    against the FP64 oracle gradient, on one 8,192-node minibatch; then the
    full BF16 adjoint solve (30 sweeps of 8,192-node minibatches, last sweep
    FP32) beside the FP32 online solve, node-updates/s."""
    if rank != 0:
        return
    mm = load_pkg()
    O = oracle_module()
    wl = dict(ADJOINT)
    t0 = time.perf_counter()
    graph = make_graph(mm, wl)
    t_gen = time.perf_counter() - t0
    k, a0, nX = wl["k"], wl["alpha0"], graph.parts[0]
    rng = np.random.default_rng(wl["seed"])
    check = {}
    # the gradient of L with theta = 1 (L = ||T - sum phi^x3||^2 - ||T||^2)
    cfg = mm.default_config(k=k, alpha0=a0, stpm_method=mm.STPM_ADJOINT, sweeps=wl["sweeps"],
                            minibatch=wl["minibatch"], seed=wl["seed"], device=local, tau=0.1,
                            precision=mm.PREC_BF16, theta=1.0)
    with mm.Pipeline(cfg) as p:
        p.upload(graph).whiten()
        y64 = {n_: np.asarray(v, dtype=np.float64) for n_, v in p.whitened().items()}
        # a point off the orthonormal manifold, where the orthogonality term
        # of L is not flat
        phi = O.qr_pos(rng.standard_normal((k, k))) + 0.05 * rng.standard_normal((k, k))
        b, cnt = 0, wl["minibatch"]
        nodes = np.arange(b, b + cnt)
        t1 = time.perf_counter()
        g_dev = p.loss_grad(phi, b, cnt)
        L_dev = p.loss(phi, b, cnt)
        t_dev = time.perf_counter() - t1
        t1 = time.perf_counter()
        g_o = O.loss_bwd(phi, y64, nodes, a0, 1.0)
        L_o = O.loss_fwd(phi, y64, nodes, a0, 1.0)
        h, errs, scale = wl["fd_step"], [], max(1.0, float(np.abs(g_o).max()))
        for _ in range(wl["directions"]):
            d = rng.standard_normal((k, k))
            d /= np.linalg.norm(d)
            fd = (O.loss_fwd(phi + h * d, y64, nodes, a0, 1.0)
                  - O.loss_fwd(phi - h * d, y64, nodes, a0, 1.0)) / (2 * h)
            errs.append(abs(float(np.sum(g_dev * d)) - fd) / scale)
        t_fd = time.perf_counter() - t1
        check = {"directions": wl["directions"], "fd_step": h, "nodes": cnt,
                 "max_abs_err_over_max_grad": float(max(errs)),
                 "median_abs_err_over_max_grad": float(np.median(errs)),
                 "grad_rel_err_vs_fp64": float(np.abs(g_dev - g_o).max() / np.abs(g_o).max()),
                 "loss_rel_err_vs_fp64": float(abs(L_dev - L_o) / max(abs(L_o), 1e-300)),
                 "device_fwd_bwd_s": t_dev, "fp64_fd_s": t_fd,
                 "note": "FP64 central differences of the FP64 loss (oracle) on the device's "
                         "whitened data; errors relative to max |dL/dPhi|"}
    forms = {}
    for name, method, prec in (("bf16_adjoint", mm.STPM_ADJOINT, mm.PREC_BF16),
                               ("fp32_online", mm.STPM_ONLINE, mm.PREC_FP32)):
        cfg = mm.default_config(k=k, alpha0=a0, stpm_method=method, sweeps=wl["sweeps"],
                                minibatch=wl["minibatch"], seed=wl["seed"], device=local,
                                tau=0.1, precision=prec)
        with mm.Pipeline(cfg) as p:
            p.upload(graph)
            for _ in range(max(1, min(args.warmup, 2))):
                p.run()
            ms, stages = [], {"whiten_ms": 0.0, "stpm_ms": 0.0, "post_ms": 0.0}
            for _ in range(max(1, args.steps)):
                p.flush_l2()
                p.synchronize()
                p.run()
                st = p.stats()
                ms.append(st["total_ms"])
                for key in stages:
                    stages[key] += st[key]
            step = statistics.mean(ms)
            forms[name] = {"value": nX * wl["sweeps"] / (step / 1e3), "unit": "node-updates/s",
                           "ms_per_step": step,
                           "stages_ms_per_step": {k_: v / len(ms) for k_, v in stages.items()},
                           "stpm_node_updates_per_s": nX * wl["sweeps"] / (stages["stpm_ms"]
                                                                            / len(ms) / 1e3)}
    line = {
        "metric": "stpm_node_updates_per_s", "value": forms["bf16_adjoint"]["value"],
        "unit": "node-updates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": forms["bf16_adjoint"]["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
        "config": {"workload": wl["name"], **{k_: v for k_, v in wl.items() if k_ != "name"},
                   "nnz_directed": int(sum(b_.nnz for b_ in graph.blocks[:3]) * 2),
                   "generation_s": t_gen, "l2": "256 MiB buffer written between timed steps"},
        "gradient_check": check, "forms": forms,
        "bf16_adjoint_over_fp32_online": forms["bf16_adjoint"]["value"] / forms["fp32_online"]["value"],
    }
    print(json.dumps(line), flush=True)


def run_io(args, ws, rank):
    """The file contract on the default graph: its five blocks written as the
    reference's COO text input (mmsb_write_coo) and read back by the parallel
    reader in the reference's compat mode, on one host thread and on all (up
    to 16), and the binary CSR container written and read; MB/s of text."""
    if rank != 0:
        return
    import tempfile
    mm = load_pkg()
    wl = dict(WORKLOAD)
    graph = make_graph(mm, wl)
    res = {}
    with tempfile.TemporaryDirectory() as td:
        files = []
        t0 = time.perf_counter()
        for b, blk in enumerate(graph.blocks):
            f = Path(td) / f"g{b}.txt"
            mm.write_coo(f, blk)
            files.append((f, blk.n_rows, blk.n_cols))
        t_write = time.perf_counter() - t0
        text_bytes = sum(f.stat().st_size for f, _, _ in files)
        for threads in (1, 0):
            env = dict(os.environ)
            code = ("import sys, time, json; sys.path.insert(0, %r); import bench; mm = bench.load_pkg(); "
                    "fs = json.loads(sys.argv[1]); ts = []\n"
                    "for r in range(%d):\n"
                    "    t0 = time.perf_counter()\n"
                    "    for f, a, b in fs: mm.read_coo(f, a, b, compat=True)\n"
                    "    ts.append(time.perf_counter() - t0)\n"
                    "print(min(ts))") % (str(ROOT), max(1, args.steps))
            if threads:
                env["MMSB_IO_THREADS"] = str(threads)
            else:
                env.pop("MMSB_IO_THREADS", None)
            out = subprocess.run([sys.executable, "-c", code, json.dumps([[str(f), a, b] for f, a, b in files])],
                                 env=env, capture_output=True, text=True, check=True)
            res["read_s_1thread" if threads else "read_s"] = float(out.stdout.strip().splitlines()[-1])
        t0 = time.perf_counter()
        for b, blk in enumerate(graph.blocks):
            mm.write_csr(Path(td) / f"g{b}.csr", blk)
        t_bw = time.perf_counter() - t0
        t0 = time.perf_counter()
        for b in range(len(graph.blocks)):
            mm.read_csr(Path(td) / f"g{b}.csr")
        t_br = time.perf_counter() - t0
        bin_bytes = sum((Path(td) / f"g{b}.csr").stat().st_size for b in range(len(graph.blocks)))
    mb = text_bytes / 1e6
    line = {"metric": "coo_text_parse_MB_per_s", "value": mb / res["read_s"], "unit": "MB/s",
            "n_gpus": 0, "steps": args.steps, "higher_is_better": True, "data": "synthetic",
            "config": {"workload": wl["name"] + "-coo-files", "text_MB": mb,
                       "nnz": int(sum(b.nnz for b in graph.blocks)), "threads": os.cpu_count()},
            "parse_MB_per_s_1_thread": mb / res["read_s_1thread"],
            "parallel_speedup": res["read_s_1thread"] / res["read_s"],
            "write_coo_MB_per_s": mb / t_write,
            "binary_csr": {"MB": bin_bytes / 1e6, "write_MB_per_s": bin_bytes / 1e6 / t_bw,
                           "read_MB_per_s": bin_bytes / 1e6 / t_br}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--clocks-csv", default=None,
                    help="also write the SM clock samples of the timed region to this CSV file")
    # --nodes, not --n alone, under torchrun: its argument parser rejects "--n" as an
    # ambiguous abbreviation of its own options even after the script name
    ap.add_argument("--nodes", "--n", dest="n", type=int, default=None,
                    help="override node count (testing)")
    ap.add_argument("--batch", action="store_true",
                    help="the batching configuration (256 graphs) instead of the default")
    ap.add_argument("--precision", action="store_true",
                    help="the precision configuration (n = 2M, k = 200, BF16 form vs FP32 vs FP64)")
    ap.add_argument("--adjoint", action="store_true",
                    help="the differentiation configuration (n = 500k, k = 100: gradient check "
                         "against FP64 finite differences, BF16 adjoint solve)")
    ap.add_argument("--spmm", action="store_true",
                    help="the whitening SpMM on panels larger than L2 (n = 2M, 2k = 400)")
    ap.add_argument("--io", action="store_true",
                    help="the file contract: COO text parse/write and binary CSR on the default graph")
    args = ap.parse_args()
    wl = dict(WORKLOAD)
    if args.n:
        wl["n"] = args.n
        wl["name"] += f"-n{args.n}"
    ws, rank, local = dist_env()
    if args.batch and args.impl != "reference":
        run_batch(args, ws, rank, local)
        return
    if args.io and args.impl != "reference":
        run_io(args, ws, rank)
        return
    if args.spmm and args.impl != "reference":
        run_spmm(args, ws, rank, local)
        return
    if args.precision and args.impl != "reference":
        run_precision(args, ws, rank, local)
        return
    if args.adjoint and args.impl != "reference":
        run_adjoint(args, ws, rank, local)
        return
    if args.impl == "reference":
        run_reference(args, wl, ws, rank)
    else:
        run_ours(args, wl, ws, rank, local)


if __name__ == "__main__":
    main()
