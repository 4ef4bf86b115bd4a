#!/usr/bin/env python
"""Benchmark of the explicit higher-order encoding operator on GB300.

Metric: E+E^H voxel·samples/s on the 200x200, 12,000-sample, 16-coil,
third-order + concomitant spiral workload (seeded synthetic inputs with the
shapes and distributions of that configuration).  One step = one forward
E x and one adjoint E^H y; it processes 2*nVox*nSam voxel·samples.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Multi-GPU: the operator runs on one GPU; under torchrun each rank runs an
independent replica (no collective on the data path), the time is the max
over ranks and ``value`` counts all ranks' work.

The ``--impl reference`` arm times the reference path's CPU restatement (the
FP64 oracle, OpenMP on all host cores) on a bounded sample of the same
workload; the reference itself is Julia and cannot run here.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "highordermri.jl_gb300"
for _p in (str(ROOT), str(PKG)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "E+E^H voxel·samples/s, TC vs plain FP32 on GB300 at <=1e-4 rel err vs FP64"
UNIT = "voxel·samples/s"
L2_FLUSH_BYTES = 256 << 20

# Per-launch ncu figures of the dominant kernels (DRAM bytes read + written,
# warp instructions issued) come from a committed capture summary,
# profiles/ncu_figures.txt, which records a hash of the kernel sources it was
# taken on.  A figure is used only when that hash equals the hash of the
# sources in this tree; otherwise the bench reports null and says why.
KERNEL_SOURCES = {
    "tc": ("hoe_tc_kernel.cuh", "hoe_tc.cu", "hoe_tcgen05.cuh"),
    "fp32": ("hoe_simt.cu", "hoe_internal.cuh"),
}
NCU_FIGURES = ROOT / "profiles" / "ncu_figures.txt"


def kernel_source_hash(engine: str) -> str:
    """sha256 (first 16 hex digits) of the sources the engine's contraction
    kernel and its tables are built from."""
    import hashlib
    h = hashlib.sha256()
    for name in KERNEL_SOURCES[engine]:
        h.update(name.encode())
        h.update((PKG / "csrc" / name).read_bytes())
    return h.hexdigest()[:16]


def ncu_figure(kind: str, workload_name: str, engine: str, direction: str):
    """(value, provenance) of one committed ncu figure: kind 'traffic' (DRAM
    bytes per launch) or 'inst' (warp instructions per launch).  value is
    None when no capture of these sources exists."""
    want = kernel_source_hash(engine)
    seen = None
    try:
        lines = NCU_FIGURES.read_text().splitlines()
    except OSError:
        return None, "no committed ncu capture"
    for ln in lines:
        f = ln.split()
        if len(f) == 6 and f[0] == kind and f[1] == workload_name and f[2] == engine and f[3] == direction:
            if f[5] == want:
                return int(f[4]), f"ncu capture of kernel sources {want}"
            seen = f[5]
    if seen:
        return None, f"stale: the committed capture is of kernel sources {seen}, this tree is {want}"
    return None, "no committed ncu capture for this workload"


# Cycles a converged warp's elected lane waits per tcgen05.mma issued back to
# back (kind::f16, M = 128, N = 64, A from TMEM), measured in isolation on
# this GPU (N = 32: 32 cycles).
MMA_ISSUE_CYCLES = 40.0
# Tensor-pipe cycles per SM of one M = 128 MMA: BF16 K = 16 and TF32 K = 8
# both run at N / 2 cycles for N >= 32 (4,096 BF16 MACs per clock per SM),
# from the same isolated probe and the ncu op counts of the capture above.


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--engine", default="auto", choices=["auto", "tc", "fp32"])
    ap.add_argument("--config", default="2", choices=["1", "2", "3", "5"],
                    help="2: 200x200 spiral (headline); 5: 24-slice batch in one persistent launch")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-compare", action="store_true", help="skip timing the second engine")
    ap.add_argument("--no-recon", action="store_true", help="skip timing the device CGNR solve")
    ap.add_argument("--recon-iterations", type=int, default=20)
    ap.add_argument("--no-recon-check", action="store_true",
                    help="skip the FP64 check of the CGNR image (about a minute of host time at 200x200)")
    ap.add_argument("--autotune", action="store_true",
                    help="time every execution plan on the workload and keep the fastest (always on for config 3)")
    a = ap.parse_args()
    a.warmup = max(a.warmup, 3)
    return a


def workload(cfg: str):
    from hoexplicit import workloads
    return {"1": workloads.config1, "2": workloads.config2, "3": workloads.config3,
            "5": lambda: workloads.config5()[0]}[cfg]()


def workload_config(w, nTermEff: int) -> dict:
    """The config dict of the JSON line, the same in both arms."""
    return {"workload": w.name, "nVox": w.nVox, "nSam": w.nSam, "nCha": w.nCha, "nTermEff": int(nTermEff),
            "l2": "GPU arm: L2 flushed between timed steps (256 MiB write)"}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(ms: float, ws: int, device) -> float:
    """The largest of the ranks' timed durations (ms): one all-reduce (MAX)
    of the process group, then a barrier; the value itself at world size 1.
    Every rank returns the same number."""
    if ws <= 1:
        return ms
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    torch.distributed.barrier()
    return float(t.item())


def replica_value(units_per_step: float, ms_per_step: float, ws: int) -> float:
    """Whole-job throughput of ws replicas that each process units_per_step
    per step, timed by the slowest rank (weak scaling)."""
    return ws * units_per_step / (ms_per_step / 1e3)


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.rows = []
        if self.proc is None:
            return
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        for row in csv.reader(io.StringIO(out)):
            if len(row) >= 9:
                self.rows.append([c.strip() for c in row])

    def summary(self):
        if not getattr(self, "rows", None):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("bf16_tflops", 1900.0), d.get("hbm_gbs", 6800.0), "measured"
    return 1900.0, 6800.0, "fallback"


def cpu_baseline(w, seconds: float, x_gpu=None, y_gpu=None, op=None):
    """Time the oracle (FP64, all host threads) on a bounded sample of rows.

    Also returns the relative error of the GPU forward/adjoint on the same
    sample (the adjoint compared for data supported on the sampled rows)."""
    import torch
    from hoexplicit import workloads
    from oracle import dense, oracle
    bf, k, t, f, c, idx = workloads.prepared_model(w)
    nthreads = oracle.max_threads()
    nSam = k.shape[1]
    rng = np.random.default_rng(0)

    def model_rows(rows):
        return oracle.Model(bf, k[:, rows], t[rows], f, c, nTerm=w.kspha.shape[0])

    xm = w.x[idx]
    probe = max(8, min(nSam, 32))
    rows = np.sort(rng.choice(nSam, probe, replace=False))
    m = model_rows(rows)
    t0 = time.perf_counter()
    yo = oracle.forward(m, xm)
    oracle.adjoint(m, yo)
    dt = time.perf_counter() - t0
    per_row = dt / probe
    n_rows = int(min(nSam, max(probe, seconds / max(per_row, 1e-9))))
    rows = np.sort(rng.choice(nSam, n_rows, replace=False))
    m = model_rows(rows)
    t0 = time.perf_counter()
    yo = oracle.forward(m, xm)
    xo = oracle.adjoint(m, yo)
    dt = time.perf_counter() - t0
    units = 2.0 * len(idx) * n_rows
    res = {"value": units / dt, "unit": UNIT, "cores": nthreads, "kind": "port",
           "sample": f"E and E^H over {n_rows} of {nSam} samples x {len(idx)} voxels x {w.nCha} coils "
                     f"(FP64 C restatement of array_operator.jl:241-348, OpenMP), {dt:.1f} s"}
    # the same restatement on one thread, on about 1 s of rows
    n1 = int(min(nSam, max(4, 1.0 / max(per_row * nthreads, 1e-9))))
    rows1 = np.sort(rng.choice(nSam, n1, replace=False))
    m1 = model_rows(rows1)
    oracle.set_threads(1)
    try:
        t0 = time.perf_counter()
        oracle.adjoint(m1, oracle.forward(m1, xm))
        dt1 = time.perf_counter() - t0
    finally:
        oracle.set_threads(nthreads)
    res["single_thread"] = {"value": 2.0 * len(idx) * n1 / dt1, "unit": UNIT, "cores": 1,
                            "sample": f"E and E^H over {n1} of {nSam} samples, {dt1:.1f} s"}
    if op is not None and x_gpu is not None:
        yg = (op * x_gpu).cpu().numpy().reshape(w.nCha, nSam)[:, rows].reshape(-1)
        res["gpu_forward_rel_err_vs_fp64"] = dense.rel(yg, yo)
        ysub = np.zeros((w.nCha, nSam), dtype=np.complex128)
        ysub[:, rows] = yo.reshape(w.nCha, n_rows)
        xg = (op.H * torch.from_numpy(ysub.reshape(-1).astype(np.complex64)).cuda()).cpu().numpy()
        res["gpu_adjoint_rel_err_vs_fp64"] = dense.rel(xg[idx], xo)
    return res


def time_engine(op, x, y, steps, warmup, flush, stream):
    """CUDA-event timing of K steps (forward + adjoint), L2 flushed between steps."""
    import torch
    yout = torch.empty(op.nrow, dtype=torch.complex64, device=x.device)
    xout = torch.empty(op.ncol, dtype=torch.complex64, device=x.device)
    for _ in range(warmup):
        op.prod_(yout, x)
        op.ctprod_(xout, y)
    torch.cuda.synchronize()
    l0 = op.timings()["launches"]
    step_ms, fk, ak = [], [], []
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    # the timed steps run without the operator's trace events
    op.set_timing(False)
    for _ in range(steps):
        flush.zero_()   # L2 flush, before ev0 in stream order; the step is queued behind it
        ev0.record(stream)
        op.prod_(yout, x)
        op.ctprod_(xout, y)
        ev1.record(stream)
        ev1.synchronize()
        step_ms.append(ev0.elapsed_time(ev1))
    launches = op.timings()["launches"] - l0
    # kernel durations from separate traced steps (same flush discipline)
    op.set_timing(True)
    for _ in range(max(3, steps // 2)):
        flush.zero_()
        torch.cuda.synchronize()
        op.prod_(yout, x)
        op.ctprod_(xout, y)
        torch.cuda.synchronize()
        tm = op.timings()
        fk.append(tm["forward_kernel_ms"])
        ak.append(tm["adjoint_kernel_ms"])
    return dict(step_ms=step_ms, fwd_kernel_ms=fk, adj_kernel_ms=ak, launches=launches)


def time_recon(op, w, y, flush, stream, iterations, reps):
    """recon_HOOp's weighted CGNR on the device (hoe_recon), as one cached CUDA
    graph and as individual launches; CUDA events around each whole solve."""
    import torch
    from hoexplicit import recon as hrecon
    dev = y.device
    kr = np.hypot(w.kspha[1], w.kspha[2])
    weight = torch.from_numpy(np.sqrt(0.05 + kr / kr.max()).astype(np.complex64)).to(dev)
    data = y.reshape(w.nCha, w.nSam).t()
    out = torch.empty(op.ncol, dtype=torch.complex64, device=dev)
    units = (2.0 * iterations + 1.0) * w.nVox * w.nSam
    res = {"iterations": iterations, "lambda": 1e-9, "weights": "sqrt-density-like, complex64",
           "units_per_solve": units}
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    for use_graph in (True, False):
        _, st = hrecon.solve(op, data, weight, iterations=iterations, rel_tol=0.0, lam=1e-9,
                             use_graph=use_graph, out=out)  # warm-up (captures the graph)
        l0 = op.timings()["launches"]
        ms = []
        for _ in range(reps):
            flush.zero_()   # L2 flush, before ev0 in stream order; the step is queued behind it
            ev0.record(stream)
            hrecon.solve(op, data, weight, iterations=iterations, rel_tol=0.0, lam=1e-9,
                         use_graph=use_graph, out=out, stats=False)
            ev1.record(stream)
            ev1.synchronize()
            ms.append(ev0.elapsed_time(ev1))
        key = "graph" if use_graph else "direct"
        m = statistics.mean(ms)
        res[key] = {"ms_per_solve": m, "ms_per_iteration": m / iterations,
                    "value": units / (m / 1e3), "unit": UNIT,
                    "launches_per_solve": (op.timings()["launches"] - l0) / reps,
                    "status": st["status"], "residual_ratio": st["residual"] / max(st["residual0"], 1e-300)}
    res["graph_speedup"] = res["direct"]["ms_per_solve"] / res["graph"]["ms_per_solve"]
    # the inputs and the image of the last solve, for the FP64 check
    res["_check"] = (data.cpu().numpy(), weight.cpu().numpy(), out.cpu().numpy())
    return res


def recon_fp64_check(w, data, weight, x_gpu, iterations: int):
    """Relative L2 error of the device CGNR image against the oracle's FP64
    CGNR of recon_HOOp on the same data and weights (the checker)."""
    from hoexplicit import workloads
    from oracle import dense, oracle
    from oracle import recon as orecon
    bf, k, t, f, c, idx = workloads.prepared_model(w)
    m = oracle.Model(bf, k, t, f, c, nTerm=w.kspha.shape[0])
    t0 = time.perf_counter()
    y = np.asarray(data, dtype=np.complex128).T.reshape(-1)   # (nSam, nCha) -> samples fastest
    xo, so = orecon.recon(m, y, np.asarray(weight, dtype=np.complex128), iterations=iterations,
                          rel_tol=0.0, lam=1e-9)
    return {"image_rel_err_vs_fp64": dense.rel(np.asarray(x_gpu, dtype=np.complex128)[idx], xo),
            "fp64_residual_ratio": so["residual"] / max(so["residual0"], 1e-300),
            "fp64_seconds": time.perf_counter() - t0,
            "note": "FP64 CGNR (same recurrence and iterations) over the oracle's operator, all host cores"}


def run_batch(a):
    """24 slices (160^2-224^2 voxels, 8,000-20,000 samples, 16 coils): all
    slices' E and E^H in one persistent launch per direction (OperatorBatch),
    and recon_HOOp's 30-iteration weighted CGNR for every slice in one graph."""
    import torch
    from hoexplicit import HighOrderExplicitOp, OperatorBatch, workloads
    ws_, rank, local = dist_env()
    if ws_ > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", init_method="env://")
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()
    engine = "fp32" if a.engine == "fp32" else "tc"
    slices = workloads.config5()
    ops = [HighOrderExplicitOp(w.grid, w.kspha, w.times, engine=engine, **w.op_kwargs()) for w in slices]
    B = OperatorBatch(ops)
    stream = torch.cuda.current_stream()
    xs = [torch.from_numpy(w.x.astype(np.complex64)).to(dev) for w in slices]
    ys = [y + 0.01 * y.abs().pow(2).mean().sqrt() * torch.randn_like(y) for y in B.forward(xs)]
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    pairs = float(sum(w.nVox * w.nSam for w in slices))
    units = 2.0 * pairs
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        ms = []
        for _ in range(steps):
            flush.zero_()   # L2 flush, before ev0 in stream order; the step is queued behind it
            ev0.record(stream)
            fn()
            ev1.record(stream)
            ev1.synchronize()
            ms.append(ev0.elapsed_time(ev1))
        return statistics.mean(ms)

    l0 = B.info()["launches"]
    with Clocks(dev) as clk:
        ms = timed(lambda: (B.forward(xs), B.adjoint(ys)), a.steps, a.warmup)
    launches = (B.info()["launches"] - l0) / (a.steps + a.warmup)
    ms = max_over_ranks(ms, ws_, dev)
    bf16_peak, _, peak_src = measured_peaks()
    flops = 8.0 * 16 * pairs  # contraction flops per direction
    out = {"metric": METRIC, "value": replica_value(units, ms, ws_), "unit": UNIT, "n_gpus": ws_,
           "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None,
           "dtype": "bf16x3/f32-acc" if engine == "tc" else "f32",
           "data": "synthetic (seeded, shapes/distributions of the named configuration)",
           "config": {"workload": f"cfg5-{len(slices)}slices-160..224sq-8k..20k-samples-16c",
                      "slices": len(slices), "voxel_samples_per_direction": pairs, "engine": engine,
                      "parallelism": f"replicas x{ws_}", "l2": "flushed between timed steps (256 MiB write)",
                      "contraction_launches_per_direction": B.info()["contraction_launches"]},
           "roofline": {"bound": "tensor", "achieved": 2 * flops / (ms / 1e3) / 1e12, "peak": bf16_peak,
                        "unit": "TFLOP/s", "frac": 2 * flops / (ms / 1e3) / 1e12 / bf16_peak,
                        "traffic": None, "kernel": "whole step (both directions, all slices)",
                        "peak_source": f"bf16_tflops ({peak_src}, burst)"},
           "clocks": clk.summary(), "gpu_launches": launches}
    # the same products slice by slice (one launch per slice and direction)
    def per_slice():
        for op, x, y in zip(ops, xs, ys):
            op * x
            op.H * y
    ms1 = timed(per_slice, max(3, a.steps // 2), 2)
    out["per_slice_launches"] = {"ms_per_step": ms1, "value": units / (ms1 / 1e3), "batched_speedup": ms1 / ms}
    if not a.no_recon:
        rng = np.random.default_rng(5)
        datas = [y.reshape(w.nCha, w.nSam).t() for w, y in zip(slices, ys)]
        weights = []
        for w in slices:
            kr = np.hypot(w.kspha[1], w.kspha[2])
            weights.append(torch.from_numpy(np.sqrt(0.05 + kr / kr.max()).astype(np.complex64)).to(dev))
        iters = 30
        outs = [torch.empty(op.ncol, dtype=torch.complex64, device=dev) for op in ops]
        _, st = B.recon(datas, weights, iterations=iters, rel_tol=0.0, lam=1e-9, out=outs)
        l0 = B.info()["launches"]
        msr = timed(lambda: B.recon(datas, weights, iterations=iters, rel_tol=0.0, lam=1e-9, out=outs,
                                    stats=False), 3, 0)
        ru = (2.0 * iters + 1.0) * pairs
        out["recon"] = {"iterations": iters, "ms_per_solve": msr, "value": ru / (msr / 1e3), "unit": UNIT,
                        "graph": True, "launches_per_solve": (B.info()["launches"] - l0) / 3,
                        "status": sorted({s["status"] for s in st}),
                        "max_residual_ratio": max(s["residual"] / max(s["residual0"], 1e-300) for s in st)}
        del rng
    if not a.no_e2e:
        xh = [x.cpu().pin_memory() for x in xs]
        yh = [y.cpu().pin_memory() for y in ys]
        xo = [torch.empty(x.shape, dtype=x.dtype).pin_memory() for x in xs]
        yo = [torch.empty(y.shape, dtype=y.dtype).pin_memory() for y in ys]
        def e2e():
            yr = B.forward([x.to(dev, non_blocking=True) for x in xh])
            xr = B.adjoint([y.to(dev, non_blocking=True) for y in yh])
            for dst, src in zip(yo, yr):
                dst.copy_(src, non_blocking=True)
            for dst, src in zip(xo, xr):
                dst.copy_(src, non_blocking=True)
        e2e()
        torch.cuda.synchronize()
        n_e2e = max(3, a.steps // 2)
        t0 = time.perf_counter()
        for _ in range(n_e2e):
            e2e()
        torch.cuda.synchronize()
        e2e_s = max_over_ranks((time.perf_counter() - t0) / n_e2e * 1e3, ws_, dev) / 1e3
        out["e2e"] = {"value": replica_value(units, e2e_s * 1e3, ws_), "unit": UNIT,
                      "h2d_bytes_per_step": int(sum(x.numel() * 8 for x in xh) + sum(y.numel() * 8 for y in yh)),
                      "d2h_bytes_per_step": int(sum(x.numel() * 8 for x in xo) + sum(y.numel() * 8 for y in yo)),
                      "ms_per_step": e2e_s * 1e3}
    if rank == 0 and ws_ == 1 and not a.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(slices[0], a.cpu_seconds)
        out["cpu_baseline"]["sample"] += " (slice 0 of the batch)"
    B.check()
    if rank == 0:
        print(json.dumps(out), flush=True)
    B.close()
    for op in ops:
        op.close()
    if ws_ > 1:
        torch.distributed.destroy_process_group()


def time_backward(op, x, y, flush, stream, reps):
    """dL/d(kspha, fieldmap, t0) of L = 0.5*||E x - y||^2 at the workload's
    shapes (hoe_backward, gradients 20 x nSam, nFull and one scalar)."""
    import torch
    r = op * x - y
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def run(n):
        op.backward(x, r)
        torch.cuda.synchronize()
        ms = []
        for _ in range(n):
            flush.zero_()   # L2 flush, before ev0 in stream order; the step is queued behind it
            ev0.record(stream)
            op.backward(x, r, kspha=True, fieldmap=True, t0_b0=True)
            ev1.record(stream)
            ev1.synchronize()
            ms.append(ev0.elapsed_time(ev1))
        return statistics.mean(ms)

    # the tensor-core backward covers up to 16 coils with residual widths <= 24
    # and up to 32 coils with widths <= 16
    rw = op.info()["residual_width"]
    tc = op.engine == "tc" and ((op.nCha <= 16 and rw <= 24) or (op.nCha <= 32 and rw <= 16))
    m = run(reps)
    pairs = float(op.nVox) * op.nSam
    out = {"ms_per_call": m, "value": pairs / (m / 1e3), "unit": UNIT,
           "outputs": f"dL/dkspha {op.nTermEff}x{op.nSam}, dL/dfieldmap {op.ncol}, dL/dt0 scalar",
           "engine": "tc (tcgen05)" if tc else "fp32 (CUDA cores)"}
    if tc:
        op.set_engine("fp32")
        m2 = run(max(2, reps // 2))
        op.set_engine("tc")
        out["fp32_engine_ms_per_call"] = m2
        out["tc_vs_fp32"] = m2 / m
    return out


def time_extras(w, x, reps=10):
    """The functions around the operator at the workload's shapes, each timed
    as the mean of `reps` synchronised calls after two warm calls: the
    derivative product B x (kspha_dt mode, FindDelay.jl:199-200), the k-dot
    stencil (FindDelay.jl:179-180), InterpTrajTime (InterpTraj.jl:18-40) on a
    (nSam, nTerm) series, and the SVD coil compression fit and apply
    (CoilCompression.jl:239-301) from 2 x nCha to nCha virtual coils."""
    import torch
    from hoexplicit import (HighOrderExplicitOp, InterpTrajTime, apply_coil_compression,
                            fit_coil_compression, kspha_dt)

    def timed_ms(fn):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / reps * 1e3

    out = {}
    if w.kspha_dt is not None:
        opd = HighOrderExplicitOp(w.grid, w.kspha, w.times, kspha_dt=w.kspha_dt, **w.op_kwargs())
        yd = torch.empty(opd.nrow, dtype=torch.complex64, device=x.device)
        ms = timed_ms(lambda: opd.prod_(yd, x))
        out["derivative"] = {"ms_per_call": ms, "value": w.nVox * w.nSam / (ms / 1e3), "unit": UNIT,
                             "engine": ("tc (one pass: phase tile scaled by 2 pi i F, F in the basis's reduced rank on the CUDA cores)" if opd.nCha <= 16
                                        else "tc (virtual-coil passes)") if opd.engine == "tc" else "fp32 (CUDA cores)"}
        opd.close()
    dt = float(w.times[1] - w.times[0])
    traj = torch.from_numpy(np.ascontiguousarray(w.kspha.T)).cuda()          # (nSam, nTerm) float64
    tq = torch.from_numpy(np.asarray(w.times, dtype=np.float64) + 0.37 * dt).cuda()
    out["kdot_stencil_ms"] = timed_ms(lambda: kspha_dt(traj, dt))
    out["interp_traj_time_ms"] = timed_ms(lambda: InterpTrajTime(traj, dt, 0.0, tq))
    rng = np.random.default_rng(7)
    nc = 2 * w.nCha
    cal = torch.from_numpy((rng.standard_normal((w.nSam, nc)) + 1j * rng.standard_normal((w.nSam, nc)))
                           .astype(np.complex64)).cuda()
    tr = fit_coil_compression(cal, n_virtual_coils=w.nCha)
    out["coil_fit_ms"] = timed_ms(lambda: fit_coil_compression(cal, n_virtual_coils=w.nCha))
    out["coil_apply_ms"] = timed_ms(lambda: apply_coil_compression(cal, tr))
    out["shapes"] = (f"derivative {w.nVox} voxels x {w.nSam} samples x {w.nCha} coils; series {w.nSam} x "
                     f"{w.kspha.shape[0]}; coils {w.nSam} x {nc} -> {w.nCha}")
    return out


def time_normal(op, w, x, flush, stream, reps):
    """E^H D E (hoe_normal) with square-root-density-like weights squared:
    2*nVox*nSam voxel.samples per application."""
    import torch
    from hoexplicit import normalOperator
    kr = np.hypot(w.kspha[1], w.kspha[2])
    D = normalOperator(op, np.tile(0.05 + kr / kr.max(), w.nCha))
    out = torch.empty(op.ncol, dtype=torch.complex64, device=x.device)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(3):
        D.prod_(out, x)
    torch.cuda.synchronize()
    ms = []
    for _ in range(reps):
        flush.zero_()   # L2 flush, before ev0 in stream order; the step is queued behind it
        ev0.record(stream)
        D.prod_(out, x)
        ev1.record(stream)
        ev1.synchronize()
        ms.append(ev0.elapsed_time(ev1))
    m = statistics.mean(ms)
    return {"ms_per_call": m, "value": 2.0 * w.nVox * w.nSam / (m / 1e3), "unit": UNIT}


def run_gb300(a):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", init_method="env://")
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()
    from hoexplicit import HighOrderExplicitOp, HoeError

    w = workload(a.config)
    engines_avail = []
    op = None
    want = ["tc", "fp32"] if a.engine == "auto" else [a.engine]
    for e in want:
        try:
            op = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine=e, **w.op_kwargs())
            engines_avail.append(e)
            break
        except HoeError:
            continue
    if op is None:
        raise SystemExit("no engine available")
    engine = engines_avail[0]
    tuned = None
    if a.autotune or a.config == "3":
        tuned = op.autotune(reps=3)
        engine = tuned["engine"]
    op.set_timing(True)
    info = op.info()
    stream = torch.cuda.current_stream()
    x = torch.from_numpy(w.x.astype(np.complex64)).to(dev)
    y = op * x
    g = torch.Generator(device=dev).manual_seed(0)
    noise = torch.randn(y.shape, dtype=torch.complex64, device=dev, generator=g)
    y = y + 0.01 * y.abs().pow(2).mean().sqrt() * noise
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    units = 2.0 * w.nVox * w.nSam

    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with Clocks(dev) as clk:
        r = time_engine(op, x, y, a.steps, a.warmup, flush, stream)
    torch.cuda.synchronize()
    total_ms = max_over_ranks(sum(r["step_ms"]), ws, dev)
    ms_per_step = total_ms / a.steps
    value = replica_value(units, ms_per_step, ws)

    # dominant kernel roofline (contraction flops: 8*nCha per voxel·sample per direction)
    fk = statistics.mean(r["fwd_kernel_ms"])
    ak = statistics.mean(r["adj_kernel_ms"])
    dom, dom_ms = ("forward", fk) if fk >= ak else ("adjoint", ak)
    flops_per_launch = 8.0 * w.nCha * w.nVox * w.nSam
    achieved = flops_per_launch / (dom_ms / 1e3) / 1e12
    bf16_peak, hbm_peak, peak_src = measured_peaks()
    traffic, traffic_src = ncu_figure("traffic", w.name, engine, dom)
    roofline = {"bound": "tensor", "achieved": achieved, "peak": bf16_peak, "unit": "TFLOP/s",
                "frac": achieved / bf16_peak, "traffic": traffic, "traffic_source": traffic_src,
                "kernel": f"{engine} {dom} contraction", "peak_source": f"bf16_tflops ({peak_src}, burst)",
                "kernel_ms": dom_ms, "flops_per_launch": flops_per_launch,
                "frac_of_split_peak": achieved / (bf16_peak / 3.0) if engine == "tc" else None,
                "share_of_step": (fk + ak) / ms_per_step}
    if engine == "tc":
        # Ceilings of the contraction kernel, each as the time it alone would
        # take; frac = that time / the measured kernel time.
        sm_mhz = clk.summary().get("sm_mhz") or 2070.0
        hz = sm_mhz * 1e6
        nsm = torch.cuda.get_device_properties(dev).multi_processor_count
        stages = -(-info["n_sample_tiles"] * info["n_voxel_tiles"] * 2 // nsm)   # 64-column stages per CTA
        nc = 2 * max(8, 1 << (w.nCha - 1).bit_length())   # N: coils padded to 8/16/32/64, re/im
        rk = info["residual_rank"]
        kp = 8 if rk <= 8 else (16 if rk <= 16 else 24)     # residual k-width
        if nc <= 64:   # hi x [B_hi | B_lo] (2N wide) and lo x B_hi, 8 k-steps each
            mma_contract, mma_busiest, pipe_contract = 16, 8, 8 * (2 * nc // 2) + 8 * max(16, nc // 2)
        else:          # 3 products of width N per k-step
            mma_contract, mma_busiest, pipe_contract = 24, 24, 24 * nc // 2
        mma_resid = 3 * (kp // 8) + 1
        pipe_cycles = pipe_contract + mma_resid * 32
        t_mma = stages * mma_busiest * MMA_ISSUE_CYCLES / hz
        t_pipe = stages * pipe_cycles / hz
        from hoexplicit.operator import sfu_rate
        sfu = sfu_rate()   # measured sin/cos lane operations per clock per SM
        t_sfu = 2.0 * w.nVox * w.nSam / (sfu * nsm * hz)
        inst, inst_src = ncu_figure("inst", w.name, engine, dom)
        t_issue = inst / (4.0 * nsm * hz) if inst else None
        dom_s = dom_ms / 1e3
        roofline["ceilings"] = [
            {"pipe": "sfu (MUFU sin/cos)", "ms": t_sfu * 1e3, "frac": t_sfu / dom_s,
             "note": f"2 MUFU ops per (voxel, sample) at the measured {sfu:.1f} per clock per SM (hoe_sfu_rate)"},
            {"pipe": "warp instruction issue", "ms": t_issue * 1e3 if t_issue else None,
             "frac": t_issue / dom_s if t_issue else None,
             "note": f"ncu warp instructions of one launch / (4 per clock per SM); {inst_src}"},
            {"pipe": "tensor pipe (all MMAs)", "ms": t_pipe * 1e3, "frac": t_pipe / dom_s,
             "note": f"{pipe_cycles} cycles per 64-column stage: contraction (3 BF16 products, "
                     f"{mma_contract} MMAs) + {mma_resid} TF32 residual-phase MMAs, {stages} stages per SM"},
            {"pipe": "tcgen05.mma issue", "ms": t_mma * 1e3, "frac": t_mma / dom_s,
             "note": f"{mma_busiest} MMAs per stage on the busiest issuer x {MMA_ISSUE_CYCLES:.0f} cycles "
                     "(converged warp, elected lane, isolated)"},
        ]
        roofline["binding"] = {"pipe": "phase generator (sfu + issue) and the stage pipeline", "frac": t_sfu / dom_s,
                               "note": "timing variants: sin/cos removed or the lo split removed each cut the "
                                       "kernel 11%; with the phase work removed it still takes 0.23 ms (the "
                                       "tensor pipe alone needs 0.11)"}
    if engine == "fp32":
        sm_mhz = clk.summary().get("sm_mhz") or 1900.0
        fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
        roofline["note"] = ("plain FP32 engine: contraction on CUDA cores; fp32 FMA issue peak "
                            f"{fp32_peak:.1f} TFLOP/s at the sampled clock, frac {achieved / fp32_peak:.3f}")
        roofline["fp32_simt_frac"] = achieved / fp32_peak

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps,
           "warmup": a.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None,
           "dtype": "bf16x3/f32-acc" if engine == "tc" else "f32",
           "data": "synthetic (seeded, shapes/distributions of the named configuration)",
           "config": workload_config(w, info["nTermEff"]),
           "parallelism": f"replicas x{ws}",
           "plan": {"engine": engine, "residual_phase_bound_cycles": info["residual_phase_bound"],
                    "residual_rank": info["residual_rank"], "residual_width": info["residual_width"]},
           "roofline": roofline, "clocks": clk.summary(),
           "gpu_launches": int(r["launches"]),
           "kernel_ms": {"forward": fk, "adjoint": ak}}

    # second engine for the TC vs plain-FP32 ratio
    if not a.no_compare and engine == "tc":
        try:
            op.set_engine("fp32")
            r2 = time_engine(op, x, y, max(3, a.steps // 4), 3, flush, stream)
            ms2 = statistics.mean(r2["step_ms"])
            out["fp32_engine"] = {"value": units / (ms2 / 1e3), "ms_per_step": ms2,
                                  "kernel_ms": {"forward": statistics.mean(r2["fwd_kernel_ms"]),
                                                "adjoint": statistics.mean(r2["adj_kernel_ms"])}}
            out["tc_vs_fp32"] = ms2 / ms_per_step
            op.set_engine("tc")
        except Exception as exc:  # report, do not substitute
            out["fp32_engine"] = {"error": str(exc)}

    if not a.no_recon:
        try:
            out["recon"] = time_recon(op, w, y, flush, stream, a.recon_iterations, max(3, a.steps // 4))
        except Exception as exc:  # report, do not substitute
            out["recon"] = {"error": str(exc)}
        try:
            out["backward"] = time_backward(op, x, y, flush, stream, max(3, a.steps // 4))
        except Exception as exc:  # report, do not substitute
            out["backward"] = {"error": str(exc)}
    try:
        out["normal"] = time_normal(op, w, x, flush, stream, max(3, a.steps // 2))
    except Exception as exc:  # report, do not substitute
        out["normal"] = {"error": str(exc)}
    if not a.no_recon:
        try:
            out["extras"] = time_extras(w, x)
        except Exception as exc:  # report, do not substitute
            out["extras"] = {"error": str(exc)}
    if tuned is not None:
        out["autotune"] = tuned

    # end-to-end through the public API with host (pinned) buffers: the
    # in-place products (the reference's mul!(y, op, x) and
    # mul!(x, adjoint(op), y)).  Every step copies its inputs in and its
    # results out and ends with the results on the host (stream synchronised).
    if not a.no_e2e:
        op.set_timing(False)
        xh = torch.from_numpy(w.x.astype(np.complex64)).pin_memory()
        yh = y.cpu().pin_memory()
        yo = torch.empty(op.nrow, dtype=torch.complex64, pin_memory=True)
        xo = torch.empty(op.ncol, dtype=torch.complex64, pin_memory=True)
        cur = torch.cuda.current_stream()

        def in_place_step():
            op.prod_(yo, xh)
            op.ctprod_(xo, yh)
            cur.synchronize()

        def alloc_step():
            op * xh
            op.H * yh

        n_e2e = max(3, a.steps // 2)
        res = {}
        for name, step in (("in_place", in_place_step), ("alloc", alloc_step)):
            for _ in range(3):
                step()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(n_e2e):
                step()
            torch.cuda.synchronize()
            res[name] = (time.perf_counter() - t0) / n_e2e
        e2e_s = max_over_ranks(res["in_place"] * 1e3, ws, dev) / 1e3
        alloc_s = max_over_ranks(res["alloc"] * 1e3, ws, dev) / 1e3
        out["e2e"] = {"value": replica_value(units, e2e_s * 1e3, ws), "unit": UNIT,
                      "h2d_bytes_per_step": int(xh.numel() * 8 + yh.numel() * 8),
                      "d2h_bytes_per_step": int(yo.numel() * 8 + xo.numel() * 8),
                      "ms_per_step": e2e_s * 1e3,
                      "api": "op.prod_(y, x) + op.ctprod_(x, y) on page-locked host tensors, one "
                             "stream synchronise per step",
                      "allocating_form": {"api": "y = op * x; x = op.H * y on page-locked host tensors",
                                          "ms_per_step": alloc_s * 1e3,
                                          "value": replica_value(units, alloc_s * 1e3, ws)}}

    check = out["recon"].pop("_check", None) if isinstance(out.get("recon"), dict) else None
    if rank == 0 and ws == 1 and not a.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(w, a.cpu_seconds, x, y, op)
        acc = {k: out["cpu_baseline"].pop(k) for k in list(out["cpu_baseline"]) if k.startswith("gpu_")}
        out["accuracy_vs_fp64"] = acc
        if check is not None and not a.no_recon_check:
            try:
                out["recon"]["accuracy"] = recon_fp64_check(w, *check, a.recon_iterations)
            except Exception as exc:  # report, do not substitute
                out["recon"]["accuracy"] = {"error": str(exc)}
    if rank == 0:
        print(json.dumps(out), flush=True)
    op.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_reference(a):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from hoexplicit import workloads
    from oracle import oracle
    w = workload(a.config)
    bf, k, t, f, c, idx = workloads.prepared_model(w)
    nSam = k.shape[1]
    xm = w.x[idx]
    rng = np.random.default_rng(0)
    # size one step to ~ (budget / (steps + warmup)) seconds, at most ~6 s
    budget = 150.0
    per_step = min(6.0, budget / (a.steps + a.warmup))
    probe = 16
    rows = np.sort(rng.choice(nSam, probe, replace=False))
    m = oracle.Model(bf, k[:, rows], t[rows], f, c)
    t0 = time.perf_counter()
    yo = oracle.forward(m, xm)
    oracle.adjoint(m, yo)
    per_row = (time.perf_counter() - t0) / probe
    n_rows = int(min(nSam, max(probe, per_step / max(per_row, 1e-9))))
    rows = np.sort(rng.choice(nSam, n_rows, replace=False))
    m = oracle.Model(bf, k[:, rows], t[rows], f, c)
    ysub = None
    for _ in range(a.warmup):
        ysub = oracle.forward(m, xm)
        oracle.adjoint(m, ysub)
    times = []
    for _ in range(a.steps):
        t0 = time.perf_counter()
        ysub = oracle.forward(m, xm)
        oracle.adjoint(m, ysub)
        times.append(time.perf_counter() - t0)
    units = 2.0 * len(idx) * n_rows
    s = statistics.mean(times)
    value = units / s
    sample = (f"each step: E and E^H over {n_rows} of {nSam} samples x {len(idx)} voxels x {w.nCha} coils "
              "(FP64 C restatement of array_operator.jl:241-348; the Julia reference cannot run here)")
    if a.config == "5":
        sample += "; slice 0 of the 24-slice batch (the reference applies slices one by one)"
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
           "steps": a.steps, "warmup": a.warmup, "ms_per_step": s * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded, shapes/distributions of the named configuration)",
           "config": workload_config(w, k.shape[0]),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": oracle.max_threads(), "kind": "port",
                            "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    a = parse_args()
    if a.impl == "reference":
        run_reference(a)
    elif a.config == "5":
        run_batch(a)
    else:
        run_gb300(a)


if __name__ == "__main__":
    main()
