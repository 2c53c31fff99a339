"""Benchmark: t-SNE optimizer iterations per second at 1M points (the 1M-point precision
workload: 1,000,000 x 50 mixture of 30 anisotropic clusters, exact KNN k = 90, perplexity 30).

One step = one optimizer iteration (grid repulsion + attractive pass + gains/momentum update)
of the resident 1M-point instance, P and state already in HBM. The line also carries:
  e2e          the same metric through the reference C ABI
               (fastembedr_cuda_opentsne_fft_from_knn_float) with pinned host buffers: H2D of
               the KNN, affinities, 250 + 750 iterations and D2H of the layout, per iteration;
  roofline     the dominant kernel (attractive CSR pass) against measured HBM bandwidth;
  cpu_baseline the CPU oracle (plain-C restatement of the reference CPU optimizer, bit-identical
               to it) on a bounded sample of the same workload on this host's cores.
`--impl reference` times that CPU implementation alone. Synthetic, seeded inputs stand in for a
dataset; inputs (P = 1.2 GB) exceed L2, so no explicit L2 flush is used.
Multi-GPU: replicas only (independent 1M instances, no collective); value is the aggregate.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

N_POINTS = 1_000_000
K = 90
PERPLEXITY = 30.0
WORKLOAD = "tsne_knn_1M_k90_perp30"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_inputs(device, n=N_POINTS):
    """The 1M-point mixture (or the same generator at n points, for profiling captures) and its
    exact KNN (torch brute force on the GPU: setup only)."""
    from fastembedr_gb300 import synthetic as S

    x, _ = S.tsne_1m(n=n)
    idx, dist = S.exact_knn_torch(x, K, device=device)
    return idx, dist


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, gpu_index=0):
        self.path = tempfile.mktemp(suffix=".csv")
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [t.strip() for t in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak_hbm():
    try:
        return float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic_per_nnz():
    """DRAM bytes per CSR entry of the attractive kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "attractive_kernel_tsne_200k.txt")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_nnz"):
                return float(line.split("=")[1])
    except OSError:
        pass
    return None


def cpu_baseline(idx_cpu, dist_cpu, iters):
    """Reference CPU optimizer (oracle, OpenMP over this host's cores) on the same workload:
    P built untimed, then `iters` iterations timed."""
    import oracle as O

    threads = O.orc().orc_set_threads(0)
    n = idx_cpu.shape[0]
    from fastembedr_gb300 import synthetic as S

    init = S.tsne_init(n)
    idx_cm = np.ascontiguousarray(idx_cpu.T).ravel()
    dist_cm = np.ascontiguousarray(dist_cpu.T).ravel()
    lib = O.orc()
    st = lib.orc_tsne_prepare(idx_cm, dist_cm, n, K, np.ascontiguousarray(init).ravel(), PERPLEXITY, 0)
    lib.orc_tsne_iterate(st, 1, 12.0, n / 12.0, 0.8, 0.01, 5.0)  # warm-up
    t = time.perf_counter()
    lib.orc_tsne_iterate(st, iters, 12.0, n / 12.0, 0.8, 0.01, 5.0)
    dt = time.perf_counter() - t
    lib.orc_tsne_free(st)
    return iters / dt, threads, dt


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import torch

    device = "cuda" if torch.cuda.is_available() else "cpu"
    if device == "cpu":
        print(json.dumps({"impl": "reference", "unavailable": "no GPU to synthesise the 1M-point exact KNN input"}))
        return 0
    idx, dist = make_inputs(device, args.n)
    idx_cpu, dist_cpu = idx.cpu().numpy(), dist.cpu().numpy()
    del idx, dist
    torch.cuda.empty_cache()
    import oracle as O

    O.build()
    lib = O.orc()
    threads = lib.orc_set_threads(0)
    n = idx_cpu.shape[0]
    from fastembedr_gb300 import synthetic as S

    init = S.tsne_init(n)
    st = lib.orc_tsne_prepare(np.ascontiguousarray(idx_cpu.T).ravel(), np.ascontiguousarray(dist_cpu.T).ravel(), n,
                              K, np.ascontiguousarray(init).ravel(), PERPLEXITY, 0)
    lib.orc_tsne_iterate(st, args.warmup, 12.0, n / 12.0, 0.8, 0.01, 5.0)
    t = time.perf_counter()
    lib.orc_tsne_iterate(st, args.steps, 12.0, n / 12.0, 0.8, 0.01, 5.0)
    dt = time.perf_counter() - t
    lib.orc_tsne_free(st)
    v = args.steps / dt
    line = {
        "impl": "reference", "metric": "tsne_iterations_per_s_1M", "value": v, "unit": "iter/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD if n == N_POINTS else f"tsne_knn_{n}_k90_perp30", "n": n, "k": K, "perplexity": PERPLEXITY, "grid": "reference CPU policy (256)",
                   "l2": "host CPU run"},
        "cpu_baseline": {"value": v, "unit": "iter/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} iterations of the 1M-point optimizer after P is built"},
        "e2e": {"value": v, "unit": "iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_gpu(args):
    import torch
    import torch.distributed as tdist

    from fastembedr_gb300 import _lib, api
    from fastembedr_gb300 import synthetic as S

    rank, world, local = dist_env()
    if world > 1:
        tdist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    device = f"cuda:{local}"
    idx, dist = make_inputs(device, args.n)
    n = idx.shape[0]
    d_idx = idx.T.contiguous()
    d_dist = dist.T.contiguous()
    init = S.tsne_init(n)
    plan = api.TsnePlan(d_idx, d_dist, n, K, PERPLEXITY, init=init)
    info = plan.info()
    lr = n / 12.0
    # untimed early-exaggeration phase, as in a real run, then the warm-up steps
    plan.run(250, 12.0, lr)
    plan.run(args.warmup, 1.0, lr)
    plan.synchronize()

    def barrier():
        if world > 1:
            tdist.barrier()
        torch.cuda.synchronize()

    stream = torch.cuda.ExternalStream(plan.stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    barrier()
    ev0.record(stream)
    plan.run(args.steps, 1.0, lr)
    ev1.record(stream)
    plan.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    # dominant kernel, timed alone with CUDA events on the plan's stream over the same number of steps
    prof = plan.profile(args.steps, 1.0, lr)
    kl = plan.kl() if not args.no_kl else None
    t_ms = torch.tensor([ms], device=device)
    if world > 1:
        tdist.all_reduce(t_ms, op=tdist.ReduceOp.MAX)
    ms = float(t_ms.item())
    plan.close()
    value = world * args.steps / (ms / 1e3)

    if args.no_e2e:
        if rank == 0:
            print(json.dumps({"metric": "tsne_iterations_per_s", "n": n, "nnz": info["nnz"], "value": value,
                              "ms_per_step": ms / args.steps,
                              "stage_ms_per_step": {k_: v / args.steps for k_, v in prof.items()}}))
        return 0
    # end to end through the reference C ABI with pinned host buffers, full 1000-iteration job
    idx_h = torch.empty((K, n), dtype=torch.int32, pin_memory=True)
    dist_h = torch.empty((K, n), dtype=torch.float32, pin_memory=True)
    idx_h.copy_(d_idx)
    dist_h.copy_(d_dist)
    init_h = torch.from_numpy(init).pin_memory()
    out_h = torch.empty((n, 2), dtype=torch.float32, pin_memory=True)
    del d_idx, d_dist, idx, dist
    torch.cuda.empty_cache()
    lib = _lib.require_gpu()
    e2e_iters = 1000
    barrier()
    t0 = time.perf_counter()
    st = lib.fastembedr_cuda_opentsne_fft_from_knn_float(
        idx_h.data_ptr(), dist_h.data_ptr(), init_h.data_ptr(), 1, n, K, 2, PERPLEXITY, 250, 750, 12.0, 1.0, lr, 0,
        0.8, 0.8, 0.01, 5.0, 4, 0, out_h.data_ptr())
    barrier()
    e2e_s = time.perf_counter() - t0
    _lib.check(st, "e2e t-SNE")
    e2e = {"value": world * e2e_iters / e2e_s, "unit": "iter/s",
           "h2d_bytes_per_step": int((idx_h.numel() * 4 + dist_h.numel() * 4 + init_h.numel() * 4) / e2e_iters),
           "d2h_bytes_per_step": int(out_h.numel() * 4 / e2e_iters), "job_seconds": e2e_s,
           "job": "H2D KNN + affinities + 250 + 750 iterations + D2H layout"}

    nnz = info["nnz"]
    alg_bytes = 8 * nnz + 24 * n + 4
    attr_ms = prof["attractive_kernel_ms"] / args.steps
    peak, peak_kind = measured_peak_hbm()
    achieved = alg_bytes / (attr_ms * 1e-3) / 1e9
    tpn = profiled_traffic_per_nnz()
    roofline = {"kernel": "attractive_kernel", "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": None if tpn is None else tpn * nnz,
                "algorithmic_bytes": alg_bytes, "avg_launch_ms": attr_ms,
                "step_fraction_of_hbm": (8 * nnz + 60 * n) / (ms / args.steps * 1e-3) / 1e9 / peak}
    launches = args.steps * info["launches_per_iteration"] + ((args.steps + 24) // 25) * 22

    line = {
        "metric": "tsne_iterations_per_s_1M", "value": value, "unit": "iter/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD if n == N_POINTS else f"tsne_knn_{n}_k90_perp30", "n": n, "k": K, "perplexity": PERPLEXITY, "nnz_P": nnz,
                   "fft_grid": info["grid_size"], "stencil": "bilinear" if info["interpolation"] == 0 else "lagrange3",
                   "phase": "normal (after 250 early-exaggeration iterations)",
                   "l2": "inputs larger than L2 (P = %.2f GB), no flush" % (8 * nnz / 1e9),
                   "parallelism": f"replicas x{world}"},
        "clocks": clk, "e2e": e2e, "roofline": roofline, "gpu_launches": launches,
        "stage_ms_per_step": {k_: v / args.steps for k_, v in prof.items()},
    }
    if kl is not None:
        line["kl_after_run"] = kl
    if rank == 0 and not args.no_cpu:
        idx_cpu, dist_cpu = idx_h.T.contiguous().numpy(), dist_h.T.contiguous().numpy()
        v, threads, dt = cpu_baseline(idx_cpu, dist_cpu, args.cpu_iters)
        line["cpu_baseline"] = {"value": v, "unit": "iter/s", "cores": threads, "kind": "port",
                                "sample": f"{args.cpu_iters} iterations of the same 1M-point instance "
                                          f"({dt:.1f} s), P built untimed, reference CPU grid policy"}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        tdist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=25)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-iters", type=int, default=20)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-kl", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--n", type=int, default=N_POINTS, help="points (profiling captures use a smaller case)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
