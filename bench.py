"""Benchmark of the KNN-input embedding optimizer: t-SNE iterations/s at 1M points, UMAP
epochs/s, batched and served forms against the plain form, p50/p99 latency.

Headline (`value`): t-SNE optimizer iterations per second on the 1M-point precision workload
(1,000,000 x 50 mixture of 30 anisotropic clusters, exact KNN k = 90, perplexity 30). One step =
one optimizer iteration (grid repulsion + attractive pass + gains/momentum update) of the resident
instance, P and state already in HBM, in the normal phase (after the 250 early-exaggeration
iterations). The line also carries:
  e2e            the same metric through the reference C ABI
                 (fastembedr_cuda_opentsne_fft_from_knn_float) with pinned host buffers: H2D of
                 the KNN, affinities, 250 + 750 iterations and D2H of the layout, per iteration;
  roofline       the dominant kernel (attractive CSR pass) against measured HBM bandwidth;
  cpu_baseline   the CPU oracle (plain-C restatement of the reference CPU optimizer, bit-identical
                 to it) timed on normal-phase iterations of the same instance on this host's cores;
  kl_parity_1M   KL and 15-NN preservation of the e2e job's layout against the reference CPU run
                 of the same workload (tests/golden/tsne_1m_cpu_run.json);
  umap           UMAP epochs/s at 100k (k = 15, 500 epochs), with its own e2e and CPU baseline;
  batched        512 instances (sizes log-uniform in [2k, 200k], half t-SNE, half UMAP) in one
                 batch against one call per instance, with per-instance KL / 15-NN parity;
  serving        transform_tsne served (500k reference, Poisson query batches of 1..50k):
                 points/s, served vs plain, p50/p99 latency.
`--headline-only` skips the last three; `--workload umap|batched|serving` runs one of them alone.
`--impl reference` times the reference CPU implementation (the oracle) on the headline workload.
Synthetic, seeded inputs stand in for a dataset; inputs (P = 1.2 GB) exceed L2, so no explicit L2
flush is used. Multi-GPU: replicas only (independent 1M instances, no collective); value is the
aggregate and the secondary workloads run only at N = 1.
"""
from __future__ import annotations

import argparse
import hashlib
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
GRADIENT_SEED = 2026  # seed of the gradient-check sample


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def replica_time_ms(ms, world, device):
    """The job's time over N replicas is the slowest replica's: max over ranks (all_reduce MAX
    on the process group; gloo on CPU tensors, NCCL on CUDA tensors)."""
    import torch

    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    if world > 1:
        import torch.distributed as tdist

        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(steps, ms, world):
    """Whole-job rate: every replica ran `steps` units in at most `ms` milliseconds."""
    return world * steps / (ms / 1e3)


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


def cpu_baseline(idx_cpu, dist_cpu, iters, start):
    """Reference CPU optimizer (oracle, OpenMP over this host's cores) on the same workload and
    phase as the GPU's timed steps: P built untimed, the GPU's normal-phase layout as the start,
    one warm-up iteration, then `iters` normal-phase iterations (exaggeration 1) timed."""
    import oracle as O

    threads = O.orc().orc_set_threads(0)
    n = idx_cpu.shape[0]
    idx_cm = np.ascontiguousarray(idx_cpu.T).ravel()
    dist_cm = np.ascontiguousarray(dist_cpu.T).ravel()
    lib = O.orc()
    st = lib.orc_tsne_prepare(idx_cm, dist_cm, n, K, np.ascontiguousarray(start, np.float32).ravel(), PERPLEXITY, 0)
    lib.orc_tsne_iterate(st, 1, 1.0, n / 12.0, 0.8, 0.01, 5.0)  # warm-up
    t = time.perf_counter()
    lib.orc_tsne_iterate(st, iters, 1.0, n / 12.0, 0.8, 0.01, 5.0)
    dt = time.perf_counter() - t
    lib.orc_tsne_free(st)
    return iters / dt, threads, dt


def gradient_summary(plan, args):
    """Grid gradient of the final layout against exact FP64-summed repulsion (all-pairs Z) at a
    seeded sample of points."""
    c = plan.gradient_check(sample=args.check_sample, seed=GRADIENT_SEED)
    return {"sample": int(c["rows"].shape[0]), "seed": GRADIENT_SEED, "grid_size": plan.info()["grid_size"],
            "gradient_rel_l2": c["gradient_rel_l2"], "repulsion_rel_l2": c["repulsion_rel_l2"],
            "repulsion_max_rel": c["repulsion_max_rel"], "z_rel_err": c["z_rel_err"]}


PARITY_FIXTURE = os.path.join(ROOT, "tests", "golden", "tsne_1m_cpu_run.json")


def _layout_quality(idx_nk, dist_nk, y, keep_stride):
    """Exact KL (all-pairs Z) of layout y under the workload's P and its 15-NN preservation over
    every keep_stride-th row (oracle)."""
    import oracle as O
    from fastembedr_gb300 import api

    with api.TsneBatch([(idx_nk, dist_nk)], perplexity=PERPLEXITY, inits=[np.ascontiguousarray(y, np.float32)]) as b:
        kl = b.kl(0)
    keep = np.arange(0, y.shape[0], keep_stride, dtype=np.int32)
    return kl, float(O.knn_preservation(y, idx_nk, keep=keep, preserve_k=15))


def kl_parity_1m(lib, idx_h, dist_h, init_h, layout_policy, lr):
    """End-to-end parity at 1M points: the final KL and 15-NN preservation of the full
    1000-iteration job against the reference CPU run of the same workload (committed fixture,
    made by tests/golden/make_tsne_1m_fixture.py). Two GPU runs: the CUDA size policy (1024 nodes,
    the e2e job above) and the reference CPU's own grid (256 nodes), the like-for-like one."""
    from fastembedr_gb300 import _lib

    try:
        ref = json.load(open(PARITY_FIXTURE))
    except OSError:
        return {"unavailable": "tests/golden/tsne_1m_cpu_run.json missing"}
    n = layout_policy.shape[0]
    idx_nk = np.ascontiguousarray(idx_h.numpy().T)
    dist_nk = np.ascontiguousarray(dist_h.numpy().T)
    same_input = (hashlib.sha256(idx_nk.tobytes()).hexdigest() == ref["knn"]["indices_sha256"]
                  and hashlib.sha256(dist_nk.tobytes()).hexdigest() == ref["knn"]["distances_sha256"])
    out = np.zeros((n, 2), np.float32)
    os.environ["FASTEMBEDR_TSNE_FFT_GRID"] = "256"
    try:
        st = lib.fastembedr_cuda_opentsne_fft_from_knn_float(
            idx_h.data_ptr(), dist_h.data_ptr(), init_h.data_ptr(), 1, n, K, 2, PERPLEXITY, 250, 750, 12.0, 1.0, lr, 0,
            0.8, 0.8, 0.01, 5.0, 4, 0, out.ctypes.data)
    finally:
        del os.environ["FASTEMBEDR_TSNE_FFT_GRID"]
    _lib.check(st, "t-SNE at the CPU grid")
    stride = int(ref["preservation_rows"].split()[1][:-2])
    res = {"reference": {"kl": ref["kl"], "preservation_15nn": ref["preservation_15nn"],
                         "run": "oracle CPU optimizer (bit-identical to the reference CPU code), 250 + 750 "
                                "iterations, 256-node grid", "cpu_seconds": ref["cpu_seconds"]},
           "same_knn_input": bool(same_input), "preservation_rows": ref["preservation_rows"],
           "bar": "KL within 1 %, 15-NN preservation within 0.01"}
    for tag, y in (("cuda_policy_grid_1024", layout_policy), ("cpu_policy_grid_256", out)):
        kl, pres = _layout_quality(idx_nk, dist_nk, y, stride)
        res[tag] = {"kl": kl, "kl_rel": (kl - ref["kl"]) / ref["kl"], "preservation_15nn": pres,
                    "preservation_diff": pres - ref["preservation_15nn"]}
    return res


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
    # the same phase as the GPU arm's timed steps: the 250 early-exaggeration iterations and the
    # warm-up run untimed, then `steps` normal-phase iterations (exaggeration 1) are timed
    t_early = time.perf_counter()
    lib.orc_tsne_iterate(st, 250, 12.0, n / 12.0, 0.8, 0.01, 5.0)
    early_s = time.perf_counter() - t_early
    lib.orc_tsne_iterate(st, args.warmup, 1.0, n / 12.0, 0.8, 0.01, 5.0)
    t = time.perf_counter()
    lib.orc_tsne_iterate(st, args.steps, 1.0, n / 12.0, 0.8, 0.01, 5.0)
    dt = time.perf_counter() - t
    lib.orc_tsne_free(st)
    v = args.steps / dt
    line = {
        "impl": "reference", "metric": "tsne_iterations_per_s_1M", "value": v, "unit": "iter/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD if n == N_POINTS else f"tsne_knn_{n}_k90_perp30", "n": n, "k": K,
                   "perplexity": PERPLEXITY, "grid": "reference CPU policy (256)",
                   "phase": "normal (after 250 early-exaggeration iterations)", "l2": "host CPU run"},
        "cpu_baseline": {"value": v, "unit": "iter/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} normal-phase iterations of the 1M-point optimizer after P is "
                                   f"built and 250 early-exaggeration iterations ({early_s:.0f} s) ran untimed"},
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
    torch.cuda.synchronize()
    t_setup = time.perf_counter()
    plan = api.TsnePlan(d_idx, d_dist, n, K, PERPLEXITY, init=init)
    setup_s = time.perf_counter() - t_setup  # validation, bisection, symmetrised P, state (synchronous)
    info = plan.info()
    lr = n / 12.0
    # the early-exaggeration phase, as in a real run (timed apart, CUDA graph captures included),
    # then the warm-up steps: at least two 25-iteration chunks and one call like the timed one, so
    # that every CUDA graph the timed call replays is captured before timing
    t_early = time.perf_counter()
    plan.run(250, 12.0, lr)
    plan.synchronize()
    early_s = time.perf_counter() - t_early
    plan.run(max(args.warmup, 50), 1.0, lr)
    # the timed call's own chunk sizes once, so its CUDA graphs are captured before timing
    plan.run(args.steps, 1.0, lr)
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
    gcheck = gradient_summary(plan, args) if not args.no_kl else None
    normal_layout = plan.layout()  # start of the CPU baseline's normal-phase iterations
    tuning = plan.tuning()
    ms = replica_time_ms(ms, world, device)
    plan.close()
    value = aggregate_rate(args.steps, ms, world)

    # the same instance under the adaptive box count (grid sizes chosen from the layout every 25
    # iterations), timed the same way; its KL is taken after as many iterations as the main plan's
    adaptive = None
    if not args.no_adaptive:
        os.environ["FASTEMBEDR_TSNE_FFT_GRID"] = "adaptive"
        try:
            plan2 = api.TsnePlan(d_idx, d_dist, n, K, PERPLEXITY, init=init)
            plan2.run(250, 12.0, lr)
            plan2.run(max(args.warmup, 50), 1.0, lr)
            plan2.run(args.steps, 1.0, lr)
            plan2.synchronize()
            st2 = torch.cuda.ExternalStream(plan2.stream)
            a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            barrier()
            a0.record(st2)
            plan2.run(args.steps, 1.0, lr)
            a1.record(st2)
            plan2.synchronize()
            ms2 = a0.elapsed_time(a1)
            plan2.run(args.steps, 1.0, lr)  # as many iterations as the main plan's profiling pass
            kl2 = plan2.kl() if not args.no_kl else None
            gcheck2 = gradient_summary(plan2, args) if not args.no_kl else None
            g2 = plan2.info()["grid_size"]
            plan2.close()
        finally:
            del os.environ["FASTEMBEDR_TSNE_FFT_GRID"]
        adaptive = {"value": world * args.steps / (ms2 / 1e3), "unit": "iter/s", "ms_per_step": ms2 / args.steps,
                    "grid_at_end": g2, "kl_after_run": kl2, "gradient_check": gcheck2,
                    "policy": "adaptive box count: node spacing <= 0.7 over the current layout, >= 128 nodes, "
                              "re-chosen every 25 iterations"}

    if args.no_e2e:
        if rank == 0:
            print(json.dumps({"metric": "tsne_iterations_per_s", "n": n, "nnz": info["nnz"], "value": value,
                              "ms_per_step": ms / args.steps, "kl_after_run": kl, "adaptive_grid": adaptive,
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
    parity = None
    if rank == 0 and not args.no_kl and n == N_POINTS:
        parity = kl_parity_1m(lib, idx_h, dist_h, init_h, out_h.numpy().copy(), lr)

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
    launches = args.steps * info["launches_per_iteration"] + ((args.steps + 24) // 25) * info["launches_per_reorder"]

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
        "attractive_launch_tuning": tuning,
        "setup": {"affinities_and_state_s": setup_s, "early_phase_ms_per_iter": early_s * 1e3 / 250,
                  "note": "device KNN -> P and optimizer state; 250 early-exaggeration iterations incl. graph capture"},
    }
    if kl is not None:
        line["kl_after_run"] = kl
    if gcheck is not None:
        line["gradient_check"] = gcheck
    if adaptive is not None:
        line["adaptive_grid"] = adaptive
    if parity is not None:
        line["kl_parity_1M"] = parity
    if rank == 0 and not args.no_cpu:
        idx_cpu, dist_cpu = idx_h.T.contiguous().numpy(), dist_h.T.contiguous().numpy()
        v, threads, dt = cpu_baseline(idx_cpu, dist_cpu, args.cpu_iters, normal_layout)
        line["cpu_baseline"] = {"value": v, "unit": "iter/s", "cores": threads, "kind": "port",
                                "sample": f"{args.cpu_iters} normal-phase iterations of the same 1M-point instance "
                                          f"({dt:.1f} s) from the GPU's layout at the timed steps, P built untimed, "
                                          "reference CPU grid policy"}
    del idx_h, dist_h, init_h, out_h
    if rank == 0 and world == 1 and not args.headline_only:
        # the other terms of the metric, each with its own timing, e2e and baselines
        torch.cuda.empty_cache()
        line["umap"] = umap_result(args, local)
        torch.cuda.empty_cache()
        line["batched"] = batched_result(args, local)
        torch.cuda.empty_cache()
        line["serving"] = serving_result(args, local)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        tdist.destroy_process_group()
    return 0


# ---------------------------------------------------------------- secondary workloads
SERVE_N_REF = 500_000
SERVE_K = 90
SERVE_ITERS = 250


def _serving_inputs(args, device):
    """Reference 500,000 x 50 (20 clusters) embedded once with t-SNE (perplexity 30, k = 90, the
    package schedule) and a 100,000-query pool with exact k = 90 KNN into the reference; the
    request list: batch sizes log-uniform in [1, 50,000], Poisson arrivals."""
    from fastembedr_gb300 import api
    from fastembedr_gb300 import synthetic as S

    n_ref = args.n_ref
    ref_x, pool_x = S.serving_transform(n_ref=n_ref)
    ridx, rdist = S.exact_knn_torch(ref_x, SERVE_K, device=device)
    fit = api.tsne_knn(ridx.cpu().numpy(), rdist.cpu().numpy(), perplexity=30.0, Y_init=S.tsne_init(n_ref))
    del ridx, rdist
    qidx, qdist = S.exact_knn_query_torch(ref_x, pool_x, SERVE_K, device=device)
    qidx = (qidx + 1).cpu().numpy()  # 1-based, as R passes them
    qdist = qdist.cpu().numpy()
    rng = np.random.default_rng(17)
    sizes = np.exp(rng.uniform(0.0, np.log(50_000), args.requests)).astype(np.int64).clip(1, 50_000)
    offsets = np.array([rng.integers(0, qidx.shape[0] - s_ + 1) for s_ in sizes])
    gaps = rng.exponential(1.0, args.requests)  # unit-rate Poisson gaps, scaled per run
    reqs = [(np.asfortranarray(qidx[o:o + s_]), np.asfortranarray(qdist[o:o + s_])) for o, s_ in zip(offsets, sizes)]
    return fit.layout.astype(np.float64), reqs, gaps


def _serve(ref_layout, reqs, arrivals, budget, slots=4):
    """Submit each request at its arrival time (None: all at once); return wall seconds,
    latencies (ms) and the server counters."""
    from fastembedr_gb300 import api

    with api.TransformServer(ref_layout, perplexity=5.0, memory_budget_bytes=budget, max_inflight=slots) as sv:
        sv.result(sv.submit(reqs[0][0][:4], reqs[0][1][:4]))  # warm-up: kernels loaded, pools touched
        ids = []
        t0 = time.perf_counter()
        for j, (qi, qd) in enumerate(reqs):
            if arrivals is not None:
                while time.perf_counter() - t0 < arrivals[j]:
                    time.sleep(0.0001)
            ids.append(sv.submit(qi, qd))
        lat = [sv.result(i)[1] for i in ids]
        wall = time.perf_counter() - t0
        stats = sv.stats()
    return wall, np.array(lat), stats


def run_serving(args):
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    print(json.dumps(serving_result(args, local)))
    return 0


def serving_result(args, local):
    """Serving form of transform_tsne (fixed-reference transform) on one GPU."""
    import torch

    from fastembedr_gb300 import api

    torch.cuda.set_device(local)
    device = f"cuda:{local}"
    ref_layout, reqs, gaps = _serving_inputs(args, device)
    torch.cuda.empty_cache()
    points = int(sum(r[0].shape[0] for r in reqs))
    budget = 40 << 30
    # warm-up, then saturation: every request queued at t = 0 (closed loop, capacity)
    _serve(ref_layout, reqs[: args.warmup], None, budget, args.serve_slots)
    clocks = ClockSampler(local)
    wall, lat_sat, st = _serve(ref_layout, reqs, None, budget, args.serve_slots)
    clk = clocks.stop()
    capacity = points / wall
    # open loop: Poisson arrivals at 70% of capacity (in requests/s)
    rate = 0.7 * len(reqs) / wall
    wall_p, lat, st_p = _serve(ref_layout, reqs, np.cumsum(gaps) / rate, budget, args.serve_slots)
    # the plain one-instance-per-call GPU form: each request through the one-shot C ABI in turn
    n_plain = min(len(reqs), args.plain_requests)
    t0 = time.perf_counter()
    for qi, qd in reqs[:n_plain]:
        api.transform_tsne(ref_layout, dict(indices=qi, distances=qd.astype(np.float64)), perplexity=5.0)
    plain_wall = time.perf_counter() - t0
    plain_points = int(sum(r[0].shape[0] for r in reqs[:n_plain]))
    # the largest group alone: iterate-kernel throughput for the roofline
    big = max(range(len(reqs)), key=lambda j: reqs[j][0].shape[0])
    _, _, st_big = _serve(ref_layout, [reqs[big]], None, budget, args.serve_slots)
    nq_big = st_big["largest_group_queries"]
    it_ms = st_big["largest_group_iterate_ms"]
    n_neg = 256
    alg_bytes = nq_big * SERVE_ITERS * (SERVE_K * 12 + n_neg * 8)
    peak, peak_kind = measured_peak_hbm()
    achieved = alg_bytes / (it_ms * 1e-3) / 1e9
    h2d = int(sum(r[0].nbytes + r[1].nbytes for r in reqs))
    line = {
        "metric": "transform_points_per_s_served", "value": capacity, "unit": "points/s", "n_gpus": 1,
        "steps": len(reqs), "warmup": args.warmup, "ms_per_step": 1e3 * wall / len(reqs), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "transform_tsne_serving_ref500k_k90", "n_reference": SERVE_N_REF if args.n_ref == SERVE_N_REF
                   else args.n_ref, "k": SERVE_K, "iterations": SERVE_ITERS, "repulsion": "sampled, 256 negatives",
                   "requests": len(reqs), "points": points, "batch_sizes": "log-uniform [1, 50000]",
                   "memory_budget_gb": 40, "groups_in_flight": args.serve_slots,
                   "l2": "reference layout is L2-resident by design; no flush"},
        "points_iterations_per_s": capacity * SERVE_ITERS,
        "latency_ms": {"rate_req_per_s": rate, "p50": float(np.percentile(lat, 50)),
                       "p99": float(np.percentile(lat, 99)), "wall_s": wall_p,
                       "saturated_p50": float(np.percentile(lat_sat, 50)),
                       "saturated_p99": float(np.percentile(lat_sat, 99))},
        "plain_gpu": {"points_per_s": plain_points / plain_wall, "requests": n_plain,
                      "form": "one fastembedr_cuda_transform_tsne call per request, in turn"},
        "served_vs_plain": capacity / (plain_points / plain_wall),
        "server": st, "clocks": clk,
        "e2e": {"value": capacity, "unit": "points/s", "h2d_bytes_per_step": h2d // len(reqs),
                "d2h_bytes_per_step": points * 16 // len(reqs),
                "note": "the serving API takes host KNN and returns host layouts: value is end to end"},
        "roofline": {"kernel": "transform_iterate_kernel", "bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind, "traffic": None,
                     "algorithmic_bytes": alg_bytes, "avg_launch_ms": it_ms, "group_queries": nq_big,
                     "note": "P/neighbour rows and the sampled reference gathers are L2-resident"},
        "gpu_launches": int(st["launches"]),
    }
    if not args.no_cpu:
        line["cpu_baseline"] = _cpu_transform_baseline(ref_layout, reqs)
    return line


def _cpu_transform_baseline(ref_layout, reqs):
    """transform_tsne_cpp restated (oracle, OpenMP over this host's cores) on the first
    requests, up to ~4,000 queries: same options as the served run."""
    import oracle as O

    O.build()
    threads = O.orc().orc_set_threads(0)
    sample, total = [], 0
    for qi, qd in reqs:
        if total >= 4000:
            break
        sample.append((qi, qd))
        total += qi.shape[0]
    t = time.perf_counter()
    for qi, qd in sample:
        O.transform_tsne(ref_layout, qi, qd.astype(np.float64), n_negatives=256, exact_threshold=4096, seed=4)
    dt = time.perf_counter() - t
    return {"value": total / dt, "unit": "points/s", "cores": threads, "kind": "port",
            "sample": f"{len(sample)} requests, {total} queries x {SERVE_ITERS} iterations ({dt:.1f} s)"}


def run_serving_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    import torch

    if not torch.cuda.is_available():
        print(json.dumps({"impl": "reference", "unavailable": "no GPU to synthesise the serving inputs"}))
        return 0
    ref_layout, reqs, _ = _serving_inputs(args, f"cuda:{local}")
    b = _cpu_transform_baseline(ref_layout, reqs)
    print(json.dumps({"impl": "reference", "metric": "transform_points_per_s_served", "value": b["value"],
                      "unit": "points/s", "n_gpus": world, "steps": 1, "warmup": 0, "higher_is_better": True,
                      "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                      "config": {"workload": "transform_tsne_serving_ref500k_k90"}, "cpu_baseline": b,
                      "e2e": {"value": b["value"], "unit": "points/s", "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0}}))
    return 0


UMAP_N = 100_000
UMAP_K = 15
UMAP_EPOCHS = 500


def _pca_init(x):
    """Top two principal components scaled to max |y| = 10 (the batched workload's start)."""
    xc = x.astype(np.float64) - x.mean(0)
    _, _, vt = np.linalg.svd(xc[:: max(1, x.shape[0] // 20000)], full_matrices=False)
    y = xc @ vt[:2].T
    return (y * (10.0 / np.abs(y).max())).astype(np.float32)


UMAP_SEED = 42


def _umap_start(idx_h, dist_h, rounds):
    """The package's spectral start of the KNN graph (computed on the GPU) and its wall time."""
    from fastembedr_gb300 import api

    api.umap_spectral_start(idx_h, dist_h, 1, UMAP_SEED)  # context and code warm-up
    t = time.perf_counter()
    start = api.umap_spectral_start(idx_h, dist_h, rounds, UMAP_SEED)
    return start, time.perf_counter() - t


def run_umap(args):
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    print(json.dumps(umap_result(args, local)))
    return 0


def umap_result(args, local):
    """UMAP epochs per second at 100,000 x 50 (20 clusters, log-normal sizes), k = 15, 500 epochs."""
    import ctypes as C

    import torch

    from fastembedr_gb300 import _lib, api
    from fastembedr_gb300 import synthetic as S

    torch.cuda.set_device(local)
    x, _ = S.plain_umap_100k(n=args.n_umap)
    idx, dist = S.exact_knn_torch(x, UMAP_K, device=f"cuda:{local}")
    idx_h = np.asfortranarray(idx.cpu().numpy())
    dist_h = np.asfortranarray(dist.cpu().numpy())
    n = idx_h.shape[0]
    rounds = api.umap_spectral_n_iter(n, UMAP_K)
    start, start_s = _umap_start(idx_h, dist_h, rounds)
    init = np.ascontiguousarray(start.astype(np.float32))
    out = np.zeros((n, 2), np.float32)
    lib = _lib.require_gpu()
    gm, sm = C.c_float(), C.c_float()

    def job(epochs):
        t = time.perf_counter()
        st = lib.fastembedr_cuda_umap_from_knn_profile(idx_h.ctypes.data, dist_h.ctypes.data, init.ctypes.data, n,
                                                       UMAP_K, 0, epochs, 5, 1.0, 0.01, 1.0, 42, out.ctypes.data,
                                                       C.byref(gm), C.byref(sm))
        _lib.check(st, "UMAP")
        return time.perf_counter() - t

    def whole_job(epochs):
        """umap_knn through the C ABI: H2D KNN, graph, spectral start, SGD, D2H layout."""
        t = time.perf_counter()
        st = lib.fastembedr_cuda_umap_knn_spectral(idx_h.ctypes.data, dist_h.ctypes.data, n, UMAP_K, 0, epochs, 5,
                                                   1.0, 0.01, 1.0, rounds, float("nan"), UMAP_SEED, out.ctypes.data)
        _lib.check(st, "UMAP")
        return time.perf_counter() - t

    for _ in range(args.warmup):
        job(25)
    whole_job(25)
    clocks = ClockSampler(local)
    job(UMAP_EPOCHS)
    wall = whole_job(UMAP_EPOCHS)
    clk = clocks.stop()
    job(UMAP_EPOCHS)
    sgd_ms, graph_ms = sm.value, gm.value
    line = {
        "metric": "umap_epochs_per_s_100k", "value": UMAP_EPOCHS / (sgd_ms * 1e-3), "unit": "epochs/s",
        "n_gpus": 1, "steps": UMAP_EPOCHS, "warmup": args.warmup, "ms_per_step": sgd_ms / UMAP_EPOCHS,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "umap_knn_100k_k15_500epochs", "n": n, "k": UMAP_K, "epochs": UMAP_EPOCHS,
                   "negative_sample_rate": 5, "min_dist": 0.01,
                   "init": f"the package's spectral start ({rounds} rounds, seed {UMAP_SEED}), computed on the GPU",
                   "l2": "edge list and layout are L2-resident (about 40 MB); no flush"},
        "graph_ms": graph_ms, "clocks": clk,
        "spectral_start": {"rounds": rounds, "gpu_wall_ms": start_s * 1e3,
                           "job": "H2D KNN + GPU fuzzy graph + spectral start + D2H"},
        "e2e": {"value": UMAP_EPOCHS / wall, "unit": "epochs/s", "h2d_bytes_per_step": (idx_h.nbytes + dist_h.nbytes)
                // UMAP_EPOCHS, "d2h_bytes_per_step": out.nbytes // UMAP_EPOCHS,
                "job": "umap_knn through fastembedr_cuda_umap_knn_spectral: H2D KNN + GPU fuzzy graph + "
                       "spectral start + 500 epochs + D2H layout"},
        "gpu_launches": 2 * UMAP_EPOCHS,
    }
    if not args.no_cpu:
        line["cpu_baseline"] = _cpu_umap_baseline(idx_h, dist_h, init)
        line["spectral_start"].update(_cpu_start_baseline(idx_h, dist_h, rounds, start))
    return line


UMAP_CPU_EPOCHS = 40


def _cpu_umap_baseline(idx_h, dist_h, init, epochs=UMAP_CPU_EPOCHS):
    """Reference CPU SGD on the same graph and start, `epochs` epochs: the oracle restatement of
    optimize_layout_csr's multi-threaded branch with the package's default worker count at this
    size (umap_default_threads: min(4, cores) at n >= 500, k >= 15; the branch runs at n >= 10000),
    or its serial branch when one worker is all the host has."""
    import oracle as O

    O.build()
    n = idx_h.shape[0]
    off, nb, w, e, mw = O.umap_graph(np.ascontiguousarray(idx_h), np.ascontiguousarray(dist_h))
    a, b = O.umap_ab(0.01)
    emb = np.ascontiguousarray(init.T.astype(np.float64)).ravel().copy()
    workers = max(1, min(4, os.cpu_count() or 1))
    threaded = workers > 1 and n >= 10000
    t = time.perf_counter()
    if threaded:
        O.orc().orc_umap_sgd_threaded(n, off, nb, w, emb, epochs, a, b, 5, 1.0, 1.0, 42, workers)
    else:
        O.orc().orc_umap_sgd_serial(n, off, nb, w, emb, epochs, a, b, 5, 1.0, 1.0, 42)
    dt = time.perf_counter() - t
    branch = f"multi-threaded branch, {workers} workers" if threaded else "serial branch"
    return {"value": epochs / dt, "unit": "epochs/s", "cores": workers if threaded else 1, "kind": "port",
            "sample": f"first {epochs} of {UMAP_EPOCHS} epochs on the same graph and start, {branch} "
                      f"({dt:.1f} s)"}


def _cpu_start_baseline(idx_h, dist_h, rounds, gpu_start):
    """The reference CPU spectral start (oracle restatement of initialize_layout_csr, one thread)
    on the graph the GPU built, and its largest difference from the GPU start (the start is
    ill-conditioned in the graph weights, so only the same graph gives a like-for-like check)."""
    import oracle as O
    from fastembedr_gb300 import api

    O.build()
    g = api.umap_graph(np.ascontiguousarray(idx_h), np.ascontiguousarray(dist_h))
    t = time.perf_counter()
    cpu = O.umap_spectral_init(g["offsets"], g["neighbors"], g["weights"], rounds, UMAP_SEED)
    dt = time.perf_counter() - t
    return {"cpu_ms": dt * 1e3, "cpu_cores": 1, "cpu_kind": "port (graph built beforehand, not timed)",
            "max_abs_diff_gpu_vs_cpu_same_graph": float(np.abs(cpu - gpu_start).max()),
            "layout_scale": "max |y| = 10"}


def run_umap_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    import torch

    from fastembedr_gb300 import synthetic as S

    if not torch.cuda.is_available():
        print(json.dumps({"impl": "reference", "unavailable": "no GPU to synthesise the KNN input"}))
        return 0
    x, _ = S.plain_umap_100k(n=args.n_umap)
    idx, dist = S.exact_knn_torch(x, UMAP_K, device=f"cuda:{local}")
    idx_h, dist_h = np.asfortranarray(idx.cpu().numpy()), np.asfortranarray(dist.cpu().numpy())
    from fastembedr_gb300 import api

    start, _ = _umap_start(idx_h, dist_h, api.umap_spectral_n_iter(idx_h.shape[0], UMAP_K))
    b = _cpu_umap_baseline(idx_h, dist_h, np.ascontiguousarray(start.astype(np.float32)))
    print(json.dumps({"impl": "reference", "metric": "umap_epochs_per_s_100k", "value": b["value"],
                      "unit": "epochs/s", "n_gpus": world, "steps": UMAP_CPU_EPOCHS, "warmup": 0,
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                      "dtype": "f32" if b["cores"] > 1 else "f64", "data": "synthetic",
                      "config": {"workload": "umap_knn_100k_k15_500epochs"}, "cpu_baseline": b,
                      "e2e": {"value": b["value"], "unit": "epochs/s", "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0}}))
    return 0


BATCH_TSNE_ITERS = (250, 750)


def _batched_instances(count, k, seed, device, with_x=False):
    """Instances of the batched workload: sizes log-uniform in [2,000, 200,000], each a 50-d
    mixture of 5-15 clusters with exact KNN (k = 90 for t-SNE, 15 for UMAP)."""
    from fastembedr_gb300 import synthetic as S

    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(2_000), np.log(200_000), count)).astype(np.int64)
    knns, xs = [], []
    for j, n in enumerate(sizes):
        x, _ = S.mixture(int(n), 50, int(rng.integers(5, 16)), seed * 1000 + j, centre_sd=4.0, lognormal_sizes=True)
        idx, dist = S.exact_knn_torch(x, k, device=device)
        knns.append((idx.cpu().numpy(), dist.cpu().numpy()))
        if with_x:
            xs.append(x)
    return (knns, xs) if with_x else knns


def _run_batched_umap(args, device):
    """UMAP half of the batched workload: instances with k = 15, 500 epochs, a data-derived start;
    one batched job against one umap_knn call per instance (size-stratified subset)."""
    import oracle as O
    from fastembedr_gb300 import api

    knns, xs = _batched_instances(args.instances - args.instances // 2, UMAP_K, 29, device, with_x=True)
    inits = [_pca_init(x) for x in xs]
    del xs
    sizes = np.array([i.shape[0] for i, _ in knns])
    api.umap_knn_batch(knns[:2], inits[:2], n_epochs=5)  # warm-up
    t0 = time.perf_counter()
    lays, sgd_ms = api.umap_knn_batch(knns, inits, n_epochs=UMAP_EPOCHS, return_time=True)
    wall = time.perf_counter() - t0
    order = np.argsort(sizes)
    subset = order[:: max(1, args.plain_stride)]
    plain_t, plain_work, pres = 0.0, 0.0, []
    for j in subset:
        idx, dist = knns[j]
        t = time.perf_counter()
        fit = api.umap_knn(idx, dist, inits[j], n_epochs=UMAP_EPOCHS)
        plain_t += time.perf_counter() - t
        plain_work += float(sizes[j]) * UMAP_EPOCHS
        if len(pres) < args.kl_instances and sizes[j] <= 60_000:
            keep = np.arange(0, sizes[j], 4, dtype=np.int32)
            pres.append({"n": int(sizes[j]),
                         "preservation_batched": O.knn_preservation(lays[j], idx, keep=keep, preserve_k=15),
                         "preservation_plain": O.knn_preservation(fit.layout, idx, keep=keep, preserve_k=15)})
    work = float(sizes.sum()) * UMAP_EPOCHS
    return {"instances": len(knns), "points": int(sizes.sum()), "epochs": UMAP_EPOCHS, "k": UMAP_K,
            "epochs_value": work / (sgd_ms * 1e-3), "unit": "points*epochs/s", "ms_per_epoch": sgd_ms / UMAP_EPOCHS,
            "e2e_value": work / wall, "job_seconds": wall,
            "plain_gpu": {"value": plain_work / plain_t, "instances": int(len(subset)),
                          "form": "fastembedr_cuda_umap_from_knn once per instance"},
            "batched_vs_plain_e2e": (work / wall) / (plain_work / plain_t), "preservation": pres}


def _run_batch(knns, inits, grid_policy, work):
    """One batched job: create (affinities of every instance), 250 + 750 iterations timed with
    CUDA events on the batch's stream, layouts back to the host; the wall clock covers it all."""
    import torch

    from fastembedr_gb300 import api

    t0 = time.perf_counter()
    b = api.TsneBatch(knns, inits=inits, grid_size=grid_policy)
    t_create = time.perf_counter() - t0
    info = b.info()
    stream = torch.cuda.ExternalStream(b.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.run(BATCH_TSNE_ITERS[0], BATCH_TSNE_ITERS[1])  # the package schedule, opt-SNE rate n_b / 12
    e1.record(stream)
    b.synchronize()
    iter_ms = e0.elapsed_time(e1)
    lays = b.layouts()
    wall = time.perf_counter() - t0
    b.final_layouts = lays
    return b, {"grid_policy": grid_policy, "grid_classes": info["grid_classes"], "nnz_P": info["nnz"],
               "iterations_value": work / (iter_ms * 1e-3), "ms_per_iteration": iter_ms / sum(BATCH_TSNE_ITERS),
               "e2e_value": work / wall, "job_seconds": wall, "create_seconds": t_create,
               "launches_per_iteration": info["launches_per_iteration"],
               "launches_per_reorder": info["launches_per_reorder"]}


def run_batched(args):
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    print(json.dumps(batched_result(args, local)))
    return 0


def batched_result(args, local):
    """Batched t-SNE: many instances per launch against one instance per call, with the CUDA
    grid-size policy and with the adaptive box count."""
    import torch

    from fastembedr_gb300 import api
    from fastembedr_gb300 import synthetic as S

    torch.cuda.set_device(local)
    knns = _batched_instances(args.instances // 2, K, 23, f"cuda:{local}")
    torch.cuda.empty_cache()
    sizes = np.array([i.shape[0] for i, _ in knns])
    iters = sum(BATCH_TSNE_ITERS)
    inits = [S.tsne_init(int(n), seed=40 + j) for j, n in enumerate(sizes)]
    work = float(sizes.sum()) * iters
    with api.TsneBatch(knns[:3], inits=inits[:3]) as w:  # warm-up
        w.iterate(5, 12.0, 1.0 / 12.0)
        w.synchronize()
    # plain form on a size-stratified subset: every `stride`-th instance by size, one call each
    order = np.argsort(sizes)
    subset = order[:: max(1, args.plain_stride)]
    # KL checks on instances spread over the whole size range (the subset is in size order)
    kl_rows = [int(subset[i]) for i in np.unique(np.linspace(0, len(subset) - 1, args.kl_instances).astype(int))]
    plain_t, plain_work, plain_kl, plain_lay = 0.0, 0.0, {}, {}
    for j in subset:
        idx, dist = knns[j]
        t = time.perf_counter()
        fit = api.tsne_knn(idx, dist, perplexity=PERPLEXITY, Y_init=inits[j], n_iter=BATCH_TSNE_ITERS[1])
        plain_t += time.perf_counter() - t
        plain_work += float(sizes[j]) * iters
        plain_lay[int(j)] = fit.layout
        if j in kl_rows:
            with api.TsneBatch([(idx, dist)], inits=[fit.layout]) as one:  # exact KL of the given layout
                plain_kl[int(j)] = one.kl(0)
    plain_rate = plain_work / plain_t
    clocks = ClockSampler(local)
    runs = {}
    for policy in ("cuda", "adaptive"):
        b, r = _run_batch(knns, inits, policy, work)
        r["kl_vs_plain"] = [{"n": int(sizes[j]), "kl_batched": b.kl(int(j)), "kl_plain": plain_kl[int(j)]}
                            for j in kl_rows]
        for e in r["kl_vs_plain"]:
            e["rel"] = (e["kl_batched"] - e["kl_plain"]) / e["kl_plain"]
        r["max_abs_kl_rel"] = max(abs(e["rel"]) for e in r["kl_vs_plain"]) if r["kl_vs_plain"] else None
        # instances of the plain subset whose batched layout equals the one-call layout bit for bit
        r["plain_subset_bit_identical"] = int(sum(np.array_equal(b.final_layouts[int(j)], plain_lay[int(j)])
                                                  for j in subset))
        r["plain_subset_size"] = int(len(subset))
        r["vs_plain_e2e"] = r["e2e_value"] / plain_rate
        b.close()
        runs[policy] = r
    umap = _run_batched_umap(args, f"cuda:{local}")
    clk = clocks.stop()
    head = runs["adaptive"]
    line = {
        "metric": "batched_tsne_points_iterations_per_s", "value": head["iterations_value"],
        "unit": "points*iterations/s", "n_gpus": 1, "steps": iters, "warmup": 1,
        "ms_per_step": head["ms_per_iteration"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "batched_tsne_knn_sizes_2k_200k_k90", "instances": len(knns),
                   "points": int(sizes.sum()), "iterations": list(BATCH_TSNE_ITERS), "perplexity": PERPLEXITY,
                   "grid_policy": "adaptive box count (node spacing <= 0.7, re-chosen every 25 iterations)",
                   "nnz_P": head["nnz_P"],
                   "l2": "P of the batch (%.1f GB) exceeds L2; no flush" % (8 * head["nnz_P"] / 1e9)},
        "e2e": {"value": head["e2e_value"], "unit": "points*iterations/s",
                "h2d_bytes_per_step": int(sum(i.nbytes + d.nbytes for i, d in knns) / iters),
                "d2h_bytes_per_step": int(sizes.sum() * 8 / iters), "job_seconds": head["job_seconds"],
                "job": "batch create (affinities of every instance) + 250 + 750 iterations + layouts"},
        "plain_gpu": {"value": plain_rate, "unit": "points*iterations/s", "instances": int(len(subset)),
                      "form": "fastembedr_cuda_opentsne_fft_from_knn_float once per instance, CUDA size policy "
                              f"(every {max(1, args.plain_stride)}th instance by size)"},
        "batched": runs, "batched_vs_plain_e2e": head["vs_plain_e2e"], "umap": umap,
        "clocks": clk, "gpu_launches": iters * head["launches_per_iteration"] + (
            (BATCH_TSNE_ITERS[0] + 24) // 25 + (BATCH_TSNE_ITERS[1] + 24) // 25) * head["launches_per_reorder"],
    }
    return line


def run_grid_calibration(args):
    """Calibration of the adaptive box count: KL, final span and time per iteration of one t-SNE
    instance per (size, grid) pair, each run as a batch of one with a fixed grid size (250 early-
    exaggeration + 750 normal iterations, opt-SNE rate n / 12; 50-d mixture of 10 log-normal
    clusters, exact k = 90 KNN, perplexity 30). One JSON line per (n, G)."""
    import torch

    from fastembedr_gb300 import api
    from fastembedr_gb300 import synthetic as S

    for n in (2000, 10000, 50000, 200000):
        x, _ = S.mixture(n, 50, 10, 11, centre_sd=4.0, lognormal_sizes=True)
        idx, dist = S.exact_knn_torch(x, K)
        knn = (idx.cpu().numpy(), dist.cpu().numpy())
        init = S.tsne_init(n, seed=5)
        for g in (64, 128, 256, 512, 1024):
            if n <= 10000 and g > 512:
                continue
            with api.TsneBatch([knn], perplexity=PERPLEXITY, inits=[init], grid_size=g) as b:
                stream = torch.cuda.ExternalStream(b.stream)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                b.iterate(250, 12.0, 1.0 / 12.0)
                b.synchronize()
                e0.record(stream)
                b.iterate(750, 1.0, 1.0 / 12.0)
                e1.record(stream)
                b.synchronize()
                lay = b.layouts()[0]
                kl = b.kl(0)
            span = float(np.ptp(lay, 0).max())
            print(json.dumps(dict(n=n, G=g, kl=kl, span=span, h=1.1 * span / (g - 1),
                                  ms_iter=e0.elapsed_time(e1) / 750)), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=25)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-iters", type=int, default=20)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-kl", action="store_true", help="skip the exact KL and the gradient check")
    ap.add_argument("--check-sample", type=int, default=20000, help="points of the gradient check")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-adaptive", action="store_true", help="skip the adaptive-grid run of the 1M instance")
    ap.add_argument("--n", type=int, default=N_POINTS, help="points (profiling captures use a smaller case)")
    ap.add_argument("--workload", default="tsne", choices=["tsne", "serving", "umap", "batched", "grid-calibration"],
                    help="tsne: the headline 1M-point optimizer; serving: transform_tsne served; umap: 100k UMAP; "
                         "batched: many t-SNE instances per launch")
    ap.add_argument("--instances", type=int, default=512, help="batched: half t-SNE (k = 90), half UMAP (k = 15)")
    ap.add_argument("--headline-only", action="store_true",
                    help="only the 1M t-SNE headline (no UMAP / batched / serving sub-objects)")
    ap.add_argument("--plain-stride", type=int, default=4)
    ap.add_argument("--kl-instances", type=int, default=6)
    ap.add_argument("--n-ref", type=int, default=SERVE_N_REF)
    ap.add_argument("--requests", type=int, default=160)
    ap.add_argument("--plain-requests", type=int, default=60)
    ap.add_argument("--serve-slots", type=int, default=4, help="serving: request groups in flight (streams)")
    ap.add_argument("--n-umap", type=int, default=UMAP_N)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.workload == "grid-calibration":
        return run_grid_calibration(args)
    if args.workload == "serving":
        return run_serving_reference(args) if args.impl == "reference" else run_serving(args)
    if args.workload == "umap":
        return run_umap_reference(args) if args.impl == "reference" else run_umap(args)
    if args.workload == "batched":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the batched form has no CPU counterpart; "
                                                                  "per-instance CPU timing is the tsne workload's"}))
            return 0
        return run_batched(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
