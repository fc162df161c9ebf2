"""Benchmark: kernel-operator matvec/s at N = 4,194,304 (the sparse-operator
workload: 16-Gaussian mixture + 20% uniform background, periodic unit box,
r = 0.02, Wendland C2 kernel, b ~ N(0,1); FP32 kernel evaluation with FP32
blocks summed in FP64 into an FP64 result).

One step = one K*b over the whole particle set.
  value : device-resident b and c, CUDA events on the launching stream, L2
          flushed (256 MB write) between timed steps.
  e2e   : the same matvec through the C ABI with pinned HOST b and c, the
          host->device copy of b and the device->host copy of c inside the
          timed region (abx_operator_matvec stages them itself).
--impl reference times the reference algorithm restated in C++ (the oracle,
FP64, OpenMP on all host threads) on the same workload: each step is one
quarter of the rows, the quarters in turn, so four steps are one whole K*b.

Multi-GPU: the path runs as independent replicas (one per rank); value is the
sum of matvecs over ranks divided by the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

N_PARTICLES = 4_194_304
RADIUS = 0.02
FLOP_PER_PAIR = 20  # FP32 FLOP per accepted pair: dx(3) d2(5) q(3) Wendland(7) accumulate(2)
WORKLOAD = ("sparse operator, 3D, N=4,194,304: 16 isotropic Gaussians (sigma 0.03, centres "
            "U[0.1,0.9]^3) + 20% uniform, periodic unit box, CellListOrdered n_leaf=10, "
            "r=0.02, Wendland C2 (1-q)^4(4q+1), b~N(0,1)")


def make_workload(seed=2024):
    import workloads
    pos = workloads.gaussian_mixture(N_PARTICLES, 3, k=16, sigma=0.03, frac_uniform=0.2,
                                     seed=seed, periodic=True)
    b_by_id = np.random.default_rng(seed + 1).standard_normal(N_PARTICLES)
    return pos, b_by_id


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


TRAFFIC_FILE = ROOT / "profiles" / "k_pairs_traffic.json"


def profile_traffic():
    """Per-launch DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of
    the pair kernel from one ncu capture of the same workload, kept as data
    next to the profile summaries."""
    if not TRAFFIC_FILE.exists():
        return None
    return float(json.loads(TRAFFIC_FILE.read_text())["dram_bytes_per_launch"])


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return world, rank, local


def slowest_rank(times, world):
    """Each entry of `times` maximised over the ranks (the job's time is the
    slowest replica's); gloo reduces on the CPU, NCCL on the GPU."""
    if world <= 1:
        return list(times)
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor(list(times), dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def cell_build_record(ctx, stream, p, pos, peaks, reps=5):
    """Cell-list build (CellListOrdered::set_domain + sort + reorder) at the
    benchmark's N, timed on the device with CUDA events (median of reps - 1
    after one warm-up): (a) a rebuild, the particles already in cell order
    (update_positions after a step that moved few particles across cells);
    (b) a build from a random order (the stored order shuffled before each
    build; the upload is outside the events).  Compulsory bytes: read
    positions (24 B) and ids (8 B), write them in cell order (32 B), write
    the bucket keys (4 B) per particle, plus bucket_begin/end (8 B) per
    cell."""
    import torch
    lo, hi, per = [0, 0, 0], [1, 1, 1], [True, True, True]

    def timed_build(prepare=None):
        bt = []
        for _ in range(reps):
            if prepare:
                prepare()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            p.init_neighbour_search(lo, hi, per, 10.0)
            e1.record(stream)
            torch.cuda.synchronize()
            bt.append(e0.elapsed_time(e1))
        return float(np.median(bt[1:]))

    ncells = p.grid()[2]
    nb = len(p) * (24 + 8 + 32 + 4) + ncells * 8
    hbm = peaks.get("hbm_gbs", 6800.0)
    rebuild_ms = timed_build()
    sorted_pos, sorted_ids = p.positions, p.ids
    rng = np.random.default_rng(11)

    def shuffle():
        perm = rng.permutation(len(sorted_pos))
        p.set(sorted_pos[perm], sorted_ids[perm])
    shuffled_ms = timed_build(shuffle)
    p.set(sorted_pos, sorted_ids)
    p.init_neighbour_search(lo, hi, per, 10.0)

    def rec(ms):
        gbs = nb / (ms / 1e3) / 1e9
        return {"ms": ms, "achieved_gbs": gbs, "frac_of_hbm": gbs / hbm}
    out = {"cells": ncells, "compulsory_bytes": nb, **rec(rebuild_ms),
           "from_random_order": rec(shuffled_ms),
           "note": "rebuild of particles in cell order (top level) and build from a random "
                   "order; median of 4 builds (CUDA events), each including the device-to-host "
                   "read of the dead count"}
    return out


def replica_throughput(world, steps, seconds):
    """Whole-job matvecs per second: every replica performs `steps` matvecs."""
    return world * steps / seconds


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def run_ours(args):
    import torch
    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    import aboria_gb300 as ab
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = ab.Context(local, stream=stream.cuda_stream)
    pos, b_by_id = make_workload()
    p = ab.Particles(3, ctx).set(pos)
    t0 = time.perf_counter()
    p.init_neighbour_search([0, 0, 0], [1, 1, 1], [True, True, True], 10.0)
    build_s = time.perf_counter() - t0
    ids0 = p.ids
    peaks, _ = measured_peaks()
    cell_build = cell_build_record(ctx, stream, p, pos, peaks)
    ncells = cell_build["cells"]
    assert np.array_equal(p.ids, ids0), "rebuild changed the order"
    ids = p.ids
    b_host = np.ascontiguousarray(b_by_id[ids])
    kern = ab.Kernel.make(ab.K_WENDLAND_C2, 1.0 / RADIUS)
    t0 = time.perf_counter()
    K = ab.create_sparse_operator(p, p, RADIUS, kern, ab.PREC_MIXED)
    layout_s = time.perf_counter() - t0

    b_dev = torch.from_numpy(b_host).cuda()
    c_dev = torch.empty_like(b_dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.int32, device="cuda")

    # correctness side-checks (outside the timed region), and the FP64 mode
    # (the reference's arithmetic for every pair) timed on the same workload
    counts = ab.radius_count(p, p.positions, RADIUS)
    pairs = int(counts.astype(np.int64).sum())
    K64 = ab.create_sparse_operator(p, p, RADIUS, kern, ab.PREC_FP64)
    c64 = K64.matvec(b_dev).cpu().numpy()
    fp64_ms = _event_ms(lambda: K64.matvec(b_dev, out=c_dev, sync=False), stream, 3)
    del K64
    c32 = K.matvec(b_dev).cpu().numpy()
    mixed_err = float(np.linalg.norm(c32 - c64) / np.linalg.norm(c64))
    mixed_maxerr = float(np.max(np.abs(c32 - c64)) / np.max(np.abs(c64)))
    fp32_peak = max(ab.fp32_peak_tflops(ctx, packed=True), ab.fp32_peak_tflops(ctx, packed=False))

    for _ in range(args.warmup):
        K.matvec(b_dev, out=c_dev)
    torch.cuda.synchronize()

    sampler = ClockSampler(local)
    sampler.start()
    barrier(world)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    for i in range(args.steps):
        flush.fill_(i)
        ev[i][0].record(stream)
        K.matvec(b_dev, out=c_dev, sync=False)
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    barrier(world)
    step_ms = [a.elapsed_time(b) for a, b in ev]
    clocks = sampler.stop()

    # e2e: host pinned buffers through the C ABI (copies inside the call)
    b_pin = torch.from_numpy(b_host).pin_memory()
    c_pin = torch.empty(N_PARTICLES, dtype=torch.float64).pin_memory()
    b_np = b_pin.numpy()
    c_np = c_pin.numpy()
    for _ in range(2):
        K.matvec(b_np, out=c_np)
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        K.matvec(b_np, out=c_np)  # returns after the D2H copy has landed
    e2e_s = time.perf_counter() - t0
    assert np.array_equal(c_np, c32), "host-buffer matvec differs from device-buffer matvec"

    ms = float(np.mean(step_ms))
    t_total, e2e_s = slowest_rank([sum(step_ms) / 1e3, e2e_s], world)
    value = replica_throughput(world, args.steps, t_total)
    e2e_value = replica_throughput(world, args.steps, e2e_s)

    peaks, peak_kind = measured_peaks()
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    comp_bytes = N_PARTICLES * (24 + 8 + 8) + ncells * 8
    achieved_gbs = comp_bytes / (ms / 1e3) / 1e9
    achieved_tflops = pairs * FLOP_PER_PAIR / (ms / 1e3) / 1e12
    tr = profile_traffic()
    out = {
        "metric": "kernel-op matvec/s (N=4M)",
        "value": value,
        "unit": "matvec/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {
            "workload": WORKLOAD,
            "n": N_PARTICLES,
            "radius": RADIUS,
            "precision": "FP32 kernel values, FP32 blocks of <=64 terms summed in FP64",
            "pairs_per_matvec": pairs,
            "mean_neighbours": pairs / N_PARTICLES,
            "l2": "flushed between timed steps (256 MB write outside the events)",
            "parallelism": f"replicas x{world}",
            "cell_build_s": build_s,
            "operator_layout_s": layout_s,
        },
        "e2e": {"value": e2e_value, "unit": "matvec/s",
                "h2d_bytes_per_step": N_PARTICLES * 8, "d2h_bytes_per_step": N_PARTICLES * 8},
        "roofline": {
            "bound": "fp32", "achieved": achieved_tflops, "peak": fp32_peak, "unit": "TFLOP/s",
            "frac": achieved_tflops / fp32_peak, "traffic": tr,
            "flop_per_pair": FLOP_PER_PAIR,
            "peak_source": "measured in this run: FP32 FMA-chain probe (abx_probe_fp32_peak, "
                           "best of scalar FFMA and packed FFMA2)",
            "note": "achieved = accepted pairs x 20 FLOP / mean step time; traffic = DRAM "
                    "read+write bytes per pair-kernel launch from one ncu capture "
                    "(profiles/k_pairs_traffic.json)",
        },
        "hbm_roofline": {
            "bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
            "frac": achieved_gbs / hbm_peak, "peak_source": peak_kind, "traffic": tr,
            "note": "compulsory bytes N*(24+8+8)+ncells*8 per matvec; not the binding bound",
        },
        "fp64": {
            "kernel": "k_pairs_fp64 (the 1e-12 mode: FP32 prefilter per candidate, FP64 distance, "
                      "kernel and product for every accepted pair)",
            "ms_per_matvec": fp64_ms, "value": 1e3 / fp64_ms, "unit": "matvec/s",
        },
        "accuracy": {"mixed_vs_fp64_rel_l2": mixed_err, "mixed_vs_fp64_rel_max": mixed_maxerr},
        "cell_build": cell_build,
        "gpu_launches": 3 * args.steps,
        "clocks": clocks,
    }
    if not args.matvec_only:
        del K
        out["cfg1"] = cfg1_section(ctx)
        out["dense"] = dense_section(ctx)
        out["rbf_as_specified"] = cfg4_as_specified(ctx)
        models = ROOT / "aboria_gb300" / "models"
        out["rbf_solve"] = rbf_section(ctx, models / "spai_mlp_2d.bin")
        out["rbf_solve_3d"] = rbf_section(ctx, models / "spai_mlp_3d.bin", dim=3, n=50000)
        # plain Schwarz is not run at 2M: its FP64 block LU took 69 s at N=500,000 (3-D)
        out["rbf_solve_3d_2M"] = rbf_section(ctx, models / "spai_mlp_3d.bin", dim=3, n=2_000_000,
                                             run_schwarz=False)
        out["fmm"] = fmm_section(ctx)
        out["fmm_16M"] = fmm_section(ctx, n=1 << 24, orders=(5,), steps=1)
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(pos, b_by_id)
        # like for like: the FP64 matvec against the FP64 port on all host cores
        out["fp64"]["vs_cpu_baseline"] = out["fp64"]["value"] / out["cpu_baseline"]["value"]
        out["e2e"]["vs_cpu_baseline"] = out["e2e"]["value"] / out["cpu_baseline"]["value"]
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


RBF_N = 200_000
RBF_EH = 2.5  # scaled shape parameter eps*h, h = N^-1/2
EXACT_PHI = 0.5  # learned preconditioner: rows with a neighbour of kernel value > 0.5 solved exactly


def _timed(fn, ctx):
    ctx.synchronize()
    t0 = time.perf_counter()
    out = fn()
    ctx.synchronize()
    return out, time.perf_counter() - t0


def rbf_section(ctx, model_path, dim=2, n=None, run_schwarz=True, seed=4040):
    """RBF interpolation solve to 1e-8 FP64 relative residual: N uniform points
    in the unit square or cube (2-D N=200,000 with the 2-D model; 3-D N=50,000
    and 2,000,000 with the 3-D model), eps*h = 2.5 (h = N^(-1/dim)),
    f = sin(4 pi x) cos(3 pi y) + 1e-3 noise, compactly supported Gaussian
    exp(-(eps |dx|)^2) cut at eps |dx| = 4, GMRES(100).

    * plain   : restricted additive Schwarz on octree leaves of 256 points,
                blocks factorised by FP64 LU, FP64 operator throughout.
    * learned : the trained MLP's sparse approximate inverse (32 k-NN columns
                per row, BF16 tensor-core inference; rows next to a neighbour
                with kernel value > 0.5 solved exactly in FP64), FP64
                operator (these systems hold 8-17 neighbours per row, so the
                FP64 matvec is cheap, and with the mixed operator the
                refinement against FP64 stalls at N >= 500k in 2-D);
                Schwarz taken as fallback when the learned preconditioner
                has not converged after 100 iterations.
    * without_network : the same, with identity rows where the network answers.
    * local_inverse : the exact FP64 local-inverse rows the network is trained
                on, as the same sparse approximate inverse (the label method).
    Every time includes the preconditioner's set-up; the residual reported is
    |b - A x| / |b| with the FP64 operator."""
    import aboria_gb300 as ab
    import workloads
    n = n or RBF_N
    eps = RBF_EH * n ** (1.0 / dim)
    r = 4.0 / eps
    pos = workloads.uniform(n, dim, seed=seed)
    p = ab.Particles(dim, ctx).set(pos)
    p.init_octree([0.0] * dim, [1.0] * dim, [False] * dim, 256)
    P = p.positions
    f = np.sin(4 * np.pi * P[:, 0]) * np.cos(3 * np.pi * P[:, 1])
    f += 1e-3 * np.random.default_rng(seed + 1).standard_normal(n)
    kern = ab.Kernel.make(ab.K_COMPACT_GAUSSIAN, eps * eps)
    K64 = ab.create_sparse_operator(p, p, r, kern, ab.PREC_FP64)
    out = {"workload": f"{dim}-D N={n} uniform, compact Gaussian eps*h={RBF_EH} (eps={eps:.1f}), "
                       f"cut-off r=4/eps={r:.3g}, f=sin(4 pi x)cos(3 pi y)+1e-3 noise, GMRES(100), "
                       f"tol 1e-8 (FP64 residual)"}

    def check(x):
        return float(np.linalg.norm(f - K64 * x) / np.linalg.norm(f))

    def plain():
        M = ab.schwarz_preconditioner(K64)
        x, it, res = ab.gmres(K64, f, M=M, restart=100, max_iters=2000, tol=1e-8)
        return x, it, M.stats()
    if run_schwarz:
        (x, it, st), t = _timed(plain, ctx)
        out["plain_schwarz_fp64"] = {"seconds": t, "iterations": it, "residual": check(x),
                                     "schwarz_setup_s": st["setup_s"], "domains": st["domains"]}

    if model_path.exists():
        mlp = ab.MLP.load(model_path, ctx=ctx)

        def learned(net):
            M = ab.learned_preconditioner(K64, net, eps, exact_phi=EXACT_PHI)
            x, it, res, fb = ab.gmres_with_fallback(K64, f, M, K64, restart=100,
                                                    learned_max_iters=100, max_iters=2000,
                                                    tol=1e-8, A_check=K64)
            return x, it, fb, M.stats()["domains"]
        (x, it, fb, nex), t = _timed(lambda: learned(mlp), ctx)
        out["learned"] = {"seconds": t, "iterations": it, "residual": check(x),
                                "fallback_taken": bool(fb), "rows_solved_exactly": nex}
        # the same method without the network: identity rows where it answers
        ident = ab.MLP.load(model_path, ctx=ctx)
        ident.params = np.zeros(ident.num_params, np.float32)
        (x, it, fb, nex), t = _timed(lambda: learned(ident), ctx)
        out["without_network"] = {"seconds": t, "iterations": it, "residual": check(x),
                                        "fallback_taken": bool(fb)}

    def local_inverse():
        cols, vals = ab.spai_local_inverse_rows(K64, 32)
        M = ab.spai_preconditioner(ctx, cols, vals)
        x, it, res = ab.gmres(K64, f, M=M, restart=100, max_iters=2000, tol=1e-8)
        return x, it
    (x, it), t = _timed(local_inverse, ctx)
    out["local_inverse"] = {"seconds": t, "iterations": it, "residual": check(x)}
    if "learned" in out and "plain_schwarz_fp64" in out:
        out["speedup_learned_vs_plain"] = (out["plain_schwarz_fp64"]["seconds"]
                                           / out["learned"]["seconds"])
    return out


RBF_GRID_EH = (0.75, 1.0, 1.5, 2.5)


def rbf_case(ctx, models, dim, n, dist, eh, seed, plain=True, fallback=True, max_iters=2000,
             methods=("learned", "without")):
    """One RBF interpolation solve to 1e-8 (FP64 residual): N points (uniform,
    or 8 Gaussians of sigma 0.05 clipped into the unit box), compact Gaussian
    exp(-(eps |dx|)^2) cut at eps |dx| = 4, eps = eh * N^(1/dim), GMRES(100).
    Methods as in rbf_section: plain Schwarz/FP64; the learned approximate
    inverse on the FP64 operator (Schwarz fallback after 100 iterations when
    ``fallback``; else its own result is reported, up to 300 iterations); the
    same without the network (identity rows where it answers).  Seconds
    include every set-up; the learned set-up is split into its phases."""
    import aboria_gb300 as ab
    import workloads
    eps = eh * n ** (1.0 / dim)
    r = 4.0 / eps
    pos = (workloads.uniform(n, dim, seed=seed) if dist == "uniform"
           else workloads.clipped_mixture(n, dim, seed=seed))
    p = ab.Particles(dim, ctx).set(pos)
    p.init_octree([0.0] * dim, [1.0] * dim, [False] * dim, 256)
    P = p.positions
    f = np.sin(4 * np.pi * P[:, 0]) * np.cos(3 * np.pi * P[:, 1])
    f += 1e-3 * np.random.default_rng(seed + 1).standard_normal(n)
    kern = ab.Kernel.make(ab.K_COMPACT_GAUSSIAN, eps * eps)
    K64 = ab.create_sparse_operator(p, p, r, kern, ab.PREC_FP64)
    row = {"dim": dim, "n": n, "dist": dist, "eh": eh, "eps": eps, "seed": seed}

    def check(x):
        return float(np.linalg.norm(f - K64 * x) / np.linalg.norm(f))

    if plain:
        def run_plain():
            M = ab.schwarz_preconditioner(K64)
            x, it, res = ab.gmres(K64, f, M=M, restart=100, max_iters=max_iters, tol=1e-8)
            return x, it, M.stats()["setup_s"]
        (x, it, su), t = _timed(run_plain, ctx)
        res = check(x)
        row["plain"] = {"s": t, "setup_s": su, "it": it, "res": res, "ok": res <= 1e-8}
    model = models / f"spai_mlp_{dim}d.bin"
    mlp = ab.MLP.load(model, ctx=ctx)
    ident = ab.MLP.load(model, ctx=ctx)
    ident.params = np.zeros(ident.num_params, np.float32)
    for name, net in (("learned", mlp), ("without", ident)):
        if name not in methods:
            continue
        def run(net=net):
            M = ab.learned_preconditioner(K64, net, eps, exact_phi=EXACT_PHI)
            if fallback:
                x, it, res, fb = ab.gmres_with_fallback(K64, f, M, K64, restart=100,
                                                        learned_max_iters=100,
                                                        max_iters=max_iters, tol=1e-8,
                                                        A_check=K64)
            else:
                x, it, res = ab.gmres(K64, f, M=M, restart=100, max_iters=300, tol=1e-8)
                fb = False
            return x, it, fb, M.stats()
        (x, it, fb, st), t = _timed(run, ctx)
        res = check(x)
        row[name] = {"s": t, "setup_s": st["setup_s"], "it": it, "fallback": bool(fb),
                     "res": res, "ok": res <= 1e-8, "exact_rows": st["domains"],
                     "phases_s": {k: st[k] for k in ("knn_s", "features_s", "infer_s",
                                                     "exact_rows_s")}}
    return row


def rbf_grid_section(ctx, models, quick=False, budget_s=900.0):
    """The RBF solve over dimension x N x point distribution x eps*h, and the
    fallback rate of the learned preconditioner over instances with eps*h
    drawn per instance.  Uniform points at N = 50k (eps*h from 0.75 in 2-D,
    from 1 in 3-D), 500k and 2M (eps*h 1.5, 2.5); the 8-Gaussian mixtures at
    N = 50k only (eps*h 1.5 and 2.5 in 2-D, 2.5 in 3-D): their clusters are
    ~100x denser than h, so at larger N the FP64 operator alone holds
    thousands of neighbours per row.  Plain Schwarz/FP64 is run where its FP64
    block LU takes seconds (2-D N <= 500k, 3-D N = 50k); larger cells report
    the approximate inverses without the Schwarz fallback.  Mixture systems
    are capped at 300 GMRES iterations (most do not reach 1e-8 with any
    preconditioner here).  Cells run in order of cost and stop at the time
    budget (the rest are listed as skipped)."""
    t_start = time.perf_counter()
    if quick:
        cells = [(2, 200_000, "uniform", eh, True, True) for eh in (1.5, 2.5)]
        cells += [(3, 50_000, "uniform", eh, True, True) for eh in (1.5, 2.5)]
    else:
        cells = [(2, 50_000, "uniform", eh, True, True) for eh in RBF_GRID_EH]
        cells += [(3, 50_000, "uniform", eh, True, True) for eh in RBF_GRID_EH[1:]]
        cells += [(2, 50_000, "mixture", eh, True, True) for eh in RBF_GRID_EH[2:]]
        cells += [(3, 50_000, "mixture", RBF_GRID_EH[-1], True, True)]
        # at N >= 500k the cells take eps*h = 1.5 and 2.5 (below, the
        # approximate inverses stall and fall back to Schwarz)
        for n in (500_000, 2_000_000):
            for eh in RBF_GRID_EH[2:]:
                cells.append((2, n, "uniform", eh, n <= 500_000, n <= 500_000))
                cells.append((3, n, "uniform", eh, False, False))
    out = {"cells": []}

    def over_budget():
        return time.perf_counter() - t_start > budget_s

    # fallback rate: instances per (dim, distribution) at N = 50k, eps*h ~ U[1, 3]
    # (mixtures: the learned preconditioner only, at most 300 iterations)
    rates = {}
    for dim in (2, 3):
        for dist in (("uniform",) if quick else ("uniform", "mixture")):
            rng = np.random.default_rng(900 + dim)
            runs = []
            mix = dist == "mixture"
            for i in range(4 if quick else 10):
                if over_budget():
                    break
                eh = float(rng.uniform(1.0, 3.0))
                c = rbf_case(ctx, models, dim, 50_000, dist, eh, seed=7000 + 10 * dim + i,
                             plain=False, fallback=True, max_iters=300 if mix else 2000,
                             methods=("learned",) if mix else ("learned", "without"))
                runs.append({"eh": eh, "fallback": c["learned"]["fallback"],
                             "it": c["learned"]["it"], "ok": c["learned"]["ok"],
                             "s": c["learned"]["s"]})
                if not mix:
                    runs[-1].update({"without_fallback": c["without"]["fallback"],
                                     "without_it": c["without"]["it"],
                                     "without_s": c["without"]["s"]})
                print(json.dumps({"dim": dim, "dist": dist, **runs[-1]}), file=sys.stderr,
                      flush=True)
            if runs:
                rates[f"{dim}d_{dist}"] = {
                    "instances": len(runs), "eh_range": [1.0, 3.0], "n": 50_000,
                    "fallback_rate": sum(r["fallback"] for r in runs) / len(runs),
                    "converged": sum(r["ok"] for r in runs), "runs": runs}
                if not mix:
                    rates[f"{dim}d_{dist}"]["without_network_fallback_rate"] = (
                        sum(r["without_fallback"] for r in runs) / len(runs))
    out["fallback"] = rates
    for dim, n, dist, eh, plain, fb in cells:
        if over_budget():
            out["cells"].append({"dim": dim, "n": n, "dist": dist, "eh": eh,
                                 "skipped": "time budget"})
            continue
        try:
            out["cells"].append(rbf_case(ctx, models, dim, n, dist, eh, seed=4040 + dim,
                                         plain=plain, fallback=fb,
                                         max_iters=300 if dist == "mixture" else 2000))
        except Exception as e:  # a cell that does not fit is recorded, not fatal
            out["cells"].append({"dim": dim, "n": n, "dist": dist, "eh": eh,
                                 "error": str(e)[:200]})
        print(json.dumps(out["cells"][-1]), file=sys.stderr, flush=True)  # progress
    out["seconds"] = time.perf_counter() - t_start
    return out


def fmm_section(ctx, n=1 << 20, orders=(3, 5, 7), n_targets=10000, steps=3):
    """Chebyshev black-box FMM, Laplace 1/(|dx| + 1e-12), N uniform points in
    the unit cube, octree leaves of 64, weights U[-1,1].  Per order: plan +
    M2L set-up time, matvec time (CUDA events, mean of ``steps``) in FP64 and
    mixed mode (3xTF32 tensor-core M2L, FP32 P2P), and the relative L2 error
    of each against an FP64 direct sum (dense operators) on 10,000 seeded
    targets, with the self term K(0) b_i = 1e12 b_i removed from both."""
    import torch
    import aboria_gb300 as ab
    import workloads
    pos = workloads.uniform(n, 3, seed=5050)
    p = ab.Particles(3, ctx).set(pos)
    p.init_octree([0.0] * 3, [1.0] * 3, [False] * 3, 64)
    P = p.positions
    b = np.random.default_rng(5051).uniform(-1, 1, n)
    tgt = np.sort(np.random.default_rng(5052).choice(n, n_targets, replace=False))
    kern = ab.Kernel.make(ab.K_LAPLACE, 1e-12)
    # FP64 direct sum without the self term K(0) b_i = 1e12 b_i (summed in, it
    # would round ~1e-4 off every later term): the sources other than the
    # targets through a targets x all dense operator with b zeroed at the
    # targets, plus the targets x targets sum with its diagonal taken out
    tp = ab.Particles(3, ctx).set(P[tgt])
    bm = b.copy()
    bm[tgt] = 0.0
    D = ab.create_dense_operator(tp, p, kern, ab.PREC_FP64)
    direct = D * bm
    del D
    D = ab.create_dense_operator(tp, tp, kern, ab.PREC_FP64)
    direct += D * b[tgt] - 1e12 * b[tgt]
    del D
    b_dev = torch.from_numpy(b).cuda()
    c_dev = torch.empty_like(b_dev)
    stream = torch.cuda.current_stream()
    res = {"workload": f"3-D N={n} uniform, Laplace 1/(|dx|+1e-12), leaf 64, "
                       f"error vs FP64 direct sum on {n_targets} targets"}
    for order in orders:
        K, t_setup = _timed(lambda: ab.create_fmm_operator(p, kern, order), ctx)
        st = ab.fmm_stats(K)
        row = {"setup_s": t_setup, "m2l_pairs": st["m2l_pairs"], "leaves": st["leaves"]}
        for prec, name in ((ab.PREC_FP64, "fp64"), (ab.PREC_MIXED, "mixed")):
            K.set_precision(prec)
            K.matvec(b_dev, out=c_dev)
            ts = []
            for _ in range(steps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                K.matvec(b_dev, out=c_dev, sync=False)
                e1.record(stream)
                torch.cuda.synchronize()
                ts.append(e0.elapsed_time(e1))
            c = c_dev.cpu().numpy()[tgt] - 1e12 * b[tgt]
            row[f"{name}_ms"] = float(np.mean(ts))
            row[f"{name}_rel_l2"] = float(np.linalg.norm(c - direct) / np.linalg.norm(direct))
        res[f"order{order}"] = row
        del K
    return res


def _event_ms(fn, stream, reps):
    import torch
    ts = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return float(np.median(ts))


def dense_section(ctx, n=65536, reps=5):
    """Dense operator (create_dense_operator, every pair): N uniform points in
    the unit cube, Gaussian exp(-|dx|^2 / 0.1^2), b U[0,1].  K*b in FP64 and
    mixed precision (CUDA events, medians), pairs per second, the FP32 compute
    roofline of the mixed kernel (FP32 FLOP per pair: dx 3, d2 5, exponent 1,
    accumulate 2, plus one exp2 on the special-function unit), and the mixed
    error against FP64."""
    import torch
    import aboria_gb300 as ab
    import workloads
    stream = torch.cuda.current_stream()
    pos = workloads.uniform(n, 3, seed=1101)
    p = ab.Particles(3, ctx).set(pos)
    kern = ab.Kernel.make(ab.K_GAUSSIAN, 1.0 / 0.1 ** 2)
    b = torch.from_numpy(np.random.default_rng(1102).uniform(0, 1, n)).cuda()
    c = torch.empty_like(b)
    out = {"workload": f"3-D N={n} uniform, dense Gaussian exp(-|dx|^2/0.1^2), {n * n:.3e} pairs"}
    res = {}
    fp32_peak = max(ab.fp32_peak_tflops(ctx, packed=True), ab.fp32_peak_tflops(ctx, packed=False))
    for prec, name in ((ab.PREC_FP64, "fp64"), (ab.PREC_MIXED, "mixed")):
        K = ab.create_dense_operator(p, p, kern, prec)
        K.matvec(b, out=c)
        ms = _event_ms(lambda: K.matvec(b, out=c, sync=False), stream, reps)
        out[f"{name}_matvec_ms"] = ms
        out[f"{name}_gpairs_per_s"] = n * n / (ms / 1e3) / 1e9
        res[name] = c.cpu().numpy()
        del K
    tflops = n * n * 11 / (out["mixed_matvec_ms"] / 1e3) / 1e12
    out["mixed_compute_roofline"] = {"achieved_tflops": tflops, "peak_tflops": fp32_peak,
                                     "frac": tflops / fp32_peak, "flop_per_pair": 11}
    out["mixed_vs_fp64_rel_l2"] = float(np.linalg.norm(res["mixed"] - res["fp64"])
                                        / np.linalg.norm(res["fp64"]))
    return out


def cfg1_section(ctx):
    """The reference's CPU-runnable case: N=100,000 uniform in the unit cube,
    non-periodic, n_leaf 10, r=0.05, Gaussian exp(-|dx|^2/(r/2)^2), b U[0,1].
    Cell build, radius counts and K*b in FP64 and mixed precision (CUDA events,
    medians), pairs per matvec and the mixed error against FP64."""
    import torch
    import aboria_gb300 as ab
    import workloads
    n, r = 100_000, 0.05
    stream = torch.cuda.current_stream()
    pos = workloads.uniform(n, 3, seed=1001)
    p = ab.Particles(3, ctx).set(pos)
    p.init_neighbour_search([0, 0, 0], [1, 1, 1], [False] * 3, 10.0)
    build_ms = _event_ms(lambda: p.init_neighbour_search([0, 0, 0], [1, 1, 1], [False] * 3, 10.0),
                         stream, 5)
    P = p.positions
    count_ms = _event_ms(lambda: ab.radius_count(p, P, r), stream, 5)
    counts = ab.radius_count(p, P, r)
    kern = ab.Kernel.make(ab.K_GAUSSIAN, 1.0 / (r / 2) ** 2)
    b = torch.from_numpy(np.random.default_rng(1002).uniform(0, 1, n)).cuda()
    c = torch.empty_like(b)
    out = {"workload": "3-D N=100000 uniform, non-periodic, r=0.05, Gaussian exp(-|dx|^2/(r/2)^2)",
           "pairs": int(counts.astype(np.int64).sum()),
           "mean_neighbours": float(counts.mean()),
           "cell_build_ms": build_ms, "radius_count_ms": count_ms}
    res = {}
    for prec, name in ((ab.PREC_FP64, "fp64"), (ab.PREC_MIXED, "mixed")):
        K = ab.create_sparse_operator(p, p, r, kern, prec)
        K.matvec(b, out=c)
        out[f"{name}_matvec_ms"] = _event_ms(lambda: K.matvec(b, out=c, sync=False), stream, 10)
        res[name] = c.cpu().numpy()
    out["mixed_vs_fp64_rel_l2"] = float(np.linalg.norm(res["mixed"] - res["fp64"])
                                        / np.linalg.norm(res["fp64"]))
    return out


def cfg4_as_specified(ctx, iters=100):
    """Configuration 4 exactly as specified: 2-D, N=200,000 uniform, compact
    Gaussian with eps=20 and cut-off 0.2 (eps*h = 0.045, ~21,000 neighbours
    per row).  The truncated flat Gaussian matrix is numerically singular; one
    GMRES(100) cycle with the plain Schwarz/FP64 preconditioner and the mixed
    operator, FP64-checked, records how far it gets."""
    import torch
    import aboria_gb300 as ab
    import workloads
    n, eps, r = 200_000, 20.0, 0.2
    stream = torch.cuda.current_stream()
    pos = workloads.uniform(n, 2, seed=4040)
    p = ab.Particles(2, ctx).set(pos)
    p.init_octree([0.0, 0.0], [1.0, 1.0], [False, False], 256)
    P = p.positions
    f = np.sin(4 * np.pi * P[:, 0]) * np.cos(3 * np.pi * P[:, 1])
    f += 1e-3 * np.random.default_rng(4041).standard_normal(n)
    kern = ab.Kernel.make(ab.K_COMPACT_GAUSSIAN, eps * eps)
    K64 = ab.create_sparse_operator(p, p, r, kern, ab.PREC_FP64)
    K32 = ab.create_sparse_operator(p, p, r, kern, ab.PREC_MIXED)
    bd = torch.from_numpy(f).cuda()
    cd = torch.empty_like(bd)
    K32.matvec(bd, out=cd)
    mv_ms = _event_ms(lambda: K32.matvec(bd, out=cd, sync=False), stream, 5)
    counts = ab.radius_count(p, P, r)
    M, t_setup = _timed(lambda: ab.schwarz_preconditioner(K64), ctx)
    st = M.stats()
    (x, it, res), t = _timed(lambda: ab.gmres(K32, f, M=M, restart=100, max_iters=iters,
                                               tol=1e-8, A_check=K64), ctx)
    return {"workload": "2-D N=200000 uniform, compact Gaussian eps=20, cut-off 0.2, GMRES(100), "
                        "Schwarz FP64 on leaves of 256",
            "mean_neighbours": float(counts.mean()), "mixed_matvec_ms": mv_ms,
            "schwarz_setup_s": t_setup, "schwarz_domains": st["domains"],
            "schwarz_max_size": st["max_size"], "gmres_iterations": it,
            "fp64_residual_after": res, "gmres_s": t,
            "note": "numerically singular at eps*h = 0.045: the solve stalls far above 1e-8"}


def _oracle_workload(pos, b_by_id):
    """The reference's cell list of the benchmark workload (oracle) and b in
    its storage order."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    t0 = time.perf_counter()
    cl = oracle.celllist_build(pos, [0, 0, 0], [1, 1, 1], [True] * 3, 10.0)
    build_s = time.perf_counter() - t0
    return oracle, cl, np.ascontiguousarray(b_by_id[cl.perm]), build_s


def _oracle_rows(oracle, cl, b, rows):
    """Rows `rows` (a slice of the storage order) of K*b, FP64, the reference's
    neighbour order, OpenMP over rows (src/Kernels.h:734-736)."""
    return oracle.sparse_matvec(cl, cl.pos[rows], RADIUS, 2, [1.0 / RADIUS], b)


def thread_sweep(oracle, cl, b, nrows=20000):
    """Rows per second of the oracle matvec on a fixed random sample of rows
    for 1, 2, 4, ... host threads up to all of them (the reference's own
    scaling harness sweeps threads the same way, tests/speed_test.h:1006-1032)."""
    full = oracle.num_threads()
    rows = np.sort(np.random.default_rng(9).choice(cl.n, nrows, replace=False))
    counts = []
    t = 1
    while t < full:
        counts.append(t)
        t *= 2
    counts.append(full)
    out = []
    try:
        for t in counts:
            oracle.set_num_threads(t)
            t0 = time.perf_counter()
            _oracle_rows(oracle, cl, b, rows)
            dt = time.perf_counter() - t0
            out.append({"threads": t, "rows_per_s": nrows / dt, "matvec_per_s": nrows / dt / cl.n})
    finally:
        oracle.set_num_threads(full)
    return out


def cpu_baseline(pos, b_by_id):
    """The oracle (the reference's OpenMP path restated in C++) timed on one
    whole FP64 matvec of all N rows on every host thread, plus a thread sweep
    on a 20,000-row sample."""
    oracle, cl, b, build_s = _oracle_workload(pos, b_by_id)
    t0 = time.perf_counter()
    _oracle_rows(oracle, cl, b, slice(0, cl.n))
    dt = time.perf_counter() - t0
    return {"value": 1.0 / dt, "unit": "matvec/s", "cores": oracle.num_threads(), "kind": "port",
            "sample": f"one whole FP64 matvec, all {cl.n} rows ({dt:.1f} s, the reference's "
                      f"neighbour order and arithmetic, OpenMP over rows); the cell-list build "
                      f"({build_s:.1f} s) is not included",
            "thread_sweep": thread_sweep(oracle, cl, b)}


def run_reference(args):
    """The reference's CPU implementation of the path (the oracle port: the
    reference's algorithm restated, FP64, OpenMP on all host threads) on the
    same workload and metric.  One step = one quarter of the rows (1,048,576,
    contiguous in storage order), the four quarters in turn, so every four
    steps are one whole K*b; value = rows per second / N.  Warm-up steps run
    1/16 of the rows each."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    pos, b_by_id = make_workload()
    oracle, cl, b, build_s = _oracle_workload(pos, b_by_id)
    n = cl.n
    q = n // 4
    for w in range(args.warmup):
        lo = (w * (n // 16)) % n
        _oracle_rows(oracle, cl, b, slice(lo, min(lo + n // 16, n)))
    times, rows_done = [], 0
    for i in range(args.steps):
        k = i % 4
        rows = slice(k * q, n if k == 3 else (k + 1) * q)
        t0 = time.perf_counter()
        _oracle_rows(oracle, cl, b, rows)
        times.append(time.perf_counter() - t0)
        rows_done += rows.stop - rows.start
    t = float(np.sum(times))
    value = rows_done / t / n
    desc = (f"{args.steps} steps of one quarter of the {n} rows each (contiguous in storage "
            f"order, the four quarters in turn; {rows_done / n:.2f} whole matvecs timed, "
            f"{t:.1f} s); FP64, the reference's neighbour order; warm-up steps of n/16 rows")
    out = {
        "impl": "reference",
        "metric": "kernel-op matvec/s (N=4M)",
        "value": value,
        "unit": "matvec/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t * 1e3 / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "n": N_PARTICLES, "radius": RADIUS,
                   "step": "one quarter of the rows (K*b restricted to 1,048,576 rows)",
                   "cell_build_s": build_s},
        "cpu_baseline": {"value": value, "unit": "matvec/s", "cores": oracle.num_threads(),
                         "kind": "port", "sample": desc,
                         "thread_sweep": thread_sweep(oracle, cl, b)},
        "e2e": {"value": value, "unit": "matvec/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--matvec-only", action="store_true",
                    help="skip the RBF-solve and FMM sections (profiling runs)")
    ap.add_argument("--only", choices=["fmm", "rbf", "rbf_grid", "cell_build"],
                    help="run one secondary section alone and print it (profiling runs)")
    ap.add_argument("--fmm-n", type=int, default=0,
                    help="with --only fmm: one problem size instead of 1M and 16M (profiling)")
    ap.add_argument("--fmm-orders", default="3,5,7", help="with --only fmm and --fmm-n")
    ap.add_argument("--grid-quick", action="store_true", help="with --only rbf_grid: 4 cells")
    ap.add_argument("--grid-budget", type=float, default=900.0,
                    help="with --only rbf_grid: seconds after which the remaining cells are skipped")
    ap.add_argument("--models", default=str(ROOT / "aboria_gb300" / "models"),
                    help="folder of the learned preconditioner's models (rbf_grid)")
    args = ap.parse_args()
    if args.only:
        import torch
        import aboria_gb300 as ab
        torch.cuda.set_device(0)
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)  # events and library calls on one stream
        ctx = ab.Context(0, stream=stream.cuda_stream)
        if args.only == "fmm" and args.fmm_n:
            orders = tuple(int(o) for o in args.fmm_orders.split(","))
            sec = {f"n{args.fmm_n}": fmm_section(ctx, n=args.fmm_n, orders=orders,
                                                 n_targets=min(10000, args.fmm_n))}
        elif args.only == "fmm":
            sec = {"n1M": fmm_section(ctx), "n16M": fmm_section(ctx, n=1 << 24, orders=(5,), steps=1)}
        elif args.only == "rbf_grid":
            sec = rbf_grid_section(ctx, Path(args.models), quick=args.grid_quick,
                                   budget_s=args.grid_budget)
        elif args.only == "cell_build":
            pos, _ = make_workload()
            p = ab.Particles(3, ctx).set(pos)
            p.init_neighbour_search([0, 0, 0], [1, 1, 1], [True, True, True], 10.0)
            sec = cell_build_record(ctx, stream, p, pos, measured_peaks()[0])
        else:
            sec = rbf_section(ctx, ROOT / "aboria_gb300" / "models" / "spai_mlp_2d.bin")
        print(json.dumps({"section": args.only, **sec}))
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
