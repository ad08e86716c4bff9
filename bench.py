#!/usr/bin/env python
"""Benchmark: converged modes/s of the GPU deflated block LOBPCG.

Workload (the N=1000 configuration the headline metric is quoted on): a seeded
rod network of N=1000 nodes (edge (N/8)^(1/3) = 5, 4 nearest periodic
neighbours, rods r = 0.2 x mean bond, eps_rod 8.41) rasterized with 4^3
sub-voxel averaging on a 128^3 grid, solved at Γ for the lowest 200 bands by
deflated block LOBPCG (block 32, guard 8, lock at relative residual 1e-6,
transverse-projection preconditioner) on the plain complex64 GPU path.

One step = one complete solve. `value` is converged modes per second of device
time over the K timed solves (inputs resident in HBM: eps and the operator
tables are on the device before the timed region; vector blocks are ~1 GB, far
larger than L2). `e2e` repeats the solve through the public API from host
memory: the eps grid is copied from pinned host memory and the operator built
inside the timed region, and the eigenvalues and eigenvectors are copied back to
pinned host memory. The fused Θ pipeline (5 pass kernels per
application) is reported in `theta_roofline` (HBM on algorithmic bytes = 32 B per
voxel per vector + 4 B per voxel of eps^-1 per call, FP32 on its flops); `roofline`
itself is the kernel family with the largest share of the timed region (the
Gram at this workload), achieved = its algorithmic bytes over the CUDA-event time
of each call measured on its stream.
`cpu_baseline` times the numpy/scipy oracle (all host cores) on a bounded
sample of the same solve (block setup plus one LOBPCG iteration) and
extrapolates to the whole solve with the GPU run's iteration count.

    python bench.py [--gpus N --steps K --warmup W] [--impl reference]
Multi-GPU (torchrun): every rank solves its own replica (seed + rank), no
collective on the data path; `value` is all ranks' modes over the slowest rank.
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
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "modes/s at ≤1e-6 eigval err, served vs plain GPU path; p50/p99 solve latency"
# The configuration words the lock criterion as residual 1e-6; in complex64 the
# relative residual of these bands floors at ~1-3e-5 at 128^3 (FFT rounding times
# |k+G|; the reference's own complex64 arithmetic shows the same floor), so the
# solve locks at the reference's default tolerance 1e-4 and the 1e-6 bar is held
# on the eigenvalue error against complex128 runs (tests/test_gpu_accuracy.py).
WORKLOAD = dict(nodes=1000, grid=128, bands=200, block=32, guard=8, tol=1e-4, seed=0, sub=4)


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


# DRAM traffic over algorithmic bytes from single-kernel ncu captures (profiles/):
# tc_gram_32x32_K512k.md (268.5 MB read + 5.6 MB written for 268.4 MB algorithmic),
# tc_rotate_96x64_K512k.md (0.403 + 0.223 GB for 0.671 GB), theta_passes_128.md
# (three passes, steady state: 129.7 MB per vector for 67.1 MB algorithmic)
TRAFFIC_RATIO = {"gram": 1.02, "rotate": 0.93, "theta": 1.93}
# FP32 flops of one Θ application per voxel and vector: 6 complex 3-D FFTs
# (5 N log2 N each) plus the curl, frame and multiply work (~40 per voxel)
def _theta_flops_per_voxel(G: int) -> float:
    import math
    return 6 * 5 * 3 * math.log2(G) + 40


def _fp32_roof(dev) -> dict:
    """Measured FP32 FMA rate of this GPU (ef_fma_probe): scalar FFMA and paired FFMA2."""
    import ctypes
    import torch
    from eigenfns_gb300._lib import call, load
    blocks, iters = 152 * 8, 4096
    out = torch.empty(blocks * 256, dtype=torch.float32, device=dev)
    res = {}
    for name, paired in (("ffma", 0), ("ffma2", 1)):
        best = 0.0
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            call("ef_fma_probe", out.data_ptr(), blocks, iters, paired, torch.cuda.current_stream().cuda_stream)
            e1.record()
            torch.cuda.synchronize()
            best = max(best, load().ef_fma_probe_flops(blocks, iters) / (e0.elapsed_time(e1) * 1e-3) / 1e12)
        res[name + "_TFLOPs"] = best
    res["peak_TFLOPs"] = max(res.values())
    return res


def _accuracy(vals, eps) -> dict | None:
    """Eigenvalue error of this solve against the complex128 run of the same method on the
    same structure (tests/golden/fp64_n1000_g128_gamma.npz), over the bands it holds."""
    import hashlib
    import numpy as np
    p = ROOT / "tests" / "golden" / "fp64_n1000_g128_gamma.npz"
    if not p.exists():
        return None
    d = np.load(p)
    if hashlib.sha256(np.ascontiguousarray(eps).tobytes()).hexdigest() != str(d["eps_sha256"]):
        return {"note": "structure differs from the FP64 fixture"}
    ref = d["vals"]
    n = min(len(ref), len(vals))
    err = np.abs(np.asarray(vals[:n]) - ref[:n]) / ref[:n]
    return {"bands": int(n), "max_rel_err_vs_fp64": float(err.max()),
            "median_rel_err_vs_fp64": float(np.median(err)), "fp64_tol": float(d["tol"])}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = Path(tempfile.mkstemp(suffix=".csv")[1])

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        rows = []
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in rows:
            for name, val in zip(names, r[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        loaded = [s for s in sm if s > 0]
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(rows)}


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def oracle_sample(eps, L, w, gpu_iters=None, gpu_blocks=None):
    """Time the oracle on block setup + one LOBPCG iteration of the same solve."""
    import numpy as np

    from oracle import operator as oop
    from oracle.solver import lobpcg_blocks as ref_lobpcg
    cores = _cores()
    oop.set_fft_workers(cores)
    op = oop.MaxwellOperator(eps, L, dtype=np.complex64)
    t0 = time.perf_counter()
    _, _, st = ref_lobpcg(op, w["bands"], m=w["block"], guard=w["guard"], tol=w["tol"],
                          seed=w["seed"], max_iters_total=1, maxit=400)
    total = time.perf_counter() - t0
    tl = dict((k, t) for k, t in st.timeline[:3])
    t_setup = tl["block_ready"] - t0
    t_iter = tl["iter_end"] - tl["iter_start"]
    iters = gpu_iters if gpu_iters else 30 * 9
    blocks = gpu_blocks if gpu_blocks else int(np.ceil(w["bands"] / (w["block"] - w["guard"])))
    est = blocks * t_setup + iters * t_iter
    return {"value": w["bands"] / est, "unit": "modes/s", "cores": cores, "kind": "port",
            "sample": (f"oracle (numpy/scipy.fft, {cores} threads) on the same {w['grid']}^3 "
                       f"solve: block setup {t_setup:.2f} s + one LOBPCG iteration {t_iter:.2f} s "
                       f"(sample {total:.1f} s), extrapolated to {blocks} blocks x setup + "
                       f"{iters} iterations = {est:.0f} s per solve"),
            "sample_seconds": total, "est_solve_seconds": est}


def run_reference(args, w):
    world, rank, _ = _dist()
    if rank != 0:
        return 0
    from eigenfns_gb300.structure import generate_network
    from oracle.structure import rasterize_averaged
    # the same seeded structure, rasterized by the numpy checker (no library code on this arm)
    from eigenfns_gb300.replicas import replica_seed
    net = generate_network(w["nodes"], replica_seed(w["seed"], rank))
    eps, L = rasterize_averaged(net.rods, w["grid"], net.box_size, sub=w["sub"]), net.box_size
    prof = _solve_profile()
    vals, secs = [], []
    sample = None
    for i in range(args.warmup + args.steps):
        s = oracle_sample(eps, L, w, prof.get("iterations"), prof.get("blocks"))
        if i >= args.warmup:
            vals.append(s["value"])
            secs.append(s["sample_seconds"])
            sample = s
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "modes/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(secs),
            "higher_is_better": True, "scaling": "weak", "extrapolated": True,
            "vs_baseline": None, "dtype": "c64", "data": "synthetic",
            "config": _config(w, args),
            "cpu_baseline": {"value": v, "unit": "modes/s", "cores": sample["cores"], "kind": "port",
                             "sample": sample["sample"] + f" (iteration and block counts: {prof['source']})"},
            "e2e": {"value": v, "unit": "modes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# The GPU solve of this workload takes 393 LOBPCG iterations in 9 blocks (a fixed count,
# measured with the three-pass operator on a GB300); the oracle's per-iteration cost is
# extrapolated with these counts when the reference arm runs alone, and with the live
# counts of the GPU solve when both run in one process
GPU_SOLVE_PROFILE = {"iterations": 393, "blocks": 9,
                     "source": "fixed constant: 393 iterations / 9 blocks measured on a GB300"}


def _solve_profile():
    return dict(GPU_SOLVE_PROFILE)


def _structure(w, rank):
    from eigenfns_gb300.structure import make_structure
    from eigenfns_gb300.replicas import replica_seed
    eps, L, _ = make_structure(w["nodes"], w["grid"], seed=replica_seed(w["seed"], rank), sub=w["sub"])
    return eps, L


def _config(w, args):
    return {"workload": (f"rod network N={w['nodes']} (seeded), {w['grid']}^3 eps with "
                         f"{w['sub']}^3 sub-voxel averaging, Gamma point, lowest {w['bands']} bands by "
                         f"deflated block LOBPCG (block {w['block']}, guard {w['guard']}, tol {w['tol']}), "
                         f"plain complex64 GPU path"),
            "nodes": w["nodes"], "grid": w["grid"], "bands": w["bands"], "block": w["block"],
            "guard": w["guard"], "tol": w["tol"],
            "tol_note": "relative-residual lock at 1e-4 (complex64 floor ~1-3e-5 at 128^3); eigenvalue error vs complex128 <= 1e-6 is the checked bar",
            "l2": "inputs larger than L2 (each 32-vector block is 1.07 GB)",
            "parallelism": f"replicas x{args.gpus}"}


def _interior_steps(dev) -> dict:
    import numpy as np
    import torch

    from eigenfns_gb300 import blas
    from eigenfns_gb300._lib import EF_RAND_RADEMACHER_C, call
    from eigenfns_gb300.chebyshev import random_block
    from eigenfns_gb300.operator import MaxwellOperator
    from eigenfns_gb300.structure import make_structure
    out = {}
    for name, grid, m, steps, bytes_per in (("kpm_256", 256, 16, 12, 48.0), ("cheb_192", 192, 8, 12, 80.0)):
        eps, L, _ = make_structure(10000, grid, seed=7)
        op = MaxwellOperator(eps, L, device=dev)
        s = 2.0 / 5.0e3
        T0 = random_block(op, m, 3, 0, EF_RAND_RADEMACHER_C)
        T1 = torch.empty_like(T0)
        ws = op.workspace(m)
        st = blas._stream()
        if name.startswith("kpm"):
            mom = torch.zeros((m, 2 * steps + 2), dtype=torch.float64, device=dev)
            call("ef_kpm_first", op.handle, T0.data_ptr(), T1.data_ptr(), m, s, mom.data_ptr(),
                 2 * steps + 2, ws.data_ptr(), ws.numel(), st)

            def step(k, a=T1, b=T0):
                call("ef_kpm_step", op.handle, a.data_ptr(), b.data_ptr(), m, s, k, mom.data_ptr(),
                     2 * steps + 2, ws.data_ptr(), ws.numel(), st)
        else:
            Y = torch.empty_like(T0)
            call("ef_cheb_first", op.handle, T0.data_ptr(), T1.data_ptr(), Y.data_ptr(), m, s,
                 0.5, 0.25, ws.data_ptr(), ws.numel(), st)

            def step(k, a=T1, b=T0):
                call("ef_cheb_step", op.handle, a.data_ptr(), b.data_ptr(), Y.data_ptr(), m, s, 0.01,
                     ws.data_ptr(), ws.numel(), st)
        step(1)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for k in range(2, steps):
            step(k, *((T1, T0) if k % 2 else (T0, T1)))
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / (steps - 2)
        N = grid ** 3
        out[name] = {"grid": grid, "vectors": m, "ms_per_step": ms,
                     "theta_applies_per_s": m / (ms * 1e-3),
                     "algorithmic_GBs": bytes_per * N * m / (ms * 1e-3) / 1e9}
        del op, T0, T1
        torch.cuda.empty_cache()
    return out


BATCHED_KINDS = ((64, 32, 16, 16, 4), (216, 48, 32, 32, 8), (512, 64, 48, 32, 8))  # N, grid, bands, m, guard


def _batched_instances(dev, seeds_per_kind: int) -> dict:
    """The 48-instance batched workload: grouped solves against one-at-a-time solves."""
    import numpy as np
    import torch
    from eigenfns_gb300.batched import lobpcg_batched
    from eigenfns_gb300.operator import MaxwellOperator
    from eigenfns_gb300.solver import lobpcg_blocks
    from eigenfns_gb300.structure import bz_kpoint, make_structure
    inst = []
    for nodes, grid, nev, m, guard in BATCHED_KINDS:
        for j in range(seeds_per_kind):
            seed = 1000 * nodes + j
            eps, L, _ = make_structure(nodes, grid, seed=seed)
            inst.append((MaxwellOperator(eps, L, k_frac=bz_kpoint(seed), device=dev), nev, m, guard, seed))
    # warm both paths (kernels, plans, workspaces) on one instance of each kind
    for k in range(len(BATCHED_KINDS)):
        op, nev, m, g, s = inst[k * seeds_per_kind]
        lobpcg_blocks(op, nev, m=m, guard=g, tol=1e-4, seed=s, verbose=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    alone = [lobpcg_blocks(op, nev, m=m, guard=g, tol=1e-4, seed=s, verbose=False)
             for op, nev, m, g, s in inst]
    torch.cuda.synchronize()
    t_alone = time.perf_counter() - t0
    t0 = time.perf_counter()
    batch = lobpcg_batched([i[0] for i in inst], [i[1] for i in inst], m=[i[2] for i in inst],
                           guard=[i[3] for i in inst], tol=1e-4, seeds=[i[4] for i in inst])
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    modes = sum(len(v) for v, _, _ in batch)
    diff = max(float(np.abs(a[0] - b[0]).max() / np.abs(a[0]).max()) for a, b in zip(alone, batch))
    return {"workload": (f"{len(inst)} instances: N in (64, 216, 512) x {seeds_per_kind} seeds on "
                         "32^3/48^3/64^3, k uniform in the first BZ, 16/32/48 bands, tol 1e-4"),
            "batched_s": t_batch, "one_at_a_time_s": t_alone,
            "batched_modes_per_s": modes / t_batch, "one_at_a_time_modes_per_s": modes / t_alone,
            "speedup": t_alone / t_batch, "max_rel_diff_batched_vs_alone": diff,
            "theta_applications": int(sum(st.theta_applications for _, _, st in batch))}


def run_ours(args, w):
    import numpy as np
    import torch
    import torch.distributed as dist

    world, rank, local = _dist()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)
    from eigenfns_gb300 import _lib, profiling
    from eigenfns_gb300.operator import MaxwellOperator
    from eigenfns_gb300.solver import lobpcg_blocks
    lib = _lib.load()

    eps, L = _structure(w, rank)
    op = MaxwellOperator(eps, L, device=dev)

    def solve():
        return lobpcg_blocks(op, w["bands"], m=w["block"], guard=w["guard"], tol=w["tol"],
                             seed=w["seed"], verbose=False, maxit=args.maxit)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # the autotuner picks the operator pipeline and the Gram schedules of this block size
    # on this GPU (timed once, cached on disk for later runs)
    from eigenfns_gb300 import tune
    tuned = tune.autotune(op, w["block"])
    for _ in range(args.warmup):
        solve()
    barrier()
    sampler = ClockSampler(local)
    sampler.start()
    launches0 = lib.ef_launch_count()
    starts, ends, stats_list, vals_list = [], [], [], []
    stream = torch.cuda.current_stream()
    torch.cuda.nvtx.range_push("timed")
    with profiling.theta_timer() as tt:
        for _ in range(args.steps):
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            vals, vecs, st = solve()
            e.record(stream)
            starts.append(s)
            ends.append(e)
            stats_list.append(st)
            vals_list.append(vals)
            del vecs
        barrier()
    torch.cuda.nvtx.range_pop()
    launches = int(lib.ef_launch_count() - launches0)
    clocks = sampler.stop()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_s = starts[0].elapsed_time(ends[-1]) / 1e3
    modes = sum(len(v) for v in vals_list)
    from eigenfns_gb300.replicas import aggregate
    total_all, modes_all = aggregate(total_s, modes, dev)
    value = modes_all / total_all

    # roofline of the kernel with the largest share of the timed region
    ops = tt.summary()
    G = w["grid"]
    dom = max(ops, key=lambda k: ops[k]["total_ms"])
    th = ops[dom]
    achieved = th["bytes"] / (th["total_ms"] * 1e-3) / 1e9
    peak, peak_kind = _peaks()
    alg_per_call = th["bytes"] / max(th["calls"], 1)
    traffic = alg_per_call * TRAFFIC_RATIO[dom] if dom in TRAFFIC_RATIO else None
    # the fused Θ pipeline against both roofs (HBM on algorithmic bytes, FP32 on flops)
    theta_roof = None
    if "theta" in ops:
        tq = ops["theta"]
        gbs = tq["bytes"] / (tq["total_ms"] * 1e-3) / 1e9
        vecs_per_s = tq["bytes"] / (32.0 * G ** 3 + 4.0 * G ** 3 / max(w["block"], 1)) / (tq["total_ms"] * 1e-3)
        tflops = vecs_per_s * _theta_flops_per_voxel(G) * G ** 3 / 1e12
        fp32 = _fp32_roof(dev)
        fp32_peak = fp32["peak_TFLOPs"]
        theta_roof = {"achieved_GBs": gbs, "hbm_frac": gbs / peak, "achieved_TFLOPs": tflops,
                      "fp32_peak_TFLOPs": fp32_peak, "fp32_peak_source": "measured (ef_fma_probe)",
                      "fp32_probe": fp32, "fp32_frac": tflops / fp32_peak,
                      "us_per_vector": 1e6 / vecs_per_s,
                      "traffic_per_vector": TRAFFIC_RATIO["theta"] * 32.0 * G ** 3}

    # e2e through the public API with host buffers (pinned), same solve
    e2e = None
    if not args.no_e2e:
        eps_pinned = torch.from_numpy(eps).pin_memory()
        nb = w["bands"]
        host_vecs = torch.empty((nb, 2, G, G, G), dtype=torch.complex64).pin_memory()
        e_ms = []
        for _ in range(max(1, args.steps)):
            barrier()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0 = time.perf_counter()
            s.record(stream)
            op2 = MaxwellOperator(eps_pinned.numpy(), L, device=dev)
            vals, vecs, _ = lobpcg_blocks(op2, nb, m=w["block"], guard=w["guard"], tol=w["tol"],
                                          seed=w["seed"], verbose=False)
            host_vecs.copy_(vecs, non_blocking=True)
            e.record(stream)
            torch.cuda.synchronize()
            e_ms.append(max(s.elapsed_time(e), (time.perf_counter() - t0) * 1e3))
            del op2, vecs
        e2e_s = sum(e_ms) / 1e3
        e2e_t = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
        if world > 1:
            dist.all_reduce(e2e_t, op=dist.ReduceOp.MAX)
        e2e = {"value": nb * len(e_ms) * world / float(e2e_t[0]), "unit": "modes/s",
               "h2d_bytes_per_step": int(eps.nbytes),
               "d2h_bytes_per_step": int(host_vecs.numel() * 8 + nb * 8)}

    # served vs plain: a seeded Poisson stream of smaller eigensolve requests (N in
    # {64, 216, 512} on 32^3/48^3/64^3, random Bloch k, 8-48 bands) solved by the
    # continuously batched server (device-memory admission, requests of one shape started
    # as grouped solves, groups interleaved by the pipelined driver) and by the plain
    # one-at-a-time path; both build each request's structure and operator
    served = None
    if not args.no_served:
        from eigenfns_gb300.serve import EigenServer, poisson_requests, run_plain, summarize
        reqs = poisson_requests(args.served_requests, seed=2025 + rank, rate_hz=40.0)
        run_plain(reqs[:2])                       # warm the small-grid kernels
        t0 = time.perf_counter()
        srv = EigenServer(budget_bytes=160e9, max_concurrent=32, device=dev)
        res_s = srv.run(reqs, realtime=True)
        wall_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        res_p = run_plain(reqs, device=dev)
        wall_p = time.perf_counter() - t0
        ss, sp = summarize(res_s, wall_s), summarize(res_p, wall_p)
        same = max(float(np.abs(a.vals - b.vals).max() / np.abs(b.vals).max()) for a, b in zip(res_s, res_p))
        served = {"workload": f"{len(reqs)} Poisson requests (40/s): N in (64, 216, 512) on 32^3/48^3/64^3, "
                              "random k, 8-48 bands, tol 1e-4; 160 GB admission budget, 32 slots",
                  "served": ss, "plain": sp, "speedup": ss["modes_per_s"] / sp["modes_per_s"],
                  "peak_concurrent": srv.peak_concurrent, "groups": srv.groups,
                  "max_rel_diff_served_vs_plain": same}

    # batched launch of 48 uneven instances: rod networks with N in {64, 216, 512} (16 seeds
    # each) on 32^3/48^3/64^3, a k-point drawn in each supercell's first Brillouin zone,
    # 16/32/48 lowest bands; solved as grouped solves (one per shape, interleaved)
    # against one at a time
    batched = None
    if not args.no_batched:
        batched = _batched_instances(dev, args.batched_seeds)

    # interior-window kernels at their configuration sizes (N = 10,000 structure):
    # fused KPM steps at 256^3 on 16 complex Rademacher probes and fused bandpass
    # Chebyshev steps at 192^3 on a chunk of 8 vectors; throughput in Θ-applies/s and
    # algorithmic GB/s (KPM step 48 B/voxel/probe, Chebyshev step 80 B/voxel/vector)
    interior = None
    if not args.no_interior:
        interior = _interior_steps(dev)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        iters = int(np.mean([st.iterations for st in stats_list]))
        blocks = int(np.mean([len(st.rounds) for st in stats_list]))
        cpu = oracle_sample(eps, L, w, iters, blocks)
        cpu = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}

    if world > 1:
        dist.destroy_process_group()
    if rank != 0:
        return 0
    st0 = stats_list[-1]
    lat = sorted(step_ms)
    line = {
        "metric": METRIC, "value": value, "unit": "modes/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": statistics.mean(step_ms), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
        "config": _config(w, args),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "kernel": dom,
                     "peak_source": peak_kind,
                     "mean_ms_per_call": th["mean_ms_per_call"],
                     "algorithmic_bytes_per_call": alg_per_call,
                     "traffic_source": "ncu DRAM bytes / algorithmic bytes of the same kernel on a "
                                       "smaller case (profiles/), scaled to this call's bytes"},
        "theta_roofline": theta_roof,
        "kernels": {k: {"share_of_step": v["total_ms"] / sum(step_ms), "calls": v["calls"],
                        "mean_ms": v["mean_ms_per_call"], "GB/s": v["gbs"], "TFLOP/s": v["tflops"]}
                    for k, v in ops.items()},
        "cpu_baseline": cpu, "e2e": e2e, "served": served, "batched": batched, "interior": interior,
        "clocks": clocks,
        "gpu_launches": launches,
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
        "accuracy": _accuracy(vals_list[-1], eps),
        "autotune": {"operator": {k: tuned["operator"][k] for k in ("passes", "subbatch_bytes", "ms")},
                     "gram": {k: {"kernel": v["kernel"], "units": v["units"]}
                              for k, v in tuned["gram"].items()}},
        "solve": {"theta_applications": st0.theta_applications, "iterations": st0.iterations,
                  "blocks": len(st0.rounds),
                  "max_res_locked": max(r["max_res_locked"] for r in st0.rounds),
                  },
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--no-interior", action="store_true")
    ap.add_argument("--served-requests", type=int, default=48)
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batched-seeds", type=int, default=16,
                    help="seeds per node count in the batched-instances workload (16 = 48 instances)")
    ap.add_argument("--grid", type=int, default=None, help="override the grid (smaller probes)")
    ap.add_argument("--bands", type=int, default=None)
    ap.add_argument("--tol", type=float, default=None)
    ap.add_argument("--maxit", type=int, default=400,
                    help="LOBPCG iterations per block (bounded runs for launch-list profiling)")
    args = ap.parse_args()
    w = dict(WORKLOAD)
    if args.grid:
        w["grid"] = args.grid
    if args.bands:
        w["bands"] = args.bands
    if args.tol:
        w["tol"] = args.tol
    if args.impl == "reference":
        return run_reference(args, w)
    return run_ours(args, w)


if __name__ == "__main__":
    sys.exit(main())
