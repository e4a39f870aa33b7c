"""Benchmark: bound levels/s of the batched FP32-compensated solver + adjoint
on the uneven 2048-potential batch (Morse / Lennard-Jones / Morse+bumps,
N ~ logU[2048, 65536], 8192 trial energies, levels up to 0.999 De), counting
only levels within 1e-9 Hartree of the FP64 reference and with the right
node count.

One step = one device-resident solve (FP32 TMA scan, FP32 Cooley refinement,
FP64 polish, normalised psi written to HBM, replayed from a CUDA graph) plus
the Hellmann-Feynman adjoint of L = sum_v w_v (E_v - T_v)^2 back to every
V(r_i).  The plain FP64 CUDA solver (FP64 scan + FP64 bisection + psi) is timed
on the same batch and is also the per-level FP64 reference (it is bit-exact
with the CPU oracle, checked here on a sample).  ``e2e`` is the same step
through the C ABI with host buffers (pinned V in, energies and dL/dV out).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun each rank solves its own batch (seed + rank): weak scaling,
no data-path collective.  ``--impl reference`` times the CPU restatement of
the path (the reference has no solver to run) on all host cores.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "bound levels/s at |dE|<=1e-9 Eh vs FP64 oracle; batched+adjoint vs plain CUDA"
UNIT = "levels/s"
E_TOL = 1e-9
CPU_SAMPLE = 96  # potentials of the workload the CPU legs time
# dram__bytes_read.sum + dram__bytes_write.sum of one scan32 launch per grid
# point, ncu on the 128-potential mixed batch (18.12 MB / 2,242,300 points)
SCAN32_DRAM_BYTES_PER_POINT = 8.08
# ncu (dram__bytes_read.sum + dram__bytes_write.sum) of refine_long_kernel per
# algorithmic point-update on the 512-potential mixed batch (64.05 MB over
# 235,987,411 point-updates: the windows' W is re-read from L2)
REFINE_LONG_DRAM_BYTES_PER_UPDATE = 0.2714


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


WORKLOADS = {
    "mixed": "mixed_batch: 2048 potentials (1/3 Morse, 1/3 LJ 12-6, 1/3 Morse+1-3 Gaussian bumps via 1024-knot "
             "natural spline), N~logU[2048,65536], mu~logU[500,1e5], 8192 trial energies, levels up to 0.999 De, "
             "psi written, adjoint dL/dV",
    "single": "morse_single: one Morse (De=0.1, a=1, re=2, mu=1000) on N=4096, r in [0.5, 27], 1024 trial "
              "energies, psi written, adjoint dL/dV",
    "morse64": "morse_batch: 64 Morse, De~U[0.02,0.2], a~U[0.5,1.5], re~U[1.5,4], mu~logU[500,1e5], N=16384 on "
               "[0.5, re+30/a], 8192 trial energies, psi written, adjoint dL/dV",
    "adjoint256": "bump_adjoint: 256 Morse+1-3 Gaussian bumps (1024-knot spline) on N=32768, 8192 trial energies; "
                  "loss sum_v w_v (E_v - T_v)^2, T_v = levels with bump amplitudes x1.1, w_v~U[0.5,1]; "
                  "gradients to every V(r_i) and to the Morse/bump parameters",
    "long": "morse_long: one Morse (De=0.15, a=0.6, re=4, mu=1e5) on N=2^20, r in [0.5, 54], 65536 trial "
            "energies, psi written, adjoint dL/dV",
}


def workload(rank: int, name: str = "mixed", **kw):
    """Rank r solves its own seeded batch (independent potentials: weak scaling).
    The single-potential workloads are replicas (the same potential per rank)."""
    from epseon_backend_gb300 import synth

    if name == "mixed":
        return synth.mixed_batch(seed=3 + 100 * rank, **kw)
    if name == "morse64":
        return synth.morse_batch(seed=2 + 100 * rank, **kw)
    if name == "adjoint256":
        return synth.bump_adjoint(seed=4 + 100 * rank, **kw)
    if name == "single":
        return synth.morse_single(**kw)
    if name == "long":
        return synth.morse_long(**kw)
    raise ValueError(f"unknown workload {name!r}")


def aggregate(ms_local: float, levels_local: int, dist=None, device=None):
    """Whole-job numbers over ranks: max of the per-rank step time, sum of the
    levels solved.  No data-path collective: only these two scalars travel."""
    if dist is None:
        return ms_local, levels_local
    import torch

    t = torch.tensor([ms_local], dtype=torch.float64, device=device)
    n = torch.tensor([levels_local], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    return float(t.item()), int(n.item())


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def count_good(b, fast_E, fast_nodes, fast_status, ref):
    """Levels of the fast solve within E_TOL of the FP64 reference with v nodes."""
    good = 0
    total = 0
    for p in range(len(b)):
        n = int(ref.n_out[p])
        total += n
        if n == 0:
            continue
        d = np.abs(fast_E[p, :n] - ref.energy[p, :n])
        ok = (d <= E_TOL) & (fast_nodes[p, :n] == np.arange(n)) & ((fast_status[p, :n] & ~4) == 0)
        # node counts are checked where the grid resolves the wavelength
        if int(ref.status[p, 0]) & 4:
            ok = (d <= E_TOL) & ((fast_status[p, :n] & ~4) == 0)
        good += int(ok.sum())
    return good, total


def cpu_oracle_leg(b, n_threads: int, seed: int = 0):
    """Times the FP64 CPU restatement (plain method) on a bounded sample."""
    from oracle import oracle as O

    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(len(b), size=min(CPU_SAMPLE, len(b)), replace=False))
    Vs = [b.V(int(i)) for i in idx]
    t = time.perf_counter()
    sols = O.solve_batch(Vs, b.r_min[idx], b.r_max[idx], b.mu[idx], b.e_cap[idx], b.n_trial, n_threads=n_threads)
    dt = time.perf_counter() - t
    levels = int(sum(s.energy.size for s in sols))
    return idx, sols, levels, dt


def run_reference(args, rank, world):
    """CPU restatement of the path on all host cores (the reference has no solver)."""
    if rank != 0:
        return 0
    from oracle import build as ob

    ob.build()
    b = workload(0, args.workload)
    cores = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_oracle_leg(b, cores, seed=0)
    t_all, lev_all = 0.0, 0
    for k in range(args.steps):
        _, _, levels, dt = cpu_oracle_leg(b, cores, seed=k)
        t_all += dt
        lev_all += levels
    v = lev_all / t_all
    sample = (f"{min(CPU_SAMPLE, len(b))} of {len(b)} potentials of {args.workload} per step (random, seeded), "
              "plain FP64 method")
    out = {
        "impl": "reference",
        "metric": METRIC,
        "value": v,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * t_all / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded PCG64)",
        "config": {"workload": WORKLOADS[args.workload], "sample": sample},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--batch", type=int, default=None,
                    help="potentials per GPU of the mixed workload (default 2048; smaller for profiler captures)")
    ap.add_argument("--long-window", type=int, default=0,
                    help="window length above which a level runs one CTA per level (0: the library's default, "
                         "chosen from the level count)")
    ap.add_argument("--mid-window", type=int, default=0,
                    help="window length above which a level runs its double-float passes one warp per level "
                         "(> 0; 0: the library's default, off)")
    ap.add_argument("--workload", default="mixed", choices=sorted(WORKLOADS),
                    help="mixed = the headline batch; the others are the single-Morse, 64-Morse, adjoint and "
                         "long-grid cases")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch

    from epseon_backend_gb300 import capi

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()

    ctx = capi.Context(local)
    fp32_peak, fp64_peak = ctx.measure_fma_peaks()
    b = workload(rank, args.workload, **({"B": args.batch} if args.batch else {}))
    Vs = b.potentials()
    cap = 512

    # ---- FP64 reference on the GPU: the plain method (bit-exact with the CPU
    # oracle, checked on a sample below) gives the per-level truth
    ref = ctx.solve(Vs, b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial, method=capi.METHOD_PLAIN_FP64,
                    level_capacity=cap)
    plain_levels = int(ref.n_out.sum())
    psi_needed = int(np.sum(ref.n_out.astype(np.int64) * b.N.astype(np.int64))) + 4096

    # ---- device-resident batch (V, outputs, psi in HBM) shared by both methods
    db = capi.DeviceBatch(ctx, Vs, b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial, cap, want_psi=True,
                          psi_capacity=psi_needed)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    # plain FP64 CUDA solver, same device-resident step (solve + psi)
    db.solve(capi.METHOD_PLAIN_FP64, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(np.nan_to_num(db.energy.cpu().numpy()), np.nan_to_num(ref.energy))
    e0.record(stream)
    db.solve(capi.METHOD_PLAIN_FP64, stream=stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    plain_ms = [e0.elapsed_time(e1)]
    db.solve(capi.METHOD_PLAIN_FP64, stage_timing=True, stream=stream.cuda_stream)
    plain_stats = ctx.stats()

    n_lev = torch.from_numpy(ref.n_out.astype(np.int64)).cuda()
    rng = np.random.default_rng(1000 + rank)
    w_np = rng.uniform(0.5, 1.0, (len(b), cap))
    w = torch.from_numpy(w_np).cuda()
    if args.workload == "adjoint256":
        # targets: the levels of the same potentials with every bump amplitude x1.1
        from epseon_backend_gb300 import synth

        tb = synth.bump_adjoint(seed=4 + 100 * rank, amp_scale=1.1)
        tsol = ctx.solve(tb.potentials(), tb.r_min, tb.r_max, tb.mu, tb.e_cap, tb.n_trial,
                         method=capi.METHOD_PLAIN_FP64, level_capacity=cap)
        target_np = np.where(np.arange(cap)[None, :] < tsol.n_out[:, None], np.nan_to_num(tsol.energy), 0.0)
    else:
        target_np = np.nan_to_num(ref.energy, nan=0.0) * 1.001
    target = torch.from_numpy(target_np).cuda()
    slot = torch.arange(cap, device="cuda")[None, :]
    mask = (slot < n_lev[:, None]).to(torch.float64)

    # the adjoint workload differentiates to the Morse / bump parameters too
    # (epscu_tabulate_adjoint: the spline transpose and the knot derivatives)
    with_params = args.workload == "adjoint256"
    if with_params:
        P_host = capi.batch_params(b)
        P_dev = torch.from_numpy(P_host).cuda()
        gP_dev = torch.zeros_like(P_dev)

    def step():
        db.solve(capi.METHOD_FAST_FP32C, long_window=args.long_window, mid_window=args.mid_window, stream=stream.cuda_stream)
        gE = 2.0 * w * (torch.nan_to_num(db.energy) - target) * mask
        db.adjoint(gE, stream=stream.cuda_stream)
        if with_params:
            db.param_adjoint(b.kind, P_dev, gP_dev, stream=stream.cuda_stream)

    db.solve(capi.METHOD_FAST_FP32C, long_window=args.long_window, mid_window=args.mid_window, tune=True, stream=stream.cuda_stream)  # autotune the scan shape
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # stage timing of one instrumented solve (per-kernel events on the solve stream)
    db.solve(capi.METHOD_FAST_FP32C, long_window=args.long_window, mid_window=args.mid_window, stage_timing=True, stream=stream.cuda_stream)
    st = ctx.stats()
    torch.cuda.synchronize()

    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms_local = e0.elapsed_time(e1) / args.steps

    fast_E = db.energy.cpu().numpy()
    fast_nodes = db.nodes.cpu().numpy()
    fast_status = db.status.cpu().numpy()
    good, total = count_good(b, fast_E, fast_nodes, fast_status, ref)
    ms, levels_all = aggregate(ms_local, good, dist, "cuda")
    plain_ms_all, plain_levels_all = aggregate(min(plain_ms), plain_levels, dist, "cuda")
    max_dE = float(np.nanmax(np.where(np.arange(cap)[None, :] < ref.n_out[:, None], np.abs(fast_E - ref.energy), 0.0)))

    # ---- adjoint check: dL/dV against the plain solve's psi on a few points
    # (exact identity of the discrete problem; FD checks live in the tests)
    gV = db.gV.cpu().numpy()

    # ---- e2e through the C ABI with host buffers: pinned V in, the solve keeps
    # psi in device memory (EPSCU_KEEP_PSI), energies out, the loss gradient
    # computed on the host, the adjoint on the kept psi, dL/dV out
    Vcat, offsets, N = capi.concat(Vs)
    V_pinned = torch.from_numpy(Vcat).pin_memory()
    gV_pinned = torch.empty(Vcat.size, dtype=torch.float64).pin_memory()
    batch_host = capi.Concatenated(V_pinned.numpy(), offsets, N)
    e2e_steps = max(2, args.steps // 2)
    maskh = (np.arange(cap)[None, :] < ref.n_out[:, None])
    w2m = 2.0 * w_np * maskh

    # page-locked host buffers, allocated once: the solve's results and the
    # loss gradient dL/dE (the host side of a training loop would keep these)
    def pinned(shape, dtype):
        return torch.empty(shape, dtype=dtype).pin_memory().numpy()

    nb = len(b)
    res_buf = capi.Solution(pinned((nb,), torch.int32), pinned((nb,), torch.int32), pinned((nb, cap), torch.float64),
                            pinned((nb, cap), torch.int32), pinned((nb, cap), torch.int32),
                            pinned((nb, cap), torch.float64), None, pinned((nb,), torch.int64), N)
    gE_pinned = pinned((nb, cap), torch.float64)

    gP_pinned = pinned((nb, 12), torch.float64) if with_params else None

    def e2e_step():
        sol = ctx.solve(batch_host, b.r_min, b.r_max, b.mu, b.e_cap, b.n_trial, method=capi.METHOD_FAST_FP32C,
                        level_capacity=cap, keep_psi=True, long_window=args.long_window, mid_window=args.mid_window, out=res_buf)
        np.subtract(np.nan_to_num(sol.energy), target_np, out=gE_pinned)
        np.multiply(gE_pinned, w2m, out=gE_pinned)
        gVh = ctx.adjoint(gE_pinned, Vcat.size, recompute=False, out=gV_pinned.numpy())
        if with_params:
            ctx.tabulate_adjoint(b.kind, P_host, N, b.r_min, b.r_max, gVh, out=gP_pinned)
        return sol, gE_pinned, gVh

    e2e_step()
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(e2e_steps):
        sol, gEh, gVh = e2e_step()
    t_e2e = (time.perf_counter() - t) / e2e_steps
    e2e_good, _ = count_good(b, sol.energy, sol.nodes, sol.status, ref)
    h2d = Vcat.nbytes + len(b) * (8 * 4 + 4 + 8) + gEh.nbytes
    d2h = len(b) * cap * (8 + 4 + 4 + 8) + len(b) * 8 + gVh.nbytes
    if with_params:  # the parameter chain: params and dL/dV in, dL/dparams out
        h2d += P_host.nbytes + gVh.nbytes + len(b) * (4 + 8 + 4 + 8 + 8)
        d2h += gP_pinned.nbytes

    # ---- CPU baseline (oracle port on the host cores, bounded sample)
    cpu = None
    if rank == 0 and not args.no_cpu:
        cores = os.cpu_count() or 1
        idx, sols, lev, dt = cpu_oracle_leg(b, cores)
        same = all(np.array_equal(s.energy, ref.energy[int(p), : s.energy.size]) for s, p in zip(sols, idx))
        cpu = {"value": lev / dt, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{len(idx)} of {len(b)} potentials (seeded random), plain FP64 method, {dt:.1f} s",
               "plain_gpu_bit_exact_on_sample": bool(same)}

    # ---- roofline of the dominant kernel: refine_long_kernel, the longest
    # single launch of the step (the long levels' CTA-per-level refinement;
    # time from its own events in the stage-timed solve, on the solve stream).
    # Unit: one Numerov point-update = 9 algorithmic flops (T, f, g, two-term
    # recurrence) in its FP32 and its double-float passes alike; the chunked
    # three-phase passes, the compensation (a double-float step issues ~10x
    # the FP32 instructions), renormalisation and sign bookkeeping are not
    # counted, so the fraction is structurally far below 1.
    rl_updates = int(st.long_fp32_point_updates + st.long_df_point_updates)
    ach = 9.0 * rl_updates / (st.ms_refine_long * 1e-3) / 1e12 if st.ms_refine_long > 0 else 0.0
    traffic = (REFINE_LONG_DRAM_BYTES_PER_UPDATE * rl_updates) if REFINE_LONG_DRAM_BYTES_PER_UPDATE else None
    roof = {"bound": "fp32_alu", "achieved": ach, "peak": fp32_peak, "unit": "TFLOP/s", "frac": ach / fp32_peak,
            "traffic": traffic,
            "traffic_unit": "bytes per launch (ncu-measured DRAM bytes per point-update x point-updates)",
            "kernel": "refine_long_kernel", "ms": st.ms_refine_long,
            "algorithmic": {"point_updates": rl_updates, "fp32_pass_point_updates": int(st.long_fp32_point_updates),
                            "double_float_pass_point_updates": int(st.long_df_point_updates),
                            "flops_per_update": 9},
            "peak_source": "measured FP32 FMA burst (epscu_measure_fma_peaks), 2 flops per FMA"}
    # the scan stage in the same unit (the coarse scan32 launch plus, on large
    # batches, the bisection rounds; scan32 alone is FP32-issue-bound)
    scan_ach = 9.0 * st.scan_point_updates / (st.ms_scan * 1e-3) / 1e12
    roof_scan = {"kernel": "scan stage (scan32_kernel" + (" on every 16th trial energy + the bisection count round)"
                                                          if len(b) >= 512 else ")"),
                 "achieved": scan_ach, "peak": fp32_peak, "unit": "TFLOP/s", "frac": scan_ach / fp32_peak,
                 "ms": st.ms_scan, "point_updates": int(st.scan_point_updates),
                 "dram_bytes_per_grid_point_scan32": SCAN32_DRAM_BYTES_PER_POINT}
    # the per-level stages in the same unit (algorithmic point-updates counted
    # by the kernels over the level windows; latency-bound lane marches)
    stage_rates = {
        "refine32_point_updates_per_s": st.refine_point_updates / (st.ms_refine32 * 1e-3) if st.ms_refine32 > 0 else None,
        "double_float_point_updates_per_s": st.fp64_point_updates / (st.ms_polish64 * 1e-3) if st.ms_polish64 > 0 else None,
        "refine32_point_updates": int(st.refine_point_updates),
        "double_float_point_updates": int(st.fp64_point_updates),
    }
    # the FP64-pipe view of the plain solver's dominant kernel, for comparison
    roof_plain = {"kernel": "scan64_kernel", "achieved": 9.0 * plain_stats.scan_point_updates
                  / (plain_stats.ms_scan * 1e-3) / 1e12, "peak": fp64_peak, "unit": "TFLOP/s"}
    roof_plain["frac"] = roof_plain["achieved"] / fp64_peak
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs")
    # the psi write-back, kernel by kernel (stage-timed solve): zero_psi
    # writes the zeros outside the level windows (8 B a point), the norm
    # passes store each window point once as a tagged float pair (8 B, inside
    # their compute-bound passes, not timed here), scale_psi reads the pairs
    # and writes the normalised doubles (16 B a window point).  Algorithmic
    # bytes: the rows written once, levels x N x 8 B.
    zero_bytes = 8 * int(st.psi_zero_points)
    scale_bytes = 16 * int(st.psi_window_points)
    pair_bytes = 8 * int(st.psi_window_points)

    def gbs(nbytes, ms_):
        return nbytes / (ms_ * 1e-3) / 1e9 if ms_ > 0 else None

    psi_write = {
        "algorithmic_bytes": int(st.psi_bytes),
        "zero_psi": {"bytes": zero_bytes, "ms": st.ms_zero_psi, "GB_per_s": gbs(zero_bytes, st.ms_zero_psi)},
        "scale_psi": {"bytes": scale_bytes, "ms": st.ms_write, "GB_per_s": gbs(scale_bytes, st.ms_write)},
        "norm_pass_pair_bytes": pair_bytes,
        "traffic_over_algorithmic": (zero_bytes + pair_bytes + scale_bytes) / st.psi_bytes if st.psi_bytes else None,
        "hbm_peak_GBs": hbm,
    }

    value = levels_all / (ms * 1e-3)
    plain_value = plain_levels_all / (plain_ms_all * 1e-3)
    out = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64",
        "data": "synthetic (seeded PCG64 potentials; no dataset)",
        "config": {
            "workload": WORKLOADS[args.workload],
            "potentials_per_gpu": len(b),
            "grid_points_per_gpu": int(b.N.sum()),
            "levels_per_gpu": total,
            "l2": "inputs larger than L2 (V 8 B x grid points, psi writes); no flush",
            "parallelism": f"independent batch per GPU (weak scaling, {world} rank(s))",
        },
        "levels_counted": good,
        "levels_total": total,
        "max_abs_dE_vs_fp64": max_dE,
        "plain_fp64": {"value": plain_value, "ms_per_step": min(plain_ms), "levels": plain_levels,
                       "ms_scan": plain_stats.ms_scan, "ms_bisect_norm": plain_stats.ms_polish64,
                       "ms_write": plain_stats.ms_write},
        "speedup_vs_plain_fp64": value / plain_value,
        "stages_ms": {"prepare": st.ms_prepare, "scan32": st.ms_scan, "refine32": st.ms_refine32,
                      "polish64": st.ms_polish64, "write64": st.ms_write, "solve_total": st.ms_total,
                      "fallbacks": st.fallbacks, "twist_searches": st.twist_searches,
                      "norm_redos": st.norm_redos, "refine_max_iters": st.refine_max_iters,
                      "refine_max_level_updates": st.refine_max_level_updates,
                      "df_max_level_updates": st.df_max_level_updates},
        "roofline": roof,
        "roofline_scan": roof_scan,
        "roofline_plain_fp64": roof_plain,
        "stage_rates": stage_rates,
        "psi_write": psi_write,
        "e2e": {"value": e2e_good * world / t_e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "steps": e2e_steps,
                "note": "host pinned V -> C ABI solve (psi kept on the device) -> energies to host -> adjoint -> dL/dV to host; wall clock per step"},
        "gpu_launches": int(args.steps * (st.kernel_launches + 1)),
        "clocks": clk.summary(),
        "peaks": {"fp32_tflops": fp32_peak, "fp64_tflops": fp64_peak, "hbm_gbs": hbm},
    }
    if cpu is not None:
        out["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(out), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
