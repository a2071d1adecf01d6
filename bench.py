"""Benchmark: DNS steps/s of the channel time step, one JSON line on stdout.

Workload: the Re_tau = 550 channel, 384 x 257 x 384 modes (576 x 257 x 576
dealiased physical points), seeded divergence-free perturbation; FP64 (the
reference's arithmetic) is the headline, the mixed-precision variant (FP32
transforms and products, FP64 solves) is measured beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--precision fp64|mixed] [--workload channel_550|channel_180]

N > 1 is launched by torchrun, one rank per GPU; every rank advances its own
independent channel (the step does not shard across GPUs here: replicas),
timed between barriers, max over ranks.  ``--impl reference`` times the CPU
restatement of the reference algorithm (oracle/owt_port.cpp: dense per-mode
LU, as src/solver.cpp does) on the host cores, rank 0 only.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "open-3d-wallturbulence_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "DNS steps/s at Re_tau=550 384x257x384: FP64 vs mixed (<=1e-6 rel RHS err)"


def metric_for(name, p):
    """The headline metric for the Re_tau=550 channel; the same measure, named by
    its own size, for the Re_tau=180 channel."""
    if name == "channel_550":
        return METRIC
    return f"DNS steps/s at Re_tau=180 {p.NX}x{p.NY}x{p.NZ}: FP64 vs mixed (<=1e-6 rel RHS err)"
DATA = ("synthetic: laminar Poiseuille + seeded divergence-free random perturbation "
        "(Gaussian amplitudes, k^-2 spectrum, RMS 0.1 U_b, zero at walls), seed 0")


def workload(name):
    from owt.params import channel_550, channel_180
    return {"channel_550": channel_550, "channel_180": channel_180}[name]()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


# ---------------------------------------------------------------------------
# clocks sampled while the timed region runs
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        self.rows = []
        if self.p is None:
            return
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
            out, _ = self.p.communicate()
        for line in out.splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 8:
                self.rows.append(parts)

    def summary(self):
        rows = getattr(self, "rows", [])
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for r in rows for q in range(4) if r[4 + q].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------
# algorithmic work per stage (fixed formulas, derived from the kernels' loops)
# ---------------------------------------------------------------------------
def stage_work(p, precision="fp64"):
    """Algorithmic flops and bytes per launch of each kernel: band solves as LAPACK counts
    them, FFTs at 5 N log2 N, 9 flops per physical point for the products, and the
    spectral fields / z-padded planes each kernel must read and write once."""
    import math
    NY, M, NXH, NZ2, NX2 = p.NY, p.NZ * p.NXH, p.NXH, p.NZ2, p.NX2
    S = 16.0 * NY * M  # bytes per spectral field (complex128)
    P = (16.0 if precision == "fp64" else 8.0) * NY * NZ2 * NXH  # one z-padded plane set
    # banded systems: v-system 4NY+4 unknowns (kl 15, ku 13: its band with the unknowns in
    # node order, kept as the fixed count), omega_y-system 2NY (6, 6); per column and
    # complex rhs: 2 * 2 * (2 kl + ku) flops (forward + backward)
    fl_modes = M * ((4 * NY + 4) * 4 * (2 * 15 + 13) + 2 * NY * 4 * (2 * 6 + 6) + 120 * NY)
    fl_fft = lambda n: 5.0 * n * math.log2(n)
    unique = NXH * (p.NZ // 2 + 1)
    factor_bytes = 8.0 * unique * ((4 * NY + 4) * (2 * 15 + 13 + 1) + 2 * NY * (2 * 6 + 6 + 1))
    return {
        "modes": {"flops": fl_modes, "bytes": 22 * S + factor_bytes},
        "zback": {"flops": 6 * NXH * NY * fl_fft(NZ2), "bytes": 6 * S + 6 * P},
        "xlamb": {"flops": 4.5 * NZ2 * NY * fl_fft(NX2) + 9.0 * NX2 * NZ2 * NY, "bytes": 9 * P},
        "zfwd": {"flops": 3 * NXH * NY * fl_fft(NZ2), "bytes": 3 * P + 3 * S},
        "nonlinear": {"flops": M * NY * 60.0, "bytes": 5 * S},
    }


# DRAM traffic per launch from ncu (dram__bytes_read.sum + dram__bytes_write.sum)
# of the 128x129x128 workload (profiles/k_zback_k_xlamb_k_zfwd_fp64_channel180.md
# and profiles/k_modes_split_k_mean_channel180.md), scaled to a launch at
# another size by the units the kernel processes (traffic grows in proportion:
# y-z lines times kx modes for the transforms, modes times NY for the mode
# kernel).
NCU_TRAFFIC_128 = {"xlamb_fp64": 198.33e6, "modes": 1.251e9}


def scaled_traffic(kernel, p, precision):
    base = {"xlamb": "xlamb_fp64" if precision == "fp64" else None, "modes": "modes"}.get(kernel)
    if not base or base not in NCU_TRAFFIC_128:
        return None
    if kernel == "xlamb":
        units, units0 = p.NY * p.NZ2 * p.NXH, 129 * 192 * 64
    else:
        units, units0 = p.NY * p.NZ * p.NXH, 129 * 128 * 64
    return NCU_TRAFFIC_128[base] * units / units0


def measure_fp64_peak():
    """cuBLAS DGEMM throughput (torch.matmul, float64) as the FP64 denominator."""
    import torch
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b
    torch.cuda.empty_cache()
    return best


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
CHUNK = 40  # longest run timed on one state (see timed_steps)


def run_ours(args, rank, world, local_rank):
    import numpy as np
    import torch
    from owt.ic import seeded_velocity
    from owt.solver import GpuSolver

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    p = workload(args.workload)
    u, v, w = seeded_velocity(p, seed=0)

    from owt.replicas import aggregate, barrier

    def timed_steps(solver, k):
        """Device time of exactly k steps.  Runs longer than CHUNK steps are timed
        in chunks, each bracketed by barrier + synchronize and CUDA events, with
        the state returned to the kept one between chunks (outside the timed
        region): from the laminar + 10% noise state the reference scheme itself
        goes unstable after ~60 steps at dt = 0.002 (explicit advection number
        ~0.76 > 0.63, its stability limit), so a long run on one state would
        time a blow-up."""
        st = torch.cuda.ExternalStream(solver.stream)
        solver.keep_state()
        total, done = 0.0, 0
        while done < k:
            n = min(CHUNK, k - done)
            if done:
                solver.restore_state()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            barrier()
            e0.record(st)
            solver.time_Integration(n)
            e1.record(st)
            solver.synchronize()
            barrier()
            ms, _ = aggregate(e0.elapsed_time(e1), n, device="cuda")
            total += ms
            done += n
        return total

    results = {}
    precisions = [args.precision] + [q for q in ("fp64", "mixed") if q != args.precision]
    solver = GpuSolver(p, precision=args.precision, device=local_rank)
    setup_report = solver.setup_report()
    solver.init_fields(u, v, w)
    solver.use_graph(True)
    clocks = None
    for prec in precisions:
        solver.set_precision(prec)
        solver.init_fields(u, v, w)
        solver.time_Integration(args.warmup)
        solver.synchronize()
        l0 = solver.launch_count
        if prec == args.precision:
            with ClockSampler(local_rank) as cs:
                ms = timed_steps(solver, args.steps)
            clocks = cs.summary()
        else:
            ms = timed_steps(solver, args.steps)
        launches = solver.launch_count - l0
        results[prec] = {"ms_per_step": ms / args.steps, "steps_per_s": 1e3 * args.steps / ms,
                         "gpu_launches": launches}
    tuning = solver.tuning_report()  # the variants were timed before the first step

    # one-step RHS error of the mixed variant against FP64 (same state)
    rhs_err = None
    if rank == 0:
        from owt.rhs import implicit_rhs
        got = {}
        for prec in ("fp64", "mixed"):
            solver.set_precision(prec)
            solver.init_fields(u, v, w)
            solver.time_Integration(1)
            got[prec] = {n: solver.get(n) for n in ("lmbx", "lmby", "lmbz", "Hv", "Hg", "vely", "vory")}
            got[prec]["source_v"], got[prec]["source_g"] = implicit_rhs(solver)
        rhs_err = {n: float(np.linalg.norm(got["mixed"][n] - got["fp64"][n]) /
                            max(np.linalg.norm(got["fp64"][n]), 1e-300)) for n in got["fp64"]}
        del got

    # per-stage timing with CUDA events on the library stream (dominant kernel)
    stage_ms, stage_ms_mixed = {}, {}
    if rank == 0:
        solver.use_graph(False)
        st = torch.cuda.ExternalStream(solver.stream)
        reps = max(3, min(10, args.steps))

        def time_stages(prec, stages, out):
            solver.set_precision(prec)
            solver.init_fields(u, v, w)
            for name, sid in stages:
                solver.enqueue_stage(sid)
                solver.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(st)
                for _ in range(reps):
                    solver.enqueue_stage(sid)
                e1.record(st)
                solver.synchronize()
                out[name] = e0.elapsed_time(e1) / reps

        time_stages("mixed", (("zback", 4), ("xlamb", 5), ("zfwd", 6), ("mean_lamb", 7)), stage_ms_mixed)
        time_stages(args.precision, (("modes", 0), ("zback", 4), ("xlamb", 5), ("zfwd", 6), ("nonlinear", 3)),
                    stage_ms)

    # end to end through the C ABI with host buffers: every step uploads the
    # full step input (12 history fields, 12 mean vectors, 6 friction values)
    # from pinned memory and reads back the new v, omega_y and friction, in
    # one owt_time_integration_host call (copies overlapped with the device
    # work inside the call; the call returns with the outputs written).
    e2e = None
    if True:
        solver.set_precision(args.precision)
        solver.init_fields(u, v, w)
        solver.time_Integration(1)
        hist = list(GpuSolver.HISTORY)
        means = ["lmbx_mean_0", "lmbx_mean_1", "lmbx_mean_2", "lmbz_mean_0", "lmbz_mean_1", "lmbz_mean_2",
                 "velx_mean_0", "velx_mean_1", "velx_mean_2", "velz_mean_0", "velz_mean_1", "velz_mean_2"]

        def pinned(shape):
            return torch.empty(tuple(shape) + (2,), dtype=torch.float64, pin_memory=True).numpy().view(
                np.complex128).reshape(shape)

        host_in = [pinned(p.spectral_shape) for _ in hist]
        for n, arr in zip(hist, host_in):
            solver.get(n, out=arr)
        host_mean = pinned((12, p.NY))
        host_mean[:] = np.stack([solver.get_cvec(n) for n in means])
        fric = solver.friction()
        out_v, out_g = pinned(p.spectral_shape), pinned(p.spectral_shape)
        k_e2e = max(3, min(args.steps, 10))
        solver.time_Integration_host(host_in, host_mean, fric, out_v, out_g)  # warm-up (first-call setup)
        bi = sum(x.nbytes for x in host_in) + host_mean.nbytes + 48
        bo = out_v.nbytes + out_g.nbytes + 48
        barrier()
        t0 = time.perf_counter()
        for _ in range(k_e2e):
            solver.time_Integration_host(host_in, host_mean, fric, out_v, out_g)
        barrier()
        dt_ms, e2e_rate = aggregate((time.perf_counter() - t0) * 1e3, k_e2e, device="cuda")
        e2e = {"value": e2e_rate, "unit": "steps/s", "h2d_bytes_per_step": int(bi),
               "d2h_bytes_per_step": int(bo), "steps": k_e2e,
               "call": "owt_time_integration_host: host state in (pinned), one step, new v, omega_y and "
                       "friction out; wall clock around the calls"}
    solver.close()

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return None

    peaks, peak_kind = load_peaks()
    fp64_peak = measure_fp64_peak()
    work = stage_work(p, args.precision)
    dom = max(stage_ms, key=lambda n: stage_ms[n])
    t_dom = stage_ms[dom] * 1e-3
    fl_dom = work[dom]["flops"]
    if args.precision == "mixed" and dom in ("zback", "xlamb", "zfwd"):
        roof = {"bound": "hbm", "achieved": work[dom]["bytes"] / t_dom / 1e9, "peak": peaks["hbm_gbs"],
                "unit": "GB/s"}
    else:
        roof = {"bound": "fp64", "achieved": fl_dom / t_dom / 1e12, "peak": fp64_peak, "unit": "TFLOP/s"}
    roof["frac"] = roof["achieved"] / roof["peak"]
    roof["kernel"] = {"modes": "k_modes", "zback": "k_zback", "xlamb": "k_xlamb", "zfwd": "k_zfwd",
                      "nonlinear": "k_nl"}[dom]
    roof["traffic"] = scaled_traffic(dom, p, args.precision)
    roof["algorithmic_bytes"] = work[dom]["bytes"]
    roof["traffic_source"] = "ncu at 128x129x128, scaled by units processed (profiles/)"
    roof["peak_source"] = ("cuBLAS DGEMM (torch.matmul float64, 4096^3) measured in this run"
                           if roof["bound"] == "fp64" else f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})")
    if roof["bound"] == "fp64":
        # second denominator: the FP64 issue rate, two DFMA (4 flops) per clock per
        # SM (ncu's sm__sass_thread_inst_executed_op_dfma_pred_on peak) at the SM
        # clock sampled during the timed steps; `frac` stays against the DGEMM
        mhz = (clocks or {}).get("sm_mhz") or 2070.0
        sms = torch.cuda.get_device_properties(local_rank).multi_processor_count
        issue_peak = 4.0 * sms * mhz * 1e6 / 1e12
        roof["peak_fp64_issue"] = {"value": round(issue_peak, 4), "unit": "TFLOP/s",
                                   "frac": round(roof["achieved"] / issue_peak, 4),
                                   "source": "2 DFMA per clock per SM x %d SMs x %.0f MHz" % (sms, mhz)}
    roof["stage_ms"] = {k: round(v, 4) for k, v in stage_ms.items()}
    roof["stage_hbm_gbs"] = {k: round(work[k]["bytes"] / (stage_ms[k] * 1e-3) / 1e9, 1) for k in stage_ms}
    roof["stage_fp64_tflops"] = {k: round(work[k]["flops"] / (stage_ms[k] * 1e-3) / 1e12, 3) for k in stage_ms}

    head = results[args.precision]
    value = world * head["steps_per_s"]
    line = {
        "metric": metric_for(args.workload, p),
        "value": round(value, 4),
        "unit": "steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(head["ms_per_step"], 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": DATA,
        "config": {
            "workload": f"{args.workload}_{p.NX}x{p.NY}x{p.NZ}",
            "modes": [p.NX, p.NY, p.NZ], "physical": [p.NX2, p.NY, p.NZ2],
            "dt": p.dt, "nu": p.nu, "precision": args.precision, "cuda_graph": True,
            "parallelism": "replicas" if world > 1 else "single",
            "l2": "inputs larger than L2 (the step streams ~40 GB of state and factors)",
            "timing": "CUDA events per chunk of <= %d steps, state restored from a device copy between "
                      "chunks outside the timed region" % CHUNK,
            "grid_point_updates_per_s": round(value * p.NX2 * p.NZ2 * p.NY, 1),
            "mode_kernel_autotune": tuning,
            "setup": setup_report,
        },
        "variants": {q: {"steps_per_s": round(world * r["steps_per_s"], 4), "ms_per_step": round(r["ms_per_step"], 4)}
                     for q, r in results.items()},
        "roofline": roof,
        "gpu_launches": head["gpu_launches"],
        "clocks": clocks,
        "e2e": e2e,
    }
    if "fp64" in results and "mixed" in results:
        line["variants"]["mixed"]["speedup_vs_fp64"] = round(results["fp64"]["ms_per_step"] /
                                                             results["mixed"]["ms_per_step"], 3)
        line["variants"]["mixed"]["rhs_rel_l2_err_vs_fp64"] = {k: float("%.3e" % x) for k, x in rhs_err.items()}
        if stage_ms_mixed:
            line["variants"]["mixed"]["transform_stage_ms"] = {k: round(x, 4) for k, x in stage_ms_mixed.items()}
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(p, args, quick=True)
    if dist is not None:
        dist.destroy_process_group()
    return line


# ---------------------------------------------------------------------------
# CPU arm: the reference algorithm (oracle restatement) on the host cores
# ---------------------------------------------------------------------------
# ---------------------------------------------------------------------------
# batch workload: 64 uneven minimal channels, one graph launch per step
# ---------------------------------------------------------------------------
def run_batch(args, rank, world, local_rank):
    import torch
    from owt.batch import Batch, minimal_channels
    from owt.replicas import aggregate, barrier
    from owt.solver import GpuSolver
    torch.cuda.set_device(local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    ps = minimal_channels(64, seed=0)
    solvers = []
    t_setup = time.perf_counter()
    for q, p in enumerate(ps):
        s = GpuSolver(p, precision="mixed", device=local_rank)
        s.init_seeded(q, 0.1)  # generated on the device
        s.use_graph(True)
        solvers.append(s)
    t_setup = time.perf_counter() - t_setup
    points = sum(p.NX2 * p.NZ2 * p.NY for p in ps)
    # serial loop: one channel after another, each its own graph
    for s in solvers:
        s.time_Integration(args.warmup)
        s.synchronize()
    k_loop = max(2, args.steps // 4)
    barrier()
    t0 = time.perf_counter()
    for _ in range(k_loop):
        for s in solvers:
            s.time_Integration(1)
            s.synchronize()
    barrier()
    loop_ms, loop_rate = aggregate((time.perf_counter() - t0) * 1e3, 64 * k_loop, device="cuda")
    # batched: one graph launch per step, each kernel over all channels
    t_batch = time.perf_counter()
    b = Batch(solvers)
    t_batch = time.perf_counter() - t_batch
    b.step(args.warmup)
    b.synchronize()
    st = torch.cuda.ExternalStream(b.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = b.launch_count
    with ClockSampler(local_rank) as cs:
        barrier()
        e0.record(st)
        b.step(args.steps)
        e1.record(st)
        b.synchronize()
        barrier()
    ms, rate = aggregate(e0.elapsed_time(e1), 64 * args.steps, device="cuda")
    launches = b.launch_count - l0
    step_launches = b.step_launches
    tuning = b.tuning_report()
    b.close()
    for s in solvers:
        s.close()
    if rank != 0:
        return None
    return {
        "metric": "channel-steps/s, 64 uneven minimal channels (Re_tau 150-250), one graph launch per step",
        "value": round(rate, 3), "unit": "channel-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic: 64 seeded minimal channels, laminar + seeded divergence-free perturbation "
                "each, generated on the device (owt_init_seeded, seed = channel index, RMS 0.1)",
        "config": {"workload": "batch64_minimal_channels", "precision": "mixed", "channels": 64,
                   "physical_points_total": points, "kernels_per_batch_step": step_launches,
                   "mode_kernel_autotune": tuning,
                   "setup_s": {"channels_create_and_init": round(t_setup, 3), "batch_create": round(t_batch, 3)},
                   "l2": "no flush; per-step state of all channels ~%.1f GB" % (
                       sum(22 * 16 * p.NY * p.NZ * p.NXH for p in ps) / 1e9)},
        "variants": {"serial_loop": {"channel_steps_per_s": round(loop_rate, 3),
                                     "ms_per_step_all_channels": round(loop_ms / k_loop, 4)},
                     "speedup_vs_serial_loop": round(rate / loop_rate, 3)},
        "gpu_launches": launches,
        "clocks": cs.summary(),
    }


def build_port():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)


def cpu_sample(p, mode_stride, fields):
    """Seconds of one full step estimated from a bounded sample: the mode
    loop over every mode_stride-th mode (the dense per-mode LU solves) and
    `fields` inverse (+ fields/2 forward) transforms, scaled up to all modes
    and 9 transforms.  A cross-check of the measured full steps only."""
    from oracle import PortOracle
    o = PortOracle()
    o.init(p.dt, p.dkx, p.dkz, p.NX, p.NY, p.NZ, p.alpha_mesh, p.nu)
    M = p.NZ * p.NXH
    n_sampled = len(range(0, M, mode_stride))
    t_modes = o.lib.port_time_modes(mode_stride, 1) * (M / n_sampled)
    t_xf = o.lib.port_time_transforms(fields) * (9.0 / (fields + fields // 2))
    return o, t_modes + t_xf


def cpu_full_steps(p, nsteps, budget_s=None):
    """Wall time of each of nsteps complete CPU steps of the oracle restatement
    (every mode's dense LU solves, solve_horizontal, the 9 dealiased
    transforms, nonlinear_source, history rotation), all host threads, from
    the same seeded state as the GPU arm after its init_fields (not timed).
    With budget_s, no further step starts once the timed steps took that
    long (at least one step is timed)."""
    from oracle import PortOracle
    from owt.ic import seeded_velocity
    build_port()
    o = PortOracle()
    threads = o.set_threads(0)
    o.init(p.dt, p.dkx, p.dkz, p.NX, p.NY, p.NZ, p.alpha_mesh, p.nu)
    o.set_velocity(*seeded_velocity(p, seed=0))
    ts = []
    for _ in range(nsteps):
        t0 = time.perf_counter()
        o.step(1)
        ts.append(time.perf_counter() - t0)
        if budget_s is not None and sum(ts) >= budget_s:
            break
    del o
    return ts, threads


def cpu_baseline(p, args, quick=False):
    """One measured full CPU step (about 25 s at 384x257x384 on 16 cores), with
    the sampled estimate beside it as a cross-check."""
    build_port()
    ts, threads = cpu_full_steps(p, 1)
    stride = max(1, (p.NZ * p.NXH) // 256)
    _, t_est = cpu_sample(p, stride, 2)
    return {"value": round(1.0 / ts[0], 6), "unit": "steps/s", "cores": threads, "kind": "port",
            "sample": f"one complete FP64 step of the oracle restatement at {p.NX}x{p.NY}x{p.NZ} "
                      f"({ts[0]:.1f} s, {threads} OpenMP threads): dense per-mode LU over all "
                      f"{p.NZ * p.NXH} modes, 9 transforms, nonlinear source",
            "sampled_estimate_s_per_step": round(t_est, 2),
            "sampled_estimate": f"cross-check only: every {stride}th mode + 3 transforms, scaled up"}


def run_adjoint(args, rank, world, local_rank):
    """Wall-drag gradient at the Re_tau=180 size (128x129x128, dt = 0.005): one
    evaluation = owt_drag_forward over a 200-step horizon (device images every
    20 steps) + owt_drag_backward (recompute of each segment + the adjoint
    steps), timed with CUDA events on the library stream.  Each evaluation is
    600 steps' work, so the run does one warm-up evaluation and at most 5."""
    import numpy as np
    import torch
    from owt.adjoint import seeded_wall_field
    from owt.ic import seeded_velocity
    from owt.params import channel_180
    from owt.replicas import aggregate, barrier
    from owt.solver import GpuSolver
    torch.cuda.set_device(local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    p = channel_180()
    horizon, interval = 200, 20
    s = GpuSolver(p, device=local_rank)
    s.use_graph(True)
    s.init_fields(*seeded_velocity(p, seed=0))
    s.keep_state()
    s.set_wall_velocity(seeded_wall_field(p, 1), seeded_wall_field(p, 2))
    st = torch.cuda.ExternalStream(s.stream)
    k = max(1, min(args.steps, 5))

    def evaluate():
        s.restore_state()
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(st)
        J = s.drag_forward(horizon, interval)
        e1.record(st)
        g = s.drag_backward()
        e2.record(st)
        s.synchronize()
        return J, g, e0.elapsed_time(e1), e1.elapsed_time(e2)

    evaluate()
    l0 = s.launch_count
    barrier()
    fwd = bwd = 0.0
    for _ in range(k):
        J, g, f, b = evaluate()
        fwd += f
        bwd += b
    barrier()
    launches = s.launch_count - l0
    ms, rate = aggregate(fwd + bwd, k, device="cuda")
    dev_bytes = s.info("device_bytes")
    s.close()
    if rank != 0:
        return None
    return {
        "metric": "wall-drag gradient evaluations/s, Re_tau=180 128x129x128, 200-step horizon",
        "value": round(rate, 4), "unit": "gradients/s", "n_gpus": world, "steps": k, "warmup": 1,
        "ms_per_step": round(ms / k, 2), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic: seeded state (seed 0), seeded wall blowing/suction RMS 1e-3 (seeds 1, 2)",
        "config": {"workload": "adjoint_channel_180_128x129x128", "horizon_steps": horizon,
                   "checkpoint_interval": interval, "forward_ms": round(fwd / k, 2),
                   "backward_ms": round(bwd / k, 2),
                   "backward_ms_per_step": round(bwd / k / horizon, 3),
                   "forward_ms_per_step": round(fwd / k / horizon, 3),
                   "objective": J, "grad_norm": float(np.sqrt(np.vdot(g[0], g[0]).real + np.vdot(g[1], g[1]).real)),
                   "handle_device_bytes_before_adjoint": dev_bytes,
                   "warmup_note": "one warm-up evaluation: each is 600 steps of work"},
        "gpu_launches": launches,
    }


def run_reference(args, rank, world):
    """The reference algorithm on the host cores: up to K timed steps (no
    further step once 120 s were timed), each a complete FP64 step of the
    oracle restatement (as src/solver.cpp:541-627 with its dense per-mode
    LU), wall-clocked one by one; at 384x257x384 a step takes about 22 s on
    16 cores.  The W warm-up steps (threads, page faults, caches) are bounded
    samples of a step: the mode loop over every 1024th mode and one
    transform."""
    if rank != 0:
        return None
    if args.workload not in ("channel_550", "channel_180"):
        return {"impl": "reference", "unavailable": f"the reference has no {args.workload} workload: it runs one "
                                                    "channel per job and has no adjoint"}
    p = workload(args.workload)
    build_port()
    for _ in range(args.warmup):
        cpu_sample(p, max(1, (p.NZ * p.NXH) // 72), 1)
    # complete steps until about two minutes of CPU work (so the run ends in a
    # few minutes: a step at 384x257x384 takes ~22 s on 16 cores)
    timed, threads = cpu_full_steps(p, args.steps, budget_s=120.0)
    total = sum(timed)
    nsteps = len(timed)
    value = nsteps / total
    return {
        "impl": "reference", "metric": metric_for(args.workload, p), "value": round(value, 6), "unit": "steps/s",
        "n_gpus": world, "steps": nsteps, "steps_requested": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total / nsteps * 1e3, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA,
        "config": {"workload": f"{args.workload}_{p.NX}x{p.NY}x{p.NZ}",
                   "modes": [p.NX, p.NY, p.NZ], "physical": [p.NX2, p.NY, p.NZ2],
                   "dt": p.dt, "nu": p.nu, "precision": "fp64", "cuda_graph": False,
                   "parallelism": f"OpenMP, {threads} host threads",
                   "timing": "wall clock per complete step, after an untimed init_fields",
                   "grid_point_updates_per_s": round(value * p.NX2 * p.NZ2 * p.NY, 1),
                   "implementation": "CPU restatement of the reference algorithm (oracle/owt_port.cpp: dense "
                                     "per-mode LU as src/solver.cpp:561-605, dense DY mat-vecs, dealiased FFT "
                                     "transforms), pinned bit for bit to the reference built from its sources"},
        "step_s": [round(t, 2) for t in timed],
        "cpu_baseline": {"value": round(value, 6), "unit": "steps/s", "cores": threads, "kind": "port",
                         "sample": f"{nsteps} complete FP64 steps at {p.NX}x{p.NY}x{p.NZ}, each timed (steps "
                                   f"stop after 120 s of timed work; warm-up: {args.warmup} bounded samples "
                                   f"of a step)"},
        "e2e": {"value": round(value, 6), "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--workload", choices=["channel_550", "channel_180", "batch64", "adjoint"], default="channel_550")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local_rank = dist_env()
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    elif args.workload == "batch64":
        line = run_batch(args, rank, world, local_rank)
    elif args.workload == "adjoint":
        line = run_adjoint(args, rank, world, local_rank)
    else:
        line = run_ours(args, rank, world, local_rank)
    if line is not None and rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
