"""A small case for kernel profilers.

Sets up one channel with the seeded initial condition, advances it two steps
(the mode kernel's autotuner runs before the first one), then enqueues the
chosen stages of the step once each inside an NVTX range named "prof", so
that a profiler restricted to that range sees exactly those launches:

    ncu --set full --nvtx --nvtx-include "prof/" -k regex:k_modes -c 1 \\
        python open-3d-wallturbulence_gb300/owt/profile_case.py --workload channel_550 --ny 33 --stages modes

Stages: modes, mean, lamb, nonlinear, zback, xlamb, zfwd, mean_lamb (the
stage numbers of owt_enqueue_stage).  Sizes default to the workload's; --nx,
--ny, --nz override them (a smaller NY keeps the device memory of a capture
to a few GB).  --adjoint N,INTERVAL profiles one wall-drag gradient instead
(owt_drag_forward over N steps with device images every INTERVAL steps, then
owt_drag_backward, with seeded wall blowing/suction), after one unprofiled
evaluation.
"""
import argparse
import dataclasses
import os
import sys

STAGES = {"modes": 0, "mean": 1, "lamb": 2, "nonlinear": 3, "zback": 4, "xlamb": 5, "zfwd": 6, "mean_lamb": 7}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--workload", choices=["channel_550", "channel_180"], default="channel_550")
    ap.add_argument("--nx", type=int)
    ap.add_argument("--ny", type=int)
    ap.add_argument("--nz", type=int)
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--stages", default="modes")
    ap.add_argument("--adjoint", help="N,INTERVAL: one wall-drag gradient evaluation")
    args = ap.parse_args(argv)
    import torch
    from owt import params
    from owt.solver import GpuSolver
    p = getattr(params, args.workload)()
    over = {k: v for k, v in (("NX", args.nx), ("NY", args.ny), ("NZ", args.nz)) if v}
    if over:
        p = dataclasses.replace(p, **over)
    stages = [STAGES[s] for s in args.stages.split(",") if s]
    s = GpuSolver(p, precision=args.precision)
    s.init_seeded(0, 0.1)
    if args.adjoint:
        from owt.adjoint import seeded_wall_field
        n, interval = (int(x) for x in args.adjoint.split(","))
        s.use_graph(True)
        s.keep_state()
        s.set_wall_velocity(seeded_wall_field(p, 1), seeded_wall_field(p, 2))
        for rep in range(2):
            s.restore_state()
            s.synchronize()
            if rep:
                torch.cuda.nvtx.range_push("prof")
            s.drag_forward(n, interval)
            s.drag_backward()
            s.synchronize()
        torch.cuda.nvtx.range_pop()
        print("profile case %dx%dx%d adjoint %s; device memory %.2f GB"
              % (p.NX, p.NY, p.NZ, args.adjoint, s.info("device_bytes") / 1e9))
        s.close()
        return
    s.time_Integration(2)
    s.synchronize()
    torch.cuda.nvtx.range_push("prof")
    for st in stages:
        s.enqueue_stage(st)
    s.synchronize()
    torch.cuda.nvtx.range_pop()
    print("profile case %dx%dx%d %s stages %s; device memory %.2f GB; mode kernel: %s"
          % (p.NX, p.NY, p.NZ, args.precision, args.stages, s.info("device_bytes") / 1e9, s.tuning_report()))
    s.close()


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    main()
