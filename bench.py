"""Benchmark of the GB300 DG residual-and-update path.

Workload (one step = one SSP-RK3 step of Solver::stepSolver, src/Solver/TimeIntegration.cpp:326-350,
including the per-step relative-error reduction): 3D compressible Euler Taylor-Green vortex, Mach 0.1,
gamma 1.4, periodic [0, 2 pi]^3, 64^3 hexahedra, P3 (64 nodes/element, 83,886,080 DOF), HLLC flux,
dt from CFL 0.2 -- seeded synthetic initial state of that shape (no dataset involved).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  value = DOF-stage updates/s with the state resident in HBM (CUDA events on the
library's stream, the step replayed as a CUDA graph); e2e = the same metric through the C ABI with host
buffers (pinned), every step taking its input state from the host and returning its new state to the host:
streamed through sdg_step_state_point_from_async (each step's input transfer overlapping the previous step),
and, under e2e.synchronous, through sdg_set_state_point + sdg_step_state_point.  The line also carries the other
workloads of the metric, each measured the same way on this GPU:
  batched      256 independent 2D Euler / Navier-Stokes Kelvin-Helmholtz solves (500..50,000 elements,
               P1..P5, quads or hybrid, Mach 0.1..0.8, Re 1e2..1e4): one batched graph step of all
               instances against the same instances stepped one after another with plain launches
  batched_small the same generator with element counts log-uniform in [500, 2,000] (the regime where one
               instance cannot fill the GPU)
  ns_hybrid    2D Navier-Stokes BR2 Kelvin-Helmholtz, Re 1e4, 256^2 jittered quads with a 50% triangle
               split, P4, Lax-Friedrichs
  vortex2d     2D Euler isentropic vortex, 40^2 quads, P3, Roe, dt 1e-3 (L2-resident, launch bound)
  tet          3D Euler Taylor-Green vortex (Mach 0.3) on periodic tetrahedra, 32^3 cubes x 6, P3, HLLC
  curved       3D Navier-Stokes BR2 (HLLC, Re 200, Mach 0.2) along a no-slip wall on 32^3 curved hexahedra of
               geometry order 3, P3: the shape of the sphere driver
  adjoint      3D Navier-Stokes BR1 Taylor-Green, Re 1600, Mach 0.1, 32^3 hexahedra, P3, Roe, 500 SSP-RK3 steps:
               forward, checkpointed adjoint (every 25 steps) of the integrated kinetic energy, reverse sweep
               of a recorded trajectory, and central-difference checks of dJ/dU0 (seeded direction) and dJ/dmu
--impl reference times the CPU restatement of the reference path (the oracle, reference-faithful
arithmetic) on the host cores.  Under torchrun (N > 1) each rank runs an independent replica on its own
GPU (the path is not sharded: replicas only).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "DOF-stage updates/s (FP64, 1 GB300)"
WORKLOAD = "tgv3d-euler-64^3-hex-P3-HLLC-SSPRK3-CFL0.2"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--elements", type=int, default=64, help="hexahedra per direction")
    ap.add_argument("--order", type=int, default=3)
    ap.add_argument("--cpu-sample", type=int, default=64, help="hexahedra per direction of the CPU baseline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="headline workload only")
    ap.add_argument("--extra", default="batched,batched_small,ns_hybrid,vortex2d,tet,curved,adjoint",
                    help="comma list of the other workloads to measure")
    ap.add_argument("--batch-count", type=int, default=256)
    ap.add_argument("--batch-max-elements", type=int, default=50000)
    ap.add_argument("--ns-elements", type=int, default=256, help="quads per direction of the NS hybrid mesh")
    ap.add_argument("--tet-elements", type=int, default=32, help="cubes per side of the tetrahedral section")
    ap.add_argument("--curved-elements", type=int, default=32, help="curved hexahedra per side of the curved section")
    ap.add_argument("--adjoint-elements", type=int, default=32)
    ap.add_argument("--adjoint-steps", type=int, default=500)
    ap.add_argument("--no-adjoint-check", action="store_true", help="skip the finite-difference checks")
    return ap.parse_args()


def dist_env():
    from subrosadg_gb300 import replicas
    return replicas.env()


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_figures():
    """Per-launch DRAM traffic and FP64 instruction counts of the element kernel from the committed ncu
    summary (profiles/), scaled to the full workload there; None when absent."""
    path = os.path.join(ROOT, "profiles", "tensor_stage_kernel_tgv_hex_p3.md")
    out = {}
    try:
        for line in open(path):
            if line.startswith("bench-figure "):
                _, key, val = line.split()[:3]
                out[key] = float(val)
    except OSError:
        pass
    return out


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 50 ms during the timed region."""

    FIELDS = "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
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
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for name, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def tgv_problem(n, p):
    import subrosadg_gb300 as sdg
    from subrosadg_gb300 import workloads as wl
    mesh = sdg.Mesh.box_3d(0, 0, 0, 2 * math.pi, 2 * math.pi, 2 * math.pi, n, n, n, periodic=True)
    cfg = wl.config(p, sdg.HLLC)
    return mesh, cfg, lambda pts: wl.tgv_primitive(pts[:, 0], pts[:, 1], pts[:, 2])


VARIANTS = {"faithful": "the reference's arithmetic: the gradient pass also for Euler (TimeIntegration.cpp:340-343) "
                        "and a dense M^-1 per element (Geometry.cpp:88-100)",
            "lean": "without the unused Euler gradient pass, one shared reference M^-1 scaled by 1/|J| on the "
                    "affine hexahedra"}


def cpu_baseline(n, p, stages, warmup, variant="faithful"):
    """Time the oracle -- the CPU restatement of the reference path -- on all host cores, on the TGV workload
    with n^3 hexahedra: `warmup` untimed RK stages, then `stages` timed ones (SSP-RK3 stages in order, one
    stage = one update of every DOF).  The mesh comes from the oracle's own generator: nothing of the GPU
    library is loaded."""
    from oracle import meshgen, orc
    from subrosadg_gb300 import _abi
    from subrosadg_gb300 import workloads as wl
    mesh = meshgen.box_3d(0, 0, 0, 2 * math.pi, 2 * math.pi, 2 * math.pi, n, n, n, periodic=True)
    cfg = wl.config(p, _abi.HLLC)
    threads = os.cpu_count() or 1
    orc.set_threads(threads)
    t0 = time.perf_counter()
    o = orc.Oracle(mesh, cfg, faithful=True, lean=variant == "lean", precision="double")
    o.initialize_primitive(wl.tgv_primitive(*o.volume_points().T))
    dt = o.delta_time(0.2)
    setup = time.perf_counter() - t0
    for s in range(warmup):
        o.stage(s % 3, dt)
    t0 = time.perf_counter()
    for s in range(warmup, warmup + stages):
        o.stage(s % 3, dt)
    t = time.perf_counter() - t0
    dof = o.dof
    return {"value": dof * stages / t, "unit": "DOF-stage/s", "cores": threads, "kind": "port",
            "sample": f"TGV {n}^3 hexahedra P{p} HLLC ({dof} DOF{', the full workload' if n == 64 else ''}), "
                      f"{stages} SSP-RK3 stages "
                      f"after {warmup} warm-up stages; oracle ({variant}: {VARIANTS[variant]}), OpenMP {threads} "
                      f"threads", "seconds": t, "setup_s": setup, "variant": variant}


def run_reference(args):
    """The reference arm: the oracle (CPU restatement of the reference path; the reference itself does not
    build here) on the host cores.  One step of this arm is one SSP-RK3 stage of the full 64^3 workload (a
    bounded sample: a whole step takes three), so the line's value is DOF-stage/s of that workload."""
    world, rank, local = dist_env()
    if rank != 0:
        return
    r = cpu_baseline(args.elements, args.order, args.steps, args.warmup, "faithful")
    lean = cpu_baseline(args.elements, args.order, max(1, min(args.steps, 3)), 1, "lean")
    line = {"impl": "reference", "metric": METRIC, "value": r["value"], "unit": "DOF-stage/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * r["seconds"] / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "elements": args.elements ** 3,
                       "step": "one SSP-RK3 stage of the full workload (a step of the GPU arm is three)",
                       "sample": r["sample"]},
            "cpu_baseline": {k: r[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "lean": {k: lean[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "setup_s": r["setup_s"],
            "e2e": {"value": r["value"], "unit": "DOF-stage/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _timed(torch, stream, fn, steps):
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        fn()
    ev1.record(stream)
    ev1.synchronize()
    return ev0.elapsed_time(ev1)


def bench_batched(args, device, torch, max_elements=None):
    """Batched workload: all instances in one batched graph step versus one instance after another."""
    import subrosadg_gb300 as sdg
    from subrosadg_gb300 import workloads as wl
    t0 = time.perf_counter()
    inst, params = wl.batch_instances(args.batch_count, max_elements=max_elements or args.batch_max_elements)
    solvers = []
    for mesh, cfg, prim in inst:
        g = sdg.GpuSolver(mesh, cfg, device=device)
        g.initialize_primitive(prim(g.volume_points()))
        solvers.append(g)
    dts = [g.calculateDeltaTime(0.2) for g in solvers]
    b = sdg.Batch(solvers)
    b.set_delta_time(dts)
    setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    b.autotune()
    tune = time.perf_counter() - t0
    c = b.counts()
    stream = torch.cuda.ExternalStream(b.stream(), device=device)
    steps = max(3, args.steps)
    b.step(args.warmup)
    with ClockSampler(device) as clocks:
        ms_batch = _timed(torch, stream, lambda: b.step_async(1), steps)
    b.synchronize()
    b.step_sequential_async(1)
    b.synchronize()
    ms_seq = _timed(torch, stream, lambda: b.step_sequential_async(1), steps)
    b.synchronize()
    # how busy the GPU is in the sequential run: every launch bracketed by CUDA events (one step), summed over
    # the instances, against the sequential step's wall time.  If batching only removed the idle gaps between
    # kernels, ms_seq / busy would bound its gain.
    import ctypes
    kms, kn = (ctypes.c_double * 5)(), (ctypes.c_int64 * 5)()
    for g in solvers:
        g.lib.sdg_set_kernel_timing(g.h, 1)
    b.step_sequential_async(1)
    b.synchronize()
    busy, launches_seq = 0.0, 0
    for g in solvers:
        g.lib.sdg_kernel_time(g.h, kms, kn)
        busy += sum(kms)
        launches_seq += sum(kn)
        g.lib.sdg_set_kernel_timing(g.h, 0)
    dof_stages = sum(g.counts.degree_of_freedom_count * 3 for g in solvers)
    out = {
        "workload": f"{len(solvers)} independent 2D Kelvin-Helmholtz solves (Euler or NS BR2, LF, SSP-RK3)",
        "instances": len(solvers), "elements": c["element_count"], "dof": c["degree_of_freedom_count"],
        "navier_stokes_instances": sum(p["navier_stokes"] for p in params),
        "orders": sorted({p["order"] for p in params}),
        "value": dof_stages * steps / (ms_batch * 1e-3), "unit": "DOF-stage/s",
        "ms_per_step": ms_batch / steps, "launches_per_step": c["launches_per_step"],
        "persistent_ctas_per_sm": c["persistent_ctas_per_sm"],
        "sequential": {"value": dof_stages * steps / (ms_seq * 1e-3), "ms_per_step": ms_seq / steps,
                       "launches_per_step": c["sequential_launches_per_step"],
                       "mode": "plain per-instance launches, instance after instance, same stream and tiles",
                       "kernel_busy_ms_per_step": busy, "busy_fraction": busy / (ms_seq / steps),
                       "gap_free_bound_speedup": (ms_seq / steps) / busy, "timed_launches": launches_seq},
        "speedup_vs_sequential": ms_seq / ms_batch,
        "setup_s": setup, "autotune_s": tune, "clocks": clocks.summary(),
    }
    b.close()
    for g in solvers:
        g.close()
    return out


def kernel_split(g, dt, steps):
    """Device time per step of each kernel class (every launch bracketed by CUDA events on the solver's stream,
    a separate pass after the timed one): element, interior face, boundary face, reduction, gradient."""
    import ctypes
    g.lib.sdg_set_kernel_timing(g.h, 1)
    for _ in range(steps):
        g.step_async(dt)
    kms = (ctypes.c_double * 5)()
    kn = (ctypes.c_int64 * 5)()
    g.lib.sdg_kernel_time(g.h, kms, kn)
    g.lib.sdg_set_kernel_timing(g.h, 0)
    g.synchronize()
    names = ("element", "interior_face", "boundary_face", "reduction", "gradient")
    return {k: kms[i] / steps for i, k in enumerate(names)}


def bench_ns_hybrid(args, device, torch):
    """2D Navier-Stokes BR2 Kelvin-Helmholtz, Re 1e4, Pr 0.71, hybrid 256^2 mesh, P4, LF."""
    import subrosadg_gb300 as sdg
    from subrosadg_gb300 import workloads as wl
    n = args.ns_elements
    mesh = sdg.Mesh.box_2d(0.0, 0.0, 1.0, 1.0, n, n, periodic=True, jitter=0.1, split_fraction=0.5, seed=11)
    cfg = wl.ns_config(4, sdg.LAX_FRIEDRICHS, sdg.BR2, 1e-4)
    g = sdg.GpuSolver(mesh, cfg, device=device)
    g.initialize_primitive(wl.kh_primitive(*g.volume_points()[:, :2].T))
    dt = g.calculateDeltaTime(0.2)
    g.autotune()
    import ctypes
    sp = ctypes.c_void_p()
    g.lib.sdg_get_stream(g.h, ctypes.byref(sp))
    stream = torch.cuda.ExternalStream(sp.value, device=device)
    for _ in range(args.warmup):
        g.step_async(dt)
    g.synchronize()
    steps = max(3, args.steps)
    ms = _timed(torch, stream, lambda: g.step_async(dt), steps)
    g.synchronize()
    dof = g.counts.degree_of_freedom_count
    out = {"workload": f"ns-kh2d-BR2-Re1e4-{n}^2-hybrid-P4-LF", "elements": g.counts.element_count, "dof": dof,
           "value": dof * 3 * steps / (ms * 1e-3), "unit": "DOF-stage/s", "ms_per_step": ms / steps,
           "tiles": [g.tile(k) for k in range(g.counts.block_count)],
           "kernel_ms_per_step": kernel_split(g, dt, 3)}
    g.close()
    return out


def bench_tet(args, device, torch):
    """3D Euler Taylor-Green vortex (Mach 0.3) on periodic tetrahedra: 32^3 cubes x 6, P3 (20 modes), HLLC."""
    import ctypes

    import subrosadg_gb300 as sdg
    from subrosadg_gb300 import workloads as wl
    n = args.tet_elements
    mesh, cfg, prim, _, _, _ = wl.tet_tgv_case(n=n, p=3, flux=sdg.HLLC)
    g = sdg.GpuSolver(mesh, cfg, device=device)
    g.initialize_primitive(prim(g.volume_points()))
    dt = g.calculateDeltaTime(0.2)
    g.autotune()
    sp = ctypes.c_void_p()
    g.lib.sdg_get_stream(g.h, ctypes.byref(sp))
    stream = torch.cuda.ExternalStream(sp.value, device=device)
    for _ in range(args.warmup):
        g.step_async(dt)
    g.synchronize()
    steps = max(3, args.steps)
    ms = _timed(torch, stream, lambda: g.step_async(dt), steps)
    g.synchronize()
    dof = g.counts.degree_of_freedom_count
    out = {"workload": f"tgv3d-euler-Ma0.3-{n}^3x6-tet-P3-HLLC", "elements": g.counts.element_count, "dof": dof,
           "value": dof * 3 * steps / (ms * 1e-3), "unit": "DOF-stage/s", "ms_per_step": ms / steps,
           "l2": f"state {8 * dof / 1e6:.0f} MB per buffer (L2 129 MB)", "tiles": [g.tile(0)],
           "kernel_ms_per_step": kernel_split(g, dt, 3)}
    g.close()
    return out


def bench_curved(args, device, torch):
    """Navier-Stokes BR2 with HLLC along a curved no-slip wall on curved hexahedra (geometry order 3), P3, Re 200,
    Mach 0.2: the shape of examples/sphere_3d_cns.cpp, n^3 elements of a warped box."""
    import ctypes

    import subrosadg_gb300 as sdg
    from subrosadg_gb300 import workloads as wl
    n = args.curved_elements
    mesh, cfg, prim, bprim, _, _ = wl.curved_wall_case(n=n, p=3, q=3)
    g = sdg.GpuSolver(mesh, cfg, device=device)
    g.initialize_primitive(prim(g.volume_points()))
    bpts, phys = g.boundary_points()
    g.set_boundary_primitive(bprim(bpts, np.repeat(phys, g.counts.face_point_count)))
    dt = g.calculateDeltaTime(0.2)
    g.autotune()
    sp = ctypes.c_void_p()
    g.lib.sdg_get_stream(g.h, ctypes.byref(sp))
    stream = torch.cuda.ExternalStream(sp.value, device=device)
    for _ in range(args.warmup):
        g.step_async(dt)
    g.synchronize()
    steps = max(3, args.steps)
    ms = _timed(torch, stream, lambda: g.step_async(dt), steps)
    g.synchronize()
    dof = g.counts.degree_of_freedom_count
    err = g.relative_error()
    out = {"workload": f"ns-curved-wall-BR2-HLLC-Re200-Ma0.2-{n}^3-hex-P3-q3", "elements": g.counts.element_count,
           "dof": dof, "value": dof * 3 * steps / (ms * 1e-3), "unit": "DOF-stage/s", "ms_per_step": ms / steps,
           "finite": bool(np.all(np.isfinite(err))), "tiles": [g.tile(0)],
           "kernel_ms_per_step": kernel_split(g, dt, 3)}
    g.close()
    return out


def bench_vortex(args, device, torch):
    """2D Euler isentropic vortex, 40^2 quads, P3, Roe, dt 1e-3: state ~0.8 MB (L2-resident)."""
    import ctypes

    import subrosadg_gb300 as sdg
    from subrosadg_gb300 import workloads as wl
    mesh, cfg, prim, _, _, _ = wl.vortex_case(n=40, p=3, flux=sdg.ROE)
    g = sdg.GpuSolver(mesh, cfg, device=device)
    g.initialize_primitive(prim(g.volume_points()))
    g.autotune()
    sp = ctypes.c_void_p()
    g.lib.sdg_get_stream(g.h, ctypes.byref(sp))
    stream = torch.cuda.ExternalStream(sp.value, device=device)
    for _ in range(20):
        g.step_async(1e-3)
    g.synchronize()
    steps = 200
    ms = _timed(torch, stream, lambda: g.step_async(1e-3), steps)
    g.synchronize()
    dof = g.counts.degree_of_freedom_count
    split = kernel_split(g, 1e-3, 20)
    out = {"workload": "vortex2d-euler-40^2-quad-P3-Roe-dt1e-3", "dof": dof, "steps": steps,
           "value": dof * 3 * steps / (ms * 1e-3), "unit": "DOF-stage/s", "us_per_step": 1e3 * ms / steps,
           "kernel_us_per_step": {k: 1e3 * v for k, v in split.items()},
           "note": "state L2-resident: latency and launch bound (graph replay of 7 launches per step); "
                   "kernel_us_per_step: device time of each class with every launch bracketed by events"}
    g.close()
    return out


def bench_adjoint(args, device, torch):
    """cfg5: gradient of the integrated kinetic energy at the final time w.r.t. U0 and mu."""
    import subrosadg_gb300 as sdg
    from subrosadg_gb300 import workloads as wl
    n, steps, K = args.adjoint_elements, args.adjoint_steps, 25
    mesh, cfg, prim, _, _, _ = wl.tgv_case(n=n, p=3, flux=sdg.ROE, viscous=sdg.BR1, mu=1.0 / 1600.0)
    s = sdg.GpuSolver(mesh, cfg, device=device)
    s.initialize_primitive(prim(s.volume_points()))
    s.autotune()
    dt = s.calculateDeltaTime(0.2)
    u0 = s.state_point()
    w = s.volume_weights()
    mu0 = s.config.dynamic_viscosity
    s.stepSolver(dt, 3)
    s.set_state_point(u0)
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    s.stepSolver(dt, steps)
    t_fwd = time.perf_counter() - t0
    J0, lamN = s.kinetic_energy(weights=w)
    s.set_state_point(u0)
    t0 = time.perf_counter()
    lam0, mubar = s.adjoint_steps(dt, steps, lamN, checkpoint_interval=K)
    t_adj = time.perf_counter() - t0
    s.set_state_point(u0)
    s.forward_steps(dt, steps, checkpoint_interval=K)
    t0 = time.perf_counter()
    lam1, mubar1 = s.adjoint_recorded(lamN)
    t_rev = time.perf_counter() - t0
    mem = ctypes_int64(s)
    # the same gradient with every stage input kept in HBM by the forward sweep (no segment recompute)
    s.set_adjoint_trajectory_store(True)
    s.set_state_point(u0)
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    lam2, mubar2 = s.adjoint_steps(dt, steps, lamN, checkpoint_interval=K)
    t_adj2 = time.perf_counter() - t0
    mem2 = ctypes_int64(s)
    stored = {"adjoint_ms_per_step": 1e3 * t_adj2 / steps, "adjoint_over_forward": t_adj2 / t_fwd,
              "equals_checkpointed": bool(np.array_equal(lam0, lam2) and mubar == mubar2), "bytes": mem2,
              "note": "sdg_set_adjoint_trajectory_store: the forward sweep keeps all steps x 3 stage inputs "
                      "when HBM has room; the reverse re-forms only each stage input's traces and gradient pass"}
    s.set_adjoint_trajectory_store(False)
    out = {"workload": f"ns-tgv3d-BR1-Roe-Re1600-Ma0.1-{n}^3-hex-P3-{steps}steps-checkpoint{K}",
           "dof": s.counts.degree_of_freedom_count, "steps": steps, "J": J0,
           "forward_ms_per_step": 1e3 * t_fwd / steps, "adjoint_ms_per_step": 1e3 * t_adj / steps,
           "adjoint_over_forward": t_adj / t_fwd, "reverse_only_over_forward": t_rev / t_fwd,
           "recorded_equals_one_call": bool(np.array_equal(lam0, lam1) and mubar == mubar1),
           "dJ_dmu": mubar, "checkpoint_bytes": mem, "trajectory_store": stored,
           "note": "wall-clock of synchronous calls; full adjoint = forward sweep with checkpoints + per-segment "
                   "recompute + reverse sweep"}
    if not args.no_adjoint_check:
        rng = np.random.default_rng(2025)
        d0 = rng.standard_normal(u0.shape) * (np.abs(u0).mean(0) + 1e-3)
        h = 1e-6

        def J(u, mu=mu0):
            s.set_viscosity(mu)
            s.set_state_point(u)
            s.stepSolver(dt, steps)
            return s.kinetic_energy(weights=w)[0]

        fd = (J(u0 + h * d0) - J(u0 - h * d0)) / (2 * h)
        ad = float(np.sum(lam0 * d0))
        hm = h * mu0
        fdm = (J(u0, mu0 + hm) - J(u0, mu0 - hm)) / (2 * hm)
        s.set_viscosity(mu0)
        out["check"] = {"direction": "seeded normal, scaled per variable by the mean |U| (seed 2025)", "h": h,
                        "dJ_dU0_dot_d": {"adjoint": ad, "central_difference": fd,
                                         "relative_difference": abs(ad - fd) / max(abs(fd), 1e-300)},
                        "dJ_dmu": {"adjoint": mubar, "central_difference": fdm,
                                   "relative_difference": abs(mubar - fdm) / max(abs(fdm), 1e-300)}}
    s.close()
    return out


def ctypes_int64(s):
    import ctypes
    v = ctypes.c_int64()
    s.lib.sdg_adjoint_memory(s.h, ctypes.byref(v))
    return v.value


def run_ours(args):
    import ctypes

    import torch

    import subrosadg_gb300 as sdg
    from subrosadg_gb300 import _abi, replicas

    world, rank, local = dist_env()
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        pg = dist
    device = local
    torch.cuda.set_device(device)
    lib = _abi.load()

    mesh, cfg, prim = tgv_problem(args.elements, args.order)
    s = sdg.GpuSolver(mesh, cfg, device=device)
    c = s.counts
    s.initialize_primitive(prim(s.volume_points()))
    dt = s.calculateDeltaTime(0.2)
    dof = c.degree_of_freedom_count
    stages = 3
    stream_ptr = ctypes.c_void_p()
    lib.sdg_get_stream(s.h, ctypes.byref(stream_ptr))
    stream = torch.cuda.ExternalStream(stream_ptr.value, device=device)

    # warm-up
    for _ in range(args.warmup):
        s.step_async(dt)
    s.synchronize()

    # timed region: K steps, state resident in HBM (state 8 * DOF bytes >> 129 MB L2: no flush needed),
    # each step one CUDA-graph replay of all stage launches and the relative-error reduction
    replicas.barrier(pg)
    torch.cuda.synchronize(device)
    n0 = s.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(device) as clocks:
        ev0.record(stream)
        for _ in range(args.steps):
            s.step_async(dt)
        ev1.record(stream)
        ev1.synchronize()
    torch.cuda.synchronize(device)
    ms = ev0.elapsed_time(ev1)
    launches = s.launch_count() - n0
    s.synchronize()
    relerr = s.relative_error()
    ms = replicas.max_over_ranks(pg, ms, device=f"cuda:{device}")
    # per-kernel device times: a separate pass with every launch bracketed by events on the stream
    ksteps = max(1, min(args.steps, 3))
    lib.sdg_set_kernel_timing(s.h, 1)
    for _ in range(ksteps):
        s.step_async(dt)
    kms = (ctypes.c_double * 5)()
    kn = (ctypes.c_int64 * 5)()
    lib.sdg_kernel_time(s.h, kms, kn)
    lib.sdg_set_kernel_timing(s.h, 0)
    s.synchronize()

    # roofline of the dominant kernel (element stage kernel): algorithmic bytes per launch =
    # 8 * (3 DOF + (d^2 + 1) N_e): read U, read U_base, write U, affine geometry
    ne = c.element_count
    elem_bytes = 8.0 * (3 * dof + 10 * ne)
    elem_avg_ms = kms[0] / max(kn[0], 1)
    achieved = elem_bytes / (elem_avg_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    prof = profile_figures()
    traffic = prof["dram_bytes_per_element"] * ne if "dram_bytes_per_element" in prof else None
    fp64 = ctypes.c_double()
    lib.sdg_measure_fp64_peak(device, 200.0, ctypes.byref(fp64))
    fp64_flops = prof["fp64_flops_per_element"] * ne if "fp64_flops_per_element" in prof else None
    fp64_achieved = fp64_flops / (elem_avg_ms * 1e-3) / 1e9 if fp64_flops else None

    # end to end through the C ABI with pinned host buffers: every step uploads its input state and returns its
    # new state.  Streamed: sdg_step_state_point_from_async, each step's input transfer (a copy kernel) running
    # while the previous step computes, the new state written by the last stage; synchronous:
    # sdg_set_state_point + sdg_step_state_point, each call waiting for its own transfers.
    e2e = None
    if not args.no_e2e:
        npts = c.volume_point_count * s.nv
        host_in = torch.empty(npts, dtype=torch.float64, pin_memory=True)
        host_out = torch.empty(npts, dtype=torch.float64, pin_memory=True)
        out_view = host_out.numpy().reshape(-1, s.nv)
        in_view = host_in.numpy().reshape(-1, s.nv)
        s.state_point(out_view)
        host_in.copy_(host_out)
        for _ in range(2):
            s.set_state_point(in_view)
            s.step_state_point(dt, out_view)
        replicas.barrier(pg)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            s.set_state_point(in_view)                  # H2D of the step's input state
            s.step_state_point(dt, out_view)            # step, its relative error and its new state (D2H)
        t_sync = replicas.max_over_ranks(pg, time.perf_counter() - t0, device=f"cuda:{device}")
        for _ in range(2):
            s.step_state_point_from(dt, in_view, out_view, asynchronous=True)
        s.synchronize()
        replicas.barrier(pg)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            s.step_state_point_from(dt, in_view, out_view, asynchronous=True)  # H2D in, step, D2H out
        s.synchronize()
        relerr_streamed = s.relative_error()                                  # D2H of the last relative error
        t_e2e = replicas.max_over_ranks(pg, time.perf_counter() - t0, device=f"cuda:{device}")
        e2e = {"value": world * dof * stages * args.steps / t_e2e, "unit": "DOF-stage/s",
               "h2d_bytes_per_step": npts * 8, "d2h_bytes_per_step": npts * 8,
               "ms_per_step": 1e3 * t_e2e / args.steps,
               "mode": "streamed: sdg_step_state_point_from_async per step (pinned input read by a copy kernel "
                       "while the previous step computes; the new state written to pinned memory by the last "
                       "stage), one synchronize at the end",
               "relative_error_finite": bool(np.all(np.isfinite(relerr_streamed))),
               "synchronous": {"value": world * dof * stages * args.steps / t_sync, "unit": "DOF-stage/s",
                               "ms_per_step": 1e3 * t_sync / args.steps,
                               "mode": "sdg_set_state_point + sdg_step_state_point per step, each waiting for "
                                       "its transfers",
                               "h2d_bytes_per_step": npts * 8, "d2h_bytes_per_step": npts * 8 + s.nv * 8}}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        # bounded samples of the same 64^3 workload on the host cores, both variants
        faithful = cpu_baseline(args.cpu_sample, args.order, 2, 1, "faithful")
        lean = cpu_baseline(args.cpu_sample, args.order, 3, 1, "lean")
        cpu = {k: faithful[k] for k in ("value", "unit", "cores", "kind", "sample")}
        cpu["lean"] = {k: lean[k] for k in ("value", "unit", "cores", "kind", "sample")}

    if rank != 0:
        return
    value = world * dof * stages * args.steps / (ms * 1e-3)
    line = {
        "metric": METRIC, "value": value, "unit": "DOF-stage/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "elements": ne, "dof": dof, "stages_per_step": stages, "dt": dt,
                   "l2": "inputs larger than L2 (state 8*DOF = %.0f MB per buffer, L2 129 MB)" % (8 * dof / 1e6),
                   "parallelism": "replicas" if world > 1 else "single-gpu"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_source": f"{peak_kind} hbm_gbs",
                     "kernel": "tensorStageKernel<3,4,affine>", "avg_launch_ms": elem_avg_ms,
                     "algorithmic_bytes_per_launch": elem_bytes,
                     "binding": "fp64 pipe (CUDA-core DFMA; neither HBM nor tensor cores)",
                     "binding_frac": (fp64_achieved / fp64.value) if fp64_achieved else None},
        "fp64": {"peak_gflops": fp64.value, "peak_source": "sdg_measure_fp64_peak (independent-chain DFMA probe)",
                 "achieved_gflops": fp64_achieved, "frac": (fp64_achieved / fp64.value) if fp64_achieved else None,
                 "achieved_source": "ncu FP64 instruction counts per element, mean of the 3 stage launches of a "
                                    "56^3 step (2 per DFMA), scaled by elements "
                                    "(profiles/tensor_stage_kernel_tgv_hex_p3.md) / the live mean launch time",
                 "pipe_active_pct": prof.get("fp64_pipe_active_pct"),
                 "note": "the DG stage kernels are FP64-issue bound on GB300"},
        "kernel_ms_per_step": {"element": kms[0] / ksteps, "interior_face": kms[1] / ksteps,
                               "boundary_face": kms[2] / ksteps, "reduction": kms[3] / ksteps,
                               "gradient": kms[4] / ksteps},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
        "e2e": e2e,
        "cpu_baseline": cpu,
        "relative_error_last_step": relerr.tolist(),
    }
    s.close()
    if not args.no_extra:
        extras = {"batched": bench_batched, "ns_hybrid": bench_ns_hybrid, "vortex2d": bench_vortex,
                  "tet": bench_tet, "curved": bench_curved,
                  "adjoint": bench_adjoint,
                  "batched_small": lambda a, d, t: bench_batched(a, d, t, max_elements=2000)}
        for name in [x for x in args.extra.split(",") if x]:
            line[name] = extras[name](args, device, torch)
    print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
