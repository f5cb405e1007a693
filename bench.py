#!/usr/bin/env python
"""Throughput of the fused fluidLB D2Q9 step on GB300.

Workload (default): flow past a cylinder, 8192 x 2048 nodes, BGK, populations
stored as FP32 shifted deviations (f - w_i), anti-bounce-back pressure
inlet/outlet, bounce-back walls and cylinder, seeded +-1e-4 velocity
perturbation.  A "step" is one time step of the whole grid (one fused kernel
launch).  Inputs (two 604 MB population buffers) are larger than L2.

Prints one JSON line.  ``--impl reference`` times the CPU restatement of the
reference's Numba-parallel CPU kernels (oracle/lbm_oracle.c, OpenMP over all
host cores) on the same case.  With torchrun (N > 1) every rank advances its own
replica of the case (the path has no exchange step on one GPU); value is the
aggregate over ranks, time the max over ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

B_LU = {"fp64": 144.0, "fp32_shifted": 72.0, "fp16_shifted": 36.0}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nx", type=int, default=8192)
    ap.add_argument("--ny", type=int, default=2048)
    ap.add_argument("--collision", default="BGK", choices=["BGK", "MRT"])
    ap.add_argument("--storage", default="fp32_shifted", choices=list(B_LU))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the FP64 / FP16 / error side measurements")
    ap.add_argument("--only", choices=["adjoint", "batch", "error-study", "aa", "config-errors"],
                    help="run one side measurement alone and print it (profiling runs)")
    ap.add_argument("--adjoint-steps", type=int, default=2000)
    return ap.parse_args()


def workload_case(args, storage):
    from pylabolt_gb300 import workloads
    scale = args.nx / 8192.0
    return workloads.cylinder(nx=args.nx, ny=args.ny, model=args.collision, storage=storage,
                              radius=128.0 * scale,
                              center=(int(2048 * scale), int(args.ny // 2 + 3)))


def workload_name(args):
    return f"cylinder_{args.nx}x{args.ny}_{args.collision.lower()}_{args.storage}"


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value, dist, device):
    """The largest `value` of all ranks (every rank receives it); `dist` is
    torch.distributed or None for one process."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_mlups(world, nodes, steps, seconds):
    """Units all ranks processed (replicas: `nodes` x `steps` each) per
    second of the slowest rank, in MLUPS."""
    return world * nodes * steps / seconds / 1e6


def reference_real(storage):
    """Field type of the reference's own case for a storage: FP64 storage is a
    "precision": "double" case; FP32 and FP16 storage stand for "precision":
    "single", whose fields are float32 (pylabolt/base/control.py:36-40)."""
    return "double" if storage == "fp64" else "float"


def cpu_measure(case_dict, steps_budget_s=20.0, max_steps=None, warmup=1, real="double"):
    """Times the C restatement of the reference CPU kernels on `case_dict`
    (real: "double", or "float" for a single-precision case)."""
    from oracle.setup import build_state
    from oracle.clib import COracle
    st = build_state(case_dict)
    co = COracle(st, real=real)
    co.initialize()
    co.run(warmup)
    t0 = time.perf_counter()
    co.run(1)
    one = time.perf_counter() - t0
    n = max(1, int(steps_budget_s / max(one, 1e-6)))
    if max_steps is not None:
        n = min(n, max_steps)
    t0 = time.perf_counter()
    co.run(n)
    dt = time.perf_counter() - t0
    nodes = st.Nx * st.Ny
    return nodes * n / dt / 1e6, n, dt


def host_link_peak(nbytes, device):
    """Pinned host <-> device copy bandwidth (GB/s, best of 5) of one
    cudaMemcpyAsync of `nbytes` each way: the floor of the end-to-end leg's
    transfers."""
    import torch
    n = nbytes // 8
    h = torch.empty(n, dtype=torch.float64, pin_memory=True)
    d = torch.empty(n, dtype=torch.float64, device=f"cuda:{device}")
    out = {}
    for name, dst, src in (("h2d", d, h), ("d2h", h, d)):
        best = float("inf")
        for _ in range(5):
            torch.cuda.synchronize(device)
            t0 = time.perf_counter()
            dst.copy_(src, non_blocking=True)
            torch.cuda.synchronize(device)
            best = min(best, time.perf_counter() - t0)
        out[name] = nbytes / best / 1e9
    del h, d
    return out


def run_reference(args, world, rank):
    if rank != 0:
        return
    from pylabolt_gb300 import workloads  # noqa: F401
    from oracle.clib import build
    real = reference_real(args.storage)
    build(real=real)
    cores = os.cpu_count()
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    case = workload_case(args, "fp64")
    from oracle.setup import build_state
    from oracle.clib import COracle
    st = build_state(case)
    co = COracle(st, real=real)
    co.initialize()
    co.run(args.warmup)
    # bounded sample: time as many of the K steps as fit in ~90 s
    t0 = time.perf_counter()
    co.run(1)
    one = time.perf_counter() - t0
    k = max(1, min(args.steps - 1, int(90.0 / max(one, 1e-6)))) + 1
    t0 = time.perf_counter()
    co.run(k - 1)
    dt = time.perf_counter() - t0 + one
    nodes = args.nx * args.ny
    mlups = nodes * k / dt / 1e6
    prec = "FP64" if real == "double" else "FP32 fields (the reference's precision single)"
    sample = (f"{k} of {args.steps} time steps of the full {args.nx}x{args.ny} grid "
              f"({prec}, 5 unfused sweeps + boundary kernels, OpenMP {cores} threads)")
    line = {
        "impl": "reference", "metric": "D2Q9 MLUPS", "value": mlups, "unit": "MLUPS",
        "n_gpus": args.gpus, "steps": k, "warmup": args.warmup,
        "ms_per_step": dt / k * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if real == "double" else "f32", "data": "synthetic",
        "config": {"workload": workload_name(args), "nx": args.nx, "ny": args.ny,
                   "collision": args.collision},
        "cpu_baseline": {"value": mlups, "unit": "MLUPS", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": mlups, "unit": "MLUPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(line), flush=True)


def run_gb300(args, world, rank, local):
    import torch
    from pylabolt_gb300.config import Case
    from pylabolt_gb300.lbm import FluidLBM
    from pylabolt_gb300 import capi

    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    device = local if world > 1 else 0
    torch.cuda.set_device(device)

    nodes = args.nx * args.ny
    case_d = workload_case(args, args.storage)
    case = Case(case_d)
    sim = FluidLBM(case, device=device)
    sim.initialize()
    sim.step(args.warmup)
    sim.step(1, residual=True)            # warms the residual step of the end-to-end leg
    sim.synchronize()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(device)

    clocks = ClockSampler(device)
    launches0 = sim.kernel_launches
    barrier()
    clocks.start()
    ms = sim.time_steps(args.steps)       # CUDA events on the handle's stream
    barrier()
    clk = clocks.stop()
    launches = sim.kernel_launches - launches0
    variant = sim.kernel_variant
    tuning = sim.tuning
    ms = max_over_ranks(ms, dist, f"cuda:{device}")
    mlups = whole_job_mlups(world, nodes, args.steps, ms / 1e3)
    per_launch_ms = ms / args.steps
    peak, peak_kind = measured_peak()
    achieved = B_LU[args.storage] * nodes / (per_launch_ms / 1e3) / 1e9

    traffic = None
    tpath = os.path.join(ROOT, "profiles", "step_kernel_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            tr = json.load(f)
        key = f"{args.collision.lower()}_{args.storage}"
        if key in tr and tr[key].get("nodes"):
            traffic = tr[key]["dram_bytes_per_launch"] * nodes / tr[key]["nodes"]

    # ---- end to end through the Python API, pinned host buffers -----------
    e2e_steps = args.steps                          # the same K steps as the device-timed leg
    # host fields as the reference's case holds them: float64 for precision
    # "double" (FP64 storage), float32 for precision "single" (the FP32 and
    # FP16 storage cases; pylabolt/base/fields.py:64-77)
    host_dt = torch.float64 if args.storage == "fp64" else torch.float32
    rho_h = torch.empty(case.density.shape, dtype=host_dt, pin_memory=True).numpy()
    u_h = torch.empty(case.velocity.shape, dtype=host_dt, pin_memory=True).numpy()
    rho_h[...] = case.density
    u_h[...] = case.velocity
    rho_out = torch.empty(case.density.shape, dtype=host_dt, pin_memory=True).numpy()
    u_out = torch.empty(case.velocity.shape, dtype=host_dt, pin_memory=True).numpy()
    def end_to_end(nsteps):
        barrier()
        t0 = time.perf_counter()
        sim.initialize(rho_h, u_h)                      # H2D of the initial fields
        for t in range(1, nsteps + 1):
            # its residual sums land in pinned host memory; the last step also
            # records the fields the final readback returns
            sim.step(1, residual=True, moments=t == nsteps)
            if t > 1:
                sim.residual(step=t - 1)                # read step t-1's while step t runs
        sim.residual(step=nsteps)
        sim.moments(out=(rho_out, u_out))               # D2H of the final fields (step nsteps)
        return max_over_ranks(time.perf_counter() - t0, dist, f"cuda:{device}")

    # three whole runs, the median reported: one run can meet a host-side
    # stall of a few ms in its transfers (seen on the shared GPU hosts)
    t_runs = [end_to_end(e2e_steps) for _ in range(3)]
    t_e2e = float(np.median(t_runs))
    io_bytes = rho_h.nbytes + u_h.nbytes
    link = host_link_peak(io_bytes, device)
    e2e = {"value": whole_job_mlups(world, nodes, e2e_steps, t_e2e), "unit": "MLUPS",
           "h2d_bytes_per_step": int(io_bytes / e2e_steps),
           "d2h_bytes_per_step": int(8 * 8 + (rho_out.nbytes + u_out.nbytes) / e2e_steps),
           "steps": e2e_steps, "ms": t_e2e * 1e3,
           "runs_ms": [round(t * 1e3, 3) for t in t_runs], "of_runs": "median",
           "host_link_gbs": link,
           "transfer_floor_ms": io_bytes / link["h2d"] / 1e6 + io_bytes / link["d2h"] / 1e6,
           "host_fields": str(rho_h.dtype),
           "what": "FluidLBM.initialize(host rho,u) + per step lbm_step_ex(RESIDUAL) + "
                   "lbm_residual_at readback (step t-1's read while step t runs) + final moments readback "
                   f"({'lbm_init_fields/lbm_get_moments' if args.storage == 'fp64' else 'lbm_init_fields_f32/lbm_get_moments_f32'})"}
    if e2e_steps != 200 and not args.no_extra:
        t200_runs = [end_to_end(200) for _ in range(3)]
        t200 = float(np.median(t200_runs))
        e2e["at_200_steps"] = {"value": whole_job_mlups(world, nodes, 200, t200), "ms": t200 * 1e3,
                               "runs_ms": [round(t * 1e3, 3) for t in t200_runs]}

    extra = {}
    if not args.no_extra and rank == 0:
        extra = side_measurements(args, case_d, sim, nodes, peak)
    sim.close()

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            from oracle.clib import build
            real = reference_real(args.storage)
            build(real=real)
            cpu_case = workload_case(args, "fp64")
            mlups_cpu, n_cpu, dt_cpu = cpu_measure(cpu_case, steps_budget_s=15.0, max_steps=200,
                                                   real=real)
            prec = "FP64" if real == "double" else "FP32 fields, the reference's precision single"
            cpu = {"value": mlups_cpu, "unit": "MLUPS", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"{n_cpu} full time steps of the same {args.nx}x{args.ny} case "
                             f"in {dt_cpu:.1f} s (C restatement of the reference CPU kernels, "
                             f"{prec}, OpenMP)"}
        except Exception as e:  # reported, never substituted
            cpu = {"value": None, "unit": "MLUPS", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"failed: {e}"}

    if rank == 0:
        line = {
            "metric": "D2Q9 MLUPS", "value": mlups, "unit": "MLUPS", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_launch_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if args.storage != "fp64" else "f64", "data": "synthetic",
            "config": {"workload": workload_name(args), "nx": args.nx, "ny": args.ny,
                       "collision": args.collision, "storage": args.storage,
                       "bytes_per_lattice_update": B_LU[args.storage],
                       "l2": "inputs larger than L2 (two population buffers of "
                             f"{9 * nodes * B_LU[args.storage] / 18 / 1e6:.0f} MB)",
                       "parallelism": f"replicas x{world}",
                       "kernel": {"kind": ["scalar", "-", "node_pair_tiles", "node_pairs"][variant[0]],
                                  "nodes_per_thread": variant[1], "block": variant[2],
                                  "stages": variant[3],
                                  "autotune_ms": [round(t, 4) for t in tuning]}},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": traffic},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": int(launches),
            "clocks": clk,
        }
        line.update(extra)
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def side_measurements(args, case_d, sim32, nodes, peak):
    """FP64 and FP16 throughput of the same step and the FP32/FP16 error
    against FP64 after a short run from the same initial state."""
    from pylabolt_gb300.config import Case
    from pylabolt_gb300.lbm import FluidLBM
    out = {}
    case = Case(case_d)
    res = {}
    for storage, steps in (("fp64", max(5, args.steps // 10)), ("fp16_shifted", args.steps)):
        with FluidLBM(case, storage=storage) as s:
            s.initialize()
            s.step(3)
            s.synchronize()
            ms = s.time_steps(steps)
            mlups = nodes * steps / (ms / 1e3) / 1e6
            res[storage] = {"mlups": mlups,
                            "roofline_frac": B_LU[storage] * nodes / (ms / steps / 1e3) / 1e9 / peak}
    # MRT (rates 1.4, 1.4, 1.2) on the same grid, FP32 shifted
    mrt_args = argparse.Namespace(**{**vars(args), "collision": "MRT"})
    with FluidLBM(Case(workload_case(mrt_args, "fp32_shifted")), storage="fp32_shifted") as s:
        s.initialize()
        s.step(3)
        s.synchronize()
        ms = s.time_steps(args.steps)
        res["mrt_fp32_shifted"] = {
            "mlups": nodes * args.steps / (ms / 1e3) / 1e6,
            "roofline_frac": B_LU["fp32_shifted"] * nodes / (ms / args.steps / 1e3) / 1e9 / peak,
            "kernel": list(s.kernel_variant)}
    out["mrt_fp32_shifted"] = res["mrt_fp32_shifted"]
    out.update(aa_measurement(args, case_d, peak))
    # the same cylinder translating at 0.02 nodes per step (moving-obstacle
    # kernels around the fused step)
    mv = dict(case_d)
    mv["obstacle_dict"] = {k: dict(v) for k, v in case_d["obstacle_dict"].items()}
    mv["obstacle_dict"]["options"] = {"compute_force_torque": True, "move_obstacles": True}
    mv["obstacle_dict"]["cylinder"].update({"static": False, "solid_motion_dict": {
        "type": "fixed_velocity", "degree_of_freedom": "translation",
        "linear_velocity": [0.02, 0.0], "angular_velocity": 0.0}})
    with FluidLBM(Case(mv), storage="fp32_shifted") as s:
        s.initialize()
        s.step(3)
        s.synchronize()
        ms = s.time_steps(args.steps)
        out["moving_cylinder_fp32_shifted"] = {
            "mlups": nodes * args.steps / (ms / 1e3) / 1e6,
            "launches_per_step": 5, "kernel": list(s.kernel_variant),
            "center_after": float(s.moving_obstacles()[0]["center"][0])}
    out["adjoint"] = adjoint_measurement()
    out["batch"] = batch_measurement()
    out["fp64"] = res["fp64"]
    out["fp16_shifted"] = res["fp16_shifted"]
    err_steps = 200
    us = {}
    for storage in ("fp64", "fp32_shifted", "fp16_shifted"):
        with FluidLBM(case, storage=storage) as s:
            s.initialize()
            s.step(err_steps, moments=True)
            us[storage] = s.moments()[1]
    ref = us["fp64"]
    fluid = ~case.solid
    for storage in ("fp32_shifted", "fp16_shifted"):
        d = us[storage][fluid] - ref[fluid]
        out.setdefault("error_vs_fp64", {})[storage] = {
            "steps": err_steps,
            "u_rel_l2": float(np.linalg.norm(d) / np.linalg.norm(ref[fluid])),
            "u_max_abs_over_max": float(np.abs(d).max() / np.abs(ref[fluid]).max())}
    return out


def aa_measurement(args, case_d=None, peak=None):
    """The same step on one population buffer updated in place (AA pattern):
    throughput, roofline fraction (same bytes per node update as two
    buffers) and device memory of both layouts."""
    from pylabolt_gb300.config import Case
    from pylabolt_gb300.lbm import FluidLBM
    case = Case(case_d or workload_case(args, "fp32_shifted"))
    peak = peak or measured_peak()[0]
    nodes = case.nx * case.ny
    out = {}
    for storage in ("fp32_shifted", "fp16_shifted"):
        rec = {}
        for layout in ("aa", "ab"):
            with FluidLBM(case, storage=storage, layout=layout) as s:
                s.initialize()
                s.step(3)
                s.synchronize()
                rec[f"device_gb_{layout}"] = s.device_bytes / 1e9
                if layout == "aa":
                    ms = s.time_steps(args.steps)
                    rec["mlups"] = nodes * args.steps / (ms / 1e3) / 1e6
                    rec["roofline_frac"] = B_LU[storage] * nodes / (ms / args.steps / 1e3) / 1e9 / peak
                    rec["kernel"] = list(s.kernel_variant)
        out[f"aa_{storage}"] = rec
    return out


def error_study(args, nsteps=10000):
    """The cylinder case, BGK and MRT, 10,000 steps from the same seeded
    start in FP64, FP32-shifted and FP16-shifted storage: throughput of each
    and the velocity error of the reduced storages against FP64 (relative L2
    and max |du| / max |u| over fluid nodes)."""
    from pylabolt_gb300.config import Case
    from pylabolt_gb300.lbm import FluidLBM
    out = {"workload": workload_name(args), "steps": nsteps}
    for coll in ("BGK", "MRT"):
        cargs = argparse.Namespace(**{**vars(args), "collision": coll})
        case = Case(workload_case(cargs, "fp64"))
        fluid = ~case.solid
        nodes = case.nx * case.ny
        us, rates = {}, {}
        for storage in ("fp64", "fp32_shifted", "fp16_shifted"):
            with FluidLBM(case, storage=storage) as s:
                s.initialize()
                s.step(1)
                s.synchronize()
                ms = s.time_steps(nsteps - 2)
                s.step(1, moments=True)
                us[storage] = s.moments()[1]
                rates[storage] = nodes * (nsteps - 2) / (ms / 1e3) / 1e6
        ref = us["fp64"][fluid]
        res = {"mlups": rates}
        for storage in ("fp32_shifted", "fp16_shifted"):
            d = us[storage][fluid] - ref
            res[storage] = {"u_rel_l2": float(np.linalg.norm(d) / np.linalg.norm(ref)),
                            "u_max_abs_over_max": float(np.abs(d).max() / np.abs(ref).max())}
        out[coll.lower()] = res
    return out


def _u_errors(u, ref, mask):
    d = u[mask] - ref[mask]
    return {"u_rel_l2": float(np.linalg.norm(d) / np.linalg.norm(ref[mask])),
            "u_max_abs_over_max": float(np.abs(d).max() / np.abs(ref[mask]).max())}


def config_errors(c1_steps=20000, c2_steps=50000):
    """Velocity error of every storage against FP64 on the two small
    configurations: the 128^2 lid-driven cavity (BGK, Re 100, lid 0.1,
    20,000 steps) and the 1024x512 gravity-driven Poiseuille channel (MRT
    rates 1.4 / 1.4 / 1.2 + Guo second order, centreline 0.05, Re 100,
    50,000 steps), the latter also against the analytic start-up profile."""
    from pylabolt_gb300 import workloads
    from pylabolt_gb300.config import Case
    from pylabolt_gb300.lbm import FluidLBM

    def run(case, storage, steps):
        with FluidLBM(case, storage=storage) as s:
            s.initialize()
            s.step(steps, moments=True)
            return s.moments()[1]

    out = {}
    case = Case(workloads.cavity(128))
    mask = np.ones((case.nx, case.ny), bool)
    u = {st: run(case, st, c1_steps) for st in ("fp64", "fp32_shifted", "fp16_shifted")}
    out["cavity_128x128_bgk"] = {"steps": c1_steps, **{
        st: _u_errors(u[st], u["fp64"], mask) for st in ("fp32_shifted", "fp16_shifted")}}
    case_d, par = workloads.poiseuille()
    case = Case(case_d)
    mask = np.ones((case.nx, case.ny), bool)
    u = {st: run(case, st, c2_steps) for st in ("fp64", "fp32_shifted", "fp16_shifted")}
    prof = workloads.poiseuille_startup_profile(case.ny, par["gx"], par["kin_visc"], c2_steps)
    ana = np.zeros_like(u["fp64"])
    ana[..., 0] = prof[None, :]
    rec = {"steps": c2_steps,
           "fp64_vs_analytic": _u_errors(u["fp64"], ana, mask)}
    for st in ("fp32_shifted", "fp16_shifted"):
        rec[st] = {**_u_errors(u[st], u["fp64"], mask),
                   "vs_analytic": _u_errors(u[st], ana, mask)}
    out["poiseuille_1024x512_mrt_guo2"] = rec
    return out


def adjoint_measurement(nsteps=2000, interval=45):
    """Adjoint case: 512x512 channel, BGK + Guo, per-node body force, tau 0.8,
    FP32-shifted forward, T = 2000, state kept every 45 steps.  Reports the
    forward time (with checkpointing), the reverse time (recompute + adjoint)
    and a gradient check of one random body-force direction against central
    differences of the FP64 forward."""
    from pylabolt_gb300 import workloads
    from pylabolt_gb300.config import Case
    from pylabolt_gb300.lbm import FluidLBM
    from pylabolt_gb300.autograd import case_with
    case = Case(workloads.adjoint_channel(seed=1))
    tgt = Case(workloads.adjoint_channel(seed=2))

    def run64(c):
        with FluidLBM(c, storage="fp64") as s:
            s.initialize()
            s.step(nsteps, moments=True)
            return s.moments()[1]

    target = run64(tgt)
    with FluidLBM(case, storage="fp32_shifted") as sim:
        sim.initialize()
        sim.step(3)
        times = []
        for _ in range(2):           # first call captures the graphs; second is steady state
            sim.initialize()
            sim.synchronize()
            t0 = time.perf_counter()
            sim.adjoint_forward(nsteps, interval)
            sim.synchronize()
            t_fwd = time.perf_counter() - t0
            _, u = sim.moments()
            t0 = time.perf_counter()
            gF, gtau, _ = sim.adjoint_backward(2.0 * (u - target) / u.size)
            t_bwd = time.perf_counter() - t0
            times.append((t_fwd, t_bwd))
        sim.initialize()
        ms_plain = sim.time_steps(nsteps)
    d = np.random.default_rng(7).standard_normal(case.body_force_field.shape)
    h = 1e-8
    lp = float(((run64(case_with(case, force=case.body_force_field + h * d)) - target) ** 2).mean())
    lm = float(((run64(case_with(case, force=case.body_force_field - h * d)) - target) ** 2).mean())
    fd = (lp - lm) / (2 * h)
    ad = float((gF * d).sum())
    return {"workload": "channel_512x512_bgk_guo2_body_force_fp32_shifted", "steps": nsteps,
            "checkpoint_interval": interval, "forward_s": t_fwd, "backward_s": t_bwd,
            "first_call_forward_s": times[0][0], "first_call_backward_s": times[0][1],
            "plain_forward_s": ms_plain / 1e3, "adjoint_over_forward": t_bwd / t_fwd,
            "adjoint_over_plain_forward": t_bwd / (ms_plain / 1e3),
            "grad_dir_vs_central_fd_rel": abs(ad - fd) / abs(fd), "grad_tau": gtau}


def batch_measurement(nsteps=5000, seq_steps=50):
    """256 lid-driven cavities (sides U{64..512}, Re U[50,1000], lid
    U[0.05,0.1], default_rng(0)) advanced together, FP32 shifted, nsteps steps
    replayed from CUDA graphs; against one launch stream per cavity run one
    after the other, and against FP64 runs of every cavity on its own."""
    from pylabolt_gb300 import workloads
    from pylabolt_gb300.batch import CavityBatch, draw_cavities
    from pylabolt_gb300.config import Case
    from pylabolt_gb300.lbm import FluidLBM
    sides, res, lids = draw_cavities()
    with CavityBatch(sides, res, lids) as b:
        b.initialize()
        b.step(3)
        b.initialize()
        b.step(1)
        ms = b.time_steps(nsteps - 2)
        b.step(1, moments=True)
        ub = b.velocities()
        variant = b.kernel_variant
        nodes = b.fluid_nodes
    batched = nodes * (nsteps - 2) / (ms / 1e3) / 1e6
    # sequential: every cavity its own handle, stepped one after the other
    sims = []
    for i in range(len(sides)):
        c = Case(workloads.cavity(int(sides[i]), re=float(res[i]), lid=float(lids[i])))
        s = FluidLBM(c, storage="fp32_shifted")
        s.initialize()
        s.step(2)
        s.synchronize()
        sims.append(s)
    t0 = time.perf_counter()
    for s in sims:
        s.step(seq_steps)
    for s in sims:
        s.synchronize()
    t_seq = time.perf_counter() - t0
    for s in sims:
        s.close()
    sequential = nodes * seq_steps / t_seq / 1e6
    # FP64 run of every cavity on its own handle; the handles' steps are
    # queued on their own streams before any result is read
    errs = []
    for lo in range(0, len(sides), 64):
        sims = []
        for i in range(lo, min(lo + 64, len(sides))):
            c = Case(workloads.cavity(int(sides[i]), re=float(res[i]), lid=float(lids[i])))
            s = FluidLBM(c, storage="fp64")
            s.initialize()
            s.step(nsteps, moments=True)
            sims.append((i, s))
        for i, s in sims:
            _, u = s.moments()
            errs.append(float(np.abs(ub[i] - u).max() / np.abs(u).max()))
            s.close()
    return {"workload": "256_cavities_U64-512_fp32_shifted", "steps": nsteps,
            "fluid_nodes": nodes, "batched_mlups": batched,
            "sequential_per_instance_mlups": sequential, "speedup": batched / sequential,
            "kernel": list(variant), "max_err_vs_fp64": max(errs),
            "median_err_vs_fp64": float(np.median(errs)), "fp64_checked": len(errs)}


def main():
    args = parse()
    if args.only:
        if args.only == "adjoint":
            out = adjoint_measurement(args.adjoint_steps)
        elif args.only == "batch":
            out = batch_measurement()
        elif args.only == "aa":
            out = aa_measurement(args)
        elif args.only == "config-errors":
            out = config_errors()
        else:
            out = error_study(args)
        print(json.dumps({"only": args.only, **out}), flush=True)
        return
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    run_gb300(args, world, rank, local)


if __name__ == "__main__":
    main()
