"""Throughput of the fused D3Q27 cumulant + Smagorinsky LES step on GB300 (GLUPS, % of HBM roofline).

Workload (default): turbulent channel 512x256x256, periodic x/z, bounce-back walls, body force for
Re_tau ~ 180, laminar profile + 5 % seeded noise; FP16-deviation population storage with FP32
collision is the headline `value`; the plain FP32-storage kernel on the same case is reported beside
it.  One "step" is one lattice time step over all 33.5 M cells.  The state (1.8 GB FP16, 3.6 GB
FP32) is far larger than the 129 MB L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs one independent replica per GPU (the path does not shard in this build); value is the
sum over ranks of cell updates divided by the slowest rank's time.  --impl reference times the CPU
restatement of the reference's pass structure (oracle/, FP32, all host threads) on the same case.
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

BYTES_PER_CELL = {"f64": 27 * 8 * 2 + 1, "f32": 27 * 4 * 2 + 1, "f16dev": 27 * 2 * 2 + 1}
METRIC = "D3Q27 GLUPS, %HBM roofline: FP16-store+learned LES vs FP32 plain, equal error"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    """Per-cell DRAM bytes of the step kernels from the committed ncu summary (or None)."""
    p = os.path.join(ROOT, "profiles", "step_kernel_traffic.json")
    if os.path.exists(p):
        with open(p) as fh:
            return json.load(fh)
    return {}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
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
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return None, 0, 1, int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    import torch.distributed as dist
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend=backend)
    return dist, dist.get_rank(), ws, local


def dist_max(dist, x):
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_sum(dist, x):
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def channel_case(shape):
    from lb_gb300 import cases
    return cases.channel(*shape, re_tau=180.0, u_max=0.05, amp=0.05)


def collision_policy(name):
    from lb_gb300 import solver
    return {"cumulant2015": solver.CollisionCumD3Q27Turbulent2015, "cumulant2017": solver.CollisionCumD3Q27Turbulent2017,
            "combined": solver.CollisionCumD3Q27TurbulentCombined, "srt": solver.CollisionSRTTurbulent}[name]


def make_solver(shape, case, storage, device, options=0, model=None, interval=1, collision="cumulant2015"):
    """Cumulant collision with the Smagorinsky closure, or with the learned closure when a model is given."""
    from lb_gb300.solver import OmegaLES, OmegaMLP, Solver
    s = Solver(shape, collision=collision_policy(collision), turbulence=OmegaMLP if model else OmegaLES,
               storage=storage, nu=case["nu"], cles=0.17, periodic=case["periodic"], force=case["force"],
               device=device, options=options, mlp_interval=interval)
    s.set_flags(case["flags"])
    s.set_bc()
    s.init_fields(case["rho"], case["u"])
    if model:
        s.load_mlp(model)
    return s


def time_storage(shape, case, storage, steps, warmup, device, dist, with_clocks, options=0, model=None, interval=1,
                 collision="cumulant2015"):
    s = make_solver(shape, case, storage, device, options, model, interval, collision)
    s.step(warmup)
    s.synchronize()
    barrier(dist)
    sampler = ClockSampler(device) if with_clocks else None
    if sampler:
        sampler.__enter__()
    ms = s.step_timed(steps)
    if sampler:
        sampler.__exit__()
    barrier(dist)
    d = s.reduce()
    d.launches_per_step = s.step_launches()
    s.close()
    return ms, d, (sampler.summary() if sampler else None)


def pinned_copy(a, dtype, keep):
    """The array in page-locked host memory (a torch pinned buffer viewed as numpy; the buffer is kept
    alive in `keep`), so the library's host-to-device copies run at the link's rate; a plain copy
    where torch has no CUDA."""
    a = np.ascontiguousarray(a, dtype=dtype)
    try:
        import torch
    except ImportError:
        return a
    if not torch.cuda.is_available():
        return a
    t = torch.empty(a.size, dtype={np.int32: torch.int32, np.float64: torch.float64}[dtype], pin_memory=True)
    keep.append(t)
    out = t.numpy().reshape(a.shape)
    out[...] = a
    return out


def e2e_run(shape, case, storage, steps, device, options=0, model=None):
    """End to end through the public API with host buffers (page-locked): upload flags + initial fields
    (and the learned closure's weights), then every step lbm_step + the reference's per-step probe
    read-back (u, rho of one cell)."""
    from lb_gb300.solver import CollisionCumD3Q27Turbulent2015, OmegaLES, OmegaMLP, Solver
    s = Solver(shape, collision=CollisionCumD3Q27Turbulent2015, turbulence=OmegaMLP if model else OmegaLES,
               storage=storage, nu=case["nu"], cles=0.17, periodic=case["periodic"], force=case["force"],
               device=device, options=options)
    keep = []
    flags = pinned_copy(case["flags"], np.int32, keep)
    rho = pinned_copy(case["rho"], np.float64, keep)
    u = pinned_copy(case["u"], np.float64, keep)
    px, py, pz = shape[0] // 2, shape[1] // 2, shape[2] // 2
    s.synchronize()
    t0 = time.perf_counter()
    s.set_flags(flags)
    s.set_bc()
    s.init_fields(rho, u)
    if model:
        s.load_mlp(model)
    for _ in range(steps):
        s.step(1)
        s.probe(px, py, pz)
    s.synchronize()
    dt = time.perf_counter() - t0
    s.close()
    h2d = flags.nbytes + rho.nbytes + u.nbytes
    return dt, h2d, 32


def cpu_reference(shape, case, steps, warmup, budget_s, threads=None):
    """The oracle's reference-structured FP32 pipeline (separate omega, collision, A-B streaming,
    boundary and moment passes) on the host cores; returns (seconds per step, steps timed, threads)."""
    from lb_gb300 import capi
    from oracle import oracle as O
    if O._lib is None:
        O.NATIVE = True  # the host-tuned build of the same sources (oracle/build.py)
    if threads:
        O.set_threads(threads)
    nth = O.max_threads()
    cfg = capi.make_config(*shape, periodic=case["periodic"], collision=capi.LBM_COLLISION_CUMULANT2015,
                           closure=capi.LBM_CLOSURE_SMAGORINSKY, nu=case["nu"], cles=0.17, force=case["force"])
    o = O.OracleSim(cfg, 32)
    o.set_flags(case["flags"])
    o.init_fields(case["rho"], case["u"])
    for _ in range(warmup):
        o.step(1)
    t0 = time.perf_counter()
    n = 0
    while n < steps:
        o.step(1)
        n += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    o.close()
    return dt / n, n, nth


def voxelizer_block(reps=3):
    """The OFF-mesh voxelizer on the C4 body (seeded perturbed icosphere, 20,480 triangles, radius 24
    cells): lbm_voxelize_mesh through the C ABI (host mesh in, host flags out, best of `reps`) against the
    CPU restatement of the reference's per-cell segment query (geometryMesherOFF.h:81-112) on all host
    cores, and whether the two agree bit for bit."""
    import ctypes as C
    from lb_gb300 import capi, cases
    from oracle import oracle as O
    v, f = cases.perturbed_icosphere(radius=24.0)
    v = np.ascontiguousarray(v, dtype=np.float64)
    f = np.ascontiguousarray(f, dtype=np.int32)
    L = capi.lib()
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int32)
    dims = np.zeros(3, np.int32)
    bbox = np.zeros(6)
    args = (v.ctypes.data_as(dp), len(v), f.ctypes.data_as(ip), len(f), 1.0, 2.0)
    capi.check(L.lbm_voxelize_mesh(*args, None, dims.ctypes.data_as(ip), bbox.ctypes.data_as(dp), 0))
    g = np.zeros(int(dims.prod()), np.int32)
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        capi.check(L.lbm_voxelize_mesh(*args, g.ctypes.data_as(ip), dims.ctypes.data_as(ip), bbox.ctypes.data_as(dp), 0))
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    if O._lib is None:
        O.NATIVE = True
    t0 = time.perf_counter()
    ref, _ = O.voxelize_mesh(v, f, 1.0, 2.0, (-300.0, -270.0, -240.0))
    t_cpu = time.perf_counter() - t0
    return {"mesh": "seeded perturbed icosphere, 20480 triangles, radius 24 cells (config 4 body)",
            "dims": dims.tolist(), "cells": int(dims.prod()), "solid_cells": int(g.sum()),
            "gpu_ms": best * 1e3, "gpu_includes": "lbm_voxelize_mesh: host mesh in, host flags out (best of %d)" % reps,
            "cpu_s": t_cpu, "cpu_cores": O.max_threads(),
            "cpu_impl": "oracle restatement of the reference's per-cell segment query, host-tuned build",
            "bit_exact": bool(np.array_equal(g.reshape(ref.shape), ref)), "speedup": t_cpu / best}


def cpu_host_info():
    """Compiler flags of the timed CPU baseline and the host's STREAM-triad bandwidth (all threads)."""
    from oracle import build as obuild
    from oracle import oracle as O
    return {"flags": obuild.flags(native=True), "host_stream_gbs": round(O.host_stream_gbs(), 1),
            "reference_pass_bytes_per_cell": 720,
            "note": "reference pass structure (omega, collision, A-B streaming, boundary and moment passes) moves "
                    "about 720 B per cell update in FP32"}


def learned_block(path, model, glups_mlp, glups_smag, interval=None, cost_table=None):
    if model is None:
        return {"model": None, "note": "no model file: headline ran the Smagorinsky closure"}
    rep = None
    jp = path.replace(".npz", ".json")
    if os.path.exists(jp):
        with open(jp) as fh:
            r = json.load(fh)
        rep = {k: r.get(k) for k in ("fine_lattice", "train_samples", "held_out_sgs_error", "in_range_fraction")}
    out = {"model": os.path.relpath(path, ROOT), "glups_f16_mlp": glups_mlp, "glups_f16_smagorinsky": glups_smag,
           "throughput_cost": 1.0 - glups_mlp / glups_smag, "training": rep}
    if interval:
        k, g = interval
        out["refresh_interval"] = {"k": k, "glups_f16_mlp": g, "throughput_cost": 1.0 - g / glups_smag,
                                   "note": "network every k-th step, nu_t kept per cell in FP16 in between"}
    if cost_table:
        out["cost_by_refresh_interval"] = {str(k): {"glups": g, "throughput_cost": 1.0 - g / glups_smag}
                                           for k, g in sorted(cost_table.items())}
        out["cost_by_refresh_interval"]["1"] = {"glups": glups_mlp, "throughput_cost": 1.0 - glups_mlp / glups_smag}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--shape", default="512,256,256")
    ap.add_argument("--cpu-budget", type=float, default=20.0, help="seconds of CPU work for the CPU arms")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-collisions", action="store_true",
                    help="skip the SRT / cumulant-2017 / combined throughput lines")
    ap.add_argument("--options", type=int, default=0, help="LBM_OPT_* bits passed to lbm_create")
    ap.add_argument("--mlp-interval", type=int, default=16,
                    help="also time the learned closure with nu_t refreshed every k-th step")
    ap.add_argument("--mlp-intervals", default="2,4,8",
                    help="further refresh intervals for the learned closure's cost table")
    ap.add_argument("--no-voxelizer", action="store_true", help="skip the voxelizer line")
    ap.add_argument("--mlp", default=os.path.join(ROOT, "lb_gb300", "data", "les_mlp_channel.npz"),
                    help="learned-closure model (lb_gb300.les_train); the headline runs FP16 storage with it")
    args = ap.parse_args()
    shape = tuple(int(v) for v in args.shape.split(","))
    N = shape[0] * shape[1] * shape[2]
    workload = f"turbulent channel {shape[0]}x{shape[1]}x{shape[2]}, D3Q27 cumulant-2015 + Smagorinsky (CLES 0.17), Re_tau 180"
    dist, rank, ws, local = dist_setup()

    if args.impl == "reference":
        # the reference's own CPU path (restated, reference-structured passes) on the host cores
        if rank != 0:
            return
        from oracle import build as obuild
        obuild.build(native=True)
        case = channel_case(shape)
        sps, n, nth = cpu_reference(shape, case, args.steps, min(args.warmup, 1), budget_s=max(args.cpu_budget, 30.0))
        glups = N / sps / 1e9
        line = {"impl": "reference", "metric": METRIC, "value": glups, "unit": "GLUPS", "n_gpus": args.gpus,
                "steps": n, "warmup": min(args.warmup, 1), "ms_per_step": sps * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": workload, "storage": "f32 (A-B, two population arrays)",
                           "impl_detail": "CPU restatement of the reference's per-hook passes (oracle/), OpenMP"},
                "cpu_baseline": dict({"value": glups, "unit": "GLUPS", "cores": nth, "kind": "port",
                                      "sample": f"{n} steps of the full {shape[0]}x{shape[1]}x{shape[2]} lattice"},
                                     **cpu_host_info()),
                "e2e": {"value": glups, "unit": "GLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    from lb_gb300 import build as lbuild
    if rank == 0 or dist is None:
        lbuild.build()
    barrier(dist)
    device = local
    case = channel_case(shape)
    hbm, peak_kind = peaks()
    traffic = ncu_traffic()

    model = None
    if args.mlp and os.path.exists(args.mlp):
        from lb_gb300 import les
        model = les.MlpModel.load(args.mlp)
    # headline: FP16-deviation storage with the learned closure (Smagorinsky when no model is present)
    ms16, d16, clk = time_storage(shape, case, "f16dev", args.steps, args.warmup, device, dist, rank == 0,
                                 args.options, model)
    ms16s, d16s, _ = time_storage(shape, case, "f16dev", args.steps, args.warmup, device, dist, False, args.options) \
        if model else (ms16, d16, None)
    ms32, d32, _ = time_storage(shape, case, "f32", args.steps, args.warmup, device, dist, False, args.options)
    ms16k = None
    if model and args.mlp_interval > 1:
        ms16k, _, _ = time_storage(shape, case, "f16dev", args.steps, args.warmup, device, dist, False, args.options,
                                   model, args.mlp_interval)
        ms16k = dist_max(dist, ms16k)
    cost_table = {}
    if model:
        for k in [int(v) for v in args.mlp_intervals.split(",") if v.strip()] + ([args.mlp_interval] if ms16k else []):
            if k <= 1:
                continue
            msk = ms16k if k == args.mlp_interval else dist_max(dist, time_storage(
                shape, case, "f16dev", args.steps, args.warmup, device, dist, False, args.options, model, k)[0])
            cost_table[k] = dist_sum(dist, float(N) * args.steps) / (msk * 1e-3) / 1e9
    ms16 = dist_max(dist, ms16)
    ms16s = dist_max(dist, ms16s)
    ms32 = dist_max(dist, ms32)
    cells = dist_sum(dist, float(N) * args.steps)
    glups16 = cells / (ms16 * 1e-3) / 1e9
    glups16s = cells / (ms16s * 1e-3) / 1e9
    glups32 = cells / (ms32 * 1e-3) / 1e9

    def roof(kind, ms, traffic_kind=None):
        per_launch = BYTES_PER_CELL[kind] * N
        achieved = per_launch / (ms * 1e-3 / args.steps) / 1e9
        t = traffic.get(traffic_kind or kind)
        return {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "peak_kind": peak_kind, "traffic": (t["dram_bytes_per_cell"] * N) if t else None,
                "algorithmic_bytes_per_launch": per_launch}

    e2e = None
    if not args.no_e2e:
        k = args.steps  # the same number of steps as the device-timed region
        dt, h2d, d2h = e2e_run(shape, case, "f16dev", k, device, args.options, model)
        dt = dist_max(dist, dt)
        e2e = {"value": dist_sum(dist, float(N) * k) / dt / 1e9, "unit": "GLUPS",
               "h2d_bytes_per_step": h2d / k, "d2h_bytes_per_step": d2h, "steps": k,
               "includes": "lbm_set_flags + lbm_set_bc + lbm_init_fields (+ lbm_mlp_load) from page-locked host buffers, "
                           "then per step lbm_step + lbm_probe (device->host read of u, rho)"}
    # the other collision operators on the same case (Smagorinsky closure), FP16 and FP32 storage
    colls = None
    if not args.no_collisions:
        colls = {}
        kc = min(args.steps, 200)
        for name in ("srt", "cumulant2017", "combined"):
            colls[name] = {}
            for st in ("f16dev", "f32"):
                msc, dc, _ = time_storage(shape, case, st, kc, args.warmup, device, dist, False, args.options,
                                          collision=name)
                msc = dist_max(dist, msc)
                colls[name][st] = {"value": dist_sum(dist, float(N) * kc) / (msc * 1e-3) / 1e9,
                                   "frac": BYTES_PER_CELL[st] * N / (msc * 1e-3 / kc) / 1e9 / hbm,
                                   "nonfinite": dc.nonfinite}
        colls["steps"] = kc
        colls["unit"] = "GLUPS"
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        from oracle import build as obuild
        obuild.build(native=True)
        cshape = (256, 128, 128)
        ccase = channel_case(cshape)
        sps, n, nth = cpu_reference(cshape, ccase, 50, 1, budget_s=args.cpu_budget)
        cpu = dict({"value": cshape[0] * cshape[1] * cshape[2] / sps / 1e9, "unit": "GLUPS", "cores": nth,
                    "kind": "port",
                    "sample": f"{n} steps of the 256x128x128 channel, FP32, reference pass structure (oracle/)"},
                   **cpu_host_info())
    vox = None
    if rank == 0 and ws == 1 and not args.no_voxelizer:
        vox = voxelizer_block()
    if rank != 0:
        return
    line = {"metric": METRIC, "value": glups16, "unit": "GLUPS", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms16 / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload, "nx": shape[0], "ny": shape[1], "nz": shape[2],
                       "storage": "f16dev (f - w rho0) * 2^10, FP32 collision",
                       "closure": "learned MLP (tensor cores, fused), Smagorinsky fallback" if model else "smagorinsky",
                       "l2": "state 1.8 GB (f16) / 3.6 GB (f32) >> 129 MB L2; no flush needed",
                       "parallelism": f"{ws} independent replica(s)", "options": args.options},
            "roofline": roof("f16dev", ms16, "f16dev_mlp" if model else None),
            "fp32_plain": {"value": glups32, "ms_per_step": ms32 / args.steps, "roofline": roof("f32", ms32),
                           "closure": "smagorinsky", "speedup_f16_over_f32": glups16 / glups32},
            "f16_smagorinsky": {"value": glups16s, "ms_per_step": ms16s / args.steps, "roofline": roof("f16dev", ms16s),
                                "speedup_over_f32": glups16s / glups32},
            "learned_closure": learned_block(args.mlp, model, glups16, glups16s,
                                             (args.mlp_interval, cells / (ms16k * 1e-3) / 1e9) if ms16k else None,
                                             cost_table),
            # one fused step kernel per step; the row-staged step adds the launch over the wall rows
            "collisions": colls,
            "voxelizer": vox,
            "gpu_launches": args.steps * d16.launches_per_step, "clocks": clk, "cpu_baseline": cpu, "e2e": e2e,
            "check": {"f16_mass": d16.mass, "f32_mass": d32.mass,
                      "nonfinite": d16.nonfinite + d32.nonfinite + d16s.nonfinite}}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
