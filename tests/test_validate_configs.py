"""Validation runs of the benchmark configurations on the GPU: long, so skipped unless pytest is given
--run-slow.  Each test writes its results as one JSON file into $LBM_VALIDATE_OUT (when set) and asserts
the bounds stated beside it.

    python -m pytest tests/test_validate_configs.py --run-slow -m gpu -k c1      (64^3, 10k steps)
    python -m pytest tests/test_validate_configs.py --run-slow -m gpu -k c3      (512x256x256, 20k steps)
    python -m pytest tests/test_validate_configs.py --run-slow -m gpu -k c4      (384x192x192, 4k steps)
    python -m pytest tests/test_validate_configs.py --run-slow -m gpu -k c5      (256^3 LES, 1024^3 fine run)
    python -m pytest tests/test_validate_configs.py --run-slow -m gpu -k c2      (learned closure a priori)

c1: lid-driven cavity 64^3, FP64 cumulant on the GPU against the CPU oracle's FP64 run of the same case
    (parity of the whole 10k-step trajectory), FP32 against FP64; centre-line profiles.
c3: channel at 512x256x256 (laminar profile + 5 % seeded noise, Re_tau 180 forcing, Smagorinsky CLES
    0.17) in FP64, FP32 and FP16-deviation storage (stochastic rounding, and round-to-nearest for
    comparison): relative L2 error of the x-z-time-averaged mean velocity and of the Reynolds stresses
    against FP64.
c4: flow past the voxelized seeded body at 384x192x192: GPU voxelizer against the CPU oracle (bit for
    bit), FP32 against FP64 drag (momentum exchange, FP64 sums).
c5: periodic decaying turbulence, coarse 256^3 and a 4x-finer run of the same seeded random-phase field
    (E(k) ~ k^4 exp(-2 (k/k0)^2), k0 = 8, divergence-free, u_rms = 0.04 per component).  A priori: the
    learned closure's and Smagorinsky's subgrid-stress and dissipation errors on the filtered fine field.
    A posteriori: coarse LES in FP16-deviation storage with each closure from the filtered initial
    field, against the filtered fine field after the same physical time.  Throughput of both closures
    on the coarse lattice.
c2 a priori: the shipped channel model on a channel realisation with another seed (1024x256x256 FP32,
    snapshots after 30k, 33k, 36k and 39k steps): subgrid-stress and dissipation errors per snapshot of
    the network, of Smagorinsky with the training samples' fitted constant, with the snapshot's own
    fitted constant and with CLES 0.17 (mean and spread over the snapshots).
LBM_VALIDATE_SMALL=1 runs reduced sizes for a quick look (the bounds are then not asserted).
"""
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import pytest  # noqa: E402

from lb_gb300 import cases  # noqa: E402
from lb_gb300.solver import OmegaLES, OmegaNo, Solver, InletVelocityEquilibrium  # noqa: E402


def c1(n, steps):
    from lb_gb300 import capi
    from oracle import oracle as O
    c = cases.cavity(n)
    out = {"config": "C1 cavity", "n": n, "steps": steps, "nu": c["nu"]}
    res = {}
    for st in ("f64", "f32"):
        s = Solver((n, n, n), turbulence=OmegaNo, storage=st, nu=c["nu"])
        s.set_flags(c["flags"])
        s.set_bc(c["inlets"])
        s.init_equilibrium(1.0, (0.0, 0.0, 0.0))
        ms = s.step_timed(steps)
        res[st] = s.moments()[1]
        out[f"gpu_{st}_seconds"] = ms * 1e-3
        s.close()
    cfg = capi.make_config(n, n, n, collision=capi.LBM_COLLISION_CUMULANT2015, closure=capi.LBM_CLOSURE_NONE,
                           nu=c["nu"])
    t0 = time.time()
    o = O.OracleSim(cfg, 64)
    o.set_flags(c["flags"])
    o.set_bc(c["inlets"])
    o.init_equilibrium(1.0, (0.0, 0.0, 0.0))
    o.step(steps)
    uo = o.moments()[1]
    o.close()
    out["oracle_seconds"] = time.time() - t0
    ulid = 0.05
    out["max_abs_du_over_ulid_gpu64_vs_oracle64"] = float(np.max(np.abs(res["f64"] - uo)) / ulid)
    out["max_abs_du_over_ulid_gpu32_vs_gpu64"] = float(np.max(np.abs(res["f32"] - res["f64"])) / ulid)
    u = res["f64"].reshape(3, n, n, n)
    out["centerline_ux_y"] = (u[0, n // 2, :, n // 2] / ulid).round(6).tolist()
    out["centerline_uy_x"] = (u[1, n // 2, n // 2, :] / ulid).round(6).tolist()
    return out


def _channel_stats(shape, storage, steps, avg, case):
    from lb_gb300 import capi
    nx, ny, nz = shape
    opt = 0
    if storage == "f16dev_rn":  # FP16 storage with round-to-nearest stores instead of stochastic rounding
        storage, opt = "f16dev", capi.LBM_OPT_F16_ROUND_NEAREST
    s = Solver(shape, turbulence=OmegaLES, storage=storage, nu=case["nu"], cles=0.17, periodic=case["periodic"],
               force=case["force"], options=opt)
    s.set_flags(case["flags"])
    s.set_bc()
    s.init_fields(case["rho"], case["u"])
    t0 = time.time()
    s.step(steps - avg + 1)
    s.timeavg_begin()
    s.step(avg - 1)
    s.timeavg_end()
    _, um, uu, cnt = s.timeavg_get()
    d = s.reduce()
    s.close()
    um = um.reshape(3, nz, ny, nx)
    uu = uu.reshape(6, nz, ny, nx)
    mean = um[0].mean(axis=(0, 2))
    R = np.stack([(uu[0] - um[0] ** 2).mean(axis=(0, 2)), (uu[1] - um[1] ** 2).mean(axis=(0, 2)),
                  (uu[2] - um[2] ** 2).mean(axis=(0, 2)), (uu[3] - um[0] * um[1]).mean(axis=(0, 2))])
    return mean, R, time.time() - t0, d, cnt


def c3(shape, steps, avg):
    case = cases.channel(*shape, re_tau=180.0, u_max=0.05, amp=0.05)
    out = {"config": "C3 channel precision", "shape": list(shape), "steps": steps, "avg_steps": avg,
           "nu": case["nu"], "force": case["force"][0]}
    stats = {st: _channel_stats(shape, st, steps, avg, case) for st in ("f64", "f32", "f16dev", "f16dev_rn")}
    m64, R64 = stats["f64"][0], stats["f64"][1]
    for st in ("f32", "f16dev", "f16dev_rn"):
        m, R = stats[st][0], stats[st][1]
        out[f"{st}_mean_velocity_rel_l2_vs_f64"] = float(np.linalg.norm(m - m64) / np.linalg.norm(m64))
        out[f"{st}_reynolds_stress_rel_l2_vs_f64"] = float(np.linalg.norm(R - R64) / max(np.linalg.norm(R64), 1e-300))
    for st in stats:
        out[f"{st}_seconds"] = stats[st][2]
        out[f"{st}_max_speed"] = stats[st][3].max_speed
        out[f"{st}_nonfinite"] = stats[st][3].nonfinite
    out["f64_reynolds_stress_norm"] = float(np.linalg.norm(R64))
    out["f64_mean_profile"] = m64.round(7).tolist()
    return out


def c4(shape, steps):
    import ctypes as C
    from lb_gb300 import capi
    from oracle import oracle as O
    nx, ny, nz = shape
    v, f = cases.perturbed_icosphere(radius=24.0)
    vv, ff = np.ascontiguousarray(v), np.ascontiguousarray(f)
    dims = np.zeros(3, np.int32)
    bbox = np.zeros(6)
    L = capi.lib()
    args = (vv.ctypes.data_as(C.POINTER(C.c_double)), len(vv), ff.ctypes.data_as(C.POINTER(C.c_int32)), len(ff),
            1.0, 2.0)
    capi.check(L.lbm_voxelize_mesh(*args, None, dims.ctypes.data_as(C.POINTER(C.c_int32)),
                                   bbox.ctypes.data_as(C.POINTER(C.c_double)), 0))
    g = np.zeros(int(np.prod(dims)), np.int32)
    t_gpu = None
    for _ in range(3):  # the first call also loads the kernel module: best of three calls
        t0 = time.time()
        capi.check(L.lbm_voxelize_mesh(*args, g.ctypes.data_as(C.POINTER(C.c_int32)),
                                       dims.ctypes.data_as(C.POINTER(C.c_int32)),
                                       bbox.ctypes.data_as(C.POINTER(C.c_double)), 0))
        dt = time.time() - t0
        t_gpu = dt if t_gpu is None else min(t_gpu, dt)
    t0 = time.time()
    ref, _ = O.voxelize_mesh(v, f, 1.0, 2.0, (-300.0, -270.0, -240.0))
    t_orc = time.time() - t0
    out = {"config": "C4 body", "shape": list(shape), "steps": steps, "triangles": len(f),
           "voxel_dims": dims.tolist(), "solid_voxels": int(g.sum()),
           "voxelizer_bit_exact": bool(np.array_equal(g.reshape(ref.shape), ref)),
           "gpu_voxelizer_seconds": t_gpu, "oracle_voxelizer_seconds": t_orc}
    body = g.reshape(dims[2], dims[1], dims[0]).astype(bool)
    center = (nx // 4 - dims[0] // 2, ny // 2 - dims[1] // 2, nz // 2 - dims[2] // 2)
    case = cases.body_in_channel(nx, ny, nz, body_flags=body, center=center)
    drag = {}
    for st in ("f64", "f32"):
        s = Solver(shape, turbulence=OmegaLES, inlet=InletVelocityEquilibrium, storage=st, nu=case["nu"], cles=0.17,
                   periodic=case["periodic"])
        s.set_flags(case["flags"])
        s.set_bc(case["inlets"], case["outlets"])
        s.init_equilibrium(1.0, (0.04, 0.0, 0.0))
        t0 = time.time()
        s.step(steps)
        d = s.reduce()
        drag[st] = np.array(d.drag)
        out[f"{st}_seconds"] = time.time() - t0
        out[f"{st}_drag"] = list(d.drag)
        out[f"{st}_nonfinite"] = d.nonfinite
        s.close()
    out["drag_x_rel_diff_f32_vs_f64"] = float(abs(drag["f32"][0] - drag["f64"][0]) / abs(drag["f64"][0]))
    return out


def _box(f, w):
    nz, ny, nx = f.shape
    return f.reshape(nz // w, w, ny // w, w, nx // w, w).mean(axis=(1, 3, 5))


def c2_a_priori(fine, warmup, every, snapshots, seed, model_path):
    """The shipped channel model on channel realisations it never saw: a run of the config-2 channel on the
    fine lattice with another seed, filtered samples at several times; per snapshot the relative
    subgrid-stress and dissipation errors of the network, of Smagorinsky with the constant fitted to the
    model's training samples (lb_gb300/data/les_mlp_channel.json), with the constant fitted to that very
    snapshot (the best any constant can do there) and with CLES 0.17."""
    from lb_gb300 import les
    model = les.MlpModel.load(model_path)
    with open(model_path.replace(".npz", ".json")) as fh:
        c_train = json.load(fh)["best_constant"]
    c = cases.channel(*fine, re_tau=180.0, u_max=0.05, amp=0.05, modes=0.25, seed=seed)
    s = Solver(fine, turbulence=OmegaLES, storage="f32", nu=c["nu"], cles=0.17, periodic=c["periodic"],
               force=c["force"])
    s.set_flags(c["flags"])
    s.set_bc()
    s.init_fields(c["rho"], c["u"])
    s.step(warmup)
    rows = []
    for k in range(snapshots):
        if k:
            s.step(every)
        smp = s.les_samples(4)
        nu_net, ok = les.evaluate(model, smp[:, :7])
        nu = np.where(ok, nu_net, les.smagorinsky_nu(smp, 0.17))
        c_self = les.best_constant(smp)
        rows.append({"step": warmup + k * every, "samples": int(smp.shape[0]), "in_range": float(ok.mean()),
                     "sgs_mlp": les.sgs_error(nu, smp),
                     "sgs_const_train": les.sgs_error(les.smagorinsky_nu(smp, c_train), smp),
                     "sgs_const_self": les.sgs_error(les.smagorinsky_nu(smp, c_self), smp),
                     "sgs_cles_0.17": les.sgs_error(les.smagorinsky_nu(smp, 0.17), smp),
                     "diss_mlp": les.sgs_dissipation_error(nu, smp),
                     "diss_const_train": les.sgs_dissipation_error(les.smagorinsky_nu(smp, c_train), smp),
                     "diss_const_self": les.sgs_dissipation_error(les.smagorinsky_nu(smp, c_self), smp)})
    s.close()
    out = {"config": "C2 channel, learned closure a priori on unseen realisations", "fine": list(fine),
           "seed": seed, "model": os.path.relpath(model_path, ROOT), "const_train": c_train, "snapshots": rows}
    for key in ("sgs_mlp", "sgs_const_train", "sgs_const_self", "diss_mlp", "diss_const_train", "diss_const_self"):
        v = np.array([r[key] for r in rows])
        out[key + "_mean"] = float(v.mean())
        out[key + "_min_max"] = [float(v.min()), float(v.max())]
    gain = np.array([r["sgs_const_self"] - r["sgs_mlp"] for r in rows])
    out["sgs_gain_over_self_fitted_constant_mean_std"] = [float(gain.mean()), float(gain.std())]
    return out


def c5(n, steps, ks, models):
    """models: {name: path of an lb_gb300.les.MlpModel}; ks: the refresh intervals run beside every step."""
    from lb_gb300 import les
    from lb_gb300.solver import OmegaMLP
    nf = 4 * n
    nets = {name: les.MlpModel.load(path) for name, path in models.items() if os.path.exists(path)}
    nu_c = 1e-3 * (n / 128.0)  # coarse lattice viscosity; the fine run has 4x this (acoustic scaling)
    nu_f = 4.0 * nu_c
    out = {"config": "C5 decaying turbulence", "coarse": n, "fine": nf, "coarse_steps": steps,
           "fine_steps": 4 * steps, "nu_coarse": nu_c, "nu_fine": nu_f, "k0": 8, "u_rms": 0.04,
           "models": {name: os.path.relpath(models[name], ROOT) for name in nets}}
    t0 = time.time()
    uf = cases.decay_field(nf)
    out["field_seconds"] = time.time() - t0
    uc0 = np.stack([_box(uf[c], 4) for c in range(3)])
    # fine run (FP32, cumulant + Smagorinsky)
    s = Solver((nf, nf, nf), turbulence=OmegaLES, storage="f32", nu=nu_f, cles=0.17, periodic=(1, 1, 1))
    s.set_flags(np.ones((nf, nf, nf), np.int32))
    s.set_bc()
    s.init_fields(np.ones(nf ** 3), uf.reshape(3, -1))
    del uf
    out["fine_seconds"] = s.step_timed(4 * steps) * 1e-3
    samples = s.les_samples(4)
    u_fine = s.moments()[1]
    s.close()
    u_ref = np.stack([_box(u_fine[c].reshape(nf, nf, nf), 4) for c in range(3)])
    del u_fine
    # a priori on the filtered fine field
    nu_s = les.smagorinsky_nu(samples, 0.17)
    cb = les.best_constant(samples)
    out["samples"] = int(samples.shape[0])
    sgs = {"smagorinsky_cles_0.17": les.sgs_error(nu_s, samples),
           "smagorinsky_best_constant_of_this_field": les.sgs_error(les.smagorinsky_nu(samples, cb), samples),
           "no_model": 1.0}
    dis = {"smagorinsky_cles_0.17": les.sgs_dissipation_error(nu_s, samples), "no_model": 1.0}
    for name, m in nets.items():
        nu_net, ok = les.evaluate(m, samples[:, :7])
        nu_m = np.where(ok, nu_net, nu_s)
        out[f"in_range_fraction_{name}"] = float(ok.mean())
        sgs[f"mlp_{name}"] = les.sgs_error(nu_m, samples)
        dis[f"mlp_{name}"] = les.sgs_dissipation_error(nu_m, samples)
    out["a_priori_sgs_error"] = sgs
    out["a_priori_dissipation_error"] = dis
    # a posteriori: coarse FP16 LES from the filtered initial field
    runs = [("smagorinsky", None, 1)]
    for name in nets:
        runs += [(f"mlp_{name}", name, 1)] + [(f"mlp_{name}_every_{k}", name, k) for k in ks]
    post, thr = {}, {}
    for label, name, interval in runs:
        g = Solver((n, n, n), turbulence=OmegaMLP if name else OmegaLES, storage="f16dev", nu=nu_c, cles=0.17,
                   periodic=(1, 1, 1), mlp_interval=interval)
        g.set_flags(np.ones((n, n, n), np.int32))
        g.set_bc()
        g.init_fields(np.ones(n ** 3), uc0.reshape(3, -1))
        if name:
            g.load_mlp(nets[name])
        g.step(steps)
        u = g.moments()[1].reshape(3, n, n, n)
        ms = g.step_timed(steps)  # throughput on warm kernels, after the compared state is read
        g.close()
        post[label] = float(np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref))
        thr[label] = n ** 3 * steps / (ms * 1e-3) / 1e9
    out["a_posteriori_rel_l2_vs_filtered_fine"] = post
    out["a_posteriori_initial_field_vs_filtered_fine"] = float(np.linalg.norm(uc0 - u_ref) / np.linalg.norm(u_ref))
    out["coarse_glups_fp16"] = thr
    out["energy_ratio_filtered_fine_T_over_0"] = float(np.sum(u_ref ** 2) / np.sum(uc0 ** 2))
    return out


pytestmark = [pytest.mark.gpu, pytest.mark.slow]
SMALL = os.environ.get("LBM_VALIDATE_SMALL") == "1"


def _record(name, r):
    out = os.environ.get("LBM_VALIDATE_OUT")
    if out:
        os.makedirs(out, exist_ok=True)
        with open(os.path.join(out, f"validate_{name}.json"), "w") as fh:
            json.dump(r, fh, indent=1)
    print(json.dumps(r))


def test_c1_cavity(built_lib, oracle_lib):
    r = c1(32 if SMALL else 64, 500 if SMALL else 10000)
    _record("c1", r)
    assert r["max_abs_du_over_ulid_gpu64_vs_oracle64"] <= 1e-12
    assert r["max_abs_du_over_ulid_gpu32_vs_gpu64"] <= 1e-3


def test_c3_channel_precision(built_lib):
    shape = (128, 64, 64) if SMALL else (512, 256, 256)
    steps, avg = (1000, 250) if SMALL else (20000, 5000)
    r = c3(shape, steps, avg)
    _record("c3", r)
    for st in ("f32", "f16dev"):
        assert r[f"{st}_nonfinite"] == 0
    if SMALL:
        return
    assert r["f32_mean_velocity_rel_l2_vs_f64"] <= 1e-3
    assert r["f16dev_mean_velocity_rel_l2_vs_f64"] <= 1e-3


def test_c4_body(built_lib, oracle_lib):
    shape = (192, 96, 96) if SMALL else (384, 192, 192)
    r = c4(shape, 500 if SMALL else 4000)
    _record("c4", r)
    assert r["voxelizer_bit_exact"]
    assert r["f64_nonfinite"] == 0 and r["f32_nonfinite"] == 0
    if not SMALL:
        assert r["drag_x_rel_diff_f32_vs_f64"] <= 1e-3


def test_c2_learned_closure_a_priori(built_lib):
    fine = (256, 64, 64) if SMALL else (1024, 256, 256)
    warmup, every = (2000, 500) if SMALL else (30000, 3000)
    r = c2_a_priori(fine, warmup, every, 4, cases.SEED + 2,
                    os.path.join(ROOT, "lb_gb300", "data", "les_mlp_channel.npz"))
    _record("c2_a_priori", r)
    if SMALL:
        return
    # the subgrid-stress error is what the network was trained on; its dissipation error on unseen
    # realisations varies from snapshot to snapshot (reported, not asserted)
    assert r["sgs_mlp_mean"] < r["sgs_const_train_mean"]
    assert r["sgs_mlp_mean"] < r["sgs_const_self_mean"]


def test_c5_learned_closure(built_lib):
    data = os.path.join(ROOT, "lb_gb300", "data")
    models = {"channel": os.path.join(data, "les_mlp_channel.npz"),
              "channel_decay": os.path.join(data, "les_mlp_channel_decay.npz")}
    r = c5(64 if SMALL else 256, 50 if SMALL else 200, (8, 16), models)
    _record("c5", r)
    if SMALL:
        return
    post = r["a_posteriori_rel_l2_vs_filtered_fine"]
    assert post["mlp_channel_decay"] < post["smagorinsky"]
    assert post["mlp_channel_decay_every_8"] < post["smagorinsky"]
    assert post["mlp_channel_decay_every_16"] < post["smagorinsky"]
