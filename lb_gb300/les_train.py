"""Train the learned LES closure on filtered samples of a 4x-finer channel run of the solver.

    python -m lb_gb300.les_train --fine 1024,256,256 --warmup 30000 --every 3000 --snapshots 5 \
        --samples 4000000 --out les_mlp_channel.npz

1. A turbulent channel (periodic x, z; bounce-back walls; body force for Re_tau = 180; laminar profile
   plus seeded 5 % cell noise and a divergence-free large-scale perturbation of 25 % rms, which trips
   the transition) runs on the fine lattice in FP32 with the cumulant collision and the Smagorinsky
   closure.
2. After `warmup` steps, every `every` steps, Solver.les_samples(4) takes the box-filtered samples of
   the state (one per coarse cell of 4^3 fine cells).  The last snapshot is held out.
3. A seeded random subset of `samples` training samples trains the network on the GPU
   (lbm_mlp_train: Adam, minibatches of `batch`).
4. The report gives the relative subgrid-stress error sum|tau_d + 2 nu S_d|^2 / sum|tau_d|^2 on the
   held-out snapshot for the trained network, for the Smagorinsky closure as the solver runs it
   (CLES 0.17) and for the least-squares Smagorinsky constant of the training samples.

With --decay-fine M, half of the training samples come instead from a periodic decaying-turbulence run
of the solver on M^3 (the seeded random-phase field of lb_gb300.cases.decay_field with its own seed,
seed + 1, snapshots after M/2, M and 2M steps; the last one held out), so that the network also covers
the strain rates of that regime (far above the channel's in lattice units).
"""
import argparse
import json
import time

import numpy as np

from . import cases, les
from .solver import OmegaLES, Solver


def decay_snapshots(nf, seed, device=0, log=print):
    """Filtered samples of a periodic decaying-turbulence run on nf^3 (FP32, cumulant + Smagorinsky) after
    nf/2, nf and 2 nf steps; the coarse lattice has nu = 1e-3 (nf / 512), the fine run 4x that."""
    nu_f = 4.0 * 1e-3 * (nf / 512.0)
    u = cases.decay_field(nf, seed=seed)
    s = Solver((nf, nf, nf), turbulence=OmegaLES, storage="f32", nu=nu_f, cles=0.17, periodic=(1, 1, 1),
               device=device)
    s.set_flags(np.ones((nf, nf, nf), np.int32))
    s.set_bc()
    s.init_fields(np.ones(nf ** 3), u.reshape(3, -1))
    del u
    out, done = [], 0
    for k in (nf // 2, nf, 2 * nf):
        s.step(k - done)
        done = k
        out.append(s.les_samples(4))
        log(f"decay snapshot at step {k}: {out[-1].shape[0]} samples")
    s.close()
    return out, nu_f


def run(fine, warmup, every, snapshots, n_samples, epochs, batch, lr, seed, device=0, log=print, decay_fine=0):
    c = cases.channel(*fine, re_tau=180.0, u_max=0.05, amp=0.05, modes=0.25, seed=seed)
    s = Solver(fine, turbulence=OmegaLES, storage="f32", nu=c["nu"], cles=0.17, periodic=c["periodic"],
               force=c["force"], device=device)
    s.set_flags(c["flags"])
    s.set_bc()
    s.init_fields(c["rho"], c["u"])
    t0 = time.time()
    s.step(warmup)
    snaps = []
    for k in range(snapshots):
        if k:
            s.step(every)
        snaps.append(s.les_samples(4))
        d = s.reduce()
        log(f"snapshot {k} at step {warmup + k * every}: {snaps[-1].shape[0]} samples, "
            f"max |u| {d.max_speed:.4f}, nonfinite {d.nonfinite}")
    s.close()
    t_fine = time.time() - t0
    held = snaps[-1]
    pool = np.concatenate(snaps[:-1]) if len(snaps) > 1 else held
    rng = np.random.default_rng(seed)
    held_decay = None
    if decay_fine > 0:
        dsnaps, nu_decay = decay_snapshots(decay_fine, seed + 1, device, log)
        held_decay = dsnaps[-1]
        dpool = np.concatenate(dsnaps[:-1])
        nd = min(n_samples // 2, dpool.shape[0])
        nc = min(n_samples - nd, pool.shape[0])
        parts = [pool[np.sort(rng.choice(pool.shape[0], size=nc, replace=False))],
                 dpool[np.sort(rng.choice(dpool.shape[0], size=nd, replace=False))]]
        train = np.ascontiguousarray(np.concatenate(parts))
    else:
        pick = rng.choice(pool.shape[0], size=min(n_samples, pool.shape[0]), replace=False)
        train = np.ascontiguousarray(pool[np.sort(pick)])
    model = les.MlpModel.init_from_samples(train, seed=seed)
    t0 = time.time()
    tr = les.Trainer(train, device=device)
    hist = tr.train(model, epochs=epochs, batch=batch, lr=lr, seed=seed)
    tr.close()
    t_train = time.time() - t0
    nu_net, ok = les.evaluate(model, held[:, :7], device=device)
    nu_smag = les.smagorinsky_nu(held, 0.17)
    nu = np.where(ok, nu_net, nu_smag)
    cbest = les.best_constant(train)
    nu_best = les.smagorinsky_nu(held, cbest)
    inr = held[ok]
    report = {
        "fine_lattice": list(fine), "nu": c["nu"], "force": list(c["force"]), "warmup_steps": warmup,
        "snapshot_every": every, "snapshots": snapshots, "train_samples": int(train.shape[0]),
        "held_out_samples": int(held.shape[0]), "epochs": epochs, "batch": batch, "lr": lr, "seed": seed,
        "loss_first_epoch": float(hist[0]), "loss_last_epoch": float(hist[-1]),
        "held_out_sgs_error": {"mlp": les.sgs_error(nu, held),
                               "smagorinsky_cles_0.17": les.sgs_error(les.smagorinsky_nu(held, 0.17), held),
                               "smagorinsky_best_constant": les.sgs_error(les.smagorinsky_nu(held, cbest), held),
                               "no_model": 1.0},
        "held_out_sgs_error_in_range": {"mlp": les.sgs_error(nu_net[ok], inr),
                                        "smagorinsky_cles_0.17": les.sgs_error(nu_smag[ok], inr),
                                        "smagorinsky_best_constant": les.sgs_error(nu_best[ok], inr)},
        "held_out_dissipation_error": {"mlp": les.sgs_dissipation_error(nu, held),
                                       "smagorinsky_cles_0.17": les.sgs_dissipation_error(nu_smag, held),
                                       "smagorinsky_best_constant": les.sgs_dissipation_error(nu_best, held),
                                       "no_model": 1.0},
        "best_constant": cbest, "in_range_fraction": float(ok.mean()),
        "seconds_fine_run": t_fine, "seconds_training": t_train,
    }
    if held_decay is not None:
        nd_net, okd = les.evaluate(model, held_decay[:, :7], device=device)
        nd_s = les.smagorinsky_nu(held_decay, 0.17)
        nd_m = np.where(okd, nd_net, nd_s)
        cbd = les.best_constant(held_decay)
        report["decay_fine_lattice"] = decay_fine
        report["decay_nu_fine"] = nu_decay
        report["decay_held_out_sgs_error"] = {
            "mlp": les.sgs_error(nd_m, held_decay),
            "smagorinsky_cles_0.17": les.sgs_error(nd_s, held_decay),
            "smagorinsky_best_constant_of_this_field": les.sgs_error(les.smagorinsky_nu(held_decay, cbd), held_decay),
            "no_model": 1.0}
        report["decay_held_out_dissipation_error"] = {"mlp": les.sgs_dissipation_error(nd_m, held_decay),
                                                      "smagorinsky_cles_0.17": les.sgs_dissipation_error(nd_s, held_decay),
                                                      "no_model": 1.0}
        report["decay_in_range_fraction"] = float(okd.mean())
    return model, report


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--fine", default="1024,256,256")
    ap.add_argument("--warmup", type=int, default=30000)
    ap.add_argument("--every", type=int, default=3000)
    ap.add_argument("--snapshots", type=int, default=5)
    ap.add_argument("--samples", type=int, default=4_000_000)
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=0x5EED2026)
    ap.add_argument("--decay-fine", type=int, default=0,
                    help="also train on a decaying-turbulence run of this fine lattice (0: channel only)")
    ap.add_argument("--out", default="les_mlp_channel.npz")
    args = ap.parse_args()
    fine = tuple(int(v) for v in args.fine.split(","))
    model, report = run(fine, args.warmup, args.every, args.snapshots, args.samples, args.epochs, args.batch,
                        args.lr, args.seed, decay_fine=args.decay_fine)
    model.save(args.out)
    with open(args.out.replace(".npz", ".json"), "w") as f:
        json.dump(report, f, indent=1)
    print(json.dumps(report))


if __name__ == "__main__":
    main()
