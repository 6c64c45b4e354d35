"""GPU checks of the learned LES closure: filtered samples, training gradients and FP16 evaluation
against the CPU oracle (oracle/les_oracle.py); the fused step kernel's fallback; and what a network
trained on the GPU gains over the Smagorinsky closure on held-out filtered data."""
import numpy as np
import pytest

from lb_gb300 import capi, cases, les
from lb_gb300.solver import OmegaLES, OmegaMLP, Solver
from oracle import les_oracle as lo

pytestmark = pytest.mark.gpu


def fine_channel(shape, steps, snapshots=(), storage="f32", seed=cases.SEED):
    """FP32 cumulant + Smagorinsky channel; returns {step: samples} at the requested steps and the solver."""
    c = cases.channel(*shape, re_tau=180.0, u_max=0.05, amp=0.3, seed=seed)
    s = Solver(shape, turbulence=OmegaLES, storage=storage, nu=c["nu"], cles=0.17, periodic=c["periodic"],
               force=c["force"])
    s.set_flags(c["flags"])
    s.set_bc()
    s.init_fields(c["rho"], c["u"])
    out = {}
    done = 0
    for k in sorted(set(snapshots) | {steps}):
        s.step(k - done)
        done = k
        if k in snapshots:
            out[k] = s.les_samples(4)
    return out, s, c


def test_samples_match_oracle(built_lib):
    shape = (64, 34, 32)  # y: 32 fluid rows between the solid rows -> ny % 4 != 0 is left out
    snaps, s, c = fine_channel(shape, 120, snapshots=(120,))
    g = snaps[120]
    rho, u = s.moments()
    nx, ny, nz = shape
    solid = c["flags"].reshape(nz, ny, nx) == 0
    ref, idx = lo.samples_from_fields(rho.reshape(nz, ny, nx), u.reshape(3, nz, ny, nx), solid, 4, (1, 0, 1))
    s.close()
    assert g.shape == ref.shape and g.shape[0] > 100
    for k in range(10):
        col = ref[:, k]
        rms = np.sqrt(np.mean(col * col)) + 1e-30
        err = np.abs(g[:, k] - col) / rms
        assert np.quantile(err, 0.999) < 2e-3, (k, np.quantile(err, 0.999))
        assert err.max() < 5e-2, (k, err.max())


def _model_and_samples(seed=7, n=4096):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((n, 7)) * np.array([1e-4, 1e-7, 1e-11, 0.5, 0.2, 1e-3, 1e-3]) + \
        np.array([0, -1e-7, 0, 0, 0.9, 1.0, 2e-3])
    b = np.abs(rng.standard_normal(n)) * 1e-6 + 1e-8
    a = -np.abs(rng.standard_normal(n)) * 1e-9
    c = a * a / b + np.abs(rng.standard_normal(n)) * 1e-12
    s = np.concatenate([x, a[:, None], b[:, None], c[:, None]], axis=1).astype(np.float32)
    m = les.MlpModel.init_from_samples(s, seed=seed)
    return m, s


def test_gradient_matches_oracle(built_lib):
    m, s = _model_and_samples()
    t = les.Trainer(s)
    K = float(np.mean(s[:, 9].astype(np.float64)))
    assert abs(t.norm - K) <= 1e-6 * K
    for first, count in ((0, 4096), (128, 1000)):
        loss, g = t.gradient(m, first, count)
        ref_loss, ref_g = lo.loss_and_grad(m.params, s[first:first + count], m.in_mean, m.in_std, m.out_scale, t.norm)
        assert abs(loss - ref_loss) <= 1e-5 * abs(ref_loss)
        assert np.linalg.norm(g - ref_g) <= 1e-4 * np.linalg.norm(ref_g), np.linalg.norm(g - ref_g) / np.linalg.norm(ref_g)
    t.close()


def test_eval_matches_fp16_oracle(built_lib):
    m, s = _model_and_samples(seed=11)
    m.params[:] = np.random.default_rng(5).standard_normal(les.NPAR).astype(np.float32) * 0.3
    x = s[:1000, :7]
    nu, ok = les.evaluate(m, x)
    ref, ref_ok = lo.infer_fp16(m.params, x, m.in_mean, m.in_std, m.in_lo, m.in_hi, m.out_scale)
    assert np.array_equal(ok, ref_ok)
    # tanh.approx.f16x2 against the exact tanh of the emulation, FP16 activations: 2 % of nu
    rel = np.abs(nu - ref) / np.abs(ref)
    assert np.quantile(rel, 0.99) < 2e-2 and rel.max() < 5e-2, (np.quantile(rel, 0.99), rel.max())
    # inputs outside the range are flagged
    xo = x.copy()
    xo[::2, 6] = m.in_hi[6] * 2 + 1
    _, ok2 = les.evaluate(m, xo)
    assert not ok2[::2].any()


def test_eval_tcgen05_matches_warp_path_and_oracle(built_lib):
    """The network on tcgen05.mma (TMEM accumulators, one CTA per 256 inputs) against the warp-level
    mma.sync path and the FP16 oracle: the same FP16 operands and activation, FP32 sums in another order, so
    the two GPU paths agree to FP16 rounding of the hidden activations; 1,000 inputs (a partial last
    CTA) and 300 (a CTA with unused rows)."""
    m, s = _model_and_samples(seed=13)
    m.params[:] = np.random.default_rng(7).standard_normal(les.NPAR).astype(np.float32) * 0.3
    for n in (1000, 300):
        x = s[:n, :7]
        nu_w, ok_w = les.evaluate(m, x, path=capi.LBM_MLP_PATH_WARP_MMA)
        nu_t, ok_t = les.evaluate(m, x, path=capi.LBM_MLP_PATH_TCGEN05)
        assert np.array_equal(ok_w, ok_t)
        assert np.all(np.isfinite(nu_t))
        d = np.abs(nu_t - nu_w) / np.abs(nu_w)
        assert np.quantile(d, 0.99) < 2e-3 and d.max() < 2e-2, (n, np.quantile(d, 0.99), d.max())
        ref, _ = lo.infer_fp16(m.params, x, m.in_mean, m.in_std, m.in_lo, m.in_hi, m.out_scale)
        rel = np.abs(nu_t - ref) / np.abs(ref)
        assert np.quantile(rel, 0.99) < 2e-2 and rel.max() < 5e-2, (n, np.quantile(rel, 0.99), rel.max())


@pytest.mark.parametrize("tc", [False, True])
@pytest.mark.parametrize("storage", ["f32", "f16dev"])
def test_fused_mlp_out_of_range_is_smagorinsky(built_lib, storage, tc):
    """A model whose training range excludes every input relaxes every cell with the Smagorinsky rate:
    the populations equal those of the Smagorinsky kernel bit for bit, with the rows beside the walls on
    the packed wall kernel (default) and on the per-cell path (LBM_OPT_NO_WALL_ROWS) in both runs."""
    shape = (64, 18, 12)
    c = cases.channel(*shape, re_tau=3.0, u_max=0.05, nu=0.01)
    m, _ = _model_and_samples()
    m.in_lo[:] = 1e30
    m.in_hi[:] = 2e30
    for wall_opt in (0, capi.LBM_OPT_NO_WALL_ROWS):
        out = []
        for clos in (OmegaLES, OmegaMLP):
            opts = wall_opt | (capi.LBM_OPT_MLP_TCGEN05 if tc else 0)
            s = Solver(shape, turbulence=clos, storage=storage, nu=c["nu"], cles=0.17, periodic=c["periodic"],
                       options=opts, force=c["force"])
            s.set_flags(c["flags"])
            s.set_bc()
            s.init_fields(c["rho"], c["u"])
            if clos is OmegaMLP:
                s.load_mlp(m)
            s.step(7)
            out.append(s.populations())
            s.close()
        assert np.array_equal(out[0], out[1]), wall_opt


@pytest.mark.parametrize("storage", ["f32", "f16dev"])
def test_interval_out_of_range_is_smagorinsky(built_lib, storage):
    """With a refresh interval the kept nu_t carry the fallback mark: an all-out-of-range model still
    reproduces the Smagorinsky kernel bit for bit (steps that run the network and steps that reuse)."""
    shape = (64, 18, 12)
    c = cases.channel(*shape, re_tau=3.0, u_max=0.05, nu=0.01)
    m, _ = _model_and_samples()
    m.in_lo[:] = 1e30
    m.in_hi[:] = 2e30
    for wall_opt in (0, capi.LBM_OPT_NO_WALL_ROWS):
        out = []
        for clos in (OmegaLES, OmegaMLP):
            s = Solver(shape, turbulence=clos, storage=storage, nu=c["nu"], cles=0.17, periodic=c["periodic"],
                       options=wall_opt, force=c["force"], mlp_interval=3)
            s.set_flags(c["flags"])
            s.set_bc()
            s.init_fields(c["rho"], c["u"])
            if clos is OmegaMLP:
                s.load_mlp(m)
            s.step(8)
            out.append(s.populations())
            s.close()
        assert np.array_equal(out[0], out[1]), wall_opt


def test_interval_tracks_every_step_evaluation(built_lib):
    """nu_t refreshed every 4th step stays close to the every-step evaluation (and is not identical)."""
    shape = (64, 34, 32)
    snaps, s, c = fine_channel(shape, 200, snapshots=(200,))
    s.close()
    m = les.MlpModel.init_from_samples(snaps[200])
    t = les.Trainer(snaps[200])
    t.train(m, epochs=20, batch=256, lr=3e-3)
    t.close()
    us = []
    for k in (1, 4):
        g = Solver(shape, turbulence=OmegaMLP, storage="f32", nu=c["nu"], cles=0.17, periodic=c["periodic"],
                   force=c["force"], mlp_interval=k)
        g.set_flags(c["flags"])
        g.set_bc()
        g.init_fields(c["rho"], c["u"])
        g.load_mlp(m)
        g.step(40)
        us.append(g.moments()[1])
        g.close()
    d = np.linalg.norm(us[0] - us[1]) / np.linalg.norm(us[0])
    assert 0.0 < d < 1e-3, d


def test_trained_closure_beats_smagorinsky(built_lib):
    """Filtered samples of a 4x-finer channel at two times train the network on the GPU; on a third,
    later time it must explain more of the filtered subgrid stress than the Smagorinsky closure (both as
    the solver runs it, CLES = 0.17, and with the constant fitted to the training samples)."""
    snaps, s, _ = fine_channel((128, 66, 64), 900, snapshots=(300, 600, 900))
    s.close()
    train = np.concatenate([snaps[300], snaps[600]])
    test = snaps[900]
    assert train.shape[0] > 4000 and test.shape[0] > 2000
    m = les.MlpModel.init_from_samples(train)
    t = les.Trainer(train)
    hist = t.train(m, epochs=150, batch=512, lr=3e-3)
    t.close()
    assert hist[-1] < hist[0]
    nu, ok = les.evaluate(m, test[:, :7])
    nu = np.where(ok, nu, les.smagorinsky_nu(test, 0.17))
    e_mlp = les.sgs_error(nu, test)
    e_smag = les.sgs_error(les.smagorinsky_nu(test, 0.17), test)
    cbest = les.best_constant(train)
    e_best = les.sgs_error(les.smagorinsky_nu(test, cbest), test)
    print(f"held-out relative SGS error: MLP {e_mlp:.4f}, Smagorinsky(0.17) {e_smag:.4f}, "
          f"Smagorinsky(C*={cbest:.4f}) {e_best:.4f}, in range {ok.mean():.3f}")
    assert e_mlp < e_best
    assert e_mlp < e_smag


def test_fused_mlp_channel_is_stable_and_conserves_mass(built_lib):
    """300 steps of the learned closure on a perturbed channel stay finite and keep the mass: to 2e-6 in
    FP32; in FP16 storage every stored value carries an independent stochastic-rounding error (zero mean,
    up to half an FP16 step, ~1e-5 in f here), so the mass does a random walk of about
    sqrt(27 x 70k stores x 300 steps) x 5e-6 ~ 0.1 (1.5e-6 relative): the bound there is 1e-5 (~6 sigma)."""
    shape = (64, 34, 32)
    snaps, s, c = fine_channel(shape, 200, snapshots=(200,))
    s.close()
    m = les.MlpModel.init_from_samples(snaps[200])
    t = les.Trainer(snaps[200])
    t.train(m, epochs=20, batch=256, lr=3e-3)
    t.close()
    for storage in ("f32", "f16dev"):
        g = Solver(shape, turbulence=OmegaMLP, storage=storage, nu=c["nu"], cles=0.17, periodic=c["periodic"],
                   force=c["force"])
        g.set_flags(c["flags"])
        g.set_bc()
        g.init_fields(c["rho"], c["u"])
        g.load_mlp(m)
        d0 = g.reduce()
        g.step(300)
        d1 = g.reduce()
        g.close()
        assert d1.nonfinite == 0
        assert abs(d1.mass - d0.mass) <= (2e-6 if storage == "f32" else 1e-5) * d0.mass


CV = np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 0, -1], [0, 0, 1], [0, -1, 0], [0, 1, 0], [1, 0, -1],
               [-1, 0, 1], [1, 0, 1], [-1, 0, -1], [-1, -1, 0], [1, 1, 0], [0, 1, -1], [0, -1, 1], [-1, 1, 0],
               [1, -1, 0], [0, 1, 1], [0, -1, -1], [-1, 1, -1], [1, -1, 1], [-1, -1, 1], [1, 1, -1], [1, -1, -1],
               [-1, 1, 1], [-1, -1, -1], [1, 1, 1]], np.float64)  # D3Q27.h:81-111 order


def oracle_learned_rate(f, force, tau, cles, m, smag_only=None):
    """The fused step's relaxation rate restated on the oracle's populations f[27, N] (float64): moments
    with the half-force velocity, Pi = M2 - rho (u u + I/3), the Smagorinsky time tau_S of OmegaLES.h:84-129,
    S = -3 Pi / (2 rho tau_S), the network's FP16 evaluation (les_oracle.infer_fp16) and
    omega = 1 / (tau + 3 nu_t) in range, 1 / tau_S outside and for the cells in `smag_only` (those beside a
    solid, which the kernel takes through its per-cell Smagorinsky path).  Returns (omega, nu_t, in_range,
    inputs)."""
    rho = f.sum(axis=0)
    j = CV.T @ f
    u = (j + 0.5 * np.asarray(force, np.float64)[:, None]) / rho
    M2 = np.einsum("va,vb,vn->abn", CV, CV, f)
    Pi = M2 - rho * (u[:, None, :] * u[None, :, :] + np.eye(3)[:, :, None] / 3.0)
    PI = np.sqrt((Pi * Pi).sum(axis=(0, 1)))
    tS = 0.5 * tau + 0.5 * np.sqrt(tau * tau + 18.0 * cles * PI / rho)
    sc = -1.5 / (rho * tS)
    S6 = np.stack([Pi[0, 0], Pi[1, 1], Pi[2, 2], Pi[0, 1], Pi[0, 2], Pi[1, 2]], axis=-1) * sc[:, None]
    x = lo.features(S6, rho)
    nu, ok = lo.infer_fp16(m.params, x, m.in_mean, m.in_std, m.in_lo, m.in_hi, m.out_scale)
    net = ok if smag_only is None else ok & ~smag_only
    om = np.where(net, 1.0 / (tau + 3.0 * np.where(net, nu, 0.0)), 1.0 / tS)
    return om, nu, ok, x


@pytest.mark.parametrize("tc", [False, True])
@pytest.mark.parametrize("storage", ["f32", "f16dev"])
def test_fused_learned_step_matches_oracle_step(built_lib, oracle_lib, storage, tc):
    """The headline kernel's learned path against the oracle: the GPU runs the network inside the
    collision kernel (k_step2_mlp, tensor-core FP16 network every step); the oracle runs the reference's
    cumulant step with, per cell and step, the relaxation rate of the same network restated on its own
    FP64 state (oracle_learned_rate), both from the oracle's state after 5 Smagorinsky steps.  The model's
    normalisation comes from the oracle's inputs there and its range covers 30 % of them (more as the
    strain decays), so both the network and the Smagorinsky fallback are exercised.
    Bounds: FP32 moments within 5e-5 u_max of the FP64 oracle after 24 steps on 99.9 % of the cells (the
    FP32 noise floor of the case is ~1e-5), 5e-4 u_max on every cell; FP16 storage 2e-3 relative L2 of u.  With a refresh interval of 2 (mode 1 on even
    steps) the kept nu_t read back from the GPU after a network step matches the oracle's nu_t of that
    step to 2 % at the 99th percentile (FP32; FP16 tanh.approx against the exact tanh), with the same
    in-range decision on >= 99 % of the cells, and the moments after 24 steps match, under the bounds
    above, a second oracle run that follows the refresh: on the odd steps each cell relaxes with
    1 / (tau + 3 nu_t) of its nu_t kept (in FP16) from the step before, the Smagorinsky rate of the current
    state where that step fell back.  tc: the network of the plain rows on tcgen05.mma
    (LBM_OPT_MLP_TCGEN05), under the same bounds."""
    from lb_gb300 import capi
    from lb_gb300.solver import CollisionCumD3Q27Turbulent2015
    from oracle import oracle as O
    shape = (48, 34, 16)
    nx, ny, nz = shape
    c = cases.channel(*shape, re_tau=180.0, u_max=0.05, amp=0.3)
    cfg = capi.make_config(*shape, periodic=c["periodic"], collision=capi.LBM_COLLISION_CUMULANT2015,
                           closure=capi.LBM_CLOSURE_SMAGORINSKY, nu=c["nu"], cles=0.17, force=c["force"])
    oracles = {}
    for interval in (1, 2):
        o = O.OracleSim(cfg, 64)
        o.set_flags(c["flags"])
        o.init_fields(c["rho"], c["u"])
        o.step(5)  # from the equilibrium start (Pi = 0 exactly) to a state with non-equilibrium stress
        oracles[interval] = o
    o = oracles[1]
    tau = 3.0 * c["nu"] + 0.5
    fl = c["flags"].reshape(-1) != 0
    # cells beside a solid take the per-cell path, which relaxes with the Smagorinsky rate
    solid = c["flags"].reshape(nz, ny, nx) == 0
    near = np.zeros_like(solid)
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                near |= np.roll(solid, (dz, dy, dx), axis=(0, 1, 2))
    smag_only = (near & ~solid).reshape(-1)[fl]
    f0 = o.populations().reshape(27, -1)
    _, _, _, x0 = oracle_learned_rate(f0[:, fl], c["force"], tau, 0.17,
                                      les.MlpModel(np.zeros(les.NPAR), np.zeros(7), np.ones(7), -np.full(7, 1e30),
                                                   np.full(7, 1e30), 1.0))
    rng = np.random.default_rng(3)
    lo_, hi_ = np.full(7, -1e30), np.full(7, 1e30)
    hi_[6] = np.quantile(x0[:, 6], 0.3)  # cells with larger |S| fall back (the strain decays over the run)
    m = les.MlpModel(rng.standard_normal(les.NPAR) * 0.3, x0.mean(axis=0), x0.std(axis=0) + 1e-30, lo_, hi_, 2e-4)
    g = {}
    for interval in (1, 2):
        s = Solver(shape, collision=CollisionCumD3Q27Turbulent2015, turbulence=OmegaMLP, storage=storage, nu=c["nu"],
                   cles=0.17, periodic=c["periodic"], force=c["force"], mlp_interval=interval,
                   options=capi.LBM_OPT_MLP_TCGEN05 if tc else 0)
        s.set_flags(c["flags"])
        s.set_bc()
        s.set_populations(f0)  # the oracle's state after its 5 Smagorinsky steps
        s.load_mlp(m)
        g[interval] = s
    steps = 24
    nu_chk = None
    nu_kept = None  # interval 2: nu_t of the last network step in FP16, -1 where it fell back
    everywhere = np.ones(int(fl.sum()), bool)
    for k in range(steps):
        f = o.populations().reshape(27, -1)
        om = np.zeros(f.shape[1])
        om_f, nu_f, ok_f, _ = oracle_learned_rate(f[:, fl], c["force"], tau, 0.17, m, smag_only)
        om[fl] = om_f
        o.set_omega_next(om)
        o.step(1)
        o2 = oracles[2]
        f2 = o2.populations().reshape(27, -1)
        om2 = np.zeros(f2.shape[1])
        if k % 2 == 0:
            om2_f, nu2, ok2, _ = oracle_learned_rate(f2[:, fl], c["force"], tau, 0.17, m, smag_only)
            nu_kept = np.where(ok2 & ~smag_only, nu2.astype(np.float16).astype(np.float64), -1.0)
        else:
            om_s, _, _, _ = oracle_learned_rate(f2[:, fl], c["force"], tau, 0.17, m, everywhere)
            om2_f = np.where(nu_kept >= 0, 1.0 / (tau + 3.0 * np.maximum(nu_kept, 0.0)), om_s)
        om2[fl] = om2_f
        o2.set_omega_next(om2)
        o2.step(1)
        for s in g.values():
            s.step(1)
        if k == steps - 2:  # interval 2: the network ran in this step (steps 0, 2, 4, ...)
            nu_chk = (nu_f, ok_f, g[2].eddy_viscosity()[fl])
    for interval, s in g.items():
        _, ug = s.moments()
        _, uo = oracles[interval].moments()
        s.close()
        oracles[interval].close()
        if storage == "f32":
            # a cell whose in-range decision differs between the GPU's FP32 features and the oracle's FP64
            # ones (allowed below on up to 1 % of the cells) relaxes at another rate in one of the two:
            # 99.9 % of the cells hold the bound, every cell 10x the bound
            d = np.abs(ug[:, fl] - uo[:, fl]).max(axis=0)
            assert np.quantile(d, 0.999) <= 5e-5 * 0.05 and d.max() <= 5e-4 * 0.05, (interval, np.quantile(d, 0.999), d.max())
        else:
            rel = np.linalg.norm(ug[:, fl] - uo[:, fl]) / np.linalg.norm(uo[:, fl])
            assert rel < 2e-3, (interval, rel)
    nu_o, ok_o, nu_g = nu_chk
    kept = np.isfinite(nu_g)  # packed bulk cells (the rows beside the walls relax with the Smagorinsky rate)
    assert kept.mean() > 0.8
    in_g = nu_g[kept] >= 0
    assert (in_g == ok_o[kept]).mean() >= 0.99
    assert 0.2 < in_g.mean() < 0.995  # both branches exercised
    if storage == "f32":
        both = kept.copy()
        both[kept] = in_g & ok_o[kept]
        rel = np.abs(nu_g[both] - nu_o[both]) / np.abs(nu_o[both])
        assert np.quantile(rel, 0.99) < 2e-2, np.quantile(rel, 0.99)
