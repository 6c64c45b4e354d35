"""CPU checks of the learned-closure oracle (oracle/les_oracle.py): the backward pass against central
finite differences of the forward pass, the invariance of the inputs under rotations, the Lode
parameter of the two axisymmetric strain states, and the filtered samples of a linear shear flow
against their closed form."""
import numpy as np
import pytest

from oracle import les_oracle as lo


def _samples(n, rng):
    x = rng.standard_normal((n, 7))
    a = -np.abs(rng.standard_normal(n)) * 1e-3
    b = np.abs(rng.standard_normal(n)) * 1e-2 + 1e-4
    c = np.abs(rng.standard_normal(n)) * 1e-4 + a * a / b  # c >= a^2/b keeps the error non-negative
    return np.concatenate([x, a[:, None], b[:, None], c[:, None]], axis=1)


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    s = _samples(64, rng)
    p = rng.standard_normal(lo.NPAR) * 0.3
    mean, std = rng.standard_normal(7) * 0.1, 1.0 + rng.random(7)
    scale, K = 0.02, float(np.mean(s[:, 9]))
    _, g = lo.loss_and_grad(p, s, mean, std, scale, K)
    h = 1e-6
    idx = np.concatenate([rng.choice(lo.NPAR, 60, replace=False), [lo.B3, lo.B1, lo.B2, lo.W3]])
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (lo.loss_and_grad(pp, s, mean, std, scale, K)[0] - lo.loss_and_grad(pm, s, mean, std, scale, K)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-8, (i, fd, g[i])


def test_features_are_rotation_invariant():
    rng = np.random.default_rng(5)
    for _ in range(20):
        A = rng.standard_normal((3, 3)) * 1e-3
        S = 0.5 * (A + A.T)
        Q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
        S2 = Q @ S @ Q.T

        def six(M):
            return np.array([M[0, 0], M[1, 1], M[2, 2], M[0, 1], M[0, 2], M[1, 2]])

        f1 = lo.features(six(S), 1.01)
        f2 = lo.features(six(S2), 1.01)
        scale = np.array([1e-3, 1e-6, 1e-9, 1, 1, 1, 1e-3])
        assert np.allclose(f1 / scale, f2 / scale, atol=1e-9)


@pytest.mark.parametrize("diag,lode", [((2.0, -1.0, -1.0), 1.0), ((-2.0, 1.0, 1.0), -1.0), ((1.0, -1.0, 0.0), 0.0)])
def test_lode_parameter(diag, lode):
    S = np.array([diag[0], diag[1], diag[2], 0.0, 0.0, 0.0]) * 1e-3
    f = lo.features(S, 1.0)
    assert abs(f[3] - lode) < 1e-12
    assert abs(f[4] - 1.0) < 1e-12  # traceless: all deviatoric
    assert abs(f[6] - np.sqrt(2.0 * np.sum(np.array(diag) ** 2)) * 1e-3) < 1e-15


def test_samples_of_linear_shear():
    """u_x = g y on a periodic box: filtered velocity is linear, S_xy = g/2 per fine cell = g w / 2 per
    coarse cell, and tau_xx = g^2 (w^2 - 1) / 12 (variance of y over w fine cells)."""
    w, g = 4, 1e-3
    nz, ny, nx = 16, 24, 20
    y = np.arange(ny, dtype=np.float64)
    u = np.zeros((3, nz, ny, nx))
    u[0] = g * y[None, :, None]
    rho = np.ones((nz, ny, nx))
    solid = np.zeros((nz, ny, nx), bool)
    s, idx = lo.samples_from_fields(rho, u, solid, w, (1, 0, 1))
    cz, cy, cx = nz // w, ny // w, nx // w
    # y is not periodic: the first and last coarse rows have no central difference
    J = (idx // cx) % cy
    assert set(J.tolist()) == set(range(1, cy - 1))
    assert len(idx) == cz * (cy - 2) * cx
    S_xy = g * w / 2.0
    tau_xx = g * g * (w * w - 1) / 12.0
    td = np.array([2.0, -1.0, -1.0]) * tau_xx / 3.0  # deviatoric diagonal of diag(tau_xx, 0, 0)
    a = 0.0  # tau_d (diagonal) : S_d (off-diagonal)
    b = 2.0 * S_xy ** 2
    c = np.sum(td ** 2)
    assert np.allclose(s[:, 7], a, atol=1e-18)
    assert np.allclose(s[:, 8], b, rtol=1e-12)
    assert np.allclose(s[:, 9], c, rtol=1e-9)
    assert np.allclose(s[:, 6], np.sqrt(2.0 * b), rtol=1e-12)  # |S| = sqrt(2 S:S)
    assert np.allclose(s[:, 3], 0.0, atol=1e-12)  # simple shear: Lode parameter 0


def test_infer_fp16_tracks_float64_forward():
    """The FP16 emulation of the step kernel stays within FP16 precision of the float64 forward."""
    rng = np.random.default_rng(9)
    p = rng.standard_normal(lo.NPAR) * 0.2
    x = rng.standard_normal((256, 7))
    mean, std = np.zeros(7), np.ones(7)
    nu64, _ = lo.forward(p, x, mean, std, 0.01)
    nu16, ok = lo.infer_fp16(p, x, mean, std, -np.full(7, 10.0), np.full(7, 10.0), 0.01)
    assert ok.all()
    assert np.max(np.abs(nu16 - nu64) / (np.abs(nu64) + 1e-4)) < 3e-2
