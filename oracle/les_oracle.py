"""CPU oracle of the learned LES closure (test infrastructure only: tests and the checker import it;
the product path never does).

There is no reference counterpart: stloufra/LB has the Smagorinsky closure only
(3D/simulation/src/solvers/turbulence/OmegaLES.h:25-137).  This file restates, in float64 numpy,
what the CUDA library computes for the learned closure, so that the GPU kernels can be checked:
  - features(): the seven inputs of the strain rate and density (order of include/lbm.h);
  - samples_from_fields(): box filter of a fine run, strain rate by central differences of the
    filtered velocity, filtered stress and the error contractions (a, b, c);
  - loss_and_grad(): the training loss and its gradient w.r.t. the FP32 parameters (the forward and
    backward pass of the GPU training kernels, in float64);
  - infer_fp16(): the step kernel's FP16 evaluation (folded activation constants, FP16 weights and
    activations, FP32 accumulation), with an exact tanh in place of tanh.approx.f16x2.
Parity of these with the GPU is "parity unpinned" by reference data; the backward pass is pinned by
central finite differences of the forward pass (tests/test_les_cpu.py).
"""
import numpy as np

NIN, NH = 7, 32
GELU_A = 1.702
NPAR = NH * NH + 10 * NH + 1
# offsets of the parameter vector (w1[H][7], b1, w2[H][H], b2, w3, b3)
W1, B1, W2 = 0, 7 * NH, 8 * NH
B2 = W2 + NH * NH
W3 = B2 + NH
B3 = W3 + NH


def features(S, rho):
    """S: (..., 6) = xx, yy, zz, xy, xz, yz; rho: (...).  Returns (..., 7)."""
    S = np.asarray(S, np.float64)
    xx, yy, zz, xy, xz, yz = (S[..., i] for i in range(6))
    tr = xx + yy + zz
    s2 = xx * xx + yy * yy + zz * zz + 2.0 * (xy * xy + xz * xz + yz * yz)

    def det3(a, b, c):
        return a * (b * c - yz * yz) - xy * (xy * c - yz * xz) + xz * (xy * yz - b * xz)

    t3 = tr / 3.0
    d2 = s2 - tr * t3
    detd = det3(xx - t3, yy - t3, zz - t3)
    with np.errstate(divide="ignore", invalid="ignore"):
        lode = np.where(d2 > 1e-30, 3.0 * np.sqrt(6.0) * detd / np.maximum(d2, 1e-30) ** 1.5, 0.0)
        frac = np.where(s2 > 1e-30, d2 / np.maximum(s2, 1e-30), 0.0)
    lode = np.clip(lode, -1.0, 1.0)
    return np.stack([tr, 0.5 * (tr * tr - s2), det3(xx, yy, zz), lode, frac, np.asarray(rho, np.float64),
                     np.sqrt(2.0 * s2)], axis=-1)


def _dd(A, B):
    return A[..., 0] * B[..., 0] + A[..., 1] * B[..., 1] + A[..., 2] * B[..., 2] + 2.0 * (
        A[..., 3] * B[..., 3] + A[..., 4] * B[..., 4] + A[..., 5] * B[..., 5])


def samples_from_fields(rho, u, solid, w, wrap):
    """rho (nz, ny, nx), u (3, nz, ny, nx), solid (nz, ny, nx) bool; w: filter width; wrap: (x, y, z).
    Returns (samples (n, 10), coarse index (n,)) in coarse-cell order, as lbm_les_samples."""
    nz, ny, nx = rho.shape
    cz, cy, cx = nz // w, ny // w, nx // w

    def box(f):
        f = f[:cz * w, :cy * w, :cx * w]
        return f.reshape(cz, w, cy, w, cx, w).mean(axis=(1, 3, 5))

    ux, uy, uz = u[0], u[1], u[2]
    R = box(rho)
    U = np.stack([box(ux), box(uy), box(uz)])
    UU = np.stack([box(ux * ux), box(uy * uy), box(uz * uz), box(ux * uy), box(ux * uz), box(uy * uz)])
    fluid = box((~solid).astype(np.float64)) == 1.0
    # wrap per coarse axis (x, y, z) only when the fine axis wraps and divides evenly
    wr = [wrap[0] and nx % w == 0, wrap[1] and ny % w == 0, wrap[2] and nz % w == 0]
    ok = fluid.copy()
    G = np.zeros((3, 3) + R.shape)  # G[a][b] = d U_b / d x_a
    for a, ax in enumerate((2, 1, 0)):  # x, y, z -> array axes
        n = R.shape[ax]
        plus = np.roll(U, -1, axis=ax + 1)
        minus = np.roll(U, 1, axis=ax + 1)
        G[a] = 0.5 * (plus - minus)
        nb_ok = np.roll(fluid, -1, axis=ax) & np.roll(fluid, 1, axis=ax)
        if not wr[a]:
            edge = np.zeros(R.shape, bool)
            sl = [slice(None)] * 3
            sl[ax] = 0
            edge[tuple(sl)] = True
            sl[ax] = n - 1
            edge[tuple(sl)] = True
            nb_ok &= ~edge
        ok &= nb_ok
    S = np.stack([G[0][0], G[1][1], G[2][2], 0.5 * (G[0][1] + G[1][0]), 0.5 * (G[0][2] + G[2][0]),
                  0.5 * (G[1][2] + G[2][1])], axis=-1)
    T = np.stack([UU[0] - U[0] * U[0], UU[1] - U[1] * U[1], UU[2] - U[2] * U[2], UU[3] - U[0] * U[1],
                  UU[4] - U[0] * U[2], UU[5] - U[1] * U[2]], axis=-1)
    Sd = S.copy()
    st = S[..., :3].sum(-1) / 3.0
    Sd[..., :3] -= st[..., None]
    tt = T[..., :3].sum(-1) / 3.0
    T[..., :3] -= tt[..., None]
    x = features(S, R)
    out = np.concatenate([x, _dd(T, Sd)[..., None], _dd(Sd, Sd)[..., None], _dd(T, T)[..., None]], axis=-1)
    idx = np.flatnonzero(ok.reshape(-1))
    return out.reshape(-1, 10)[idx], idx


# ---- training model (float64) --------------------------------------------------------------------------
def _sig(x):
    return 1.0 / (1.0 + np.exp(-x))


def _gelu(x):
    return x * _sig(GELU_A * x)


def _gelu_grad(x):
    s = _sig(GELU_A * x)
    return s + GELU_A * x * s * (1.0 - s)


def _softplus(z):
    return np.maximum(z, 0.0) + np.log1p(np.exp(-np.abs(z)))


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[W1:B1].reshape(NH, NIN), p[B1:W2], p[W2:B2].reshape(NH, NH), p[B2:W3], p[W3:B3], p[B3])


def forward(p, x, mean, std, scale):
    w1, b1, w2, b2, w3, b3 = unpack(p)
    xh = (np.asarray(x, np.float64) - mean) / std
    pre1 = xh @ w1.T + b1
    h1 = _gelu(pre1)
    pre2 = h1 @ w2.T + b2
    h2 = _gelu(pre2)
    z = h2 @ w3 + b3
    return scale * _softplus(z), (xh, pre1, h1, pre2, h2, z)


def loss_and_grad(p, samples, mean, std, scale, K):
    """Mean over samples of (c + 4 nu a + 4 nu^2 b) / K and its gradient (float64)."""
    s = np.asarray(samples, np.float64)
    a, b, c = s[:, 7], s[:, 8], s[:, 9]
    nu, (xh, pre1, h1, pre2, h2, z) = forward(p, s[:, :NIN], mean, std, scale)
    n = s.shape[0]
    loss = np.mean(c + 4.0 * nu * a + 4.0 * nu * nu * b) / K
    dnu = (4.0 * a + 8.0 * nu * b) / K / n
    dz = dnu * scale * _sig(z)
    w1, b1, w2, b2, w3, b3 = unpack(p)
    g = np.zeros(NPAR)
    g[W3:B3] = dz @ h2
    g[B3] = dz.sum()
    d2 = (dz[:, None] * w3[None, :]) * _gelu_grad(pre2)
    g[W2:B2] = (d2.T @ h1).reshape(-1)
    g[B2:W3] = d2.sum(0)
    d1 = (d2 @ w2) * _gelu_grad(pre1)
    g[W1:B1] = (d1.T @ xh).reshape(-1)
    g[B1:W2] = d1.sum(0)
    return loss, g


# ---- the step kernel's FP16 evaluation -------------------------------------------------------------
def _h(x):
    return np.asarray(x, np.float64).astype(np.float16).astype(np.float64)


def infer_fp16(p, x, mean, std, lo, hi, scale):
    """nu_t and in-range flags as the step kernel computes them: FP16 inputs and folded FP16 weights
    (z = 0.851 x, the activation z (1 + tanh z) with the 1/1.702 in the next layer's weights), sums in
    float64, each activation rounded to FP16, with an exact tanh in place of tanh.approx.f16x2."""
    w1, b1, w2, b2, w3, b3 = unpack(p)
    hA = 0.5 * GELU_A
    x = np.asarray(x, np.float64)
    # normalised input = fma(x, isd, nmi) in FP32: the product of two floats is exact in float64
    isd = (np.float32(1.0) / np.asarray(std, np.float32)).astype(np.float64)
    nmi = (-(np.asarray(mean, np.float32) * isd.astype(np.float32))).astype(np.float64)

    def fma32(a):
        return (np.asarray(a, np.float32).astype(np.float64) * isd + nmi).astype(np.float32).astype(np.float64)

    xn = fma32(x)
    lo_n, hi_n = fma32(lo), fma32(hi)
    ok = np.all((xn >= lo_n) & (xn <= hi_n), axis=1)
    xin = np.concatenate([_h(xn), np.ones((x.shape[0], 1))], axis=1)
    W1e = _h(np.concatenate([(hA * w1).astype(np.float32), (hA * b1).astype(np.float32)[:, None]], axis=1))
    W2e = _h((hA / GELU_A * w2).astype(np.float32))
    B2e = (hA * b2).astype(np.float32).astype(np.float64)
    W3e = _h((w3 / GELU_A).astype(np.float32))

    def act(v):
        zq = _h(v)
        t = _h(np.tanh(zq))
        return _h(zq * t + zq)

    a1 = act(xin @ W1e.T)
    a2 = act(a1 @ W2e.T + B2e)
    zz = a2 @ W3e
    return scale * _softplus(zz + b3), ok
