"""Seeded synthetic cases (lattice units) built on the reference's flag encoding.

Flag fields are int32 [z, y, x] (x fastest in memory, as the reference's mesh matrix,
postprocesors/outputerMesh.h:45-53): 0 solid, >0 fluid (after the wall pass, 1 + number of solid
cells in the 26-neighbourhood, geometry/geometryMesherBoundary.h:439-484), -1 inlet / moving-wall
node, -2 outlet node.  Random numbers come from a counter-based splitmix64 of (seed, cell, component)
so any process reproduces them.
"""
import math

import numpy as np

from . import capi

SEED = 0x5EED2026
_M64 = (1 << 64) - 1


def splitmix64(x):
    """Vectorised splitmix64 finaliser on uint64 arrays."""
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(_M64)
    z = x
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def uniform(seed, index, component):
    """U[0,1) per (seed, index, component); index is an integer array."""
    with np.errstate(over="ignore"):
        key = np.uint64(seed) * np.uint64(0x100000001B3) + np.asarray(index, dtype=np.uint64) * np.uint64(8) + np.uint64(component)
        r = splitmix64(splitmix64(key))
    return (r >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))


def wall_pass(flags):
    """geometryMesherBoundary::meshingBoundaryWall via the C ABI (host code)."""
    import ctypes as C
    f = np.ascontiguousarray(flags, dtype=np.int32)
    nz, ny, nx = f.shape
    capi.check(capi.lib().lbm_mesher_wall_pass(f.ctypes.data_as(C.POINTER(C.c_int32)), nx, ny, nz))
    return f


def write_mesh_matrix(path, flags, resolution, additional, bbox):
    """flags [z, y, x] to the reference's mesh-matrix text file (lbm_mesh_matrix_write)."""
    import ctypes as C
    f = np.ascontiguousarray(flags, dtype=np.int32)
    nz, ny, nx = f.shape
    dims = np.array([nx, ny, nz], np.int32)
    bb = np.ascontiguousarray(bbox, dtype=np.float64)
    L = capi.lib()
    st = L.lbm_mesh_matrix_write(path.encode(), f.ctypes.data_as(C.POINTER(C.c_int32)),
                                 dims.ctypes.data_as(C.POINTER(C.c_int32)), float(resolution), float(additional),
                                 bb.ctypes.data_as(C.POINTER(C.c_double)))
    if st:
        raise capi.LbmError(st, L.lbm_mesh_matrix_last_error().decode())


def read_mesh_matrix(path):
    """The reference's mesh-matrix text file: (flags [z, y, x] int32, resolution, additional, bbox)."""
    import ctypes as C
    L = capi.lib()
    dims = np.zeros(3, np.int32)
    res, add = C.c_double(0), C.c_double(0)
    bb = np.zeros(6)
    args = (dims.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(res), C.byref(add), bb.ctypes.data_as(C.POINTER(C.c_double)))
    st = L.lbm_mesh_matrix_read(path.encode(), None, 0, *args)
    if st:
        raise capi.LbmError(st, L.lbm_mesh_matrix_last_error().decode())
    f = np.zeros(int(dims.prod()), np.int32)
    st = L.lbm_mesh_matrix_read(path.encode(), f.ctypes.data_as(C.POINTER(C.c_int32)), f.size, *args)
    if st:
        raise capi.LbmError(st, L.lbm_mesh_matrix_last_error().decode())
    return f.reshape(dims[2], dims[1], dims[0]), res.value, add.value, bb


def wall_pass_numpy(flags):
    """Same count in numpy (no library needed): fluid cells get 1 + #solid 26-neighbours."""
    f = np.asarray(flags, dtype=np.int32).copy()
    solid = (f == 0)
    pad = np.pad(solid, 1, constant_values=False)
    cnt = np.zeros_like(f)
    nz, ny, nx = f.shape
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                cnt += pad[1 + dz:1 + dz + nz, 1 + dy:1 + dy + ny, 1 + dx:1 + dx + nx]
    m = f > 0
    f[m] += cnt[m]
    return f


# ---- config 1: lid-driven cavity --------------------------------------------------------------------
def cavity(n=64, u_lid=0.05, re=1000.0, wall=wall_pass_numpy):
    """n^3 box: solid at x=0, x=n-1, y=0, z=0, z=n-1; the top plane y=n-1 (inside the side walls) is
    moving-wall nodes (flag -1, normal +y, velocity (u_lid,0,0)); nu = u_lid * n / Re."""
    f = np.ones((n, n, n), dtype=np.int32)
    f[:, :, 0] = 0; f[:, :, -1] = 0
    f[:, 0, :] = 0
    f[0, :, :] = 0; f[-1, :, :] = 0
    f[1:-1, -1, 1:-1] = -1
    f = wall(f)
    lid = [capi.make_inlet(i, n - 1, k, (0, 1, 0), (u_lid, 0, 0)) for k in range(1, n - 1) for i in range(1, n - 1)]
    return {"flags": f, "inlets": lid, "outlets": [], "nu": u_lid * n / re, "periodic": (0, 0, 0)}


# ---- configs 2/3: turbulent channel -------------------------------------------------------------------
def channel_modes(nx, ny, nz, h, rms, seed, n_modes=12):
    """Divergence-free large-scale perturbation that vanishes at the walls: u = curl(chi, 0, psi) with
    psi, chi = sum of g(eta) sin(k_x x + k_z z + phase), g = sin^2(pi eta), eta = (y - 0.5) / (2h), over
    seeded modes k_x = 2 pi m_x / nx, k_z = 2 pi m_z / nz (m = 1..4).  Each component is a y-profile
    times an (x, z) plane, so the field costs O(N).  Returns (3, nz, ny, nx) scaled to the given rms."""
    rng = np.random.default_rng(seed)
    y = np.arange(ny, dtype=np.float64)
    eta = np.clip((y - 0.5) / (2.0 * h), 0.0, 1.0)
    g = np.sin(np.pi * eta) ** 2
    dg = np.pi * np.sin(2.0 * np.pi * eta) / (2.0 * h)  # d g / d y
    dg[(eta <= 0.0) | (eta >= 1.0)] = 0.0
    x = np.arange(nx, dtype=np.float64)[None, :]
    z = np.arange(nz, dtype=np.float64)[:, None]
    pu = np.zeros((nz, nx))
    pv = np.zeros((nz, nx))
    pw = np.zeros((nz, nx))
    for _ in range(n_modes):
        kx = 2.0 * np.pi * rng.integers(1, 5) / nx
        kz = 2.0 * np.pi * rng.integers(1, 5) / nz
        a, b = rng.standard_normal(2)
        ph1, ph2 = rng.uniform(0.0, 2.0 * np.pi, 2)
        t1 = kx * x + kz * z + ph1
        t2 = kx * x + kz * z + ph2
        pu += a * np.sin(t1)                              # u = d psi / d y
        pv += -a * kx * np.cos(t1) + b * kz * np.cos(t2)  # v = -d psi / d x + d chi / d z
        pw += -b * np.sin(t2)                             # w = -d chi / d y
    u = np.empty((3, nz, ny, nx))
    u[0] = dg[None, :, None] * pu[:, None, :]
    u[1] = g[None, :, None] * pv[:, None, :]
    u[2] = dg[None, :, None] * pw[:, None, :]
    cur = np.sqrt(np.mean(u * u))
    if cur > 0:
        u *= rms / cur
    return u


def channel(nx, ny, nz, re_tau=180.0, u_max=0.05, amp=0.05, seed=SEED, nu=None, wall=wall_pass_numpy, modes=0.0):
    """Periodic in x and z, bounce-back solid rows y=0 and y=ny-1 (walls at y=0.5 and ny-1.5, half
    height h=(ny-2)/2).  Body force F_x = u_tau^2/h for Re_tau = u_tau h / nu.  nu (builder's
    choice when not given): the turbulent centre-line velocity of a Re_tau = 180 channel is about
    18.3 u_tau, so u_tau = u_max / 18.3 and nu = u_tau h / Re_tau (tau = 0.5058 at h = 127).
    Initial velocity: laminar profile, uniform seeded noise of amplitude amp * u_max per cell and
    component, and (modes > 0) the divergence-free large-scale perturbation of rms modes * u_max."""
    f = np.ones((nz, ny, nx), dtype=np.int32)
    f[:, 0, :] = 0
    f[:, -1, :] = 0
    f = wall(f)
    h = (ny - 2) / 2.0
    if nu is None:
        nu = (u_max / 18.3) * h / re_tau
    u_tau = re_tau * nu / h
    force = (u_tau * u_tau / h, 0.0, 0.0)
    y = np.arange(ny, dtype=np.float64)
    yc = (ny - 1) / 2.0
    prof = u_max * (1.0 - ((y - yc) / h) ** 2)
    prof[[0, -1]] = 0.0
    N = nx * ny * nz
    idx = np.arange(N, dtype=np.uint64)
    u = np.zeros((3, N))
    for a in range(3):
        u[a] = (uniform(seed, idx, a) * 2.0 - 1.0) * amp * u_max
    u[0] += np.broadcast_to(prof[None, :, None], (nz, ny, nx)).reshape(-1)
    if modes > 0.0:
        u += channel_modes(nx, ny, nz, h, modes * u_max, seed).reshape(3, -1)
    solid = f.reshape(-1) == 0
    u[:, solid] = 0.0
    rho = np.ones(N)
    return {"flags": f, "inlets": [], "outlets": [], "nu": nu, "periodic": (1, 0, 1), "force": force,
            "rho": rho, "u": u, "h": h, "u_tau": u_tau}


def symmetric_channel(nx, h_rows, nz, u_max=0.05, amp=0.05, seed=SEED, nu=0.02, re_tau=3.0, wall=wall_pass_numpy):
    """A periodic (x, z) channel cut at its mid-plane by a BounceSymmetryHalf plane, and the full channel
    it stands for.  Half: solid row y=0, fluid rows 1..h_rows with the last one -2 symmetry nodes (normal
    +y; regular when the wall pass gave them 10), solid row h_rows+1 across the plane.  Full: fluid rows
    1..2 h_rows between solid rows 0 and 2 h_rows+1; its initial field is the half's mirrored about
    y = h_rows + 1/2 (u_y changes sign), so the two runs agree on rows 0..h_rows.  Laminar profile plus
    seeded noise, body force F_x = u_tau^2 / h for Re_tau = u_tau h / nu.  Returns (half, full)."""
    H = int(h_rows)
    h = float(H)
    u_tau = re_tau * nu / h
    force = (u_tau * u_tau / h, 0.0, 0.0)
    fh = np.ones((nz, H + 2, nx), dtype=np.int32)
    fh[:, 0, :] = 0
    fh[:, H + 1, :] = 0
    fh = wall(fh)
    regular = fh[:, H, :] == 10
    fh[:, H, :] = -2
    sym = [capi.make_symmetry(i, H, k, (0, 1, 0), int(regular[k, i])) for k in range(nz) for i in range(nx)]
    y = np.arange(H + 2, dtype=np.float64)
    prof = u_max * (1.0 - ((y - (H + 0.5)) / h) ** 2)
    prof[[0, -1]] = 0.0
    Nh = nx * (H + 2) * nz
    idx = np.arange(Nh, dtype=np.uint64)
    uh = np.zeros((3, Nh))
    for a in range(3):
        uh[a] = (uniform(seed, idx, a) * 2.0 - 1.0) * amp * u_max
    uh[0] += np.broadcast_to(prof[None, :, None], (nz, H + 2, nx)).reshape(-1)
    uh[:, (fh.reshape(-1) == 0)] = 0.0
    half = {"flags": fh, "inlets": [], "outlets": [], "symmetry": sym, "nu": nu, "periodic": (1, 0, 1),
            "force": force, "rho": np.ones(Nh), "u": uh}
    ff = np.ones((nz, 2 * H + 2, nx), dtype=np.int32)
    ff[:, 0, :] = 0
    ff[:, -1, :] = 0
    ff = wall(ff)
    u3 = uh.reshape(3, nz, H + 2, nx)
    uf = np.zeros((3, nz, 2 * H + 2, nx))
    uf[:, :, :H + 1, :] = u3[:, :, :H + 1, :]
    mir = u3[:, :, H:0:-1, :].copy()        # rows H..1 -> rows H+1..2H
    mir[1] *= -1.0
    uf[:, :, H + 1:2 * H + 1, :] = mir
    full = {"flags": ff, "inlets": [], "outlets": [], "nu": nu, "periodic": (1, 0, 1), "force": force,
            "rho": np.ones(nx * (2 * H + 2) * nz), "u": uf.reshape(3, -1)}
    return half, full


def duct(nx, ny, nz, u_in=0.04, rho_out=1.0, nu=0.02, amp=0.3, seed=SEED):
    """Inlet plane x=0 (-1 nodes, normal -x, u=(u_in,0,0)), outlet plane x=nx-1 (-2 nodes, normal +x,
    rho_out), periodic y and z, no walls; initial field u_in plus seeded noise of amplitude amp * u_in
    per component (enough for some outlet nodes to start with u_x < 0)."""
    f = np.ones((nz, ny, nx), dtype=np.int32)
    f[:, :, 0] = -1
    f[:, :, -1] = -2
    inl = [capi.make_inlet(0, j, k, (-1, 0, 0), (u_in, 0, 0)) for k in range(nz) for j in range(ny)]
    out = [capi.make_outlet(nx - 1, j, k, (1, 0, 0), rho_out) for k in range(nz) for j in range(ny)]
    N = nx * ny * nz
    idx = np.arange(N, dtype=np.uint64)
    u = np.zeros((3, N))
    for a in range(3):
        u[a] = (uniform(seed, idx, a) * 2.0 - 1.0) * amp * u_in
    u[0] += u_in
    rho = 1.0 + 0.01 * (uniform(seed + 1, idx, 0) * 2.0 - 1.0)
    return {"flags": f, "inlets": inl, "outlets": out, "nu": nu, "periodic": (0, 1, 1), "rho": rho, "u": u}


# ---- config 4: flow past a seeded body ------------------------------------------------------------------
def icosphere(subdiv):
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    v = [np.asarray(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdiv):
        cache = {}
        nf = []

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                p = v[a] + v[b]
                v.append(p / np.linalg.norm(p))
                cache[key] = len(v) - 1
            return cache[key]

        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.asarray(v), np.asarray(faces, dtype=np.int32)


def _real_sph_harm(l, m, theta, phi):
    """Real spherical harmonic (unnormalised associated Legendre with Condon-Shortley phase)."""
    from scipy.special import lpmv
    x = np.cos(theta)
    am = abs(m)
    norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
    p = lpmv(am, l, x)
    if m > 0:
        return math.sqrt(2) * norm * p * np.cos(am * phi)
    if m < 0:
        return math.sqrt(2) * norm * p * np.sin(am * phi)
    return norm * p


def perturbed_icosphere(radius=24.0, subdiv=5, lmax=6, amp=0.15, seed=SEED, center=(0.0, 0.0, 0.0)):
    """Icosphere (20*4^subdiv faces) with r(theta,phi) = R (1 + s(theta,phi)), s = sum a_lm Y_lm over
    1 <= l <= lmax with a_lm ~ U(-1,1) from the seed, scaled so max |s| over the vertices = amp."""
    v, f = icosphere(subdiv)
    theta = np.arccos(np.clip(v[:, 2], -1, 1))
    phi = np.arctan2(v[:, 1], v[:, 0])
    s = np.zeros(len(v))
    k = 0
    for l in range(1, lmax + 1):
        for m in range(-l, l + 1):
            a = uniform(seed, np.asarray([k]), 7)[0] * 2.0 - 1.0
            s += a * _real_sph_harm(l, m, theta, phi)
            k += 1
    s *= amp / np.abs(s).max()
    r = radius * (1.0 + s)
    return v * r[:, None] + np.asarray(center)[None, :], f


def write_off(path, verts, faces):
    with open(path, "w") as fh:
        fh.write("OFF\n%d %d 0\n" % (len(verts), len(faces)))
        for p in verts:
            fh.write("%.17g %.17g %.17g\n" % tuple(p))
        for t in faces:
            fh.write("3 %d %d %d\n" % tuple(t))


def body_in_channel(nx=384, ny=192, nz=192, u_in=0.04, rho_out=1.0, nu=None, body_flags=None, center=None,
                    wall=wall_pass_numpy):
    """Inlet plane x=0 (-1 nodes, normal -x, u=(u_in,0,0)), outlet plane x=nx-1 (-2 nodes, normal +x,
    rho_out), periodic y and z, solid body cells from `body_flags` (True = solid) placed with its
    grid origin at `center` offset.  nu default: Re = u_in * D / nu = 200 with D = 48."""
    f = np.ones((nz, ny, nx), dtype=np.int32)
    if body_flags is not None:
        bz, by, bx = body_flags.shape
        ox, oy, oz = center
        f[oz:oz + bz, oy:oy + by, ox:ox + bx][body_flags] = 0
    f = wall(f)
    f[:, :, 0] = -1
    f[:, :, -1] = -2
    inl = [capi.make_inlet(0, j, k, (-1, 0, 0), (u_in, 0, 0)) for k in range(nz) for j in range(ny)]
    out = [capi.make_outlet(nx - 1, j, k, (1, 0, 0), rho_out) for k in range(nz) for j in range(ny)]
    if nu is None:
        nu = u_in * 48.0 / 200.0
    return {"flags": f, "inlets": inl, "outlets": out, "nu": nu, "periodic": (0, 1, 1)}


# ---- config 5: periodic decaying turbulence ------------------------------------------------------------
def decay_field(n, k0=8.0, urms=0.04, seed=SEED):
    """Random-phase solenoidal field on n^3 (box wavenumbers k = 2 pi m / n): amplitude
    sqrt(E(k) / (4 pi k^2)), E ~ k^4 exp(-2 (k/k0)^2), random complex vector projected normal to k,
    scaled to urms per component.  Returns u (3, n, n, n) float64 [z, y, x]."""
    try:
        from scipy import fft as sfft
        irfftn = lambda a: sfft.irfftn(a, s=(n, n, n), axes=(1, 2, 3), workers=-1)  # noqa: E731
    except ImportError:
        irfftn = lambda a: np.fft.irfftn(a, s=(n, n, n), axes=(1, 2, 3))  # noqa: E731
    rng = np.random.default_rng(seed)
    kz = np.fft.fftfreq(n, 1.0 / n).astype(np.float32)[:, None, None]
    ky = np.fft.fftfreq(n, 1.0 / n).astype(np.float32)[None, :, None]
    kx = np.fft.rfftfreq(n, 1.0 / n).astype(np.float32)[None, None, :]
    k2 = kx * kx + ky * ky + kz * kz
    k = np.sqrt(k2)
    with np.errstate(divide="ignore", invalid="ignore"):
        amp = np.where(k2 > 0, np.sqrt(k ** 4 * np.exp(-2.0 * (k / k0) ** 2) / (4.0 * np.pi * k2)), 0.0).astype(np.float32)
    shape = (n, n, n // 2 + 1)
    a = (rng.standard_normal((3,) + shape, dtype=np.float32) + 1j * rng.standard_normal((3,) + shape, dtype=np.float32))
    kv = (np.broadcast_to(kx, shape), np.broadcast_to(ky, shape), np.broadcast_to(kz, shape))
    with np.errstate(divide="ignore", invalid="ignore"):
        dot = (kv[0] * a[0] + kv[1] * a[1] + kv[2] * a[2]) / np.where(k2 > 0, k2, 1.0)
    for c in range(3):
        a[c] = (a[c] - kv[c] * dot) * amp
    u = irfftn(a)  # components x, y, z on [z, y, x]
    u *= urms / np.sqrt(np.mean(u * u))
    return u.astype(np.float64)
