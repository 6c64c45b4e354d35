"""Learned LES closure: model container, GPU training, evaluation and the a-priori subgrid error.

The network and its inputs are defined in include/lbm.h (lbm_mlp_model).  Training data are the
filtered samples of a run of the solver on a `width`-times finer lattice (Solver.les_samples): per
coarse cell the inputs x[7] of the filtered strain rate and density, and a = tau_d:S_d, b = S_d:S_d,
c = tau_d:tau_d, so that the subgrid-stress error of an eddy viscosity nu is c + 4 nu a + 4 nu^2 b.

Everything here calls the CUDA library (lb_gb300/liblbm_gb300.so); numpy is used only for set-up and
for the a-priori error sums.
"""
import ctypes as C

import numpy as np

from . import capi
from .capi import check, lib

NIN, NH, NPAR = capi.LBM_MLP_INPUTS, capi.LBM_MLP_HIDDEN, capi.LBM_MLP_PARAMS
# offsets of the parameter vector (w1[H][7], b1, w2[H][H], b2, w3, b3)
W1, B1, W2 = 0, 7 * NH, 8 * NH
B2 = W2 + NH * NH
W3 = B2 + NH
B3 = W3 + NH
FEATURES = ("tr S", "I2", "I3 = det S", "Lode parameter", "S_d:S_d / S:S", "rho", "|S|")


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class MlpModel:
    """Parameters (FP32), input normalisation and range, output scale."""

    def __init__(self, params, in_mean, in_std, in_lo, in_hi, out_scale):
        self.params = np.ascontiguousarray(params, np.float32).reshape(NPAR).copy()
        self.in_mean = np.asarray(in_mean, np.float32).reshape(NIN).copy()
        self.in_std = np.asarray(in_std, np.float32).reshape(NIN).copy()
        self.in_lo = np.asarray(in_lo, np.float32).reshape(NIN).copy()
        self.in_hi = np.asarray(in_hi, np.float32).reshape(NIN).copy()
        self.out_scale = float(out_scale)

    @classmethod
    def init_from_samples(cls, samples, seed=0x5EED2026, range_quantile=0.0):
        """Seeded Glorot-uniform weights; normalisation from the samples' inputs; training range =
        [quantile, 1 - quantile] of each input; output scale = median least-squares nu of the samples."""
        x = samples[:, :NIN].astype(np.float64)
        mean, std = x.mean(0), x.std(0)
        std = np.where(std > 0, std, 1.0)
        lo = np.quantile(x, range_quantile, axis=0)
        hi = np.quantile(x, 1.0 - range_quantile, axis=0)
        a, b = samples[:, 7].astype(np.float64), samples[:, 8].astype(np.float64)
        nu_ls = np.clip(-a / (2.0 * np.maximum(b, 1e-300)), 0.0, None)
        scale = float(np.median(nu_ls[b > 0])) if np.any(b > 0) else 1e-3
        scale = scale if scale > 0 else 1e-3
        rng = np.random.default_rng(seed)
        p = np.zeros(NPAR, np.float32)

        def glorot(n_out, n_in):
            lim = np.sqrt(6.0 / (n_in + n_out))
            return rng.uniform(-lim, lim, size=(n_out, n_in)).astype(np.float32)

        p[W1:B1] = glorot(NH, NIN).reshape(-1)
        p[W2:B2] = glorot(NH, NH).reshape(-1)
        p[W3:B3] = glorot(1, NH).reshape(-1)
        return cls(p, mean, std, lo, hi, scale)

    def struct(self):
        m = capi.LbmMlpModel()
        C.memmove(m.params, self.params.ctypes.data, NPAR * 4)
        for name in ("in_mean", "in_std", "in_lo", "in_hi"):
            arr = getattr(self, name)
            C.memmove(getattr(m, name), arr.ctypes.data, NIN * 4)
        m.out_scale = self.out_scale
        return m

    def copy(self):
        return MlpModel(self.params, self.in_mean, self.in_std, self.in_lo, self.in_hi, self.out_scale)

    ACTIVATION = "gelu"  # hidden activation of the network the library evaluates (files without the key: gelu)

    def save(self, path):
        np.savez(path, params=self.params, in_mean=self.in_mean, in_std=self.in_std, in_lo=self.in_lo,
                 in_hi=self.in_hi, out_scale=np.float32(self.out_scale), activation=np.array(self.ACTIVATION))

    def save_raw(self, path):
        """The lbm_mlp_model struct as raw bytes (the C++ driver's --mlp file)."""
        with open(path, "wb") as fh:
            fh.write(bytes(self.struct()))

    @classmethod
    def load(cls, path):
        """A model saved by save(); a file whose hidden activation is not the library's is refused."""
        d = np.load(path)
        act = str(d["activation"]) if "activation" in d.files else "gelu"
        if act != cls.ACTIVATION:
            raise ValueError(f"{path}: trained with a {act} activation; the library evaluates {cls.ACTIVATION}")
        return cls(d["params"], d["in_mean"], d["in_std"], d["in_lo"], d["in_hi"], float(d["out_scale"]))


def evaluate(model, x, device=0, path=capi.LBM_MLP_PATH_WARP_MMA):
    """nu_t and the in-range flag of raw inputs x (n x 7) on the GPU (FP16 tensor-core path: warp-level
    mma.sync, or tcgen05.mma with TMEM accumulators for path=capi.LBM_MLP_PATH_TCGEN05)."""
    x = np.ascontiguousarray(x, np.float32).reshape(-1, NIN)
    n = x.shape[0]
    nu = np.zeros(n, np.float32)
    ok = np.zeros(n, np.int32)
    m = model.struct()
    check(lib().lbm_mlp_eval_path(C.byref(m), _fp(x), n, _fp(nu), ok.ctypes.data_as(C.POINTER(C.c_int32)), path,
                                  device), mlp=True)
    return nu, ok.astype(bool)


class Trainer:
    """The GPU trainer of include/lbm.h (samples resident on the device)."""

    def __init__(self, samples, device=0):
        self.samples = np.ascontiguousarray(samples, np.float32).reshape(-1, capi.LBM_MLP_SAMPLE)
        self._t = C.c_void_p()
        check(lib().lbm_mlp_trainer_create(_fp(self.samples), self.samples.shape[0], device, C.byref(self._t)),
              mlp=True)

    @property
    def norm(self):
        return lib().lbm_mlp_trainer_norm(self._t)

    def gradient(self, model, first=0, count=None):
        count = self.samples.shape[0] - first if count is None else count
        g = np.zeros(NPAR, np.float32)
        loss = C.c_double(0)
        check(lib().lbm_mlp_gradient(self._t, C.byref(model.struct()), first, count, _fp(g), C.byref(loss)), mlp=True)
        return float(loss.value), g

    def train(self, model, epochs, batch=4096, lr=2e-3, seed=0x5EED2026):
        """Adam epochs on the GPU; returns the per-epoch mean loss and updates model.params."""
        m = model.struct()
        hist = np.zeros(max(epochs, 1), np.float32)
        check(lib().lbm_mlp_train(self._t, C.byref(m), epochs, batch, lr, seed, _fp(hist)), mlp=True)
        model.params[:] = np.frombuffer(m.params, np.float32)
        return hist[:epochs]

    def close(self):
        if self._t:
            lib().lbm_mlp_trainer_destroy(self._t)
            self._t = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sgs_error(nu, samples):
    """Relative a-priori subgrid-stress error sum|tau_d + 2 nu S_d|^2 / sum|tau_d|^2 (FP64 sums)."""
    s = np.asarray(samples, np.float64)
    nu = np.asarray(nu, np.float64)
    a, b, c = s[:, 7], s[:, 8], s[:, 9]
    return float(np.sum(c + 4.0 * nu * a + 4.0 * nu * nu * b) / np.sum(c))


def sgs_dissipation_error(nu, samples):
    """Relative error of the subgrid dissipation: the model transfers 2 nu S_d:S_d = 2 nu b, the filtered
    field -tau_d:S_d = -a; returns sum (2 nu b + a)^2 / sum a^2."""
    s = np.asarray(samples, np.float64)
    nu = np.asarray(nu, np.float64)
    a, b = s[:, 7], s[:, 8]
    return float(np.sum((2.0 * nu * b + a) ** 2) / np.sum(a * a))


def smagorinsky_nu(samples, cles):
    """The eddy viscosity of the Smagorinsky closure as the solver runs it (OmegaLES.h:117-124):
    tau_S = tau/2 + sqrt(tau^2 + 18 CLES |Pi|/rho)/2 with |Pi| = 2/3 rho tau_S |S|_F gives
    nu_t = CLES |S|_F, |S|_F = sqrt(S:S) = x[6] / sqrt(2)."""
    return cles * np.asarray(samples, np.float64)[:, 6] / np.sqrt(2.0)


def best_constant(samples):
    """Least-squares constant C of nu_t = C |S|_F over the samples (the best Smagorinsky constant)."""
    s = np.asarray(samples, np.float64)
    sf = s[:, 6] / np.sqrt(2.0)
    return float(-np.sum(sf * s[:, 7]) / (2.0 * np.sum(sf * sf * s[:, 8])))
