// mlp.cu - learned LES closure: training kernels (forward, backward, Adam) in FP32, the batch
// evaluation through the step kernel's tensor-core path, the filtered training samples of a fine run,
// and their C ABI (lbm_mlp_*).
//
// Loss of one minibatch: the mean over its samples of the normalised subgrid-stress error of the model
// tau_d = -2 nu_t S_d against the filtered stress,
//     e = (c + 4 nu_t a + 4 nu_t^2 b) / K,   a = tau_d:S_d, b = S_d:S_d, c = tau_d:tau_d,
// K = the mean of c over the trainer's samples (e = 1 for nu_t = 0).
// Gradients: one thread per sample computes its forward pass and back-propagates to the hidden
// layers; the block then forms its parameter gradients as sums over its 128 samples from shared
// memory (no atomics), and a second kernel adds the blocks in a fixed order and applies Adam.  The
// result is deterministic for a given sample order.

#include "../../include/lbm.h"
#include "lbm_device.cuh"
#include "lbm_launch.h"
#include "lbm_mlp_host.h"
#include "lbm_mlp_tc.cuh"

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

using namespace lbm;

namespace {

constexpr int kBlk = 128;   // samples per training block
constexpr int kPad = kMlpHid + 1;  // row stride of the per-sample hidden arrays in shared memory
constexpr int kGradLen = kMlpParams + 1;  // the gradients and the loss

struct TrainNorm {
    float mu[7], isd[7];
    float scale, invK;
};

// shared memory of k_mlp_grad (floats)
constexpr int kSmW = kMlpParams + 3;
constexpr size_t kSmemGrad =
    sizeof(float) * ((size_t)kSmW + 4 * (size_t)kBlk * kPad + (size_t)kBlk * 8 + 2 * (size_t)kBlk);

__global__ void __launch_bounds__(kBlk) k_mlp_grad(const float* __restrict__ samples, const int32_t* __restrict__ perm,
                                                   long long first, int count, const float* __restrict__ params,
                                                   TrainNorm nm, float* __restrict__ gpart, int* tick) {
    extern __shared__ float sm[];
    float* W = sm;                          // parameters
    float* H1 = W + kSmW;                   // [kBlk][kPad] layer-1 activations
    float* D1 = H1 + kBlk * kPad;           // gelu'(pre1), then delta1
    float* H2 = D1 + kBlk * kPad;           // layer-2 activations
    float* D2 = H2 + kBlk * kPad;           // gelu'(pre2), then delta2
    float* X = D2 + kBlk * kPad;            // [kBlk][8] normalised inputs and 1
    float* DZ = X + kBlk * 8;               // dL/dz per sample
    float* LS = DZ + kBlk;                  // loss per sample
    const int t = threadIdx.x;
    if (tick && blockIdx.x == 0 && t == 0) atomicAdd(tick, 1);  // Adam step counter for the next update
    for (int i = t; i < kMlpParams; i += kBlk) W[i] = params[i];
    __syncthreads();
    const int j = blockIdx.x * kBlk + t;
    const bool live = j < count;
    float a = 0.f, b = 0.f, c = 0.f;
    float* x = X + t * 8;
    if (live) {
        const long long s = first + j;
        const float* r = samples + (perm ? (long long)perm[s] : s) * kMlpSample;
        for (int i = 0; i < 7; i++) x[i] = (r[i] - nm.mu[i]) * nm.isd[i];
        a = r[7]; b = r[8]; c = r[9];
    } else {
        for (int i = 0; i < 7; i++) x[i] = 0.f;
    }
    x[7] = live ? 1.f : 0.f;
    float* h1 = H1 + t * kPad;
    float* d1 = D1 + t * kPad;
    float* h2 = H2 + t * kPad;
    float* d2 = D2 + t * kPad;
    for (int i = 0; i < kMlpHid; i++) {
        float pre = W[kMlpB1 + i];
        for (int k = 0; k < 7; k++) pre = fmaf(W[kMlpW1 + i * 7 + k], x[k], pre);
        h1[i] = live ? gelu_s(pre) : 0.f;
        d1[i] = live ? gelu_s_grad(pre) : 0.f;
    }
    float zz = W[kMlpB3];
    for (int o = 0; o < kMlpHid; o++) {
        float pre = W[kMlpB2 + o];
        for (int i = 0; i < kMlpHid; i++) pre = fmaf(W[kMlpW2 + o * kMlpHid + i], h1[i], pre);
        h2[o] = live ? gelu_s(pre) : 0.f;
        d2[o] = live ? gelu_s_grad(pre) : 0.f;
        zz = fmaf(W[kMlpW3 + o], h2[o], zz);
    }
    float dz = 0.f, loss = 0.f;
    if (live) {
        const float nu = nm.scale * softplusf_(zz);
        loss = (c + 4.f * nu * a + 4.f * nu * nu * b) * nm.invK;
        const float dnu = (4.f * a + 8.f * nu * b) * nm.invK;
        dz = dnu * nm.scale * sigmoidf_(zz);
    }
    DZ[t] = dz;
    LS[t] = loss;
    for (int o = 0; o < kMlpHid; o++) d2[o] *= dz * W[kMlpW3 + o];
    for (int i = 0; i < kMlpHid; i++) {
        float s = 0.f;
        for (int o = 0; o < kMlpHid; o++) s = fmaf(d2[o], W[kMlpW2 + o * kMlpHid + i], s);
        d1[i] *= s;
    }
    __syncthreads();
    float* g = gpart + (size_t)blockIdx.x * kGradLen;
    // w2 [o][i] and b2 [o]
    for (int q = t; q < kMlpHid * kMlpHid + kMlpHid; q += kBlk) {
        float s = 0.f;
        if (q < kMlpHid * kMlpHid) {
            const int o = q / kMlpHid, i = q % kMlpHid;
            for (int n = 0; n < kBlk; n++) s = fmaf(D2[n * kPad + o], H1[n * kPad + i], s);
            g[kMlpW2 + q] = s;
        } else {
            const int o = q - kMlpHid * kMlpHid;
            for (int n = 0; n < kBlk; n++) s += D2[n * kPad + o];
            g[kMlpB2 + o] = s;
        }
    }
    // w1 [i][k] and b1 [i] (input 7 = 1)
    for (int q = t; q < kMlpHid * 8; q += kBlk) {
        const int i = q >> 3, k = q & 7;
        float s = 0.f;
        for (int n = 0; n < kBlk; n++) s = fmaf(D1[n * kPad + i], X[n * 8 + k], s);
        if (k < 7) g[kMlpW1 + i * 7 + k] = s;
        else g[kMlpB1 + i] = s;
    }
    // w3, b3, loss
    if (t < kMlpHid) {
        float s = 0.f;
        for (int n = 0; n < kBlk; n++) s = fmaf(DZ[n], H2[n * kPad + t], s);
        g[kMlpW3 + t] = s;
    } else if (t == kMlpHid) {
        float s = 0.f;
        for (int n = 0; n < kBlk; n++) s += DZ[n];
        g[kMlpB3] = s;
    } else if (t == kMlpHid + 1) {
        float s = 0.f;
        for (int n = 0; n < kBlk; n++) s += LS[n];
        g[kMlpParams] = s;
    }
}

// sum of the block gradients in block order, divided by the batch size; optional Adam update
__global__ void k_mlp_reduce(const float* __restrict__ gpart, int nblk, float inv_batch, float* params, float* m,
                             float* v, const int* tick, float lr, float beta1, float beta2, float eps, int apply,
                             float* grad_out, double* loss_acc) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q > kMlpParams) return;
    double s = 0.0;
    for (int b = 0; b < nblk; b++) s += (double)gpart[(size_t)b * kGradLen + q];
    const float gq = (float)(s * inv_batch);
    if (q == kMlpParams) {
        if (loss_acc) *loss_acc += s * inv_batch;
        return;
    }
    if (grad_out) grad_out[q] = gq;
    if (!apply) return;
    const int n = *tick;
    const float mq = beta1 * m[q] + (1.f - beta1) * gq;
    const float vq = beta2 * v[q] + (1.f - beta2) * gq * gq;
    m[q] = mq;
    v[q] = vq;
    const float mh = mq / (1.f - powf(beta1, (float)n));
    const float vh = vq / (1.f - powf(beta2, (float)n));
    params[q] -= lr * mh / (sqrtf(vh) + eps);
}

// nu_t of raw inputs through the step kernel's FP16 tensor-core path; 64 samples per warp
__global__ void __launch_bounds__(128) k_mlp_eval(const float* __restrict__ x, long long n, const uint4* __restrict__ frag,
                                                  MlpNorm nm, float* __restrict__ nu, int32_t* __restrict__ in_range) {
    __shared__ uint4 wf[kMlpFragRows][32];
    __shared__ uint4 stage[4][64];
    for (int i = threadIdx.x; i < kMlpFragRows * 32; i += blockDim.x) (&wf[0][0])[i] = frag[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long base = ((long long)blockIdx.x * 4 + warp) * 64;
    const long long sA = base + lane, sB = base + 32 + lane;
    uint4 rA = make_uint4(0, 0, 0, 0), rB = rA;
    bool okA = false, okB = false;
    float xr[7];
    if (sA < n) {
        for (int i = 0; i < 7; i++) xr[i] = x[sA * 7 + i];
        rA = mlp_row(xr, nm, okA);
    }
    if (sB < n) {
        for (int i = 0; i < 7; i++) xr[i] = x[sB * 7 + i];
        rB = mlp_row(xr, nm, okB);
    }
    const float2 z = mlp_warp(rA, rB, stage[warp], wf);
    if (sA < n) { nu[sA] = mlp_nu(z.x, nm); if (in_range) in_range[sA] = okA; }
    if (sB < n) { nu[sB] = mlp_nu(z.y, nm); if (in_range) in_range[sB] = okB; }
}

// the same through the tcgen05 path: one CTA of 128 threads per 256 samples (thread t: samples 2t, 2t+1)
__global__ void __launch_bounds__(128) k_mlp_eval_tc(const float* __restrict__ x, long long n, const uint4* __restrict__ img,
                                                     MlpNorm nm, float* __restrict__ nu, int32_t* __restrict__ in_range,
                                                     int* err) {
    __shared__ TcSmem ts;
    const uint32_t tm = tc_setup(ts, img);
    const long long sA = (long long)blockIdx.x * 256 + 2 * threadIdx.x, sB = sA + 1;
    uint4 rA = make_uint4(0, 0, 0, 0), rB = rA;
    bool okA = false, okB = false;
    float xr[7];
    if (sA < n) {
        for (int i = 0; i < 7; i++) xr[i] = x[sA * 7 + i];
        rA = mlp_row(xr, nm, okA);
    }
    if (sB < n) {
        for (int i = 0; i < 7; i++) xr[i] = x[sB * 7 + i];
        rB = mlp_row(xr, nm, okB);
    }
    const float2 z = tc_mlp(ts, tm, rA, rB, nm, err, 0u);
    tc_teardown(tm);
    if (sA < n) { nu[sA] = mlp_nu(z.x, nm); if (in_range) in_range[sA] = okA; }
    if (sB < n) { nu[sB] = mlp_nu(z.y, nm); if (in_range) in_range[sB] = okB; }
}

// ---- filtered samples -------------------------------------------------------------------------------
// coarse cell = w^3 fine cells: mean rho and u, the filtered stress <u_i u_j> - <u_i><u_j> (FP64 sums,
// the difference taken in FP64), and whether every fine cell is fluid.  cf: [11][Nc] =
// rho, ux, uy, uz, tau_xx, tau_yy, tau_zz, tau_xy, tau_xz, tau_yz, fluid
__global__ void k_les_filter(const double* __restrict__ rho, const double* __restrict__ u, const uint8_t* __restrict__ cls,
                             int nx, int ny, int nz, int w, float* __restrict__ cf, int ncx, int ncy, int ncz) {
    const long long Nc = (long long)ncx * ncy * ncz;
    const long long ic = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (ic >= Nc) return;
    const int I = (int)(ic % ncx), J = (int)((ic / ncx) % ncy), K = (int)(ic / ((long long)ncx * ncy));
    const long long N = (long long)nx * ny * nz;
    double s[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    bool fluid = true;
    for (int dz = 0; dz < w; dz++)
        for (int dy = 0; dy < w; dy++)
            for (int dx = 0; dx < w; dx++) {
                const long long i = (long long)(I * w + dx) + nx * ((long long)(J * w + dy) + (long long)ny * (K * w + dz));
                fluid = fluid && (cls[i] & CLS_MASK) != CLS_SOLID;
                const double ux = u[i], uy = u[N + i], uz = u[2 * N + i];
                s[0] += rho[i]; s[1] += ux; s[2] += uy; s[3] += uz;
                s[4] += ux * ux; s[5] += uy * uy; s[6] += uz * uz;
                s[7] += ux * uy; s[8] += ux * uz; s[9] += uy * uz;
            }
    const double inv = 1.0 / ((double)w * w * w);
    double m[10];
    for (int k = 0; k < 10; k++) m[k] = s[k] * inv;
    m[4] -= m[1] * m[1]; m[5] -= m[2] * m[2]; m[6] -= m[3] * m[3];
    m[7] -= m[1] * m[2]; m[8] -= m[1] * m[3]; m[9] -= m[2] * m[3];
    for (int k = 0; k < 10; k++) cf[k * Nc + ic] = (float)m[k];
    cf[10 * Nc + ic] = fluid ? 1.f : 0.f;
}

// per coarse cell: strain rate of the filtered velocity (central differences, coarse lattice units),
// the filtered stress, inputs and (a, b, c); out[ic][11], [10] = valid
__global__ void k_les_samples(const float* __restrict__ cf, int ncx, int ncy, int ncz, int wx, int wy, int wz,
                              float* __restrict__ out) {
    const long long Nc = (long long)ncx * ncy * ncz;
    const long long ic = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (ic >= Nc) return;
    const int I = (int)(ic % ncx), J = (int)((ic / ncx) % ncy), K = (int)(ic / ((long long)ncx * ncy));
    float* o = out + ic * 11;
    const int n[3] = {ncx, ncy, ncz}, wr[3] = {wx, wy, wz}, c0[3] = {I, J, K};
    long long nb[3][2];
    bool ok = cf[10 * Nc + ic] > 0.5f;
    for (int a = 0; a < 3 && ok; a++)
        for (int sgn = 0; sgn < 2; sgn++) {
            int cc[3] = {c0[0], c0[1], c0[2]};
            cc[a] += sgn ? 1 : -1;
            if (cc[a] < 0 || cc[a] >= n[a]) {
                if (!wr[a]) { ok = false; break; }
                cc[a] = (cc[a] + n[a]) % n[a];
            }
            nb[a][sgn] = cc[0] + (long long)ncx * (cc[1] + (long long)ncy * cc[2]);
            ok = ok && cf[10 * Nc + nb[a][sgn]] > 0.5f;
        }
    if (!ok) {
        for (int k = 0; k < 11; k++) o[k] = 0.f;
        return;
    }
    float G[3][3];  // G[a][b] = d u_b / d x_a
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) G[a][b] = 0.5f * (cf[(1 + b) * Nc + nb[a][1]] - cf[(1 + b) * Nc + nb[a][0]]);
    const float S[6] = {G[0][0], G[1][1], G[2][2], 0.5f * (G[0][1] + G[1][0]), 0.5f * (G[0][2] + G[2][0]),
                        0.5f * (G[1][2] + G[2][1])};
    const float r = cf[ic];
    float T[6] = {cf[4 * Nc + ic], cf[5 * Nc + ic], cf[6 * Nc + ic], cf[7 * Nc + ic], cf[8 * Nc + ic], cf[9 * Nc + ic]};
    const float tt = (T[0] + T[1] + T[2]) * (1.f / 3.f), st = (S[0] + S[1] + S[2]) * (1.f / 3.f);
    float Sd[6] = {S[0] - st, S[1] - st, S[2] - st, S[3], S[4], S[5]};
    T[0] -= tt; T[1] -= tt; T[2] -= tt;
    auto dd = [](const float* A, const float* B) {
        return A[0] * B[0] + A[1] * B[1] + A[2] * B[2] + 2.f * (A[3] * B[3] + A[4] * B[4] + A[5] * B[5]);
    };
    float x[7];
    mlp_features(S, r, x);
    for (int k = 0; k < 7; k++) o[k] = x[k];
    o[7] = dd(T, Sd);
    o[8] = dd(Sd, Sd);
    o[9] = dd(T, T);
    o[10] = 1.f;
}

std::string g_mlp_err;

lbm_status mfail(lbm_status s, const std::string& m) {
    g_mlp_err = m;
    return s;
}
#define MCU(call)                                                                                        \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess)                                                                           \
            return mfail(e_ == cudaErrorMemoryAllocation ? LBM_ERR_OOM : LBM_ERR_CUDA,                   \
                         std::string(#call) + ": " + cudaGetErrorString(e_));                           \
    } while (0)

bool model_ok(const lbm_mlp_model* m) {
    if (!m || !(m->out_scale > 0.f) || !std::isfinite(m->out_scale)) return false;
    for (int i = 0; i < 7; i++)
        if (!(m->in_std[i] > 0.f) || !std::isfinite(m->in_mean[i]) || !(m->in_lo[i] <= m->in_hi[i])) return false;
    for (int i = 0; i < kMlpParams; i++)
        if (!std::isfinite(m->params[i])) return false;
    return true;
}

// splitmix64 of the seed: Fisher-Yates order of the samples for one epoch
uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

}  // namespace

namespace lbm {

// host: FP16 fragment table with the activation constants folded in, and the uniform normalisation
void mlp_pack(const lbm_mlp_model& m, uint4* frag, MlpNorm& nm) {
    constexpr int H = kMlpHid;
    // the activation constants folded into the weights: z = 0.851 x, the next layer takes g = z (1 + tanh z)
    // / 1.702 (mlp_act returns z (1 + tanh z))
    const float h = 0.5f * kGeluA;
    auto W1 = [&](int n, int k) { return h * (k < 7 ? m.params[kMlpW1 + n * 7 + k] : m.params[kMlpB1 + n]); };
    auto W2 = [&](int n, int k) { return (h / kGeluA) * m.params[kMlpW2 + n * H + k]; };
    auto W3 = [&](int k) { return m.params[kMlpW3 + k] / kGeluA; };
    auto hb = [](float a, float b) {
        const __half2 v = __floats2half2_rn(a, b);
        uint32_t u;
        std::memcpy(&u, &v, 4);
        return u;
    };
    auto fb = [](float a) {
        uint32_t u;
        std::memcpy(&u, &a, 4);
        return u;
    };
    // warp fragment table: lane (g = lane / 4, c = lane % 4) holds, per n-tile j of 8 units, the B fragment
    // of output unit 8 j + g at inputs (2c, 2c + 1) and (2c + 8, 2c + 9) of each k16 step; unused slots 0
    for (int i = 0; i < kMlpFragRows * 32; i++) frag[i] = make_uint4(0, 0, 0, 0);
    for (int lane = 0; lane < 32; lane++) {
        const int g = lane >> 2, c = lane & 3;
        uint32_t r[4] = {0, 0, 0, 0};
        for (int j = 0; j < kMlpNT; j++) r[j] = hb(W1(8 * j + g, 2 * c), W1(8 * j + g, 2 * c + 1));
        frag[0 * 32 + lane] = make_uint4(r[0], r[1], r[2], r[3]);
        for (int j = 0; j < kMlpNT; j++) {
            const int n = 8 * j + g;
            uint32_t w[4] = {0, 0, 0, 0};
            for (int ks = 0; ks < kMlpKS; ks++) {
                w[2 * ks] = hb(W2(n, 16 * ks + 2 * c), W2(n, 16 * ks + 2 * c + 1));
                w[2 * ks + 1] = hb(W2(n, 16 * ks + 2 * c + 8), W2(n, 16 * ks + 2 * c + 9));
            }
            frag[(1 + j) * 32 + lane] = make_uint4(w[0], w[1], w[2], w[3]);
        }
        uint32_t w3[4] = {0, 0, 0, 0};
        if (g == 0)
            for (int ks = 0; ks < kMlpKS; ks++) {
                w3[2 * ks] = hb(W3(16 * ks + 2 * c), W3(16 * ks + 2 * c + 1));
                w3[2 * ks + 1] = hb(W3(16 * ks + 2 * c + 8), W3(16 * ks + 2 * c + 9));
            }
        frag[5 * 32 + lane] = make_uint4(w3[0], w3[1], w3[2], w3[3]);
        uint32_t b[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int j = 0; j < kMlpNT; j++) {
            b[2 * j] = fb(h * m.params[kMlpB2 + 8 * j + 2 * c]);
            b[2 * j + 1] = fb(h * m.params[kMlpB2 + 8 * j + 2 * c + 1]);
        }
        frag[6 * 32 + lane] = make_uint4(b[0], b[1], b[2], b[3]);
        frag[7 * 32 + lane] = make_uint4(b[4], b[5], b[6], b[7]);
    }
    for (int i = 0; i < 7; i++) {
        nm.isd[i] = 1.0f / m.in_std[i];
        nm.nmi[i] = -(m.in_mean[i] * nm.isd[i]);
        nm.lo[i] = std::fma(m.in_lo[i], nm.isd[i], nm.nmi[i]);
        nm.hi[i] = std::fma(m.in_hi[i], nm.isd[i], nm.nmi[i]);
    }
    nm.b3 = m.params[kMlpB3];
    nm.scale = m.out_scale;
    for (int n = 0; n < H; n++) nm.b2[n] = h * m.params[kMlpB2 + n];
    // the tcgen05 weight image after the table, with the same folded constants: W1 (k 0..6 weights, k 7 =
    // b1, 8..15 zero), W2, W3 (row 0 = w3), FP16, K-major core matrices of 8 rows x 8 halves (lbm_mlp_tc.cuh)
    std::vector<__half> img(kTcWBytes / 2, __float2half(0.0f));
    auto put = [&](int base, int KG, int n, int k, float v) {
        img[(base + tc_off(n, k >> 3, KG)) / 2 + (k & 7)] = __float2half_rn(v);
    };
    for (int n = 0; n < H; n++) {
        for (int k = 0; k < 8; k++) put(kTcW1, 2, n, k, W1(n, k));
        for (int k = 0; k < H; k++) put(kTcW2, kTcKG, n, k, W2(n, k));
    }
    for (int k = 0; k < H; k++) put(kTcW3, kTcKG, 0, k, W3(k));
    std::memcpy(frag + kMlpFragRows * 32, img.data(), kTcWBytes);
}

bool mlp_model_valid(const lbm_mlp_model* m) { return model_ok(m); }

cudaError_t launch_les_samples(const double* rho, const double* u, const uint8_t* cls, int nx, int ny, int nz, int w,
                               const int wrap[3], float* cf, float* out, cudaStream_t st) {
    const int ncx = nx / w, ncy = ny / w, ncz = nz / w;
    const long long Nc = (long long)ncx * ncy * ncz;
    const int B = 256;
    const unsigned g = (unsigned)((Nc + B - 1) / B);
    k_les_filter<<<g, B, 0, st>>>(rho, u, cls, nx, ny, nz, w, cf, ncx, ncy, ncz);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // a coarse axis wraps only if the fine axis wraps and divides evenly
    k_les_samples<<<g, B, 0, st>>>(cf, ncx, ncy, ncz, wrap[0] && nx % w == 0, wrap[1] && ny % w == 0,
                                   wrap[2] && nz % w == 0, out);
    return cudaGetLastError();
}

}  // namespace lbm

// ---- C ABI ----------------------------------------------------------------------------------------------
struct lbm_mlp_trainer {
    int device = 0;
    long long n = 0;
    float* d_samples = nullptr;
    int32_t* d_perm = nullptr;
    float *d_params = nullptr, *d_m = nullptr, *d_v = nullptr, *d_grad = nullptr, *d_gpart = nullptr;
    int* d_tick = nullptr;
    double* d_loss = nullptr;
    int gpart_blocks = 0;
    double K = 1.0;  // mean of c
    cudaStream_t st = nullptr;
};

extern "C" {

const char* lbm_mlp_last_error(void) { return g_mlp_err.c_str(); }

lbm_status lbm_mlp_eval(const lbm_mlp_model* m, const float* x, int64_t n, float* nu, int32_t* in_range,
                        int32_t device) {
    return lbm_mlp_eval_path(m, x, n, nu, in_range, LBM_MLP_PATH_WARP_MMA, device);
}

lbm_status lbm_mlp_eval_path(const lbm_mlp_model* m, const float* x, int64_t n, float* nu, int32_t* in_range,
                             int32_t path, int32_t device) {
    if (!model_ok(m) || n < 0 || (n > 0 && (!x || !nu)) || (path != LBM_MLP_PATH_WARP_MMA && path != LBM_MLP_PATH_TCGEN05))
        return mfail(LBM_ERR_INVALID, "lbm_mlp_eval: bad arguments");
    if (n == 0) return LBM_OK;
    MCU(cudaSetDevice(device));
    std::vector<uint4> frag(kMlpFragTotal);
    MlpNorm nm;
    mlp_pack(*m, frag.data(), nm);
    uint4* d_frag = nullptr;
    float *d_x = nullptr, *d_nu = nullptr;
    int32_t* d_in = nullptr;
    int* d_err = nullptr;
    cudaError_t e = cudaMalloc(&d_frag, frag.size() * sizeof(uint4));
    if (e == cudaSuccess) e = cudaMalloc(&d_err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(d_err, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&d_x, (size_t)n * 7 * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&d_nu, (size_t)n * sizeof(float));
    if (e == cudaSuccess && in_range) e = cudaMalloc(&d_in, (size_t)n * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMemcpy(d_frag, frag.data(), frag.size() * sizeof(uint4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_x, x, (size_t)n * 7 * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const long long blocks = (n + 255) / 256;
        if (path == LBM_MLP_PATH_TCGEN05)
            k_mlp_eval_tc<<<(unsigned)blocks, 128>>>(d_x, n, d_frag + kMlpFragRows * 32, nm, d_nu, d_in, d_err);
        else
            k_mlp_eval<<<(unsigned)blocks, 128>>>(d_x, n, d_frag, nm, d_nu, d_in);
        e = cudaGetLastError();
    }
    int herr = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(nu, d_nu, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && in_range) e = cudaMemcpy(in_range, d_in, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost);
    cudaFree(d_frag); cudaFree(d_x); cudaFree(d_nu); cudaFree(d_in); cudaFree(d_err);
    if (e != cudaSuccess) return mfail(LBM_ERR_CUDA, std::string("lbm_mlp_eval: ") + cudaGetErrorString(e));
    if (herr) return mfail(LBM_ERR_TIMEOUT, "lbm_mlp_eval: a CTA gave up waiting for its tensor-core products");
    return LBM_OK;
}

lbm_status lbm_mlp_trainer_create(const float* samples, int64_t n, int32_t device, lbm_mlp_trainer** out) {
    if (!out || !samples || n <= 0 || n > (int64_t)INT32_MAX) return mfail(LBM_ERR_INVALID, "trainer: bad arguments");
    *out = nullptr;
    double K = 0.0;
    for (int64_t i = 0; i < n; i++) K += samples[i * kMlpSample + 9];
    K /= (double)n;
    if (!(K > 0.0) || !std::isfinite(K)) return mfail(LBM_ERR_INVALID, "trainer: samples carry no subgrid stress");
    MCU(cudaSetDevice(device));
    auto* t = new lbm_mlp_trainer();
    t->device = device;
    t->n = n;
    t->K = K;
    cudaError_t e = cudaStreamCreateWithFlags(&t->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&t->d_samples, (size_t)n * kMlpSample * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&t->d_perm, (size_t)n * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&t->d_params, kMlpParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&t->d_m, kMlpParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&t->d_v, kMlpParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&t->d_grad, kMlpParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&t->d_tick, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&t->d_loss, sizeof(double));
    if (e == cudaSuccess)
        e = cudaMemcpy(t->d_samples, samples, (size_t)n * kMlpSample * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemGrad);
    if (e != cudaSuccess) {
        lbm_mlp_trainer_destroy(t);
        return mfail(e == cudaErrorMemoryAllocation ? LBM_ERR_OOM : LBM_ERR_CUDA,
                     std::string("trainer: ") + cudaGetErrorString(e));
    }
    *out = t;
    return LBM_OK;
}

lbm_status lbm_mlp_trainer_destroy(lbm_mlp_trainer* t) {
    if (!t) return LBM_OK;
    cudaSetDevice(t->device);
    if (t->st) cudaStreamSynchronize(t->st);
    cudaFree(t->d_samples); cudaFree(t->d_perm); cudaFree(t->d_params); cudaFree(t->d_m); cudaFree(t->d_v);
    cudaFree(t->d_grad); cudaFree(t->d_gpart); cudaFree(t->d_tick); cudaFree(t->d_loss);
    if (t->st) cudaStreamDestroy(t->st);
    delete t;
    return LBM_OK;
}

double lbm_mlp_trainer_norm(const lbm_mlp_trainer* t) { return t ? t->K : 0.0; }

static TrainNorm train_norm(const lbm_mlp_model* m, double K) {
    TrainNorm nm;
    for (int i = 0; i < 7; i++) {
        nm.mu[i] = m->in_mean[i];
        nm.isd[i] = 1.0f / m->in_std[i];
    }
    nm.scale = m->out_scale;
    nm.invK = (float)(1.0 / K);
    return nm;
}

static cudaError_t ensure_gpart(lbm_mlp_trainer* t, int blocks) {
    if (blocks <= t->gpart_blocks) return cudaSuccess;
    cudaFree(t->d_gpart);
    t->d_gpart = nullptr;
    t->gpart_blocks = 0;
    cudaError_t e = cudaMalloc(&t->d_gpart, (size_t)blocks * kGradLen * sizeof(float));
    if (e == cudaSuccess) t->gpart_blocks = blocks;
    return e;
}

lbm_status lbm_mlp_gradient(lbm_mlp_trainer* t, const lbm_mlp_model* m, int64_t first, int64_t count, float* grad,
                            double* loss) {
    if (!t || !model_ok(m) || first < 0 || count <= 0 || first + count > t->n || count > (1 << 24))
        return mfail(LBM_ERR_INVALID, "lbm_mlp_gradient: bad arguments");
    MCU(cudaSetDevice(t->device));
    const int blocks = (int)((count + kBlk - 1) / kBlk);
    MCU(ensure_gpart(t, blocks));
    MCU(cudaMemcpyAsync(t->d_params, m->params, kMlpParams * sizeof(float), cudaMemcpyHostToDevice, t->st));
    MCU(cudaMemsetAsync(t->d_loss, 0, sizeof(double), t->st));
    const TrainNorm nm = train_norm(m, t->K);
    k_mlp_grad<<<blocks, kBlk, kSmemGrad, t->st>>>(t->d_samples, nullptr, first, (int)count, t->d_params, nm, t->d_gpart,
                                                  nullptr);
    MCU(cudaGetLastError());
    k_mlp_reduce<<<(kGradLen + 127) / 128, 128, 0, t->st>>>(t->d_gpart, blocks, 1.0f / (float)count, t->d_params, nullptr,
                                                           nullptr, nullptr, 0.f, 0.f, 0.f, 0.f, 0, t->d_grad, t->d_loss);
    MCU(cudaGetLastError());
    if (grad) MCU(cudaMemcpyAsync(grad, t->d_grad, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost, t->st));
    double l = 0.0;
    MCU(cudaMemcpyAsync(&l, t->d_loss, sizeof(double), cudaMemcpyDeviceToHost, t->st));
    MCU(cudaStreamSynchronize(t->st));
    if (loss) *loss = l;
    return LBM_OK;
}

// Adam over shuffled minibatches of `batch` samples (the remainder of an epoch is left out).  The
// launches of one epoch are captured once into a CUDA graph and replayed per epoch; each epoch only
// uploads its sample order first.
lbm_status lbm_mlp_train(lbm_mlp_trainer* t, lbm_mlp_model* m, int32_t epochs, int32_t batch, float lr, uint64_t seed,
                         float* loss_per_epoch) {
    if (!t || !model_ok(m) || epochs < 0 || batch < kBlk || batch % kBlk || batch > t->n || !(lr > 0.f))
        return mfail(LBM_ERR_INVALID, "lbm_mlp_train: bad arguments (batch: a multiple of 128, <= samples)");
    MCU(cudaSetDevice(t->device));
    const int blocks = batch / kBlk;
    const long long nb = t->n / batch;
    MCU(ensure_gpart(t, blocks));
    MCU(cudaMemcpyAsync(t->d_params, m->params, kMlpParams * sizeof(float), cudaMemcpyHostToDevice, t->st));
    MCU(cudaMemsetAsync(t->d_m, 0, kMlpParams * sizeof(float), t->st));
    MCU(cudaMemsetAsync(t->d_v, 0, kMlpParams * sizeof(float), t->st));
    MCU(cudaMemsetAsync(t->d_tick, 0, sizeof(int), t->st));
    const TrainNorm nm = train_norm(m, t->K);
    const float inv_batch = 1.0f / (float)batch;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    MCU(cudaStreamBeginCapture(t->st, cudaStreamCaptureModeThreadLocal));
    cudaError_t ce = cudaSuccess;
    for (long long b = 0; b < nb && ce == cudaSuccess; b++) {
        k_mlp_grad<<<blocks, kBlk, kSmemGrad, t->st>>>(t->d_samples, t->d_perm, b * batch, batch, t->d_params, nm,
                                                      t->d_gpart, t->d_tick);
        k_mlp_reduce<<<(kGradLen + 127) / 128, 128, 0, t->st>>>(t->d_gpart, blocks, inv_batch, t->d_params, t->d_m, t->d_v,
                                                               t->d_tick, lr, 0.9f, 0.999f, 1e-8f, 1, nullptr, t->d_loss);
        ce = cudaGetLastError();
    }
    cudaError_t ee = cudaStreamEndCapture(t->st, &graph);
    if (ce != cudaSuccess || ee != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return mfail(LBM_ERR_CUDA, std::string("lbm_mlp_train capture: ") +
                                       cudaGetErrorString(ce != cudaSuccess ? ce : ee));
    }
    cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
    std::vector<int32_t> perm((size_t)t->n);
    uint64_t s = seed;
    for (int ep = 0; ep < epochs && e == cudaSuccess; ep++) {
        for (long long i = 0; i < t->n; i++) perm[i] = (int32_t)i;
        for (long long i = t->n - 1; i > 0; i--) {
            const long long j = (long long)(splitmix(s) % (uint64_t)(i + 1));
            std::swap(perm[i], perm[j]);
        }
        e = cudaMemcpyAsync(t->d_perm, perm.data(), perm.size() * sizeof(int32_t), cudaMemcpyHostToDevice, t->st);
        if (e == cudaSuccess) e = cudaMemsetAsync(t->d_loss, 0, sizeof(double), t->st);
        if (e == cudaSuccess) e = cudaGraphLaunch(exec, t->st);
        double l = 0.0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&l, t->d_loss, sizeof(double), cudaMemcpyDeviceToHost, t->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(t->st);
        if (loss_per_epoch) loss_per_epoch[ep] = (float)(l / (double)(nb > 0 ? nb : 1));
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(m->params, t->d_params, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost, t->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(t->st);
    if (exec) cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return mfail(LBM_ERR_CUDA, std::string("lbm_mlp_train: ") + cudaGetErrorString(e));
    return LBM_OK;
}

}  // extern "C"
