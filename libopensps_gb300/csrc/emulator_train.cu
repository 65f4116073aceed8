// The emulator's training and its host side: the training set from this library's own CSP, the PCA of the log
// spectra, the ensemble's training (forward, reverse and Adam on the device), the weights file, and prediction with
// the fallback to the plain CSP.
//
// Training set: n samples drawn uniformly (seed) over the box of the ten inputs (log10 tau uniform), the spectra and
// magnitudes from opensps_context_compute_csp_batch on the context (SSP operators with a Kroupa IMF per model, the
// delayed-tau SFH formed on the device). Targets: the first 64 PCA coefficients of log10 of the spectrum (floored
// at 1e-6 of its peak, the exclusion rule of the spectral comparisons) and the magnitudes less the distance term
// (which the inference adds back exactly).
//
// Training: the five members in one set of launches (the grouped GEMMs of gemm_bf16x3.cu; each member its own
// minibatch order), bf16 operands with f32 accumulation as in the inference, f32 masters and Adam moments, a cosine
// learning rate. The reverse pass: dZ = dH * silu'(Z) (fused with the transposed copies the weight GEMMs read),
// dW = dZ^T A (split over K), dA = dZ W.
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cublas_v2.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>
#include "context.h"
#include "sm103_ptx.cuh"

namespace sps {

cudaError_t run_emu_infer(const Emulator &e, const EmuInferArgs &a, int num_sms, cudaStream_t st);
int emu_weight_box_rows();
int emu_weight_box_rows4();
int csp_batch_mags(Context &c, int n, int n_params, const char *const *names, const double *const *values,
                   double *mags, std::string &err);

static const char *const EMU_NAMES[EMU_NIN] = {"tau", "tage", "logzsol", "dust2", "dust_index", "zred",
                                               "sigma_smooth", "imf1", "imf2", "imf3"};
// The training box (raw values; tau drawn log-uniform, the others uniform): the delayed-tau SFH of the plain FP64
// configuration, the mixed configuration's dust, redshift and velocity ranges, the IMF slopes of the operator
// configuration.
static const double EMU_BOX_LO[EMU_NIN] = {0.1, 1.0, -2.0, 0.0, -1.0, 0.0, 50.0, 0.3, 1.3, 1.8};
static const double EMU_BOX_HI[EMU_NIN] = {10.0, 13.7, 0.5, 3.0, -0.4, 6.0, 300.0, 1.8, 2.8, 3.3};
constexpr double EMU_CLIP = 18.0;            // magnitude targets: at most this much fainter than the brightest band
constexpr float EMU_PCA_WEIGHT = 0.0625f;    // loss weight of a PCA coefficient (a magnitude: 1)

long long emu_param_count() {
    return EMU_MEMBERS * (EMU_W0 + 3 * EMU_WH + EMU_W4) + (long long)EMU_MEMBERS * EMU_NBIAS;
}
static long long n_w0() { return EMU_MEMBERS * EMU_W0; }
static long long n_wh() { return 3LL * EMU_MEMBERS * EMU_WH; }
static long long n_w4() { return EMU_MEMBERS * EMU_W4; }
static long long n_b() { return (long long)EMU_MEMBERS * EMU_NBIAS; }

void Emulator::release() {
    for (void *p : {(void *)w0, (void *)wh, (void *)w4, (void *)wht, (void *)w4t, (void *)bias, (void *)d_par,
                    (void *)d_pca_mean, (void *)d_pca_basis, (void *)master, (void *)adam_m, (void *)adam_v,
                    (void *)d_x, (void *)d_mags, (void *)d_coef, (void *)d_spread, (void *)d_flag, (void *)d_nflag,
                    (void *)d_flagged, (void *)d_scratch})
        if (p) cudaFree(p);
    w0 = wh = w4 = nullptr;
    wht = w4t = nullptr;
    bias = d_par = d_pca_mean = d_pca_basis = master = adam_m = adam_v = nullptr;
    d_x = d_mags = d_coef = d_spread = d_scratch = nullptr;
    d_flag = d_nflag = d_flagged = nullptr;
    cap = 0;
    ready = trainable = false;
    adam_t = 0;
    info.clear();
}

// ============================================================================================== kernels
__device__ __forceinline__ float silu_t(float z) {
    const float hz = 0.5f * z;
    return fmaf(hz, tanh_approx(hz), hz);
}
__device__ __forceinline__ float silu_grad(float z) {
    const float s = 0.5f + 0.5f * tanh_approx(0.5f * z);
    return s + z * s * (1.f - s);
}
__device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
    return x;
}
// A pseudo-random permutation of [0, n): a 4-round Feistel network on 2 * half bits, cycle-walked into [0, n).
__device__ __forceinline__ uint32_t emu_perm(uint32_t i, uint32_t n, int half, uint32_t key) {
    const uint32_t mask = (1u << half) - 1u;
    uint32_t x = i;
    do {
        uint32_t L = x >> half, R = x & mask;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const uint32_t t = L ^ (mix32(R ^ (key + (uint32_t)r * 0x9e3779b9u)) & mask);
            L = R;
            R = t;
        }
        x = (L << half) | R;
    } while (x >= n);
    return x;
}

struct EmuGatherArgs {
    int B, n_train, half, given;       // given: rows are the caller's (idx = row within the member)
    long long offset;                  // first position of this step in the epoch's order
    uint32_t key[EMU_MEMBERS];
    const float *xraw, *par;           // N x EMU_NIN, the parameter block
    const float *xstd;                 // given: B x EMU_NFEAT standardised features
    __half *X;                         // 5B x 64 f16: the features' hi parts at 0..11, lo parts at 16..27, zeros
    __nv_bfloat16 *Xt;                 // 5*64 x B bf16: the features at rows 0..11 (the weight gradient's operand)
    int *idx;                          // 5B
};
__global__ void emu_gather_kernel(EmuGatherArgs a) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= EMU_MEMBERS * a.B) return;
    const int g = row / a.B, i = row - g * a.B;
    float xs[EMU_NFEAT];
    int id;
    if (a.given) {
        id = i;
        for (int k = 0; k < EMU_NFEAT; ++k) xs[k] = a.xstd[(size_t)i * EMU_NFEAT + k];
    } else {
        id = (int)emu_perm((uint32_t)((a.offset + i) % a.n_train), (uint32_t)a.n_train, a.half, a.key[g]);
        float x[EMU_NIN];
        for (int k = 0; k < EMU_NIN; ++k) x[k] = a.xraw[(size_t)id * EMU_NIN + k];
        emu_features(x, a.par, xs);
    }
    a.idx[row] = id;
    for (int k = 0; k < EMU_NFEAT; ++k) {
        const __half hi = __float2half_rn(xs[k]);
        a.X[(size_t)row * EMU_KIN + k] = hi;
        a.X[(size_t)row * EMU_KIN + 16 + k] = __float2half_rn(xs[k] - __half2float(hi));
        a.Xt[(size_t)(g * EMU_KIN + k) * a.B + i] = __float2bfloat16_rn(xs[k]);
    }
}

// Z (f32, from the GEMM) + bias -> Z in place, H = silu(Z) (f16, the next layer's input) and its bf16 transpose
// per member (the weight gradient's operand); 64 x 64 tiles.
struct EmuActArgs {
    int B, C, bias_off;
    float *z;
    const float *bias;
    __half *h;
    __nv_bfloat16 *ht;
};
__global__ void __launch_bounds__(256) emu_act_fwd_kernel(EmuActArgs a) {
    __shared__ __nv_bfloat16 tt[64][66];
    const int c0 = blockIdx.x * 64, r0 = blockIdx.y * 64;
    const int g = r0 / a.B, b0 = r0 - g * a.B;
    const int cc = threadIdx.x & 63, rg = threadIdx.x >> 6;
    const float bv = a.bias[(size_t)g * EMU_NBIAS + a.bias_off + c0 + cc];
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const int rr = rg + 4 * k;
        const size_t o = (size_t)(r0 + rr) * a.C + c0 + cc;
        const float z = a.z[o] + bv;
        a.z[o] = z;
        const float hv = silu_t(z);
        a.h[o] = __float2half_rn(hv);
        tt[cc][rr] = __float2bfloat16_rn(hv);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const int c = rg + 4 * k, rr = cc;
        a.ht[(size_t)(g * a.C + c0 + c) * a.B + b0 + rr] = tt[c][rr];
    }
}

// dZ = dH silu'(Z) -> bf16 and its transpose per member, bias gradients (column sums); 64 x 64 tiles.
struct EmuBwdArgs {
    int B, C, bias_off;
    const float *dh, *z;
    __nv_bfloat16 *dz, *dzt;
    float *db;
};
__global__ void __launch_bounds__(256) emu_act_bwd_kernel(EmuBwdArgs a) {
    __shared__ __nv_bfloat16 tt[64][66];
    __shared__ float cs[4][64];
    const int c0 = blockIdx.x * 64, r0 = blockIdx.y * 64;
    const int g = r0 / a.B, b0 = r0 - g * a.B;
    const int cc = threadIdx.x & 63, rg = threadIdx.x >> 6;
    float sum = 0.f;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const int rr = rg + 4 * k;
        const size_t o = (size_t)(r0 + rr) * a.C + c0 + cc;
        const float d = a.dh[o] * silu_grad(a.z[o]);
        const __nv_bfloat16 dv = __float2bfloat16_rn(d);
        a.dz[o] = dv;
        tt[cc][rr] = dv;
        sum += __bfloat162float(dv);
    }
    cs[rg][cc] = sum;
    __syncthreads();
    if (threadIdx.x < 64)
        atomicAdd(&a.db[(size_t)g * EMU_NBIAS + a.bias_off + c0 + cc], cs[0][cc] + cs[1][cc] + cs[2][cc] + cs[3][cc]);
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const int c = rg + 4 * k, rr = cc;
        a.dzt[(size_t)(g * a.C + c0 + c) * a.B + b0 + rr] = tt[c][rr];
    }
}

// The output layer: Z + bias against the standardised targets -> the loss per member and dZ (bf16, transposed).
struct EmuOutArgs {
    int B;
    float scale;                         // 2 / (B sum_k w_k)
    float *z;                            // 5B x 128
    const float *bias, *y, *rw, *lossw;  // y: N x 128 (by idx), rw: N, lossw: 128
    const int *idx;
    __nv_bfloat16 *dz, *dzt;
    float *db, *loss;
};
__global__ void __launch_bounds__(256) emu_out_grad_kernel(EmuOutArgs a) {
    __shared__ __nv_bfloat16 tt[64][66];
    __shared__ float cs[4][64];
    __shared__ float ls[256];
    const int c0 = blockIdx.x * 64, r0 = blockIdx.y * 64;
    const int g = r0 / a.B, b0 = r0 - g * a.B;
    const int cc = threadIdx.x & 63, rg = threadIdx.x >> 6;
    const int col = c0 + cc;
    const float bv = a.bias[(size_t)g * EMU_NBIAS + 4 * EMU_H + col];
    const float wk = a.lossw[col];
    float sum = 0.f, lsum = 0.f;
#pragma unroll 4
    for (int k = 0; k < 16; ++k) {
        const int rr = rg + 4 * k;
        const size_t o = (size_t)(r0 + rr) * EMU_NOUT + col;
        const int id = a.idx[r0 + rr];
        const float z = a.z[o] + bv;
        a.z[o] = z;
        const float w = wk * a.rw[id];
        const float diff = w > 0.f ? z - a.y[(size_t)id * EMU_NOUT + col] : 0.f;   // excluded rows may hold non-finite targets
        lsum += w * diff * diff;
        const __nv_bfloat16 dv = __float2bfloat16_rn(a.scale * w * diff);
        a.dz[o] = dv;
        tt[cc][rr] = dv;
        sum += __bfloat162float(dv);
    }
    cs[rg][cc] = sum;
    ls[threadIdx.x] = lsum;
    __syncthreads();
    if (threadIdx.x < 64)
        atomicAdd(&a.db[(size_t)g * EMU_NBIAS + 4 * EMU_H + col], cs[0][cc] + cs[1][cc] + cs[2][cc] + cs[3][cc]);
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) ls[threadIdx.x] += ls[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(&a.loss[g], ls[0]);
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const int c = rg + 4 * k, rr = cc;
        a.dzt[(size_t)(g * EMU_NOUT + c0 + c) * a.B + b0 + rr] = tt[c][rr];
    }
}

// Adam on one tensor [members][rows][cols] (gradient = the sum of nsplit partials); writes the f16 copy (with
// tie16, columns < 12 also at column + 16: the features' lo parts) and, if wt, the bf16 transpose per member. With
// grad_out, only the summed gradient is stored (no update).
struct EmuAdamArgs {
    long long size;
    int rows, cols, nsplit, tie16;
    long long gstride;
    float *p, *m, *v;
    const float *g;
    __half *wb;
    __nv_bfloat16 *wt;
    float lr, b1, b2, eps, bc1, bc2;
    float *grad_out;
};
__device__ __forceinline__ void emu_store_weight(long long e, float p, int rows, int cols, int tie16, __half *wb,
                                                 __nv_bfloat16 *wt) {
    if (wb) {
        const __half h = __float2half_rn(p);
        wb[e] = h;
        if (tie16 && (e % cols) < EMU_NFEAT) wb[e + 16] = h;
    }
    if (wt) {
        const long long per = (long long)rows * cols;
        const long long mem = e / per, rem = e - mem * per;
        const int r = (int)(rem / cols), c = (int)(rem - (long long)r * cols);
        wt[mem * per + (long long)c * rows + r] = __float2bfloat16_rn(p);
    }
}
__global__ void emu_adam_kernel(EmuAdamArgs a) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= a.size) return;
    float gr = 0.f;
    for (int s = 0; s < a.nsplit; ++s) gr += a.g[s * a.gstride + e];
    if (a.grad_out) { a.grad_out[e] = gr; return; }
    const float m = a.b1 * a.m[e] + (1.f - a.b1) * gr;
    const float v = a.b2 * a.v[e] + (1.f - a.b2) * gr * gr;
    a.m[e] = m;
    a.v[e] = v;
    const float p = a.p[e] - a.lr * (m * a.bc1) / (sqrtf(v * a.bc2) + a.eps);
    a.p[e] = p;
    emu_store_weight(e, p, a.rows, a.cols, a.tie16, a.wb, a.wt);
}

// f32 masters -> f16 copies and bf16 transposes, after initialisation or a parameter upload (columns 16.. of the
// input layer are the tied lo-part weights: not copied from the masters).
__global__ void emu_cast_kernel(long long size, int rows, int cols, int tie16, const float *p, __half *wb,
                                __nv_bfloat16 *wt) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= size) return;
    if (tie16 && (e % cols) >= 16) return;
    emu_store_weight(e, p[e], rows, cols, tie16, wb, wt);
}

// log10 of each spectrum floored at 1e-6 of its peak (one block per model); rows that are not finite or have no
// positive pixel get weight 0 and zeros.
__global__ void __launch_bounds__(256) emu_logspec_kernel(int ns, const float *spec, float *out, float *rw) {
    __shared__ float red[256];
    __shared__ int badf;
    const int m = blockIdx.x;
    const float *s = spec + (size_t)m * ns;
    float mx = 0.f;
    int bad = 0;
    for (int j = threadIdx.x; j < ns; j += 256) {
        const float v = s[j];
        if (!isfinite(v)) bad = 1;
        mx = fmaxf(mx, v);
    }
    if (threadIdx.x == 0) badf = 0;
    red[threadIdx.x] = mx;
    __syncthreads();
    if (bad) badf = 1;
    for (int k = 128; k > 0; k >>= 1) {
        if (threadIdx.x < k) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + k]);
        __syncthreads();
    }
    const float peak = red[0];
    const bool ok = !badf && peak > 0.f;
    const float fl = peak * 1e-6f;
    float *o = out + (size_t)m * ns;
    for (int j = threadIdx.x; j < ns; j += 256) o[j] = ok ? log10f(fmaxf(s[j], fl)) : 0.f;
    if (threadIdx.x == 0 && !ok) rw[m] = 0.f;
}

// x -= mean per column (rows with weight 0 -> 0)
__global__ void emu_center_kernel(long long n, int ns, float *x, const float *mean, const float *rw) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * ns) return;
    const long long m = e / ns;
    const int j = (int)(e - m * ns);
    x[e] = rw[m] > 0.f ? x[e] - mean[j] : 0.f;
}

// Column sums and sums of squares (FP64) of y (rows x 128) over rows with weight > 0.
__global__ void emu_colstats_kernel(long long rows, const float *y, const float *rw, double *s1, double *s2,
                                    double *cnt) {
    const int col = threadIdx.x;
    double a = 0.0, b = 0.0, c = 0.0;
    for (long long r = blockIdx.x; r < rows; r += gridDim.x) {
        if (rw[r] > 0.f) {
            const double v = y[r * EMU_NOUT + col];
            a += v; b += v * v; c += 1.0;
        }
    }
    atomicAdd(&s1[col], a);
    atomicAdd(&s2[col], b);
    if (col == 0) atomicAdd(cnt, c);
}

__global__ void emu_standardise_y_kernel(long long rows, float *y, const float *mu, const float *sig) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= rows * EMU_NOUT) return;
    const int k = (int)(e % EMU_NOUT);
    y[e] = (y[e] - mu[k]) / sig[k];
}

// ============================================================================================== host helpers
namespace {

struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    double normal() {
        const double u1 = std::max(uniform(), 1e-300), u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
    }
};

template <class T>
cudaError_t dalloc(T **p, size_t count) {
    return cudaMalloc(reinterpret_cast<void **>(p), sizeof(T) * std::max<size_t>(count, 1));
}

std::string cmsg(const char *what, cudaError_t e) { return std::string(what) + ": " + cudaGetErrorString(e); }

int blocks(long long n, int t = 256) { return (int)((n + t - 1) / t); }

// Cyclic Jacobi eigen-decomposition of a symmetric k x k matrix (row-major, FP64): eigenvalues w, eigenvectors as
// the columns of V (row-major).
void jacobi_eigen(std::vector<double> A, int k, std::vector<double> &w, std::vector<double> &V) {
    V.assign((size_t)k * k, 0.0);
    for (int i = 0; i < k; ++i) V[(size_t)i * k + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0;
        for (int i = 0; i < k; ++i)
            for (int j = i + 1; j < k; ++j) off += A[(size_t)i * k + j] * A[(size_t)i * k + j];
        if (off < 1e-30) break;
        for (int p = 0; p < k; ++p)
            for (int q = p + 1; q < k; ++q) {
                const double apq = A[(size_t)p * k + q];
                if (std::fabs(apq) < 1e-300) continue;
                const double app = A[(size_t)p * k + p], aqq = A[(size_t)q * k + q];
                const double theta = (aqq - app) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int r = 0; r < k; ++r) {
                    const double arp = A[(size_t)r * k + p], arq = A[(size_t)r * k + q];
                    A[(size_t)r * k + p] = c * arp - s * arq;
                    A[(size_t)r * k + q] = s * arp + c * arq;
                }
                for (int r = 0; r < k; ++r) {
                    const double apr = A[(size_t)p * k + r], aqr = A[(size_t)q * k + r];
                    A[(size_t)p * k + r] = c * apr - s * aqr;
                    A[(size_t)q * k + r] = s * apr + c * aqr;
                }
                for (int r = 0; r < k; ++r) {
                    const double vrp = V[(size_t)r * k + p], vrq = V[(size_t)r * k + q];
                    V[(size_t)r * k + p] = c * vrp - s * vrq;
                    V[(size_t)r * k + q] = s * vrp + c * vrq;
                }
            }
    }
    w.resize(k);
    for (int i = 0; i < k; ++i) w[i] = A[(size_t)i * k + i];
}

// Orthonormal columns (modified Gram-Schmidt, twice) of Y (ns x k, column-major, FP64).
void orthonormalise(std::vector<double> &Y, int ns, int k) {
    for (int j = 0; j < k; ++j) {
        double *v = Y.data() + (size_t)j * ns;
        for (int pass = 0; pass < 2; ++pass)
            for (int i = 0; i < j; ++i) {
                const double *q = Y.data() + (size_t)i * ns;
                double d = 0.0;
                for (int t = 0; t < ns; ++t) d += q[t] * v[t];
                for (int t = 0; t < ns; ++t) v[t] -= d * q[t];
            }
        double nr = 0.0;
        for (int t = 0; t < ns; ++t) nr += v[t] * v[t];
        nr = std::sqrt(nr);
        for (int t = 0; t < ns; ++t) v[t] = nr > 0 ? v[t] / nr : 0.0;
    }
}

}  // namespace

// ---------------------------------------------------------------------------------------------- state setup
static int emu_alloc(Emulator &e, bool trainable, std::string &err) {
    cudaError_t r;
    if (!e.w0) {
        if ((r = dalloc(&e.w0, n_w0())) != cudaSuccess || (r = dalloc(&e.wh, n_wh())) != cudaSuccess ||
            (r = dalloc(&e.w4, n_w4())) != cudaSuccess || (r = dalloc(&e.bias, n_b())) != cudaSuccess ||
            (r = dalloc(&e.d_par, EMU_PAR)) != cudaSuccess) {
            err = cmsg("emulator weights", r);
            return ST_DATA_MISSING;
        }
        cudaMemset(e.w0, 0, sizeof(__half) * n_w0());
        cudaMemset(e.w4, 0, sizeof(__half) * n_w4());
        cudaMemset(e.bias, 0, sizeof(float) * n_b());
    }
    if (trainable && !e.master) {
        const long long np = n_w0() + n_wh() + n_w4();
        if ((r = dalloc(&e.wht, n_wh())) != cudaSuccess || (r = dalloc(&e.w4t, n_w4())) != cudaSuccess ||
            (r = dalloc(&e.master, np)) != cudaSuccess || (r = dalloc(&e.adam_m, np + n_b())) != cudaSuccess ||
            (r = dalloc(&e.adam_v, np + n_b())) != cudaSuccess) {
            err = cmsg("emulator training state", r);
            return ST_DATA_MISSING;
        }
        cudaMemset(e.adam_m, 0, sizeof(float) * (np + n_b()));
        cudaMemset(e.adam_v, 0, sizeof(float) * (np + n_b()));
        e.trainable = true;
        e.adam_t = 0;
    }
    // the inference kernel's boxes: a whole hidden-layer tile (256 rows) and a whole output-layer tile (128 rows)
    const uint32_t rows = (uint32_t)emu_weight_box_rows(), rows4 = (uint32_t)emu_weight_box_rows4();
    cudaError_t r1 = encode_tmap_2d_16(&e.tm_w0, e.w0, EMU_KIN, (uint64_t)EMU_MEMBERS * EMU_H, 64, rows, true);
    cudaError_t r2 = encode_tmap_2d_16(&e.tm_wh, e.wh, EMU_H, 3ull * EMU_MEMBERS * EMU_H, 64, rows, true);
    cudaError_t r3 = encode_tmap_2d_16(&e.tm_w4, e.w4, EMU_H, (uint64_t)EMU_MEMBERS * EMU_NOUT, 64, rows4, true);
    if (r1 != cudaSuccess || r2 != cudaSuccess || r3 != cudaSuccess) {
        err = "emulator weight tensor maps";
        return ST_DATA_MISSING;
    }
    return 0;
}

// the standardisation of the inputs from the box, the cosmology table of the context
static void emu_set_box(Context &c, Emulator &e) {
    for (int i = 0; i < EMU_NIN; ++i) {
        e.box_lo[i] = EMU_BOX_LO[i];
        e.box_hi[i] = EMU_BOX_HI[i];
        const double flo = emu_feature(i, (float)e.box_lo[i]), fhi = emu_feature(i, (float)e.box_hi[i]);
        e.par[EMU_P_INC + i] = (float)(0.5 * (flo + fhi));
        e.par[EMU_P_INS + i] = (float)(2.0 / (fhi - flo));
    }
    for (int i = EMU_NIN; i < EMU_NFEAT; ++i) {     // the grid clocks, in [0, 1]
        e.par[EMU_P_INC + i] = 0.5f;
        e.par[EMU_P_INS + i] = 2.f;
    }
    // the clocks' grids (off when a grid is not evenly spaced)
    auto uniform_step = [](const std::vector<double> &v) -> double {
        if (v.size() < 2) return 0.0;
        const double d = (v.back() - v.front()) / (double)(v.size() - 1);
        for (size_t i = 1; i < v.size(); ++i)
            if (std::fabs((v[i] - v[i - 1]) - d) > 1e-6 * std::fabs(d)) return 0.0;
        return d;
    };
    std::vector<double> lz(c.zlegend.size());
    for (size_t i = 0; i < lz.size(); ++i) lz[i] = std::log10(c.zlegend[i] / c.zsol);
    e.par[EMU_P_CLK] = c.log_age.empty() ? 0.f : (float)c.log_age.front();
    e.par[EMU_P_CLK + 1] = (float)uniform_step(c.log_age);
    e.par[EMU_P_CLK + 2] = lz.empty() ? 0.f : (float)lz.front();
    e.par[EMU_P_CLK + 3] = (float)uniform_step(lz);
    for (int i = 0; i < 500; ++i) {
        e.par[EMU_P_ZT + i] = (float)c.zt[i];
        e.par[EMU_P_DL + i] = (float)c.dl[i];
    }
}

// Random initial weights (member-specific): uniform with variance 2 / fan_in (hidden, input), 0.1 / fan_in
// (output); zero biases; zero pads.
static int emu_init_params(Context &c, Emulator &e, uint64_t seed, std::string &err) {
    (void)c;
    const long long np = n_w0() + n_wh() + n_w4();
    std::vector<float> h((size_t)np, 0.f);
    Rng rng(seed * 0x2545F4914F6CDD1Dull + 7);
    float *w0 = h.data(), *wh = w0 + n_w0(), *w4 = wh + n_wh();
    for (int g = 0; g < EMU_MEMBERS; ++g)
        for (int o = 0; o < EMU_H; ++o)
            for (int k = 0; k < EMU_NFEAT; ++k)
                w0[((size_t)g * EMU_H + o) * EMU_KIN + k] = (float)((2.0 * rng.uniform() - 1.0) * std::sqrt(6.0 / EMU_NFEAT));
    for (long long i = 0; i < n_wh(); ++i) wh[i] = (float)((2.0 * rng.uniform() - 1.0) * std::sqrt(6.0 / EMU_H));
    for (int g = 0; g < EMU_MEMBERS; ++g)
        for (int o = 0; o < EMU_NPC + e.nb; ++o)
            for (int k = 0; k < EMU_H; ++k)
                w4[((size_t)g * EMU_NOUT + o) * EMU_H + k] = (float)((2.0 * rng.uniform() - 1.0) * std::sqrt(0.3 / EMU_H));
    cudaError_t r;
    if ((r = cudaMemcpy(e.master, h.data(), sizeof(float) * np, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (r = cudaMemset(e.bias, 0, sizeof(float) * n_b())) != cudaSuccess) {
        err = cmsg("emulator initial weights", r);
        return ST_DATA_MISSING;
    }
    return 0;
}

// bf16 copies of the masters
static cudaError_t emu_cast_all(Emulator &e, cudaStream_t st) {
    float *m0 = e.master, *mh = m0 + n_w0(), *m4 = mh + n_wh();
    emu_cast_kernel<<<blocks(n_w0()), 256, 0, st>>>(n_w0(), EMU_H, EMU_KIN, 1, m0, e.w0, nullptr);
    for (int l = 0; l < 3; ++l)
        emu_cast_kernel<<<blocks(EMU_MEMBERS * EMU_WH), 256, 0, st>>>(EMU_MEMBERS * EMU_WH, EMU_H, EMU_H, 0,
                                                                      mh + l * EMU_MEMBERS * EMU_WH,
                                                                      e.wh + l * EMU_MEMBERS * EMU_WH,
                                                                      e.wht + l * EMU_MEMBERS * EMU_WH);
    emu_cast_kernel<<<blocks(n_w4()), 256, 0, st>>>(n_w4(), EMU_NOUT, EMU_H, 0, m4, e.w4, e.w4t);
    return cudaGetLastError();
}

static int emu_upload_par(Emulator &e, std::string &err) {
    cudaError_t r = cudaMemcpy(e.d_par, e.par, sizeof(float) * EMU_PAR, cudaMemcpyHostToDevice);
    if (r != cudaSuccess) { err = cmsg("emulator parameters", r); return ST_DATA_MISSING; }
    return 0;
}

// ---------------------------------------------------------------------------------------------- one training step
// Scratch of the training steps at minibatch B.
struct EmuTrainBufs {
    int B = 0, S = 8;
    __half *X = nullptr, *H[5] = {};                                   // forward operands (f16)
    __nv_bfloat16 *Xt = nullptr, *Ht[5] = {}, *dz = nullptr, *dzt = nullptr;   // reverse operands (bf16)
    float *Z[5] = {}, *dh = nullptr, *gpart = nullptr, *db = nullptr, *loss = nullptr, *lossw = nullptr;
    int *idx = nullptr;
    CUtensorMap tmX, tmXt, tmH[5], tmHt[5], tmDz, tmDz4, tmDzt, tmDzt4, tmW0, tmWh[3], tmW4, tmWht[3], tmW4t;
    void release() {
        for (void *p : {(void *)X, (void *)Xt, (void *)dz, (void *)dzt, (void *)dh, (void *)gpart, (void *)db,
                        (void *)loss, (void *)lossw, (void *)idx})
            if (p) cudaFree(p);
        for (int i = 0; i < 5; ++i) {
            if (H[i]) cudaFree(H[i]);
            if (Ht[i]) cudaFree(Ht[i]);
            if (Z[i]) cudaFree(Z[i]);
            H[i] = nullptr;
            Ht[i] = nullptr;
            Z[i] = nullptr;
        }
        X = nullptr;
        Xt = dz = dzt = nullptr;
        dh = gpart = db = loss = lossw = nullptr;
        idx = nullptr;
    }
};

static int emu_bufs(Emulator &e, EmuTrainBufs &b, int B, std::string &err) {
    b.B = B;
    b.S = std::min(8, B / 64);
    const size_t R = (size_t)EMU_MEMBERS * B;
    cudaError_t r = cudaSuccess;
    auto ok = [&](cudaError_t x) { if (x != cudaSuccess && r == cudaSuccess) r = x; };
    ok(dalloc(&b.X, R * EMU_KIN));
    ok(dalloc(&b.Xt, R * EMU_KIN));
    for (int l = 1; l <= 4; ++l) { ok(dalloc(&b.H[l], R * EMU_H)); ok(dalloc(&b.Ht[l], R * EMU_H)); }
    for (int l = 0; l < 4; ++l) ok(dalloc(&b.Z[l], R * EMU_H));
    ok(dalloc(&b.Z[4], R * EMU_NOUT));
    ok(dalloc(&b.dz, R * EMU_H));
    ok(dalloc(&b.dzt, R * EMU_H));
    ok(dalloc(&b.dh, R * EMU_H));
    ok(dalloc(&b.gpart, (size_t)b.S * EMU_MEMBERS * EMU_WH));
    ok(dalloc(&b.db, (size_t)n_b()));
    ok(dalloc(&b.loss, 8));
    ok(dalloc(&b.lossw, EMU_NOUT));
    ok(dalloc(&b.idx, R));
    if (r != cudaSuccess) { err = cmsg("emulator training buffers", r); return ST_DATA_MISSING; }
    cudaMemset(b.X, 0, sizeof(__half) * R * EMU_KIN);
    cudaMemset(b.Xt, 0, sizeof(__nv_bfloat16) * R * EMU_KIN);
    const int bm = gemm_bm(), bn = gemm_bn(), bk = gemm_bk();
    cudaError_t t = cudaSuccess;
    auto tm = [&](CUtensorMap *m, const void *p, uint64_t inner, uint64_t outer, uint32_t box_outer, bool f16 = false) {
        cudaError_t x = encode_tmap_2d_16(m, p, inner, outer, bk, box_outer, f16);
        if (x != cudaSuccess && t == cudaSuccess) t = x;
    };
    // A operands (box 64 x 128) and B operands (box 64 x 256)
    tm(&b.tmX, b.X, EMU_KIN, R, bm, true);
    tm(&b.tmXt, b.Xt, B, (uint64_t)EMU_MEMBERS * EMU_KIN, bn);
    for (int l = 1; l <= 4; ++l) {
        tm(&b.tmH[l], b.H[l], EMU_H, R, bm, true);
        tm(&b.tmHt[l], b.Ht[l], B, (uint64_t)EMU_MEMBERS * EMU_H, bn);
    }
    tm(&b.tmDz, b.dz, EMU_H, R, bm);
    tm(&b.tmDz4, b.dz, EMU_NOUT, R, bm);
    tm(&b.tmDzt, b.dzt, B, (uint64_t)EMU_MEMBERS * EMU_H, bm);
    tm(&b.tmDzt4, b.dzt, B, (uint64_t)EMU_MEMBERS * EMU_NOUT, bm);
    tm(&b.tmW0, e.w0, EMU_KIN, (uint64_t)EMU_MEMBERS * EMU_H, bn, true);
    for (int l = 0; l < 3; ++l) {
        tm(&b.tmWh[l], e.wh + (size_t)l * EMU_MEMBERS * EMU_WH, EMU_H, (uint64_t)EMU_MEMBERS * EMU_H, bn, true);
        tm(&b.tmWht[l], e.wht + (size_t)l * EMU_MEMBERS * EMU_WH, EMU_H, (uint64_t)EMU_MEMBERS * EMU_H, bn);
    }
    tm(&b.tmW4, e.w4, EMU_H, (uint64_t)EMU_MEMBERS * EMU_NOUT, bn, true);
    tm(&b.tmW4t, e.w4t, EMU_NOUT, (uint64_t)EMU_MEMBERS * EMU_H, bn);
    if (t != cudaSuccess) { err = cmsg("emulator training tensor maps", t); return ST_DATA_MISSING; }
    return 0;
}

static cudaError_t gemm1(const CUtensorMap &ta, const CUtensorMap &tb, int M, int N, int K, float *D, int ldd,
                         long long a_grp, long long b_grp, long long d_grp, int ksplit, long long d_split,
                         int num_sms, int *status, cudaStream_t st, int f16 = 0) {
    GemmPlan pl;
    pl.tm_a_hi = ta; pl.tm_a_lo = ta; pl.tm_b_hi = tb; pl.tm_b_lo = tb;
    pl.num_sms = num_sms;
    GemmArgs g;
    g.M = M; g.N = N; g.K = K; g.ldd = ldd; g.b_row0 = 0; g.D = D; g.status = status;
    g.groups = EMU_MEMBERS; g.ksplit = ksplit; g.a_grp = a_grp; g.b_grp = b_grp; g.d_grp = d_grp; g.d_split = d_split;
    g.f16 = f16;
    return run_gemm_bf16(pl, g, st);
}

struct EmuStepCfg {
    float lr = 1e-3f;
    bool apply = true;           // false: store the gradients (grad_out) instead of an Adam step
    float *grad_out = nullptr;   // device, emu_param_count() floats: [w0 | wh | w4 | bias]
};

// One forward and reverse pass of the five members over the minibatch already gathered into b.X / b.Xt / b.idx,
// then Adam (or the gradients into cfg.grad_out). y, rw: the standardised targets and row weights.
static int emu_step(Context &c, Emulator &e, EmuTrainBufs &b, const float *y, const float *rw, float scale,
                    const EmuStepCfg &cfg, std::string &err) {
    cudaStream_t st = c.stream;
    const int B = b.B, S = b.S;
    const long long R = (long long)EMU_MEMBERS * B;
    int *status = c.d_status.p;
    cudaError_t r;
#define EMU_CHECK(x, what) if ((r = (x)) != cudaSuccess) { err = cmsg(what, r); return ST_DATA_MISSING; }
    // ---- forward
    for (int L = 0; L < 4; ++L) {
        const CUtensorMap &ta = L == 0 ? b.tmX : b.tmH[L];
        const CUtensorMap &tb = L == 0 ? b.tmW0 : b.tmWh[L - 1];
        EMU_CHECK(gemm1(ta, tb, B, EMU_H, L == 0 ? EMU_KIN : EMU_H, b.Z[L], EMU_H, B, EMU_H, (long long)B * EMU_H, 1, 0,
                        c.num_sms, status, st, 1), "emulator forward GEMM");
        EmuActArgs aa;
        aa.B = B; aa.C = EMU_H; aa.bias_off = L * EMU_H; aa.z = b.Z[L]; aa.bias = e.bias; aa.h = b.H[L + 1]; aa.ht = b.Ht[L + 1];
        emu_act_fwd_kernel<<<dim3(EMU_H / 64, (unsigned)(R / 64)), 256, 0, st>>>(aa);
        EMU_CHECK(cudaGetLastError(), "emulator activation kernel");
    }
    EMU_CHECK(gemm1(b.tmH[4], b.tmW4, B, EMU_NOUT, EMU_H, b.Z[4], EMU_NOUT, B, EMU_NOUT, (long long)B * EMU_NOUT, 1, 0,
                    c.num_sms, status, st, 1), "emulator output GEMM");
    cudaMemsetAsync(b.db, 0, sizeof(float) * n_b(), st);
    cudaMemsetAsync(b.loss, 0, sizeof(float) * 8, st);
    EmuOutArgs oa;
    oa.B = B; oa.scale = scale; oa.z = b.Z[4]; oa.bias = e.bias; oa.y = y; oa.rw = rw; oa.lossw = b.lossw;
    oa.idx = b.idx; oa.dz = b.dz; oa.dzt = b.dzt; oa.db = b.db; oa.loss = b.loss;
    emu_out_grad_kernel<<<dim3(EMU_NOUT / 64, (unsigned)(R / 64)), 256, 0, st>>>(oa);
    EMU_CHECK(cudaGetLastError(), "emulator output gradient kernel");

    // ---- reverse, layer 4 down to 0; each layer's weights are updated right after their last use
    ++e.adam_t;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = (float)(1.0 / (1.0 - std::pow((double)b1, (double)e.adam_t)));
    const float bc2 = (float)(1.0 / (1.0 - std::pow((double)b2, (double)e.adam_t)));
    float *m0 = e.master, *mh = m0 + n_w0(), *m4 = mh + n_wh();
    const long long off_h = n_w0(), off_4 = n_w0() + n_wh(), off_b = n_w0() + n_wh() + n_w4();
    auto adam = [&](long long size, int rows, int cols, float *p, long long moff, const float *gsrc, int nsplit,
                    long long gstride, __half *wb, __nv_bfloat16 *wt, long long goff, int tie16) -> cudaError_t {
        EmuAdamArgs ad;
        ad.size = size; ad.rows = rows; ad.cols = cols; ad.nsplit = nsplit; ad.gstride = gstride;
        ad.p = p; ad.m = e.adam_m + moff; ad.v = e.adam_v + moff; ad.g = gsrc; ad.wb = wb; ad.wt = wt; ad.tie16 = tie16;
        ad.lr = cfg.lr; ad.b1 = b1; ad.b2 = b2; ad.eps = 1e-8f; ad.bc1 = bc1; ad.bc2 = bc2;
        ad.grad_out = cfg.apply ? nullptr : cfg.grad_out + goff;
        emu_adam_kernel<<<blocks(size), 256, 0, st>>>(ad);
        return cudaGetLastError();
    };
    // layer 4 (output): dW4 = dZ4^T H4, dH4 = dZ4 W4
    EMU_CHECK(gemm1(b.tmDzt4, b.tmHt[4], EMU_NOUT, EMU_H, B, b.gpart, EMU_H, EMU_NOUT, EMU_H, EMU_W4, S, n_w4(),
                    c.num_sms, status, st), "emulator weight-gradient GEMM");
    EMU_CHECK(gemm1(b.tmDz4, b.tmW4t, B, EMU_H, EMU_NOUT, b.dh, EMU_H, B, EMU_H, (long long)B * EMU_H, 1, 0,
                    c.num_sms, status, st), "emulator input-cotangent GEMM");
    EMU_CHECK(adam(n_w4(), EMU_NOUT, EMU_H, m4, off_4, b.gpart, S, n_w4(), e.w4, e.w4t, off_4, 0), "emulator Adam");
    for (int L = 3; L >= 0; --L) {
        EmuBwdArgs ba;
        ba.B = B; ba.C = EMU_H; ba.bias_off = L * EMU_H; ba.dh = b.dh; ba.z = b.Z[L]; ba.dz = b.dz; ba.dzt = b.dzt; ba.db = b.db;
        emu_act_bwd_kernel<<<dim3(EMU_H / 64, (unsigned)(R / 64)), 256, 0, st>>>(ba);
        EMU_CHECK(cudaGetLastError(), "emulator activation reverse kernel");
        if (L > 0) {
            const int l = L - 1;
            const long long per = (long long)EMU_MEMBERS * EMU_WH;
            EMU_CHECK(gemm1(b.tmDzt, b.tmHt[L], EMU_H, EMU_H, B, b.gpart, EMU_H, EMU_H, EMU_H, EMU_WH, S, per,
                            c.num_sms, status, st), "emulator weight-gradient GEMM");
            EMU_CHECK(gemm1(b.tmDz, b.tmWht[l], B, EMU_H, EMU_H, b.dh, EMU_H, B, EMU_H, (long long)B * EMU_H, 1, 0,
                            c.num_sms, status, st), "emulator input-cotangent GEMM");
            EMU_CHECK(adam(per, EMU_H, EMU_H, mh + l * per, off_h + l * per, b.gpart, S, per, e.wh + l * per,
                           e.wht + l * per, off_h + l * per, 0), "emulator Adam");
        } else {
            EMU_CHECK(gemm1(b.tmDzt, b.tmXt, EMU_H, EMU_KIN, B, b.gpart, EMU_KIN, EMU_H, EMU_KIN, EMU_W0, S, n_w0(),
                            c.num_sms, status, st), "emulator weight-gradient GEMM");
            EMU_CHECK(adam(n_w0(), EMU_H, EMU_KIN, m0, 0, b.gpart, S, n_w0(), e.w0, nullptr, 0, 1), "emulator Adam");
        }
    }
    EMU_CHECK(adam(n_b(), 1, EMU_NBIAS, e.bias, off_b, b.db, 1, n_b(), nullptr, nullptr, off_b, 0), "emulator Adam");
#undef EMU_CHECK
    return 0;
}

// ---------------------------------------------------------------------------------------------- inference scratch
static int emu_scratch(Emulator &e, int n, std::string &err) {
    if (n <= e.cap) return 0;
    for (void *p : {(void *)e.d_x, (void *)e.d_mags, (void *)e.d_coef, (void *)e.d_spread, (void *)e.d_flag,
                    (void *)e.d_flagged})
        if (p) cudaFree(p);
    e.d_x = e.d_mags = e.d_coef = e.d_spread = nullptr;
    e.d_flag = e.d_flagged = nullptr;
    cudaError_t r = cudaSuccess;
    auto ok = [&](cudaError_t x) { if (x != cudaSuccess && r == cudaSuccess) r = x; };
    ok(dalloc(&e.d_x, (size_t)n * EMU_NIN));
    ok(dalloc(&e.d_mags, (size_t)n * EMU_MAX_BANDS));
    ok(dalloc(&e.d_coef, (size_t)n * EMU_NPC));
    ok(dalloc(&e.d_spread, (size_t)n));
    ok(dalloc(&e.d_flag, (size_t)n));
    ok(dalloc(&e.d_flagged, (size_t)n));
    if (!e.d_nflag) ok(dalloc(&e.d_nflag, 4));
    if (r != cudaSuccess) { err = cmsg("emulator scratch", r); e.cap = 0; return ST_DATA_MISSING; }
    e.cap = n;
    return 0;
}

// The ensemble on n device inputs (n x 10 floats): outputs into the given device arrays.
int emu_infer_device(Context &c, int n, const float *d_x, float *d_mags, float *d_coef, float *d_spread, int *d_flag,
                     int *d_nflag, int *d_flagged, std::string &err) {
    Emulator &e = c.emu;
    if (!e.ready) { err = "no emulator on the context (opensps_gb300_emulator_load / _train)"; return ST_NO_OPERATOR; }
    if (e.nb != c.nbands) { err = "the emulator was trained for another band set"; return ST_UNSUPPORTED; }
    if (!e.d_scratch) {
        const cudaError_t r = dalloc(&e.d_scratch, (size_t)c.num_sms * EMU_SCRATCH_CTA);
        if (r != cudaSuccess) { err = cmsg("emulator scratch", r); return ST_DATA_MISSING; }
    }
    EmuInferArgs a;
    a.n = n; a.nb = e.nb; a.x = d_x; a.bias = e.bias; a.par = e.d_par; a.spread_max = e.spread_max; a.faint = e.faint;
    a.scratch = e.d_scratch;
    a.mags = d_mags; a.coef = d_coef; a.spread = d_spread; a.flag = d_flag; a.nflag = d_nflag; a.flagged = d_flagged;
    a.status = c.d_status.p;
    cudaMemsetAsync(c.d_status.p, 0, sizeof(int), c.stream);
    cudaMemsetAsync(d_nflag, 0, sizeof(int), c.stream);
    cudaError_t r = run_emu_infer(e, a, c.num_sms, c.stream);
    if (r != cudaSuccess) { err = cmsg("emulator kernel", r); return ST_DATA_MISSING; }
    return 0;
}

static int check_status(Context &c, std::string &err) {
    int s = 0;
    cudaError_t r = cudaMemcpyAsync(&s, c.d_status.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream);
    if (r == cudaSuccess) r = cudaStreamSynchronize(c.stream);
    if (r != cudaSuccess) { err = cmsg("emulator", r); return ST_DATA_MISSING; }
    if (s != 0) {
        char b[96];
        std::snprintf(b, sizeof b, "emulator kernel gave up waiting (code 0x%x)", s);
        err = b;
        return ST_DATA_MISSING;
    }
    return 0;
}

// ---------------------------------------------------------------------------------------------- PCA
// Mean and the first EMU_NPC principal directions of the rows of L (P x ns, f32, weights rw): covariance by SGEMM,
// subspace iteration (96 vectors) with FP64 Gram-Schmidt on the host, Rayleigh-Ritz with Jacobi.
static int emu_pca(Context &c, Emulator &e, float *L, const float *rw, long long P, std::vector<double> &explained,
                   std::string &err) {
    const int ns = c.nspec, k = 96;
    cudaStream_t st = c.stream;
    if (!c.cublas) {
        cublasHandle_t h;
        if (cublasCreate(&h) != CUBLAS_STATUS_SUCCESS) { err = "cuBLAS could not be initialised"; return ST_DATA_MISSING; }
        c.cublas = h;
    }
    cublasHandle_t h = static_cast<cublasHandle_t>(c.cublas);
    cublasSetStream(h, st);
    float *mean = nullptr, *C = nullptr, *Q = nullptr, *Y = nullptr;
    cudaError_t r = cudaSuccess;
    auto ok = [&](cudaError_t x) { if (x != cudaSuccess && r == cudaSuccess) r = x; };
    ok(dalloc(&mean, ns)); ok(dalloc(&C, (size_t)ns * ns)); ok(dalloc(&Q, (size_t)ns * k)); ok(dalloc(&Y, (size_t)ns * k));
    if (r != cudaSuccess) { err = cmsg("PCA buffers", r); return ST_DATA_MISSING; }
    int rc = 0;
    std::vector<float> rwh((size_t)P);
    cudaMemcpy(rwh.data(), rw, sizeof(float) * P, cudaMemcpyDeviceToHost);
    double wsum = 0.0;
    for (float v : rwh) wsum += v;
    const float inv = wsum > 0 ? (float)(1.0 / wsum) : 0.f, zero = 0.f, one = 1.f;
    std::vector<double> Yh((size_t)ns * k), Qh((size_t)ns * k);
    std::vector<float> f((size_t)ns * k);
    Rng rng(12345);
    if (cublasSgemv(h, CUBLAS_OP_N, ns, (int)P, &inv, L, ns, rw, 1, &zero, mean, 1) != CUBLAS_STATUS_SUCCESS) {
        err = "PCA mean"; rc = ST_DATA_MISSING; goto done;
    }
    emu_center_kernel<<<blocks(P * ns), 256, 0, st>>>(P, ns, L, mean, rw);
    if (cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_T, ns, ns, (int)P, &inv, L, ns, L, ns, &zero, C, ns) != CUBLAS_STATUS_SUCCESS) {
        err = "PCA covariance"; rc = ST_DATA_MISSING; goto done;
    }
    for (auto &v : Qh) v = rng.normal();
    orthonormalise(Qh, ns, k);
    for (int it = 0; it < 30; ++it) {
        for (size_t i = 0; i < f.size(); ++i) f[i] = (float)Qh[i];
        cudaMemcpyAsync(Q, f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice, st);
        cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, ns, k, ns, &one, C, ns, Q, ns, &zero, Y, ns);
        cudaMemcpyAsync(f.data(), Y, sizeof(float) * f.size(), cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        for (size_t i = 0; i < f.size(); ++i) Qh[i] = f[i];
        orthonormalise(Qh, ns, k);
    }
    {
        // Rayleigh-Ritz: T = Q^T C Q
        for (size_t i = 0; i < f.size(); ++i) f[i] = (float)Qh[i];
        cudaMemcpyAsync(Q, f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice, st);
        cublasSgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, ns, k, ns, &one, C, ns, Q, ns, &zero, Y, ns);
        cudaMemcpyAsync(f.data(), Y, sizeof(float) * f.size(), cudaMemcpyDeviceToHost, st);
        std::vector<float> diag((size_t)ns);
        cudaMemcpy2DAsync(diag.data(), sizeof(float), C, sizeof(float) * (ns + 1), sizeof(float), ns, cudaMemcpyDeviceToHost, st);
        std::vector<float> mh((size_t)ns);
        cudaMemcpyAsync(mh.data(), mean, sizeof(float) * ns, cudaMemcpyDeviceToHost, st);
        if ((r = cudaStreamSynchronize(st)) != cudaSuccess) { err = cmsg("PCA", r); rc = ST_DATA_MISSING; goto done; }
        std::vector<double> T((size_t)k * k, 0.0);
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j) {
                double s = 0.0;
                for (int t = 0; t < ns; ++t) s += Qh[(size_t)i * ns + t] * (double)f[(size_t)j * ns + t];
                T[(size_t)i * k + j] = s;
            }
        for (int i = 0; i < k; ++i)
            for (int j = i + 1; j < k; ++j) T[(size_t)i * k + j] = T[(size_t)j * k + i] = 0.5 * (T[(size_t)i * k + j] + T[(size_t)j * k + i]);
        std::vector<double> w, V;
        jacobi_eigen(T, k, w, V);
        std::vector<int> order(k);
        for (int i = 0; i < k; ++i) order[i] = i;
        std::sort(order.begin(), order.end(), [&](int a, int b) { return w[a] > w[b]; });
        double trace = 0.0;
        for (float d : diag) trace += d;
        e.pca_basis.assign((size_t)EMU_NPC * ns, 0.f);
        explained.clear();
        double cum = 0.0;
        for (int pc = 0; pc < EMU_NPC; ++pc) {
            const int col = order[pc];
            cum += w[col];
            explained.push_back(trace > 0 ? cum / trace : 0.0);
            for (int t = 0; t < ns; ++t) {
                double s = 0.0;
                for (int i = 0; i < k; ++i) s += Qh[(size_t)i * ns + t] * V[(size_t)i * k + col];
                e.pca_basis[(size_t)pc * ns + t] = (float)s;
            }
        }
        e.pca_mean = mh;
    }
done:
    cudaFree(mean); cudaFree(C); cudaFree(Q); cudaFree(Y);
    return rc;
}

// coefficients (rows x EMU_NPC, written into y with row stride EMU_NOUT) of centred log spectra L (rows x ns)
static int emu_project(Context &c, const float *L, long long rows, float *y, std::string &err) {
    cublasHandle_t h = static_cast<cublasHandle_t>(c.cublas);
    cublasSetStream(h, c.stream);
    const float one = 1.f, zero = 0.f;
    if (cublasSgemm(h, CUBLAS_OP_T, CUBLAS_OP_N, EMU_NPC, (int)rows, c.nspec, &one, c.emu.d_pca_basis, c.nspec, L,
                    c.nspec, &zero, y, EMU_NOUT) != CUBLAS_STATUS_SUCCESS) {
        err = "PCA projection";
        return ST_DATA_MISSING;
    }
    return 0;
}

// ---------------------------------------------------------------------------------------------- validation
// Errors of the ensemble's magnitudes against the CSP's over nv models: fills info entries.
static int emu_validate(Context &c, const float *d_xval, const std::vector<double> &mags_true, int nv,
                        std::vector<double> &out, std::string &err) {
    Emulator &e = c.emu;
    if (int rc = emu_scratch(e, nv, err)) return rc;
    if (int rc = emu_infer_device(c, nv, d_xval, e.d_mags, e.d_coef, e.d_spread, e.d_flag, e.d_nflag, e.d_flagged, err)) return rc;
    if (int rc = check_status(c, err)) return rc;
    const int nb = e.nb;
    std::vector<float> mg((size_t)nv * nb);
    std::vector<int> fl(nv);
    cudaMemcpy(mg.data(), e.d_mags, sizeof(float) * mg.size(), cudaMemcpyDeviceToHost);
    cudaMemcpy(fl.data(), e.d_flag, sizeof(int) * nv, cudaMemcpyDeviceToHost);
    double se = 0.0, cnt = 0.0, mx_all = 0.0, mx_ok = 0.0;
    int nflag = 0;
    std::vector<double> errs;
    for (int m = 0; m < nv; ++m) {
        double mmin = 1e300;
        for (int b = 0; b < nb; ++b) mmin = std::min(mmin, mags_true[(size_t)b + (size_t)nb * m]);
        double em = 0.0;
        for (int b = 0; b < nb; ++b) {
            const double t = mags_true[(size_t)b + (size_t)nb * m];
            if (!(t < mmin + e.faint) || !std::isfinite(t)) continue;
            const double d = std::fabs((double)mg[(size_t)m * nb + b] - t);
            se += d * d; cnt += 1.0;
            em = std::max(em, d);
        }
        errs.push_back(em);
        mx_all = std::max(mx_all, em);
        if (fl[m]) ++nflag; else mx_ok = std::max(mx_ok, em);
    }
    std::sort(errs.begin(), errs.end());
    out = {cnt > 0 ? std::sqrt(se / cnt) : 0.0, mx_all, errs.empty() ? 0.0 : errs[(size_t)(0.99 * (errs.size() - 1))],
           nv > 0 ? (double)nflag / nv : 0.0, mx_ok};
    return 0;
}

// ---------------------------------------------------------------------------------------------- weights file
static const char EMU_MAGIC[8] = {'O', 'P', 'S', 'E', 'M', 'U', '0', '4'};

static int emu_save(Context &c, const std::string &path, std::string &err) {
    Emulator &e = c.emu;
    std::vector<__half> w0((size_t)n_w0()), wh((size_t)n_wh()), w4((size_t)n_w4());
    std::vector<float> bias((size_t)n_b());
    cudaMemcpy(w0.data(), e.w0, sizeof(__half) * w0.size(), cudaMemcpyDeviceToHost);
    cudaMemcpy(wh.data(), e.wh, sizeof(__half) * wh.size(), cudaMemcpyDeviceToHost);
    cudaMemcpy(w4.data(), e.w4, sizeof(__half) * w4.size(), cudaMemcpyDeviceToHost);
    cudaError_t r = cudaMemcpy(bias.data(), e.bias, sizeof(float) * bias.size(), cudaMemcpyDeviceToHost);
    if (r != cudaSuccess) { err = cmsg("emulator weights", r); return ST_DATA_MISSING; }
    std::ofstream f(path, std::ios::binary);
    if (!f) { err = "cannot write " + path; return ST_BAD_ARG; }
    const int32_t hdr[9] = {1, EMU_NIN, EMU_KIN, EMU_H, EMU_NOUT, EMU_NPC, e.nb, EMU_MEMBERS, e.ns};
    f.write(EMU_MAGIC, 8);
    f.write(reinterpret_cast<const char *>(hdr), sizeof hdr);
    f.write(reinterpret_cast<const char *>(e.box_lo), sizeof e.box_lo);
    f.write(reinterpret_cast<const char *>(e.box_hi), sizeof e.box_hi);
    f.write(reinterpret_cast<const char *>(e.par), sizeof(float) * (EMU_P_ZT));
    const float thr[2] = {e.spread_max, e.faint};
    f.write(reinterpret_cast<const char *>(thr), sizeof thr);
    f.write(reinterpret_cast<const char *>(bias.data()), sizeof(float) * bias.size());
    f.write(reinterpret_cast<const char *>(w0.data()), sizeof(__half) * w0.size());
    f.write(reinterpret_cast<const char *>(wh.data()), sizeof(__half) * wh.size());
    f.write(reinterpret_cast<const char *>(w4.data()), sizeof(__half) * w4.size());
    f.write(reinterpret_cast<const char *>(e.pca_mean.data()), sizeof(float) * e.ns);
    f.write(reinterpret_cast<const char *>(e.pca_basis.data()), sizeof(float) * (size_t)EMU_NPC * e.ns);
    const int32_t ni = (int32_t)e.info.size();
    f.write(reinterpret_cast<const char *>(&ni), sizeof ni);
    f.write(reinterpret_cast<const char *>(e.info.data()), sizeof(double) * e.info.size());
    if (!f) { err = "write error on " + path; return ST_BAD_ARG; }
    return 0;
}

static int emu_upload_pca(Emulator &e, std::string &err) {
    cudaError_t r;
    if (!e.d_pca_mean && (r = dalloc(&e.d_pca_mean, e.ns)) != cudaSuccess) { err = cmsg("PCA", r); return ST_DATA_MISSING; }
    if (!e.d_pca_basis && (r = dalloc(&e.d_pca_basis, (size_t)EMU_NPC * e.ns)) != cudaSuccess) { err = cmsg("PCA", r); return ST_DATA_MISSING; }
    cudaMemcpy(e.d_pca_mean, e.pca_mean.data(), sizeof(float) * e.ns, cudaMemcpyHostToDevice);
    r = cudaMemcpy(e.d_pca_basis, e.pca_basis.data(), sizeof(float) * (size_t)EMU_NPC * e.ns, cudaMemcpyHostToDevice);
    if (r != cudaSuccess) { err = cmsg("PCA", r); return ST_DATA_MISSING; }
    return 0;
}

int emu_load(Context &c, const std::string &path, std::string &err) {
    std::ifstream f(path, std::ios::binary);
    if (!f) { err = "cannot read " + path; return ST_DATA_MISSING; }
    char magic[8];
    int32_t hdr[9];
    f.read(magic, 8);
    f.read(reinterpret_cast<char *>(hdr), sizeof hdr);
    if (!f || std::memcmp(magic, EMU_MAGIC, 8) != 0 || hdr[0] != 1 || hdr[1] != EMU_NIN || hdr[2] != EMU_KIN ||
        hdr[3] != EMU_H || hdr[4] != EMU_NOUT || hdr[5] != EMU_NPC || hdr[7] != EMU_MEMBERS) {
        err = path + " is not an emulator file of this library";
        return ST_BAD_ARG;
    }
    if (hdr[6] != c.nbands || hdr[8] != c.nspec) {
        err = "the emulator in " + path + " was trained for another band set or wavelength grid";
        return ST_UNSUPPORTED;
    }
    Emulator &e = c.emu;
    e.release();
    e.nb = hdr[6];
    e.ns = hdr[8];
    f.read(reinterpret_cast<char *>(e.box_lo), sizeof e.box_lo);
    f.read(reinterpret_cast<char *>(e.box_hi), sizeof e.box_hi);
    emu_set_box(c, e);
    f.read(reinterpret_cast<char *>(e.par), sizeof(float) * (EMU_P_ZT));
    float thr[2];
    f.read(reinterpret_cast<char *>(thr), sizeof thr);
    e.spread_max = thr[0];
    e.faint = thr[1];
    std::vector<__half> w0((size_t)n_w0()), wh((size_t)n_wh()), w4((size_t)n_w4());
    std::vector<float> bias((size_t)n_b());
    f.read(reinterpret_cast<char *>(bias.data()), sizeof(float) * bias.size());
    f.read(reinterpret_cast<char *>(w0.data()), sizeof(__half) * w0.size());
    f.read(reinterpret_cast<char *>(wh.data()), sizeof(__half) * wh.size());
    f.read(reinterpret_cast<char *>(w4.data()), sizeof(__half) * w4.size());
    e.pca_mean.resize(e.ns);
    e.pca_basis.resize((size_t)EMU_NPC * e.ns);
    f.read(reinterpret_cast<char *>(e.pca_mean.data()), sizeof(float) * e.ns);
    f.read(reinterpret_cast<char *>(e.pca_basis.data()), sizeof(float) * e.pca_basis.size());
    int32_t ni = 0;
    f.read(reinterpret_cast<char *>(&ni), sizeof ni);
    if (!f || ni < 0 || ni > 4096) { err = path + ": truncated"; e.release(); return ST_BAD_ARG; }
    e.info.resize(ni);
    f.read(reinterpret_cast<char *>(e.info.data()), sizeof(double) * ni);
    if (!f) { err = path + ": truncated"; e.release(); return ST_BAD_ARG; }
    if (int rc = emu_alloc(e, false, err)) { e.release(); return rc; }
    cudaMemcpy(e.w0, w0.data(), sizeof(__half) * w0.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(e.wh, wh.data(), sizeof(__half) * wh.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(e.w4, w4.data(), sizeof(__half) * w4.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(e.bias, bias.data(), sizeof(float) * bias.size(), cudaMemcpyHostToDevice);
    if (int rc = emu_upload_par(e, err)) { e.release(); return rc; }
    if (int rc = emu_upload_pca(e, err)) { e.release(); return rc; }
    e.ready = true;
    return 0;
}

// ---------------------------------------------------------------------------------------------- training
int emu_train(Context &c, long long n_train, int n_val, int epochs, int batch, int seed,
              const std::string &path, std::string &err) {
    if (!c.ops.ready) { err = "the emulator is trained on the SSP-operator path: build the operators first"; return ST_NO_OPERATOR; }
    if (c.sfh != 4) { err = "the emulator is trained on the delayed-tau SFH: set sfh = 4"; return ST_UNSUPPORTED; }
    if (c.nbands < 1 || c.nbands > EMU_MAX_BANDS) { err = "the emulator needs 1 .. 48 bands"; return ST_UNSUPPORTED; }
    if (batch < 128 || batch % 128 != 0 || n_train < batch || n_val < 1 || epochs < 0 || n_train > (1LL << 30)) {
        err = "emulator training: batch must be a multiple of 128, n_train >= batch, n_val >= 1";
        return ST_BAD_ARG;
    }
    const int ns = c.nspec, nb = c.nbands;
    Emulator &e = c.emu;
    e.release();
    e.nb = nb;
    e.ns = ns;
    emu_set_box(c, e);
    cudaStream_t st = c.stream;
    const long long N = n_train + n_val;
    // spectra of the PCA: the first P training models, P a multiple of the chunk of CSP models per batch
    const long long P0 = std::min<long long>(n_train, 131072);
    const int chunk = (int)std::min<long long>(65536, P0);
    const long long P = (P0 / chunk) * chunk;
    float *xraw = nullptr, *Y = nullptr, *rw = nullptr, *Lp = nullptr, *Lc = nullptr;
    cudaError_t r = cudaSuccess;
    auto ok = [&](cudaError_t x) { if (x != cudaSuccess && r == cudaSuccess) r = x; };
    ok(dalloc(&xraw, (size_t)N * EMU_NIN));
    ok(dalloc(&Y, (size_t)N * EMU_NOUT));
    ok(dalloc(&rw, (size_t)N));
    ok(dalloc(&Lp, (size_t)P * ns));
    ok(dalloc(&Lc, (size_t)chunk * ns));
    EmuTrainBufs tb;
    int rc = 0;
    std::vector<double> mags_val((size_t)n_val * nb);
    std::vector<double> explained, val;
    double s1h[EMU_NOUT], s2h[EMU_NOUT], cnth = 0.0;
    double *s1 = nullptr, *s2 = nullptr, *cnt = nullptr;
    float *mu = nullptr, *sig = nullptr;
    std::vector<float> muh(EMU_NOUT, 0.f), sigh(EMU_NOUT, 1.f), lw(EMU_NOUT, 0.f);
    double t_gen = 0.0, t_train = 0.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    if (r != cudaSuccess) { err = cmsg("emulator training set", r); rc = ST_DATA_MISSING; goto cleanup; }
    cudaMemsetAsync(Y, 0, sizeof(float) * N * EMU_NOUT, st);
    {
        // ---- the training set from the CSP
        cudaEventRecord(e0, st);
        Rng rng((uint64_t)seed);
        std::vector<double> vals((size_t)EMU_NIN * chunk), mags((size_t)nb * chunk), dist(chunk);
        std::vector<float> xh((size_t)chunk * EMU_NIN), yh((size_t)chunk * EMU_NOUT), rwh(chunk);
        bool pca_done = false;
        for (long long row0 = 0; row0 < N; row0 += chunk) {
            const int nc = (int)std::min<long long>(chunk, N - row0);
            for (int m = 0; m < nc; ++m)
                for (int i = 0; i < EMU_NIN; ++i) {
                    double u;
                    if (i == 0)   // tau log-uniform
                        u = std::pow(10.0, std::log10(e.box_lo[i]) + (std::log10(e.box_hi[i]) - std::log10(e.box_lo[i])) * rng.uniform());
                    else
                        u = e.box_lo[i] + (e.box_hi[i] - e.box_lo[i]) * rng.uniform();
                    vals[(size_t)i * chunk + m] = u;
                    xh[(size_t)m * EMU_NIN + i] = (float)u;
                }
            const double *vp[EMU_NIN];
            for (int i = 0; i < EMU_NIN; ++i) vp[i] = vals.data() + (size_t)i * chunk;
            if ((rc = csp_batch_mags(c, nc, EMU_NIN, EMU_NAMES, vp, mags.data(), err))) {
                err = "emulator training set: " + err;
                goto cleanup;
            }
            cudaMemcpy(dist.data(), c.d_dist.p, sizeof(double) * nc, cudaMemcpyDeviceToHost);
            for (int m = 0; m < nc; ++m) {
                // bands fainter than the brightest by more than EMU_CLIP mag (or not finite: no flux) are clipped
                // there: they are outside the accuracy gate and the spread, and keep the targets finite
                double mmin = INFINITY;
                for (int b = 0; b < nb; ++b) {
                    const double v = mags[(size_t)b + (size_t)nb * m];
                    if (std::isfinite(v)) mmin = std::min(mmin, v);
                }
                const bool fin = std::isfinite(mmin) && std::isfinite(dist[m]);
                for (int b = 0; b < nb; ++b) {
                    double v = mags[(size_t)b + (size_t)nb * m];
                    if (!std::isfinite(v) || v > mmin + EMU_CLIP) v = mmin + EMU_CLIP;
                    yh[(size_t)m * EMU_NOUT + EMU_NPC + b] = fin ? (float)(v - dist[m]) : 0.f;
                }
                rwh[m] = fin ? 1.f : 0.f;
                if (row0 + m >= n_train)
                    for (int b = 0; b < nb; ++b) mags_val[(size_t)b + (size_t)nb * (row0 + m - n_train)] = mags[(size_t)b + (size_t)nb * m];
            }
            cudaMemcpyAsync(xraw + row0 * EMU_NIN, xh.data(), sizeof(float) * nc * EMU_NIN, cudaMemcpyHostToDevice, st);
            cudaMemcpy2DAsync(Y + row0 * EMU_NOUT + EMU_NPC, sizeof(float) * EMU_NOUT, yh.data() + EMU_NPC,
                              sizeof(float) * EMU_NOUT, sizeof(float) * nb, nc, cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(rw + row0, rwh.data(), sizeof(float) * nc, cudaMemcpyHostToDevice, st);
            float *L = row0 < P ? Lp + row0 * ns : Lc;
            emu_logspec_kernel<<<nc, 256, 0, st>>>(ns, c.d_spec.p, L, rw + row0);
            if ((r = cudaGetLastError()) != cudaSuccess) { err = cmsg("log spectra", r); rc = ST_DATA_MISSING; goto cleanup; }
            if (row0 + nc >= P && !pca_done) {
                if ((rc = emu_pca(c, e, Lp, rw, P, explained, err))) goto cleanup;
                if ((rc = emu_upload_pca(e, err))) goto cleanup;
                if ((rc = emu_project(c, Lp, P, Y, err))) goto cleanup;
                pca_done = true;
                if (row0 < P) continue;      // this chunk was part of the PCA set
            }
            if (pca_done && row0 >= P) {
                emu_center_kernel<<<blocks((long long)nc * ns), 256, 0, st>>>(nc, ns, Lc, e.d_pca_mean, rw + row0);
                if ((rc = emu_project(c, Lc, nc, Y + row0 * EMU_NOUT, err))) goto cleanup;
            }
            if ((r = cudaStreamSynchronize(st)) != cudaSuccess) { err = cmsg("training set", r); rc = ST_DATA_MISSING; goto cleanup; }
        }
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        t_gen = ms * 1e-3;
    }
    {
        // ---- standardisation of the targets (training rows): PCA columns on the first coefficient's scale
        ok(dalloc(&s1, EMU_NOUT)); ok(dalloc(&s2, EMU_NOUT)); ok(dalloc(&cnt, 1)); ok(dalloc(&mu, EMU_NOUT)); ok(dalloc(&sig, EMU_NOUT));
        if (r != cudaSuccess) { err = cmsg("statistics", r); rc = ST_DATA_MISSING; goto cleanup; }
        cudaMemsetAsync(s1, 0, sizeof(double) * EMU_NOUT, st);
        cudaMemsetAsync(s2, 0, sizeof(double) * EMU_NOUT, st);
        cudaMemsetAsync(cnt, 0, sizeof(double), st);
        emu_colstats_kernel<<<1024, EMU_NOUT, 0, st>>>(n_train, Y, rw, s1, s2, cnt);
        cudaMemcpyAsync(s1h, s1, sizeof s1h, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(s2h, s2, sizeof s2h, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(&cnth, cnt, sizeof(double), cudaMemcpyDeviceToHost, st);
        if ((r = cudaStreamSynchronize(st)) != cudaSuccess) { err = cmsg("statistics", r); rc = ST_DATA_MISSING; goto cleanup; }
        const double nrow = std::max(cnth, 1.0);
        std::fprintf(stderr, "emulator training set: %lld models (%.0f used, %.0f excluded: no finite magnitude or spectrum), %.1f s\n",
                     n_train, cnth, (double)n_train - cnth, t_gen);
        double pc_sig = 1.0;
        for (int k = 0; k < EMU_NOUT; ++k) {
            const double m = s1h[k] / nrow, v = std::max(s2h[k] / nrow - m * m, 0.0);
            if (k < EMU_NPC) {
                muh[k] = (float)m;
                if (k == 0) pc_sig = std::sqrt(v) > 0 ? std::sqrt(v) : 1.0;
            } else if (k < EMU_NPC + nb) {
                muh[k] = (float)m;
                sigh[k] = (float)(std::sqrt(v) > 1e-6 ? std::sqrt(v) : 1.0);
            }
        }
        for (int k = 0; k < EMU_NPC; ++k) sigh[k] = (float)pc_sig;
        for (int k = 0; k < EMU_NOUT; ++k) {
            e.par[EMU_P_OMU + k] = muh[k];
            e.par[EMU_P_OSIG + k] = sigh[k];
            lw[k] = k < EMU_NPC ? EMU_PCA_WEIGHT : (k < EMU_NPC + nb ? 1.f : 0.f);
        }
        cudaMemcpyAsync(mu, muh.data(), sizeof(float) * EMU_NOUT, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(sig, sigh.data(), sizeof(float) * EMU_NOUT, cudaMemcpyHostToDevice, st);
        emu_standardise_y_kernel<<<blocks(n_train * EMU_NOUT), 256, 0, st>>>(n_train, Y, mu, sig);
    }
    if ((rc = emu_alloc(e, true, err))) goto cleanup;
    if ((rc = emu_upload_par(e, err))) goto cleanup;
    if ((rc = emu_init_params(c, e, (uint64_t)seed, err))) goto cleanup;
    if ((r = emu_cast_all(e, st)) != cudaSuccess) { err = cmsg("emulator weights", r); rc = ST_DATA_MISSING; goto cleanup; }
    e.ready = true;
    if ((rc = emu_bufs(e, tb, batch, err))) goto cleanup;
    cudaMemcpyAsync(tb.lossw, lw.data(), sizeof(float) * EMU_NOUT, cudaMemcpyHostToDevice, st);
    {
        // ---- training
        const long long steps = n_train / batch, total = steps * epochs;
        const float lr0 = 2e-3f, lr1 = 2e-6f;
        const long long warm = std::min<long long>(500, total / 10 + 1);
        int half = 1;
        while ((1LL << (2 * half)) < n_train) ++half;
        float lsum_w = 0.f;
        for (float v : lw) lsum_w += v;
        const float scale = 2.f / ((float)batch * lsum_w);
        std::vector<float> lossh(8);
        long long t = 0;
        cudaEventRecord(e0, st);
        for (int ep = 0; ep < epochs; ++ep) {
            EmuGatherArgs ga;
            ga.B = batch; ga.n_train = (int)n_train; ga.half = half; ga.given = 0; ga.xraw = xraw; ga.par = e.d_par;
            ga.xstd = nullptr; ga.X = tb.X; ga.Xt = tb.Xt; ga.idx = tb.idx;
            for (int g = 0; g < EMU_MEMBERS; ++g) ga.key[g] = (uint32_t)(0x9e3779b1u * (uint32_t)(ep * EMU_MEMBERS + g + 1) ^ (uint32_t)seed);
            double ep_loss = 0.0;
            for (long long s = 0; s < steps; ++s, ++t) {
                ga.offset = s * batch;
                emu_gather_kernel<<<blocks((long long)EMU_MEMBERS * batch), 256, 0, st>>>(ga);
                const double frac = (double)t / (double)std::max<long long>(total, 1);
                float lr = (float)(lr1 + 0.5 * (lr0 - lr1) * (1.0 + std::cos(M_PI * frac)));
                if (t < warm) lr *= (float)(t + 1) / (float)warm;
                EmuStepCfg sc;
                sc.lr = lr;
                if ((rc = emu_step(c, e, tb, Y, rw, scale, sc, err))) goto cleanup;
                if (s == steps - 1) {
                    cudaMemcpyAsync(lossh.data(), tb.loss, sizeof(float) * 8, cudaMemcpyDeviceToHost, st);
                    if ((r = cudaStreamSynchronize(st)) != cudaSuccess) { err = cmsg("training", r); rc = ST_DATA_MISSING; goto cleanup; }
                    for (int g = 0; g < EMU_MEMBERS; ++g) ep_loss += lossh[g] / ((double)batch * lsum_w) / EMU_MEMBERS;
                }
            }
            if ((rc = check_status(c, err))) goto cleanup;
            if (ep == epochs - 1 || (ep + 1) % 10 == 0) {
                if ((rc = emu_validate(c, xraw + n_train * EMU_NIN, mags_val, n_val, val, err))) goto cleanup;
                std::fprintf(stderr, "emulator epoch %d: loss %.3e  val rms %.4f mag  max %.4f  p99 %.4f  flagged %.4f  max(unflagged) %.4f\n",
                             ep + 1, ep_loss, val[0], val[1], val[2], val[3], val[4]);
            }
        }
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        t_train = ms * 1e-3;
        if (epochs == 0 && (rc = emu_validate(c, xraw + n_train * EMU_NIN, mags_val, n_val, val, err))) goto cleanup;
    }
    e.info = {(double)n_train, (double)n_val, (double)epochs, (double)batch, (double)seed, t_gen, t_train};
    for (double v : val) e.info.push_back(v);
    e.info.push_back(explained.empty() ? 0.0 : explained.back());
    if (!path.empty() && (rc = emu_save(c, path, err))) goto cleanup;
cleanup:
    cudaStreamSynchronize(st);
    tb.release();
    for (void *p : {(void *)xraw, (void *)Y, (void *)rw, (void *)Lp, (void *)Lc, (void *)s1, (void *)s2, (void *)cnt,
                    (void *)mu, (void *)sig})
        if (p) cudaFree(p);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) e.release();
    return rc;
}

// ---------------------------------------------------------------------------------------------- tests' entry points
// A fresh ensemble with random weights (no training set): for the gradient check and the inference tests.
int emu_init(Context &c, int seed, std::string &err) {
    if (c.nbands < 1 || c.nbands > EMU_MAX_BANDS) { err = "the emulator needs 1 .. 48 bands"; return ST_UNSUPPORTED; }
    Emulator &e = c.emu;
    e.release();
    e.nb = c.nbands;
    e.ns = c.nspec;
    emu_set_box(c, e);
    for (int k = 0; k < EMU_NOUT; ++k) { e.par[EMU_P_OMU + k] = 0.f; e.par[EMU_P_OSIG + k] = 1.f; }
    if (int rc = emu_alloc(e, true, err)) { e.release(); return rc; }
    if (int rc = emu_upload_par(e, err)) { e.release(); return rc; }
    if (int rc = emu_init_params(c, e, (uint64_t)seed, err)) { e.release(); return rc; }
    cudaError_t r = emu_cast_all(e, c.stream);
    if (r == cudaSuccess) r = cudaStreamSynchronize(c.stream);
    if (r != cudaSuccess) { err = cmsg("emulator weights", r); e.release(); return ST_DATA_MISSING; }
    e.pca_mean.assign(e.ns, 0.f);
    e.pca_basis.assign((size_t)EMU_NPC * e.ns, 0.f);
    if (int rc = emu_upload_pca(e, err)) { e.release(); return rc; }
    e.ready = true;
    return 0;
}

// The FP32 masters and biases [w0 | wh | w4 | bias] (emu_param_count floats): get (set = 0) or set (set = 1).
int emu_params(Context &c, int set, float *host, std::string &err) {
    Emulator &e = c.emu;
    if (!e.ready || !e.trainable) { err = "no trainable emulator on the context (opensps_gb300_emulator_init)"; return ST_NO_OPERATOR; }
    const long long nw = n_w0() + n_wh() + n_w4();
    cudaError_t r;
    if (set) {
        if ((r = cudaMemcpy(e.master, host, sizeof(float) * nw, cudaMemcpyHostToDevice)) == cudaSuccess &&
            (r = cudaMemcpy(e.bias, host + nw, sizeof(float) * n_b(), cudaMemcpyHostToDevice)) == cudaSuccess &&
            (r = emu_cast_all(e, c.stream)) == cudaSuccess)
            r = cudaStreamSynchronize(c.stream);
    } else {
        if ((r = cudaMemcpy(host, e.master, sizeof(float) * nw, cudaMemcpyDeviceToHost)) == cudaSuccess)
            r = cudaMemcpy(host + nw, e.bias, sizeof(float) * n_b(), cudaMemcpyDeviceToHost);
    }
    if (r != cudaSuccess) { err = cmsg("emulator parameters", r); return ST_DATA_MISSING; }
    return 0;
}

// The training kernels' loss and gradients of every member on one minibatch (the same n rows for each member):
// x_std (n x 12 standardised features), y_std (n x 128 standardised targets), lossw (128). loss: 5 floats (the
// members' weighted mean squared errors), grads: emu_param_count floats.
int emu_grads(Context &c, int n, const float *x_std, const float *y_std, const float *lossw, float *loss, float *grads,
              std::string &err) {
    Emulator &e = c.emu;
    if (!e.ready || !e.trainable) { err = "no trainable emulator on the context (opensps_gb300_emulator_init)"; return ST_NO_OPERATOR; }
    if (n < 128 || n % 128 != 0) { err = "emulator gradients: n must be a positive multiple of 128"; return ST_BAD_ARG; }
    cudaStream_t st = c.stream;
    EmuTrainBufs tb;
    float *xs = nullptr, *y = nullptr, *rw = nullptr, *g = nullptr;
    int rc = 0;
    cudaError_t r = cudaSuccess;
    auto ok = [&](cudaError_t x) { if (x != cudaSuccess && r == cudaSuccess) r = x; };
    ok(dalloc(&xs, (size_t)n * EMU_NFEAT)); ok(dalloc(&y, (size_t)n * EMU_NOUT)); ok(dalloc(&rw, (size_t)n));
    ok(dalloc(&g, (size_t)emu_param_count()));
    std::vector<float> ones(n, 1.f), lh(8);
    float wsum = 0.f;
    EmuGatherArgs ga{};
    EmuStepCfg sc;
    if (r != cudaSuccess) { err = cmsg("emulator gradients", r); rc = ST_DATA_MISSING; goto out; }
    if ((rc = emu_bufs(e, tb, n, err))) goto out;
    cudaMemcpy(xs, x_std, sizeof(float) * n * EMU_NFEAT, cudaMemcpyHostToDevice);
    cudaMemcpy(y, y_std, sizeof(float) * n * EMU_NOUT, cudaMemcpyHostToDevice);
    cudaMemcpy(rw, ones.data(), sizeof(float) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(tb.lossw, lossw, sizeof(float) * EMU_NOUT, cudaMemcpyHostToDevice);
    for (int k = 0; k < EMU_NOUT; ++k) wsum += lossw[k];
    ga.B = n; ga.n_train = n; ga.given = 1; ga.xstd = xs; ga.par = e.d_par; ga.X = tb.X; ga.Xt = tb.Xt; ga.idx = tb.idx;
    emu_gather_kernel<<<blocks((long long)EMU_MEMBERS * n), 256, 0, st>>>(ga);
    cudaMemsetAsync(g, 0, sizeof(float) * emu_param_count(), st);
    sc.apply = false;
    sc.grad_out = g;
    if ((rc = emu_step(c, e, tb, y, rw, 2.f / ((float)n * wsum), sc, err))) goto out;
    --e.adam_t;
    if ((rc = check_status(c, err))) goto out;
    cudaMemcpy(grads, g, sizeof(float) * emu_param_count(), cudaMemcpyDeviceToHost);
    cudaMemcpy(lh.data(), tb.loss, sizeof(float) * 8, cudaMemcpyDeviceToHost);
    for (int k = 0; k < EMU_MEMBERS; ++k) loss[k] = lh[k] / ((float)n * wsum);
out:
    cudaStreamSynchronize(st);
    tb.release();
    for (void *p : {(void *)xs, (void *)y, (void *)rw, (void *)g})
        if (p) cudaFree(p);
    return rc;
}

// ---------------------------------------------------------------------------------------------- prediction
// Host inputs (EMU_NIN x n, column-major doubles, the order of EMU_NAMES) -> magnitudes (nb x n), and optionally
// the PCA coefficients (64 x n), the spread (n) and the source of each model (0 emulator, 1 outside the box,
// 2 spread, 3 not finite: the last three from the plain CSP when fallback != 0).
int emu_predict(Context &c, int n, const double *inputs, int fallback, double *mags, double *pca,
                double *spread, int *source, int *n_fallback, std::string &err) {
    Emulator &e = c.emu;
    if (!e.ready) { err = "no emulator on the context (opensps_gb300_emulator_load / _train)"; return ST_NO_OPERATOR; }
    if (c.dust_type != 0) { err = "emulator: trained with the power-law dust curve (dust_type 0)"; return ST_UNSUPPORTED; }
    if (n <= 0) { if (n_fallback) *n_fallback = 0; return 0; }
    if (!inputs) { err = "emulator: inputs are NULL"; return ST_BAD_ARG; }
    if (int rc = emu_scratch(e, n, err)) return rc;
    const int nb = e.nb;
    std::vector<float> xh((size_t)n * EMU_NIN);
    for (int m = 0; m < n; ++m)
        for (int i = 0; i < EMU_NIN; ++i) xh[(size_t)m * EMU_NIN + i] = (float)inputs[(size_t)i + (size_t)EMU_NIN * m];
    cudaMemcpyAsync(e.d_x, xh.data(), sizeof(float) * xh.size(), cudaMemcpyHostToDevice, c.stream);
    if (int rc = emu_infer_device(c, n, e.d_x, e.d_mags, pca ? e.d_coef : nullptr, e.d_spread, e.d_flag, e.d_nflag,
                                  e.d_flagged, err))
        return rc;
    std::vector<float> mg((size_t)n * nb), cf(pca ? (size_t)n * EMU_NPC : 0), sp(spread ? n : 0);
    std::vector<int> fl(n);
    int nf = 0;
    cudaMemcpyAsync(mg.data(), e.d_mags, sizeof(float) * mg.size(), cudaMemcpyDeviceToHost, c.stream);
    cudaMemcpyAsync(fl.data(), e.d_flag, sizeof(int) * n, cudaMemcpyDeviceToHost, c.stream);
    cudaMemcpyAsync(&nf, e.d_nflag, sizeof(int), cudaMemcpyDeviceToHost, c.stream);
    if (pca) cudaMemcpyAsync(cf.data(), e.d_coef, sizeof(float) * cf.size(), cudaMemcpyDeviceToHost, c.stream);
    if (spread) cudaMemcpyAsync(sp.data(), e.d_spread, sizeof(float) * n, cudaMemcpyDeviceToHost, c.stream);
    if (int rc = check_status(c, err)) return rc;
    if (mags)
        for (int m = 0; m < n; ++m)
            for (int b = 0; b < nb; ++b) mags[(size_t)b + (size_t)nb * m] = mg[(size_t)m * nb + b];
    if (pca)
        for (int m = 0; m < n; ++m)
            for (int k = 0; k < EMU_NPC; ++k) pca[(size_t)k + (size_t)EMU_NPC * m] = cf[(size_t)m * EMU_NPC + k];
    if (spread)
        for (int m = 0; m < n; ++m) spread[m] = sp[m];
    if (source)
        for (int m = 0; m < n; ++m) source[m] = fl[m];
    if (n_fallback) *n_fallback = nf;
    if (!fallback || nf == 0) return 0;
    // ---- the flagged models through the plain CSP (in model order)
    std::vector<int> idx;
    idx.reserve(nf);
    for (int m = 0; m < n; ++m)
        if (fl[m]) idx.push_back(m);
    const int nfb = (int)idx.size();
    std::vector<double> vals((size_t)EMU_NIN * nfb), mf((size_t)nb * nfb);
    for (int j = 0; j < nfb; ++j)
        for (int i = 0; i < EMU_NIN; ++i) vals[(size_t)i * nfb + j] = inputs[(size_t)i + (size_t)EMU_NIN * idx[j]];
    const double *vp[EMU_NIN];
    for (int i = 0; i < EMU_NIN; ++i) vp[i] = vals.data() + (size_t)i * nfb;
    if (int rc = csp_batch_mags(c, nfb, EMU_NIN, EMU_NAMES, vp, mf.data(), err)) {
        err = "emulator fallback: " + err;
        return rc;
    }
    if (mags)
        for (int j = 0; j < nfb; ++j)
            for (int b = 0; b < nb; ++b) mags[(size_t)b + (size_t)nb * idx[j]] = mf[(size_t)b + (size_t)nb * j];
    if (pca && nfb > 0) {
        // the CSP spectra's own coefficients
        float *L = nullptr, *rw = nullptr, *cy = nullptr;
        cudaError_t r = cudaSuccess;
        auto ok = [&](cudaError_t x) { if (x != cudaSuccess && r == cudaSuccess) r = x; };
        ok(dalloc(&L, (size_t)nfb * c.nspec)); ok(dalloc(&rw, nfb)); ok(dalloc(&cy, (size_t)nfb * EMU_NOUT));
        int rc = 0;
        if (r != cudaSuccess) { err = cmsg("emulator fallback", r); rc = ST_DATA_MISSING; }
        if (!rc) {
            std::vector<float> ones(nfb, 1.f), cyh((size_t)nfb * EMU_NOUT);
            cudaMemcpy(rw, ones.data(), sizeof(float) * nfb, cudaMemcpyHostToDevice);
            emu_logspec_kernel<<<nfb, 256, 0, c.stream>>>(c.nspec, c.d_spec.p, L, rw);
            emu_center_kernel<<<blocks((long long)nfb * c.nspec), 256, 0, c.stream>>>(nfb, c.nspec, L, e.d_pca_mean, rw);
            if (!c.cublas) {
                cublasHandle_t h;
                if (cublasCreate(&h) != CUBLAS_STATUS_SUCCESS) { err = "cuBLAS could not be initialised"; rc = ST_DATA_MISSING; }
                else c.cublas = h;
            }
            if (!rc) rc = emu_project(c, L, nfb, cy, err);
            if (!rc) {
                cudaMemcpyAsync(cyh.data(), cy, sizeof(float) * cyh.size(), cudaMemcpyDeviceToHost, c.stream);
                cudaStreamSynchronize(c.stream);
                for (int j = 0; j < nfb; ++j)
                    for (int k = 0; k < EMU_NPC; ++k) pca[(size_t)k + (size_t)EMU_NPC * idx[j]] = cyh[(size_t)j * EMU_NOUT + k];
            }
        }
        cudaFree(L); cudaFree(rw); cudaFree(cy);
        if (rc) return rc;
    }
    return 0;
}

}  // namespace sps
