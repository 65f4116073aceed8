// The reverse pass of the batched CSP (compute_csp_batch_grad): analytic adjoints of the magnitudes, the observed
// frame, the velocity smoothing, the IGM and the attenuation, recomputing the forward's attenuated spectrum and its
// smoothing from the young and old age sums instead of storing them (OpenSPS batch_backward,
// src/physics/opensps_csp_batch.f90:4743-5135: the cotangent scale cscale :4870-4897, backward_observed_frame :6958,
// backward_attenuation :6368; smooth_columns_adjoint and smooth_sigma_adjoint
// src/spectra/opensps_batch_photometry.f90:607-700; distance_term_dz :798-814), then the weights' cotangent as a
// tensor-core GEMM against the transposed basis (backward_age_sums_w :5288-5322) with the mass and L_bol terms
// (:1140-1150, :4958-4963).
//
// adjoint_kernel: one CTA per model. Shared memory holds the model's recomputed pre-smoothing spectrum (TOT, later
// the cotangent of TOT), its smoothed spectrum (S), the cotangent of S (SB) and the observed-frame cotangent (VB).
// The cotangents of the young and old sums leave as the bf16 hi / lo A operands of the weight GEMM; the parameter
// gradients are block reductions. Every cotangent is divided by a power of two at least the model's largest one
// (cscale) so that the FP32 arithmetic stays in range; the results are multiplied back in FP64.
#include <climits>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>
#include "context.h"
#include "sm103_ptx.cuh"

namespace sps {

constexpr int ADJ_THREADS = 384;
constexpr int ADJ_WARPS = ADJ_THREADS / 32;
constexpr int ADJ_MAX_BANDS = 256;
constexpr double ADJ_C_KMS = 2.99792458e5;           // C_LIGHT 1e-13: km/s
constexpr double DMAG_DF = -1.0857362047581294;       // -2.5 / ln 10
constexpr int NBGRAD = 44;

// gradient rows of params_bar (opensps.h)
enum { R_DUST1 = 1, R_DUST2 = 2, R_DUST3 = 3, R_DUST_INDEX = 4, R_DUST1_INDEX = 5, R_FRAC_OBRUN = 6,
       R_FRAC_NODUST = 7, R_MWR = 8, R_UVB = 9, R_ZRED = 22, R_SIGMA = 23, R_IGM_FACTOR = 32 };
enum { G_DUST2 = 0, G_DUST_INDEX, G_FNODUST, G_DUST1, G_DUST1_INDEX, G_FOBRUN, G_DUST3, G_ZRED, G_IGMF, G_SIGMA,
       G_OBS, G_MWR, G_UVB, G_WQ, G_WU, G_GAM, NG };
// rows of the dust emission and the AGN torus (opensps.h)
enum { R_FAGN = 0, R_DUSTE_QPAH = 10, R_DUSTE_UMIN = 11, R_DUSTE_GAMMA = 12, R_AGN_TAU = 31 };

// The per-model block of the reverse pass (floats; KOBS and DDIST are doubles at 8-byte offsets), written by
// adjoint_prep_kernel: the redshift factors b_k = (1 + z)^p_k and d b_k / dz, the smoothing taps' d / dsigma, the
// observed frame's d t / dz factor and the distance term's d / dz.
enum { AP_B = 0, AP_DB = 6, AP_DTAP = 12, AP_KOBS = 22, AP_DDIST = 24, AP_FLOATS = 32 };

__device__ __forceinline__ float adj_ex2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// e^y - 1 as the forward's epilogue forms it: the Taylor series to y^6 below |y| = 1/8, else e^y - 1
__device__ __forceinline__ float adj_expm1(float y) {
    if (fabsf(y) < 0.125f) {
        float r = 1.f + y * (1.f / 6.f);
        r = 1.f + y * (1.f / 5.f) * r;
        r = 1.f + y * (1.f / 4.f) * r;
        r = 1.f + y * (1.f / 3.f) * r;
        r = 1.f + y * (1.f / 2.f) * r;
        return y * r;
    }
    return adj_ex2(y * 1.4426950408889634f) - 1.f;
}

// The dust emission's template at pixel i for a model's cell (dl07_shape, src/physics/opensps_csp_batch.f90:4103-4122:
// bilinear in the q_PAH and U_min weights, the two components mixed by gamma, floored at the smallest normal), and
// its derivatives in wq, wu and gamma (zero where the floor holds). tab: (2 numin x nqpah) columns of nspec, column
// (2 u + c) nqpah + q.
struct Dl07Val {
    float shape, d_wq, d_wu, d_gam;
};
__device__ __forceinline__ Dl07Val dl07_eval(const float *tab, int ns, int nq, int i, const DustEmModel &d) {
    const int k0 = 2 * d.iu, k1 = 2 * (d.iu + 1);
    const float *a = tab + (size_t)i;
    auto T = [&](int k, int q) { return __ldg(a + ((size_t)k * nq + q) * ns); };
    const float a0 = T(k0, d.iq), a1 = T(k0, d.iq + 1), a2 = T(k1, d.iq + 1), a3 = T(k1, d.iq);
    const float b0 = T(k0 + 1, d.iq), b1 = T(k0 + 1, d.iq + 1), b2 = T(k1 + 1, d.iq + 1), b3 = T(k1 + 1, d.iq);
    const float wq = d.wq, wu = d.wu;
    const float w00 = (1.f - wq) * (1.f - wu), w10 = wq * (1.f - wu), w11 = wq * wu, w01 = (1.f - wq) * wu;
    const float lo = w00 * a0 + w10 * a1 + w11 * a2 + w01 * a3, hi = w00 * b0 + w10 * b1 + w11 * b2 + w01 * b3;
    const float v = (1.f - d.gam) * lo + d.gam * hi;
    Dl07Val r;
    r.shape = fmaxf(v, FLT_MIN);
    if (v < FLT_MIN) {
        r.d_wq = r.d_wu = r.d_gam = 0.f;
        return r;
    }
    const float lq = (1.f - wu) * (a1 - a0) + wu * (a2 - a3), hq = (1.f - wu) * (b1 - b0) + wu * (b2 - b3);
    const float lu = (1.f - wq) * (a3 - a0) + wq * (a2 - a1), hu = (1.f - wq) * (b3 - b0) + wq * (b2 - b1);
    r.d_wq = (1.f - d.gam) * lq + d.gam * hq;
    r.d_wu = (1.f - d.gam) * lu + d.gam * hu;
    r.d_gam = hi - lo;
    return r;
}

// x 2^-k as FP32 on the integer pipes (GB300 has little FP64): round to nearest even on the dropped mantissa bits; a
// result below FP32's smallest normal is a signed 0, above its largest an infinity; infinities and NaNs carry over.
__device__ __forceinline__ float scaled_to_f32(double x, int k) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const uint32_t hi32 = (uint32_t)(b >> 32), lo32 = (uint32_t)b;
    const uint32_t sign = hi32 & 0x80000000u;
    const int de = (int)((hi32 >> 20) & 0x7ff);
    if (de == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (((hi32 & 0xfffffu) | lo32) ? 0x400000u : 0u));
    const int fe = de - 896 - k;                                        // FP32 biased exponent of x 2^-k
    if (de == 0 || fe < 1) return __uint_as_float(sign);
    if (fe > 254) return __uint_as_float(sign | 0x7f800000u);
    uint32_t m = ((hi32 & 0xfffffu) << 3) | (lo32 >> 29);
    const uint32_t rem = lo32 & 0x1fffffffu;
    m += (rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) ? 1u : 0u;
    return __uint_as_float(sign | (((uint32_t)fe << 23) + m));         // a mantissa carry moves into the exponent
}

// ---------------------------------------------------------------------------------------------- per-model scalars
// One thread per model, FP64 (igm_tau_z_terms_dz src/physics/opensps_cosmology.f90:511-522; smooth_sigma_adjoint's
// d C / d sigma = C (x^2 - <x^2>) / (sigma_beta^3 c); backward_observed_frame's d t / dz; distance_term_dz).
__global__ void __launch_bounds__(256) adjoint_prep_kernel(AdjointPrepArgs a) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= a.n_models) return;
    const double *pr = a.par + (size_t)PAR_DEVICE * m;
    const float *mp = a.mpar + (size_t)MODEL_PAR_FLOATS * m;
    float blk[AP_FLOATS];
#pragma unroll
    for (int i = 0; i < AP_FLOATS; ++i) blk[i] = 0.f;
    const double z = pr[PF_ZRED];
    if (mp[MP_IGM_ON] != 0.f) {
        const double pk[6] = {3.46, 1.68, 3.0 + 0.46, 1.5 + 0.18, 3.0 - 1.32, 1.68};
        const double l1z = log1p(z);
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const double bk = exp(pk[k] * l1z);
            blk[AP_B + k] = (float)bk;
            blk[AP_DB + k] = (float)(pk[k] * bk / (1.0 + z));
        }
    }
    const int R = __float_as_int(mp[MP_SMOOTH_R]);
    const double sig = pr[PF_SIGMA_SMOOTH];
    if (R >= 0 && sig > 0.0) {
        const double sb = sig / ADJ_C_KMS;
        const double inv = 1.0 / (sb * sb * sb * ADJ_C_KMS);
        double av[9], mean = 0.0;
#pragma unroll
        for (int d = -4; d <= 4; ++d) {
            const int j = min(max(a.sm_lo + d, 0), a.nspec - 1);
            const double dd = a.lnlam[a.sm_lo] - a.lnlam[j];
            av[d + 4] = dd * dd * inv;
            mean += (double)mp[MP_TAPS + d + 4] * av[d + 4];
        }
#pragma unroll
        for (int d = 0; d < 9; ++d) blk[AP_DTAP + d] = (float)((double)mp[MP_TAPS + d] * (av[d] - mean));
    }
    double kobs = 0.0, ddist = 0.0;
    const float4 zi = a.zinfo[m];
    if (zi.w == 1.f) {
        // t = (lambda_j / (1 + z) - lambda_il) / (lambda_(il+1) - lambda_il): dt/dz = -lambda_j / ((1 + z)^2 dlambda_il),
        // lambda_j / dlambda_il = e^((j - il) dlnl) / (e^dlnl - 1), j - il = nsh on the grid's interior
        const int nsh = __float_as_int(zi.x) + ((zi.y > 0.f) ? 1 : 0);
        const double opz = 1.0 + z;
        kobs = -exp((double)nsh * a.dlnl) / (opz * opz * a.em1);
        const int idx = max(0, min(find_interval0(a.zt, 500, z), 498));
        const double slope = (a.dl[idx + 1] - a.dl[idx]) / (a.zt[idx + 1] - a.zt[idx]);
        const double dm = a.dl[idx] + slope * (z - a.zt[idx]);
        if (dm == dm && dm > SAFE_FLOOR) ddist = 5.0 / log(10.0) * slope / dm - 2.5 / (log(10.0) * opz);
    }
    float *o = a.apar + (size_t)AP_FLOATS * m;
#pragma unroll
    for (int i = 0; i < AP_FLOATS; i += 4)
        reinterpret_cast<float4 *>(o)[i / 4] = make_float4(blk[i], blk[i + 1], blk[i + 2], blk[i + 3]);
    reinterpret_cast<double *>(o)[AP_KOBS / 2] = kobs;
    reinterpret_cast<double *>(o)[AP_DDIST / 2] = ddist;
}

// ---------------------------------------------------------------------------------------------- the adjoint
// The forward's per-pixel factors of a model (as the contraction's epilogue forms them).
struct PixFwd {
    float curve, ltab, td, c1, tb, to, D, ssfac_y;
    float dci, dcm, dcu;   // the diffuse curve's derivatives in dust_index, mwr and uvb
    float tau, dtau;   // IGM optical depth at unit igm_factor and its derivative in z (0 without IGM)
    bool igm;
};

struct ModelConst {
    float kd2, one_m_fnd, fnd, dust_index, kd1, dust1_index, one_m_fo, fo, kd3;
    float cs1, cs2, cs3;   // the tabulated curve's scalars (dust_index: its power)
    float b[6], db[6];
    int jmax;
    bool igm_model;
};

__device__ __forceinline__ PixFwd pix_forward(const AdjointArgs &a, const ModelConst &mc, int p) {
    PixFwd f;
    const float ltab2 = fmaf((float)p, a.lt_step, a.lt_base);   // ln(lambda / 5500) log2(e) on the log-uniform grid
    f.ltab = ltab2 * 0.6931471805599453f;                        // ln(lambda / 5500)
    if (a.dust_type != 0) {
        // the tabulated curve (T0 + s1 T1 + s2 T2 + s3 T3) (lambda / 5500)^ed and its derivatives: in dust_index
        // (Kriek & Conroy: s1 = ed = dust_index), in mwr and uvb (CCM89: s = (1 / mwr, uvb, uvb / mwr))
        const float4 t = __ldg(reinterpret_cast<const float4 *>(a.pix + (size_t)p * PIX_FLOATS + PIX_T));
        const float pl = mc.dust_index != 0.f ? adj_ex2(mc.dust_index * ltab2) : 1.f;
        f.curve = fmaf(mc.cs1, t.y, fmaf(mc.cs2, t.z, fmaf(mc.cs3, t.w, t.x))) * pl;
        f.dci = a.dust_type == 4 ? fmaf(t.y, pl, f.curve * f.ltab) : 0.f;
        f.dcm = a.dust_type == 1 ? -(t.y + mc.cs2 * t.w) * mc.cs1 * mc.cs1 : 0.f;
        f.dcu = a.dust_type == 1 ? fmaf(mc.cs1, t.w, t.z) : 0.f;
    } else {
        f.curve = adj_ex2(mc.dust_index * ltab2);
        f.dci = f.curve * f.ltab; f.dcm = 0.f; f.dcu = 0.f;
    }
    f.td = adj_ex2(mc.kd2 * f.curve);
    f.c1 = adj_ex2(mc.dust1_index * ltab2);
    f.tb = (mc.kd1 != 0.f) ? adj_ex2(mc.kd1 * f.c1) : 1.f;
    f.to = (mc.kd3 != 0.f) ? adj_ex2(mc.kd3 * f.curve) : 1.f;
    f.D = fmaf(f.td, mc.one_m_fnd, mc.fnd);
    f.ssfac_y = f.tb * mc.one_m_fo + mc.fo;
    f.igm = mc.igm_model && p < a.jtop;
    f.tau = 0.f;
    f.dtau = 0.f;
    if (f.igm) {
        // pixels below the one of the largest depth take its depth (apply_igm_z's cap)
        const int jc = (p < mc.jmax) ? mc.jmax - 1 : p;
        const float4 w0 = __ldg(reinterpret_cast<const float4 *>(a.pix + (size_t)jc * PIX_FLOATS));
        const float4 w1 = __ldg(reinterpret_cast<const float4 *>(a.pix + (size_t)jc * PIX_FLOATS) + 1);
        const float ia[6] = {w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            f.tau = fmaf(ia[k], mc.b[k], f.tau);
            f.dtau = fmaf(ia[k], mc.db[k], f.dtau);
        }
    }
    return f;
}

// A cotangent of the diffuse curve at one pixel into the dust_index, mwr and uvb rows.
__device__ __forceinline__ void curve_rows(const PixFwd &f, float cbar, float *g) {
    g[G_DUST_INDEX] = fmaf(cbar, f.dci, g[G_DUST_INDEX]);
    g[G_MWR] = fmaf(cbar, f.dcm, g[G_MWR]);
    g[G_UVB] = fmaf(cbar, f.dcu, g[G_UVB]);
}

// The reverse pass of one pixel: from dL / dTOT (tb), the forward's sums (y, o), the gradient accumulators and the
// cotangents of y and o.
__device__ __forceinline__ void pixel_adjoint(const AdjointArgs &a, const ModelConst &mc, const PixFwd &f, float y,
                                              float o, float tb, float f_igm, float kf, float d1, float d2, float d3,
                                              float pre_extra, float *g, float &yb, float &ob, float &T) {
    const float ss = y * f.ssfac_y + o * f.to;
    const float pre = ss * f.D;
    float pb = tb;
    T = 1.f;
    if (f.igm) {
        // T = exp(-igm_factor tau): dT/dz = -igm_factor T dtau/dz, dT/d igm_factor = -tau T (the dust emission's
        // escaping light, pre_extra, passes through the IGM with the rest)
        T = adj_ex2(f.tau * kf);
        const float gT = pb * (pre + pre_extra);
        g[G_ZRED] = fmaf(gT, -f_igm * T * f.dtau, g[G_ZRED]);
        g[G_IGMF] = fmaf(gT, -f.tau * T, g[G_IGMF]);
        pb *= T;
    }
    // pre = ss D, D = T_d (1 - fnd) + fnd, ss = y (T_b (1 - fo) + fo) + o T_o; the curve's cotangent through the
    // diffuse and old-star screens into dust_index, mwr and uvb
    g[G_DUST2] = fmaf(pb * ss * mc.one_m_fnd, -f.td * f.curve, g[G_DUST2]);
    curve_rows(f, pb * (ss * mc.one_m_fnd * f.td * -d2 + f.D * o * f.to * -d3), g);
    g[G_FNODUST] = fmaf(pb * ss, 1.f - f.td, g[G_FNODUST]);
    const float ybase = pb * f.D * y;
    g[G_DUST1] = fmaf(ybase * mc.one_m_fo, -f.tb * f.c1, g[G_DUST1]);
    g[G_DUST1_INDEX] = fmaf(ybase * mc.one_m_fo, -f.tb * d1 * f.c1 * f.ltab, g[G_DUST1_INDEX]);
    g[G_FOBRUN] = fmaf(ybase, 1.f - f.tb, g[G_FOBRUN]);
    g[G_DUST3] = fmaf(pb * f.D * o, -f.to * f.curve, g[G_DUST3]);
    yb = pb * f.D * f.ssfac_y;
    ob = pb * f.D * f.to;
}

__device__ __forceinline__ __nv_bfloat162 bf16_hi2(float a, float b) { return __floats2bfloat162_rn(a, b); }
__device__ __forceinline__ __nv_bfloat162 bf16_lo2(float a, float b, __nv_bfloat162 h) {
    return __floats2bfloat162_rn(a - __low2float(h), b - __high2float(h));
}

// floats per staged row: the row plus the unit offsets at either end, in 16-byte units
__host__ __device__ int adj_row_pad(int ns);

__global__ void __launch_bounds__(ADJ_THREADS, 2) adjoint_kernel(AdjointArgs a) {
    extern __shared__ __align__(16) float sh[];
    const int ns = a.nspec;
    const int rowpad = adj_row_pad(ns);
    // YS, OS: the model's young and old sums (bulk copies of the 16-byte units that hold the rows); TOT: the
    // pre-smoothing spectrum, later dL / dTOT; S: the smoothed spectrum, later dL / dS; VB: pixels j0 .. j1
    float *YS = sh, *OS = sh + rowpad, *TOT = sh + 2 * rowpad, *S = TOT + ns, *VB = S + ns;
    __shared__ float fbs[ADJ_MAX_BANDS];
    __shared__ uint64_t rows_bar;
    __shared__ float red[NG][ADJ_WARPS];
    __shared__ unsigned long long wmax[ADJ_WARPS];
    __shared__ double wsum[ADJ_WARPS];
    __shared__ float emsum[3][ADJ_WARPS];   // the dust emission's and the AGN's per-warp sums
    const int m = blockIdx.x, tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const float *mp = a.mpar + (size_t)MODEL_PAR_FLOATS * m;
    const float *ap = a.apar + (size_t)AP_FLOATS * m;
    const double *pr = a.par + (size_t)PAR_DEVICE * m;
    // the rows' 16-byte units: from the unit holding the first pixel through the one holding the last
    const uintptr_t y0 = reinterpret_cast<uintptr_t>(a.young + (size_t)m * ns);
    const uintptr_t o0 = reinterpret_cast<uintptr_t>(a.old + (size_t)m * ns);
    const uintptr_t yb0 = y0 & ~uintptr_t(15), ob0 = o0 & ~uintptr_t(15);
    const uint32_t ybytes = (uint32_t)(((y0 + 4 * (uintptr_t)ns + 15) & ~uintptr_t(15)) - yb0);
    const uint32_t obytes = (uint32_t)(((o0 + 4 * (uintptr_t)ns + 15) & ~uintptr_t(15)) - ob0);
    if (tid == 0) {
        mbar_init(&rows_bar, 1);
        fence_mbar_init();
        mbar_arrive_expect_tx(&rows_bar, ybytes + obytes);
        bulk_load(YS, reinterpret_cast<const void *>(yb0), ybytes, &rows_bar);
        bulk_load(OS, reinterpret_cast<const void *>(ob0), obytes, &rows_bar);
    }
    const float *yv = YS + (y0 - yb0) / 4, *ov = OS + (o0 - ob0) / 4;
    const double *mb = a.mags_bar ? a.mags_bar + (size_t)m * a.nbands : nullptr;
    const double *fbd = a.fband + (size_t)m * a.nbands;
    const double *sbar = a.spec_bar ? a.spec_bar + (size_t)m * ns : nullptr;
    const bool even = (ns & 1) == 0;   // rows start on 8-byte (float2) and 16-byte (double2) boundaries

    // ---- the cotangent scale 2^ks >= the largest band-flux and spectrum cotangent of the model (a power of two, so
    // that scaling is exact); magnitudes of doubles compared as their bit patterns
    unsigned long long amax = 0ull;
    double msum = 0.0;   // the magnitudes' cotangents over the bands computed (the distance term's share of d / dz)
    if (mb)
        for (int b = tid; b < a.nbands; b += ADJ_THREADS) {
            const double f = fbd[b];
            if ((a.do_band == nullptr || a.do_band[b] != 0) && f > 0.0) {
                amax = max(amax, (unsigned long long)__double_as_longlong(mb[b] * DMAG_DF / f) & 0x7fffffffffffffffull);
                msum += mb[b];
            }
        }
    if (sbar) {
        if (even) {
            const double2 *s2 = reinterpret_cast<const double2 *>(sbar);
#pragma unroll 4
            for (int i = tid; i < ns / 2; i += ADJ_THREADS) {
                const double2 v = __ldg(s2 + i);
                amax = max(amax, (unsigned long long)__double_as_longlong(v.x) & 0x7fffffffffffffffull);
                amax = max(amax, (unsigned long long)__double_as_longlong(v.y) & 0x7fffffffffffffffull);
            }
        } else {
            for (int i = tid; i < ns; i += ADJ_THREADS)
                amax = max(amax, (unsigned long long)__double_as_longlong(sbar[i]) & 0x7fffffffffffffffull);
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        amax = max(amax, __shfl_xor_sync(0xffffffffu, amax, off));
        msum += __shfl_xor_sync(0xffffffffu, msum, off);
    }
    if (lane == 0) { wmax[warp] = amax; wsum[warp] = msum; }
    ModelConst mc;
    {
        const float4 d0 = __ldg(reinterpret_cast<const float4 *>(mp));        // kd2, 1 - fnd, fnd, dust_index
        const float4 d1v = __ldg(reinterpret_cast<const float4 *>(mp) + 1);   // kd1, dust1_index, 1 - fo, fo
        const float4 d2v = __ldg(reinterpret_cast<const float4 *>(mp) + 2);   // igm on, jmax, kcap, kd3
        mc.kd2 = d0.x; mc.one_m_fnd = d0.y; mc.fnd = d0.z; mc.dust_index = d0.w;
        mc.kd1 = d1v.x; mc.dust1_index = d1v.y; mc.one_m_fo = d1v.z; mc.fo = d1v.w;
        mc.igm_model = d2v.x != 0.f; mc.jmax = __float_as_int(d2v.y); mc.kd3 = d2v.w;
        mc.cs1 = __ldg(mp + MP_CS1); mc.cs2 = __ldg(mp + MP_CS1 + 1); mc.cs3 = __ldg(mp + MP_CS1 + 2);
#pragma unroll
        for (int k = 0; k < 6; ++k) { mc.b[k] = __ldg(ap + AP_B + k); mc.db[k] = __ldg(ap + AP_DB + k); }
    }
    __syncthreads();
    unsigned long long u = 0ull;
#pragma unroll
    for (int w = 0; w < ADJ_WARPS; ++w) u = max(u, wmax[w]);
    // 2^ks with ks = the exponent of frexp (2^ks >= the maximum); 1 for a zero or non-finite maximum
    const int de = (int)(u >> 52);
    const int ks = (u == 0ull || de == 0x7ff) ? 0 : de - 1022;
    if (mb)
        for (int b = tid; b < a.nbands; b += ADJ_THREADS) {
            const double f = fbd[b];
            fbs[b] = ((a.do_band == nullptr || a.do_band[b] != 0) && f > 0.0) ? scaled_to_f32(mb[b] * DMAG_DF / f, ks)
                                                                              : 0.f;
        }
    const float f_igm = (float)pr[PF_IGM_FACTOR];
    const float kf = -f_igm * 1.4426950408889634f;
    // dust emission and the AGN torus of this model (the forward's per-model epilogue, parts_epilogue_kernel)
    DustEmModel dm{};
    if (a.dem) dm = a.dem[m];
    const bool emis = a.dem != nullptr && dm.on != 0;
    const bool agn = a.dem != nullptr && dm.agn != 0;
    double lsum_m = 1.0;
    float lagn = 0.f;
    if (agn) {
        const double ls = a.lsum[(size_t)a.lsum_stride * m];
        lsum_m = ls > SAFE_FLOOR ? ls : 1.0;
        lagn = (float)(lsum_m * (double)dm.fagn);
    }
    const float *ag0 = agn ? a.agn_spec + (size_t)dm.ita * ns : nullptr, *ag1 = agn ? ag0 + ns : nullptr;
    constexpr float LN2 = 0.6931471805599453f;
    // 1 - T of each screen from its exponent (the forward's absorbed light, without cancellation)
    auto one_minus = [&](const PixFwd &f, float &omb, float &omo, float &omd) {
        omb = (mc.kd1 != 0.f) ? -adj_expm1(mc.kd1 * f.c1 * LN2) : 0.f;
        omo = (mc.kd3 != 0.f) ? -adj_expm1(mc.kd3 * f.curve * LN2) : 0.f;
        omd = mc.one_m_fnd * -adj_expm1(mc.kd2 * f.curve * LN2);
    };
    // block sums of up to three per-thread values into emsum, then every thread reads them
    auto block_sums = [&](float v0, float v1, float v2, float *out) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            v0 += __shfl_xor_sync(0xffffffffu, v0, off);
            v1 += __shfl_xor_sync(0xffffffffu, v1, off);
            v2 += __shfl_xor_sync(0xffffffffu, v2, off);
        }
        if (lane == 0) { emsum[0][warp] = v0; emsum[1][warp] = v1; emsum[2][warp] = v2; }
        __syncthreads();
        out[0] = out[1] = out[2] = 0.f;
        for (int w = 0; w < ADJ_WARPS; ++w) { out[0] += emsum[0][w]; out[1] += emsum[1][w]; out[2] += emsum[2][w]; }
        __syncthreads();
    };

    // ---- pass 0: the pre-smoothing spectrum TOT = ss D T_igm (the forward's epilogue, recomputed), with dust
    // emission the energy-balance sums and its escaping template through the IGM (in S, free until pass 1), with the
    // AGN its template through the diffuse dust
    mbar_wait(&rows_bar, 0, a.status, ERR_TIMEOUT_ADJOINT, false);
    float s_abs = 0.f, s_esc = 0.f, R_em = 0.f;
#pragma unroll 2
    for (int p = tid; p < ns; p += ADJ_THREADS) {
        const PixFwd f = pix_forward(a, mc, p);
        const float T = f.igm ? adj_ex2(f.tau * kf) : 1.f;
        float tot = (yv[p] * f.ssfac_y + ov[p] * f.to) * f.D * T;
        if (emis) {
            float omb, omo, omd;
            one_minus(f, omb, omo, omd);
            const float absorbed = yv[p] * (mc.one_m_fo * omb + f.ssfac_y * omd) + ov[p] * (omo + f.to * omd);
            const float e = dl07_eval(a.dtab, ns, a.nqpah, p, dm).shape * f.td;
            const float cn = __ldg(a.cnu + p);
            s_abs = fmaf(cn, absorbed, s_abs);
            s_esc = fmaf(cn, e, s_esc);
            S[p] = e * T;
        }
        if (agn) tot = fmaf(lagn * fmaf(dm.wta, __ldg(ag1 + p) - __ldg(ag0 + p), __ldg(ag0 + p)), f.td, tot);
        TOT[p] = tot;
    }
    if (emis) {
        float sums[3];
        block_sums(s_abs, s_esc, 0.f, sums);
        s_abs = sums[0];
        s_esc = sums[1];
        R_em = s_esc > SAFE_FLOOR ? s_abs / s_esc : 0.f;
        for (int p = tid; p < ns; p += ADJ_THREADS) TOT[p] = fmaf(S[p], R_em, TOT[p]);
    }
    __syncthreads();
    // ---- pass 1: the smoothed spectrum S (pixels sm_lo .. sm_hi with the model's taps)
    const int R = __float_as_int(mp[MP_SMOOTH_R]);
    float tap[9];
#pragma unroll
    for (int d = 0; d < 9; ++d) tap[d] = __ldg(mp + MP_TAPS + d);
    for (int p = tid; p < ns; p += ADJ_THREADS) {
        float v = TOT[p];
        if (R >= 0 && p >= a.sm_lo && p <= a.sm_hi) {
            float s = 0.f;
#pragma unroll
            for (int d = -4; d <= 4; ++d) s = fmaf(tap[d + 4], TOT[p + d], s);
            v = s;
        }
        S[p] = v;
    }
    __syncthreads();
    // ---- pass 2: band fluxes -> observed frame: VB(j) = dL / dv_j, v_j the rest spectrum interpolated at
    // lambda_j / (1 + z); Fobs_j = max(v_j, 0) / lambda_j
    const float4 zi = a.zinfo[m];
    const bool shifted = zi.w == 1.f;
    const int nsh = __float_as_int(zi.x) + ((zi.y > 0.f) ? 1 : 0);   // observed pixel j reads interval j - nsh
    const float tin = zi.y;
    float gobs = 0.f;   // sum of VB_j (S(il + 1) - S(il)) lambda_j / lambda_(il + nsh)
    if (mb) {
        for (int j = a.j0 + tid; j <= a.j1; j += ADJ_THREADS) {
            // dL / dFobs_j = sum over the bands reaching j of C(j, b) dL / dfband_b: the warp's 32 pixels form one
            // chunk, whose bands are read as coalesced rows of the band-major matrix
            float fo_bar = 0.f;
            const int2 br = __ldg(a.bchunk + ((j - a.j0) >> 5));
            for (int b = br.x; b <= br.y; ++b) {
                const int4 bm = __ldg(a.bmeta + b);
                if (j >= bm.x && j <= bm.y) fo_bar = fmaf(__ldg(a.bc + bm.z + (j - bm.x)), fbs[b], fo_bar);
            }
            float v;
            int cl = j;
            float xf = 1.f;
            if (shifted) {
                const int il = j - nsh;
                cl = min(max(il, 0), ns - 2);
                float t = tin;
                if (cl != il) {
                    // outside the grid: the first / last interval extrapolated
                    t = (adj_ex2(((float)(j - cl) - zi.z) * a.dl2) - 1.f) * a.inv_em1;
                    xf = adj_ex2((float)(il - cl) * a.dl2);
                }
                v = fmaf(t, S[cl + 1] - S[cl], S[cl]);
            } else {
                v = S[j];
            }
            const float vb = (v > 0.f) ? fo_bar * __ldg(a.wl + j) : 0.f;   // (NaN v: 0, as the forward)
            VB[j - a.j0] = vb;
            if (shifted && vb != 0.f) gobs = fmaf(vb * (S[cl + 1] - S[cl]), xf, gobs);
        }
    }
    __syncthreads();
    // ---- pass 3: dL / dS (into S): the spectrum's own cotangent and the transpose of the observed-frame
    // interpolation
    for (int p = 2 * tid; p < ns; p += 2 * ADJ_THREADS) {
        float sb[2] = {0.f, 0.f};
        if (sbar) {
            if (even && p + 1 < ns) {
                const double2 v = __ldg(reinterpret_cast<const double2 *>(sbar + p));
                sb[0] = scaled_to_f32(v.x, ks);
                sb[1] = scaled_to_f32(v.y, ks);
            } else {
                sb[0] = scaled_to_f32(sbar[p], ks);
                if (p + 1 < ns) sb[1] = scaled_to_f32(sbar[p + 1], ks);
            }
        }
#pragma unroll
        for (int u2 = 0; u2 < 2; ++u2) {
            const int q = p + u2;
            if (q >= ns) break;
            float x = sb[u2];
            if (mb) {
                if (!shifted) {
                    if (q >= a.j0 && q <= a.j1) x += VB[q - a.j0];
                } else {
                    const int ja = q + nsh;        // interval q, weight 1 - t
                    const int jb = q - 1 + nsh;    // interval q - 1, weight t
                    if (q <= ns - 2 && ja >= a.j0 && ja <= a.j1) x = fmaf(1.f - tin, VB[ja - a.j0], x);
                    if (q >= 1 && jb >= a.j0 && jb <= a.j1) x = fmaf(tin, VB[jb - a.j0], x);
                }
            }
            S[q] = x;
        }
    }
    __syncthreads();
    if (tid == 0 && mb && shifted) {
        // observed pixels whose interval lies outside the grid (extrapolated from the first / last interval)
        const int lo_end = min(a.j1, nsh - 1), hi_beg = max(a.j0, ns - 1 + nsh);
        for (int j = a.j0; j <= lo_end; ++j) {
            const float t = (adj_ex2(((float)j - zi.z) * a.dl2) - 1.f) * a.inv_em1;
            S[0] = fmaf(1.f - t, VB[j - a.j0], S[0]);
            S[1] = fmaf(t, VB[j - a.j0], S[1]);
        }
        for (int j = hi_beg; j <= a.j1; ++j) {
            const int cl = ns - 2;
            const float t = (adj_ex2(((float)(j - cl) - zi.z) * a.dl2) - 1.f) * a.inv_em1;
            S[cl] = fmaf(1.f - t, VB[j - a.j0], S[cl]);
            S[cl + 1] = fmaf(t, VB[j - a.j0], S[cl + 1]);
        }
    }
    __syncthreads();
    // ---- pass 4: d / dsigma of the taps (dtap from the per-model block; they sum to zero, so the differences from
    // the centre keep the FP32 sum clear of cancellation), then the smoothing's transpose into TOT
    float gs = 0.f;
    if (R >= 0) {
        float dtap[9];
#pragma unroll
        for (int d = 0; d < 9; ++d) dtap[d] = __ldg(ap + AP_DTAP + d);
        for (int p = max(a.sm_lo, 0) + tid; p <= a.sm_hi; p += ADJ_THREADS) {
            const float t0 = TOT[p];
            float ds = 0.f;
#pragma unroll
            for (int d = -4; d <= 4; ++d) ds = fmaf(dtap[d + 4], TOT[p + d] - t0, ds);
            gs = fmaf(S[p], ds, gs);
        }
    }
    __syncthreads();
    for (int p = tid; p < ns; p += ADJ_THREADS) {
        const bool act = R >= 0 && p >= a.sm_lo && p <= a.sm_hi;
        float tb = act ? 0.f : S[p];
        if (R >= 0) {
#pragma unroll
            for (int d = -4; d <= 4; ++d) {
                const int r = p - d;   // S(r) reads TOT(r + d) = TOT(p)
                if (r >= a.sm_lo && r <= a.sm_hi) tb = fmaf(tap[d + 4], S[r], tb);
            }
        }
        TOT[p] = tb;
    }
    __syncthreads();
    // ---- pass 5: the IGM and attenuation adjoints; the young / old cotangents (bf16 hi / lo); parameter gradients
    float g[NG];
#pragma unroll
    for (int k = 0; k < NG; ++k) g[k] = 0.f;
    const float d2 = a.dust_type == 3 ? 1.f : (float)pr[PF_DUST2], d3 = (float)pr[PF_DUST3], d1 = (float)pr[PF_DUST1];
    // the dust emission's and the AGN's sums over the pixels (backward_emission_sums / backward_agn,
    // src/physics/opensps_csp_batch.f90:6667-6845): R_bar = sum dL/dTOT T_igm shape T_d (E = R shape T_d T_igm is linear
    // in R = s_abs / s_esc), s1 = sum dL/dTOT tmpl T_d, s2 = sum dL/dTOT (tmpl_hi - tmpl_lo) T_d
    float em_sums[3] = {0.f, 0.f, 0.f};
    if (emis || agn) {
        float rb = 0.f, s1 = 0.f, s2 = 0.f;
        for (int p = tid; p < ns; p += ADJ_THREADS) {
            const PixFwd f = pix_forward(a, mc, p);
            const float sb = TOT[p];
            if (emis) {
                const float T = f.igm ? adj_ex2(f.tau * kf) : 1.f;
                rb = fmaf(sb * T, dl07_eval(a.dtab, ns, a.nqpah, p, dm).shape * f.td, rb);
            }
            if (agn) {
                const float t0 = __ldg(ag0 + p), t1 = __ldg(ag1 + p);
                s1 = fmaf(sb, fmaf(dm.wta, t1 - t0, t0) * f.td, s1);
                s2 = fmaf(sb, (t1 - t0) * f.td, s2);
            }
        }
        block_sums(rb, s1, s2, em_sums);
    }
    // s_abs_bar = R_bar / s_esc, s_esc_bar = -R_bar s_abs / s_esc^2 (zero where the forward added no emission)
    const bool em_on = emis && s_esc > SAFE_FLOOR;
    const float sab = em_on ? em_sums[0] / s_esc : 0.f;
    const float seb = em_on ? -em_sums[0] * (s_abs / s_esc) / s_esc : 0.f;
    __nv_bfloat162 *yh = reinterpret_cast<__nv_bfloat162 *>(a.ybar_hi + (size_t)m * a.ppad);
    __nv_bfloat162 *yl = reinterpret_cast<__nv_bfloat162 *>(a.ybar_lo + (size_t)m * a.ppad);
    __nv_bfloat162 *oh = reinterpret_cast<__nv_bfloat162 *>(a.obar_hi + (size_t)m * a.ppad);
    __nv_bfloat162 *ol = reinterpret_cast<__nv_bfloat162 *>(a.obar_lo + (size_t)m * a.ppad);
    for (int p = 2 * tid; p < a.ppad; p += 2 * ADJ_THREADS) {
        float yb[2] = {0.f, 0.f}, ob[2] = {0.f, 0.f};
        if (p < ns) {
#pragma unroll
            for (int u2 = 0; u2 < 2; ++u2) {
                const int q = p + u2;
                if (q >= ns) break;
                const PixFwd f = pix_forward(a, mc, q);
                const float y = yv[q], o = ov[q], sb = TOT[q];
                Dl07Val dv{};
                if (em_on) dv = dl07_eval(a.dtab, ns, a.nqpah, q, dm);
                float T;
                pixel_adjoint(a, mc, f, y, o, sb, f_igm, kf, d1, d2, d3, em_on ? R_em * dv.shape * f.td : 0.f, g,
                              yb[u2], ob[u2], T);
                if (em_on || agn) {
                    float td_bar = 0.f;
                    if (em_on) {
                        // the escaping template E = R shape T_d T_igm, s_esc = sum cn shape T_d, and the absorbed
                        // light in s_abs = sum cn (y A_y + o A_o), A_y = (1 - fo) (1 - T_b) + (T_b (1 - fo) + fo)
                        // (1 - T_d) (1 - fnd), A_o = (1 - T_o) + T_o (1 - T_d) (1 - fnd)
                        const float cn = __ldg(a.cnu + q), sbt = sb * T;
                        td_bar = sbt * R_em * dv.shape + seb * cn * dv.shape;
                        const float shape_bar = (sbt * R_em + seb * cn) * f.td;
                        g[G_WQ] = fmaf(shape_bar, dv.d_wq, g[G_WQ]);
                        g[G_WU] = fmaf(shape_bar, dv.d_wu, g[G_WU]);
                        g[G_GAM] = fmaf(shape_bar, dv.d_gam, g[G_GAM]);
                        float omb, omo, omd;
                        one_minus(f, omb, omo, omd);
                        const float A = sab * cn, yo = y * f.ssfac_y + o * f.to;
                        yb[u2] = fmaf(A, mc.one_m_fo * omb + f.ssfac_y * omd, yb[u2]);
                        ob[u2] = fmaf(A, omo + f.to * omd, ob[u2]);
                        td_bar = fmaf(A * yo, -mc.one_m_fnd, td_bar);
                        g[G_FOBRUN] = fmaf(A * y, omb * (omd - 1.f), g[G_FOBRUN]);
                        g[G_FNODUST] = fmaf(A * yo, -(1.f - f.td), g[G_FNODUST]);
                        if (mc.kd1 != 0.f) {
                            const float tbb = A * y * mc.one_m_fo * (omd - 1.f);
                            g[G_DUST1] = fmaf(tbb, -f.c1 * f.tb, g[G_DUST1]);
                            g[G_DUST1_INDEX] = fmaf(tbb, -d1 * f.c1 * f.ltab * f.tb, g[G_DUST1_INDEX]);
                        }
                        if (mc.kd3 != 0.f) {
                            const float tob = A * o * (omd - 1.f);
                            g[G_DUST3] = fmaf(tob, -f.curve * f.to, g[G_DUST3]);
                            curve_rows(f, tob * -d3 * f.to, g);
                        }
                    }
                    // the AGN: lagn tmpl T_d
                    if (agn) td_bar = fmaf(sb * lagn, fmaf(dm.wta, __ldg(ag1 + q) - __ldg(ag0 + q), __ldg(ag0 + q)), td_bar);
                    // T_d = exp(-dust2 curve)
                    g[G_DUST2] = fmaf(td_bar, -f.curve * f.td, g[G_DUST2]);
                    curve_rows(f, td_bar * -d2 * f.td, g);
                }
            }
        }
        const __nv_bfloat162 hy = bf16_hi2(yb[0], yb[1]), ho = bf16_hi2(ob[0], ob[1]);
        yh[p >> 1] = hy;
        yl[p >> 1] = bf16_lo2(yb[0], yb[1], hy);
        oh[p >> 1] = ho;
        ol[p >> 1] = bf16_lo2(ob[0], ob[1], ho);
    }
    g[G_SIGMA] = gs;
    g[G_OBS] = gobs;
#pragma unroll
    for (int k = 0; k < NG; ++k) {
        float v = g[k];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if (lane == 0) red[k][warp] = v;
    }
    __syncthreads();
    if (tid < NBGRAD) {
        const double c = ldexp(1.0, ks);
        // (row_of[k]: the params_bar row of accumulator k; G_OBS goes into the zred row below)
        constexpr int NROW = 13;
        const int row_of[NROW] = {R_DUST2, R_DUST_INDEX, R_FRAC_NODUST, R_DUST1, R_DUST1_INDEX, R_FRAC_OBRUN,
                                  R_DUST3, R_ZRED, R_IGM_FACTOR, R_SIGMA, -1, R_MWR, R_UVB};
        static_assert(G_OBS == 10 && G_MWR == 11 && G_UVB == 12, "row_of follows the accumulators' order");
        double v = 0.0;
        int k = -1;
#pragma unroll
        for (int i = 0; i < NROW; ++i)
            if (row_of[i] == tid) k = i;
        // the dust emission's rows: d / d(wq, wu, gam) times the chain factors to q_PAH, U_min, gamma
        float chain = 0.f;
        if (emis && a.dchain) {
            const float4 dc = a.dchain[m];
            if (tid == R_DUSTE_QPAH) { k = G_WQ; chain = dc.x; }
            if (tid == R_DUSTE_UMIN) { k = G_WU; chain = dc.y; }
            if (tid == R_DUSTE_GAMMA) { k = G_GAM; chain = dc.z; }
        }
        if (k >= 0) {
            for (int w = 0; w < ADJ_WARPS; ++w) v += (double)red[k][w];
            v *= c;
            if (k >= G_WQ) v *= (double)chain;
        }
        if (agn && tid == R_FAGN) v = c * lsum_m * (double)em_sums[1];
        if (agn && tid == R_AGN_TAU && a.dchain) v = c * lsum_m * (double)dm.fagn * (double)em_sums[2] * (double)a.dchain[m].w;
        // (dust_type 3: the optical depth is the curve itself, dust2 has no effect: its row zero)
        if (tid == R_DUST2 && a.dust_type == 3) v = 0.0;
        if (tid == R_ZRED) {
            // the observed frame's share (its factor formed in FP64 per model) and the distance term's
            double go = 0.0, ms = 0.0;
            for (int w = 0; w < ADJ_WARPS; ++w) { go += (double)red[G_OBS][w]; ms += wsum[w]; }
            const double *apd = reinterpret_cast<const double *>(ap);
            v += c * go * apd[AP_KOBS / 2];
            if (mb) v += ms * apd[AP_DDIST / 2];
        }
        a.params_bar[(size_t)m * NBGRAD + tid] = v;
    }
    if (tid == 0) {
        a.cscale[m] = ldexp(1.0, ks);
        // the AGN's cotangent of the linear L_bol (fagn s1 where the forward did not floor it), unscaled
        if (a.lsum_bar) {
            const double ls = agn ? a.lsum[(size_t)a.lsum_stride * m] : 0.0;
            a.lsum_bar[m] = (agn && ls > SAFE_FLOOR) ? ldexp(1.0, ks) * (double)dm.fagn * (double)em_sums[1] : 0.0;
        }
        // (a wait above that gave up leaves the bulk copies to be waited for here, before the CTA exits)
        mbar_wait(&rows_bar, 0, a.status, ERR_TIMEOUT_ADJOINT, false);
    }
}

__host__ __device__ int adj_row_pad(int ns) { return (ns + 8 + 3) / 4 * 4; }

// ---------------------------------------------------------------------------------------------- transposed basis
// t(k, p) = basis(p, k): kpad x ppad from the first kpad columns of ns rows of ld (zero for p >= ns), 32 x 32 tiles
// through shared memory.
__global__ void transpose_bf16_kernel(const __nv_bfloat16 *__restrict__ src, __nv_bfloat16 *__restrict__ dst, int ns,
                                      int kpad, int ld, int ppad) {
    __shared__ __nv_bfloat16 tile[32][33];
    const int k0 = blockIdx.x * 32, p0 = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int p = p0 + r, k = k0 + threadIdx.x;
        tile[r][threadIdx.x] = (p < ns && k < kpad) ? src[(size_t)p * ld + k] : __float2bfloat16_rn(0.f);
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int k = k0 + r, p = p0 + threadIdx.x;
        if (k < kpad && p < ppad) dst[(size_t)k * ppad + p] = tile[threadIdx.x][r];
    }
}

cudaError_t run_transpose_bf16(const __nv_bfloat16 *src, __nv_bfloat16 *dst, int ns, size_t kpad, size_t ld, int ppad,
                               cudaStream_t st) {
    if (kpad > (size_t)INT_MAX - 32 || ld > (size_t)INT_MAX) return cudaErrorInvalidValue;
    const dim3 grid((unsigned)((kpad + 31) / 32), (unsigned)((ppad + 31) / 32)), block(32, 8);
    transpose_bf16_kernel<<<grid, block, 0, st>>>(src, dst, ns, (int)kpad, (int)ld, ppad);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------- weights' cotangent
// wzb(t + nt z, m) = cscale_m D(m, col(t, z)) + mass_bar_m M(t, z) + lsum_bar_m L(t, z), lsum_bar = lbol_bar /
// (ln 10 L_bol) plus the AGN's (backward_age_sums_w; the ssp_weights_z branch of compute_csp_batch's reverse pass).
struct WzbArgs {
    int n_models, ntz, ldd;
    const float *D;
    const int *col_of;
    const double *cscale, *mass_bar, *lbol_bar, *sums, *mass, *llin;
    const double *lsum_bar = nullptr;   // n_models: the AGN's cotangent of the linear L_bol (null: none)
    double *wzb;
};
__global__ void wzbar_kernel(WzbArgs a) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)a.n_models * a.ntz) return;
    const int m = (int)(i / a.ntz), k = (int)(i % a.ntz);
    double v = 0.0;
    if (a.D) v = a.cscale[m] * (double)a.D[(size_t)m * a.ldd + a.col_of[k]];
    if (a.mass_bar) v += a.mass_bar[m] * a.mass[k];
    if (a.lbol_bar) {
        const double ls = a.sums[(size_t)6 * m + 1];
        if (ls > SAFE_FLOOR) v += a.lbol_bar[m] / (ls * 2.302585092994046) * a.llin[k];
    }
    if (a.lsum_bar) v += a.lsum_bar[m] * a.llin[k];
    a.wzb[i] = v;
}

// The reverse of nebular emission's escaping ionizing light (the forward adds fesc sum_k w_k ion_k(p) to the young
// or old sums at the ionizing pixels p, fesc = clamp(frac_obrun, 0, 1)): per model and nebular (age, metallicity) k
// the sum s_k = sum_p ybar(p) ion_k(p) (obar for the old ages), one warp per k; the weights' cotangent gains
// fesc s_k and the frac_obrun row sum_k w_k s_k (where 0 < frac_obrun < 1).
struct IonRevArgs {
    int whl, ntneb, nt, nz, itesc, ppad, ntz;
    const float *ion;
    const double *wz, *par, *cscale;
    const __nv_bfloat16 *ybh, *ybl, *obh, *obl;
    double *wzbar;         // n x ntz (source order t + nt z), or null
    double *params_bar;    // n x NBGRAD
};

__global__ void __launch_bounds__(256) ion_rev_kernel(IonRevArgs a) {
    extern __shared__ float sb[];          // the ionizing pixels' young then old cotangents (scaled by 1 / cscale)
    __shared__ double red[8];
    const int m = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const double fo = a.par[(size_t)PAR_DEVICE * m + PF_FRAC_OBRUN];
    const double fesc = fmin(fmax(fo, 0.0), 1.0);
    const bool dfo = fo > 0.0 && fo < 1.0;
    if (fesc <= 0.0 && !dfo) return;
    const __nv_bfloat16 *yh = a.ybh + (size_t)m * a.ppad, *yl = a.ybl + (size_t)m * a.ppad;
    const __nv_bfloat16 *oh = a.obh + (size_t)m * a.ppad, *ol = a.obl + (size_t)m * a.ppad;
    for (int p = tid; p < a.whl; p += blockDim.x) {
        sb[p] = __bfloat162float(yh[p]) + __bfloat162float(yl[p]);
        sb[a.whl + p] = __bfloat162float(oh[p]) + __bfloat162float(ol[p]);
    }
    __syncthreads();
    const double cs = a.cscale[m];
    double part = 0.0;
    for (int k = warp; k < a.nz * a.ntneb; k += (int)(blockDim.x >> 5)) {
        const int z = k / a.ntneb, t = k - z * a.ntneb;
        const float *ik = a.ion + (size_t)k * a.whl, *bar = sb + (t < a.itesc ? 0 : a.whl);
        float s = 0.f;
        for (int p = lane; p < a.whl; p += 32) s = fmaf(bar[p], __ldg(ik + p), s);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (lane == 0) {
            const double sk = (double)s * cs;
            if (a.wzbar) a.wzbar[(size_t)m * a.ntz + t + (size_t)a.nt * z] += fesc * sk;
            const double w = a.wz[(size_t)m * a.nz * a.nt + (size_t)z * a.nt + t];
            if (w > SAFE_FLOOR) part += w * sk;
        }
    }
    if (lane == 0) red[warp] = part;
    __syncthreads();
    if (tid == 0 && dfo) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w];
        a.params_bar[(size_t)m * NBGRAD + R_FRAC_OBRUN] += v;
    }
}

cudaError_t run_adjoint(const AdjointPrepArgs &pa, const AdjointArgs &a, cudaStream_t st) {
    if (a.n_models <= 0) return cudaSuccess;
    adjoint_prep_kernel<<<(pa.n_models + 255) / 256, 256, 0, st>>>(pa);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int nj = a.j1 - a.j0 + 1;
    const size_t smem = sizeof(float) * (2 * (size_t)adj_row_pad(a.nspec) + 2 * (size_t)a.nspec + (size_t)(nj > 0 ? nj : 1));
    e = cudaFuncSetAttribute(adjoint_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    adjoint_kernel<<<a.n_models, ADJ_THREADS, smem, st>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------- the driver
static std::string msg(const char *what, cudaError_t e) { return std::string(what) + ": " + cudaGetErrorString(e); }

int run_grad_batch(Context &c, const BatchIO &io_in, const double *mags_bar, const double *spec_bar,
                   const double *mass_bar, const double *lbol_bar, double *params_bar, int params_bar_rows,
                   double *weights_z_bar, double *weights_bar, std::string &err) {
    if (!params_bar && !weights_z_bar && !weights_bar) return run_batch(c, io_in, err);
    const int n = io_in.n, ns = c.nspec, nb = c.nbands, ntz = c.nt * c.nz;
    if (mags_bar && (c.fast_mode || nb == 0)) {
        err = "mags_bar needs the magnitudes (fast mode off, a filter library)";
        return ST_UNSUPPORTED;
    }
    if (nb > ADJ_MAX_BANDS) { err = "more than 256 bands"; return ST_UNSUPPORTED; }
    cudaError_t e;
    // ---- the cotangents to the device on their own stream, beside the forward (from page-locked memory the copies
    // overlap its weight copy and kernels; the reverse pass waits for them on the batch's stream)
    auto put = [&](DevBuf<double> &d, const double *h, size_t cnt) -> cudaError_t {
        cudaError_t r = d.reserve(cnt);
        if (r != cudaSuccess) return r;
        return cudaMemcpyAsync(d.p, h, sizeof(double) * cnt, cudaMemcpyHostToDevice, c.side3);
    };
    // (every return waits for these copies first: the caller may reuse its buffers once the call returns)
    struct CopiesDone {
        cudaStream_t s;
        ~CopiesDone() { cudaStreamSynchronize(s); }
    } copies_done{c.side3};
    if ((mags_bar && (e = put(c.d_mags_bar, mags_bar, (size_t)n * nb)) != cudaSuccess) ||
        (spec_bar && (e = put(c.d_spec_bar, spec_bar, (size_t)n * ns)) != cudaSuccess) ||
        (mass_bar && (e = put(c.d_mass_bar, mass_bar, n)) != cudaSuccess) ||
        (lbol_bar && (e = put(c.d_lbol_bar, lbol_bar, n)) != cudaSuccess) ||
        (e = cudaEventRecord(c.ev_cot, c.side3)) != cudaSuccess) {
        err = msg("cotangent copy", e);
        return ST_DATA_MISSING;
    }
    // ---- the forward, keeping the young and old sums and the band fluxes on the device
    if ((e = c.d_fband.reserve((size_t)n * std::max(nb, 1))) != cudaSuccess) { err = msg("device memory", e); return ST_DATA_MISSING; }
    BatchIO io = io_in;
    io.keep_parts = true;
    io.fband_dev = nb > 0 ? c.d_fband.p : nullptr;
    int st = run_batch(c, io, err);
    if (st) return st;
    // with the SSP operators the age sums came from the operator (no basis operand): the reverse pass goes through
    // the transposed library and the reverse fold instead
    const bool ops = c.ops.ready;
    BasisOperand *bop = c.geom.bop;
    if ((!ops && !bop) || (ops && !c.geom.wz) || c.geom.nacc != 2 || c.geom.n != n) {
        err = "reverse pass: the forward's state is missing";
        return ST_DATA_MISSING;
    }
    cudaStream_t s = c.stream;
    // (the weights' cotangent is over the young and old columns: the escaping light's columns repeat nebular entries,
    // whose reverse is ion_rev_kernel's; ld_basis is the forward operand's row length)
    const int kpad = ops ? 0 : bop->kmain, ld_basis = ops ? 0 : bop->kpad;

    // ---- the transposed library (once per operator): the B operand of the template cotangents' GEMM
    if (ops && !c.ops.lib_thi.p) {
        SspOps &o = c.ops;
        const int ppad = (ns + gemm_bk() - 1) / gemm_bk() * gemm_bk();
        if ((e = o.lib_thi.reserve((size_t)o.ntpad * ppad)) != cudaSuccess ||
            (e = o.lib_tlo.reserve((size_t)o.ntpad * ppad)) != cudaSuccess) {
            err = msg("device memory", e);
            o.lib_thi.release(); o.lib_tlo.release();
            return ST_DATA_MISSING;
        }
        const dim3 grid((o.ntpad + 31) / 32, (ppad + 31) / 32), block(32, 8);
        transpose_bf16_kernel<<<grid, block, 0, s>>>(o.lib_hi.p, o.lib_thi.p, ns, o.ntpad, o.ntpad, ppad);
        transpose_bf16_kernel<<<grid, block, 0, s>>>(o.lib_lo.p, o.lib_tlo.p, ns, o.ntpad, o.ntpad, ppad);
        if ((e = cudaGetLastError()) != cudaSuccess ||
            (e = encode_tmap_2d_bf16(&o.tm_lib_thi, o.lib_thi.p, ppad, o.ntpad, gemm_bk(), gemm_bn())) != cudaSuccess ||
            (e = encode_tmap_2d_bf16(&o.tm_lib_tlo, o.lib_tlo.p, ppad, o.ntpad, gemm_bk(), gemm_bn())) != cudaSuccess) {
            err = msg("transposed library", e);
            o.lib_thi.release(); o.lib_tlo.release();
            return ST_DATA_MISSING;
        }
        o.ppad = ppad;
    }
    // ---- the transposed basis (once per operand) and its column map
    if (!ops && !bop->thi.p) {
        const int ppad = (ns + gemm_bk() - 1) / gemm_bk() * gemm_bk();
        std::vector<int> kmap(kpad), col_of(ntz, 0);
        if ((e = cudaMemcpy(kmap.data(), bop->kmap.p, sizeof(int) * kpad, cudaMemcpyDeviceToHost)) != cudaSuccess) {
            err = msg("basis map", e);
            return ST_DATA_MISSING;
        }
        for (int k = 0; k < kpad; ++k)
            if (kmap[k] >= 0) col_of[kmap[k] & KMAP_SRC] = k;
        if ((e = bop->thi.reserve((size_t)kpad * ppad)) != cudaSuccess ||
            (e = bop->tlo.reserve((size_t)kpad * ppad)) != cudaSuccess ||
            (e = bop->col_of.reserve(ntz)) != cudaSuccess ||
            (e = cudaMemcpy(bop->col_of.p, col_of.data(), sizeof(int) * ntz, cudaMemcpyHostToDevice)) != cudaSuccess) {
            err = msg("device memory", e);
            bop->thi.release(); bop->tlo.release();
            return ST_DATA_MISSING;
        }
        const dim3 grid((kpad + 31) / 32, (ppad + 31) / 32), block(32, 8);
        transpose_bf16_kernel<<<grid, block, 0, s>>>(bop->hi.p, bop->thi.p, ns, kpad, ld_basis, ppad);
        transpose_bf16_kernel<<<grid, block, 0, s>>>(bop->lo.p, bop->tlo.p, ns, kpad, ld_basis, ppad);
        if ((e = cudaGetLastError()) != cudaSuccess ||
            (e = encode_tmap_2d_bf16(&bop->tm_thi, bop->thi.p, ppad, kpad, gemm_bk(), gemm_bn())) != cudaSuccess ||
            (e = encode_tmap_2d_bf16(&bop->tm_tlo, bop->tlo.p, ppad, kpad, gemm_bk(), gemm_bn())) != cudaSuccess) {
            err = msg("transposed basis", e);
            bop->thi.release(); bop->tlo.release();
            return ST_DATA_MISSING;
        }
        bop->ppad = ppad;
    }
    const int ppad = ops ? c.ops.ppad : bop->ppad;

    // ---- the cotangents (copied beside the forward) before the reverse pass's kernels
    if ((e = cudaStreamWaitEvent(s, c.ev_cot, 0)) != cudaSuccess) { err = msg("cotangent copy", e); return ST_DATA_MISSING; }
    if ((e = c.d_cscale.reserve(n)) != cudaSuccess || (e = c.d_pbar.reserve((size_t)NBGRAD * n)) != cudaSuccess ||
        (e = c.d_ybh.reserve((size_t)n * ppad)) != cudaSuccess || (e = c.d_ybl.reserve((size_t)n * ppad)) != cudaSuccess ||
        (e = c.d_obh.reserve((size_t)n * ppad)) != cudaSuccess || (e = c.d_obl.reserve((size_t)n * ppad)) != cudaSuccess) {
        err = msg("device memory", e);
        return ST_DATA_MISSING;
    }
    cudaMemsetAsync(c.d_status.p, 0, sizeof(int), s);

    // ---- the per-model adjoint
    if ((e = c.d_apar.reserve((size_t)32 * n)) != cudaSuccess) { err = msg("device memory", e); return ST_DATA_MISSING; }
    AdjointPrepArgs pa;
    pa.n_models = n; pa.nspec = ns; pa.sm_lo = c.geom.sm_lo; pa.dlnl = c.dlnl; pa.em1 = std::expm1(c.dlnl);
    pa.par = c.d_params.p; pa.mpar = c.d_mpar.p; pa.zinfo = c.d_zinfo.p; pa.lnlam = c.d_lnlam.p;
    pa.zt = c.d_zt.p; pa.dl = c.d_dl.p; pa.apar = c.d_apar.p;
    AdjointArgs a;
    a.n_models = n; a.nspec = ns; a.ppad = ppad; a.nbands = nb; a.jtop = c.jtop;
    a.j0 = c.band_j0; a.j1 = nb > 0 ? c.band_j1 : c.band_j0 - 1;
    a.sm_lo = c.geom.sm_lo; a.sm_hi = c.geom.sm_hi; a.uniform_index = c.geom.uniform_index;
    a.dl2 = (float)(c.dlnl * 1.4426950408889634); a.inv_em1 = (float)(1.0 / std::expm1(c.dlnl));
    a.young = ops ? c.d_yo.p : c.d_young.p;
    a.old = ops ? c.d_yo.p + (size_t)n * ns : c.d_old.p;
    a.mpar = c.d_mpar.p; a.apar = c.d_apar.p; a.par = c.d_params.p;
    a.zinfo = c.d_zinfo.p; a.fband = c.d_fband.p;
    a.mags_bar = mags_bar ? c.d_mags_bar.p : nullptr;
    a.spec_bar = spec_bar ? c.d_spec_bar.p : nullptr;
    a.dust_type = c.dust_type;
    a.do_band = c.mag_mask.empty() ? nullptr : c.d_do_band.p;
    a.pix = c.d_pix.p; a.wl = c.d_wl.p; a.bc = c.d_bc.p; a.bmeta = c.d_bmeta.p; a.bchunk = c.d_bchunk.p;
    a.lt_base = (float)(std::log(c.lam[0] / 5500.0) * 1.4426950408889634);
    a.lt_step = (float)(c.dlnl * 1.4426950408889634);
    a.ybar_hi = c.d_ybh.p; a.ybar_lo = c.d_ybl.p; a.obar_hi = c.d_obh.p; a.obar_lo = c.d_obl.p;
    a.cscale = c.d_cscale.p; a.params_bar = c.d_pbar.p; a.status = c.d_status.p;
    if (c.geom.emis || c.geom.agn) {
        // the forward's dust emission / AGN (the AGN's L_bol: the batch's linear FP64 sum)
        a.dem = c.d_dem.p; a.dchain = c.d_dchain.p;
        a.dtab = c.dustem.tab.p; a.cnu = c.dustem.cnu.p; a.nqpah = c.dustem.nqpah;
        a.agn_spec = c.agn.spec.p;
        // (weights blended on the device without the operators: the log-blended L_bol the forward's AGN took)
        const bool blend = io_in.sfh_par != nullptr && !ops;
        a.lsum = blend ? c.d_lblend.p : c.d_sums.p + 1;
        a.lsum_stride = blend ? 3 : 6;
        if (c.geom.agn) {
            if ((e = c.d_lsum_bar.reserve(n)) != cudaSuccess) { err = msg("device memory", e); return ST_DATA_MISSING; }
            a.lsum_bar = c.d_lsum_bar.p;
        }
    }
    prof_mark(c, 6);
    if ((e = run_adjoint(pa, a, s)) != cudaSuccess) { err = msg("adjoint kernel", e); return ST_DATA_MISSING; }
    prof_mark(c, 7);
    int launches = 2;

    // ---- the weights' cotangent: young and old pixel cotangents against the transposed basis (over ages and
    // metallicities; with weights formed on the device, then through the blend and the SFH below)
    const bool dev_blend = io_in.sfh_par != nullptr;
    const bool sfh_rev = dev_blend && (weights_bar || params_bar);
    if (ops) {
        // ---- the operator: template cotangents (young and old pixel cotangents against the transposed library),
        // then the reverse fold: the weights' cotangent at every grid point (when wanted) and the slopes' rows
        const SspOps &o = c.ops;
        const bool want_wzb = weights_z_bar || sfh_rev;
        if ((e = c.d_vbar.reserve((size_t)2 * n * o.ntpad)) != cudaSuccess ||
            (e = c.d_apart.reserve((size_t)c.nz * n * 3)) != cudaSuccess ||
            (want_wzb && (e = c.d_wzbar.reserve((size_t)n * ntz)) != cudaSuccess)) {
            err = msg("device memory", e);
            return ST_DATA_MISSING;
        }
        for (int part = 0; part < 2; ++part) {
            GemmArgs g;
            g.M = n; g.N = o.ntpad; g.K = ppad; g.ldd = o.ntpad; g.b_row0 = 0; g.status = c.d_status.p;
            g.D = c.d_vbar.p + (size_t)part * n * o.ntpad;
            GemmPlan pl;
            pl.num_sms = c.num_sms;
            pl.tm_b_hi = o.tm_lib_thi;
            pl.tm_b_lo = o.tm_lib_tlo;
            const __nv_bfloat16 *ah = part == 0 ? c.d_ybh.p : c.d_obh.p, *al = part == 0 ? c.d_ybl.p : c.d_obl.p;
            if ((e = encode_tmap_2d_bf16(&pl.tm_a_hi, ah, ppad, n, gemm_bk(), gemm_bm())) != cudaSuccess ||
                (e = encode_tmap_2d_bf16(&pl.tm_a_lo, al, ppad, n, gemm_bk(), gemm_bm())) != cudaSuccess) {
                err = msg("cotangent tensor map", e);
                return ST_DATA_MISSING;
            }
            if ((e = run_gemm_bf16x3(pl, g, s)) != cudaSuccess) { err = msg("template cotangent GEMM", e); return ST_DATA_MISSING; }
            ++launches;
        }
        prof_mark(c, 8);
        OpsRevArgs r;
        r.n = n; r.nt = c.nt; r.nz = c.nz; r.npt = o.npt; r.ntpad = o.ntpad; r.itesc = c.geom.itesc; r.imf_type = c.imf_type;
        if (int rc = ops_imf_limits(c, c.imf_type, r.lim, err)) return rc;   // (the forward's limits and user IMF)
        r.wz = c.geom.wz; r.alpha = c.d_alpha.p; r.pts = o.pts.p; r.pidx = o.pidx.p; r.pcoef = o.pcoef.p;
        r.vbar = c.d_vbar.p; r.cscale = c.d_cscale.p;
        r.mass_bar = mass_bar ? c.d_mass_bar.p : nullptr;
        r.lbol_bar = lbol_bar ? c.d_lbol_bar.p : nullptr;   // (L_bol with the operators: the linear row, always)
        r.lsum_bar = c.geom.agn ? c.d_lsum_bar.p : nullptr;
        r.sums = c.d_sums.p;
        r.wzb = want_wzb ? c.d_wzbar.p : nullptr;
        r.apart = c.d_apart.p;
        r.params_bar = c.d_pbar.p; r.rows = NBGRAD; r.row_imf1 = PB_IMF1;
        // (the reverse of the fold the forward took: the interpolated one as GEMMs against the transposed basis)
        if (c.ops_last_interp) {
            if (int rc = run_ops_interp_reverse(c, r, err)) return rc;
            launches += 1 + (n + 2047) / 2048 * (1 + (r.itesc > 0 ? 1 : 0) + (r.itesc < c.nt ? 1 : 0));
        } else {
            if ((e = run_ops_reverse(r, s)) != cudaSuccess) { err = msg("operator reverse kernel", e); return ST_DATA_MISSING; }
            launches += 2;
        }
        prof_mark(c, 9);
        if (weights_z_bar &&
            (e = cudaMemcpyAsync(weights_z_bar, c.d_wzbar.p, sizeof(double) * n * ntz, cudaMemcpyDeviceToHost, s)) != cudaSuccess) {
            err = msg("weights cotangent copy", e);
            return ST_DATA_MISSING;
        }
    } else if (weights_z_bar || sfh_rev) {
        if ((e = c.d_wzb32.reserve((size_t)n * kpad)) != cudaSuccess || (e = c.d_wzbar.reserve((size_t)n * ntz)) != cudaSuccess) {
            err = msg("device memory", e);
            return ST_DATA_MISSING;
        }
        for (int part = 0; part < 2; ++part) {
            GemmArgs g;
            g.M = n; g.K = ppad; g.ldd = kpad; g.status = c.d_status.p;
            g.N = part == 0 ? bop->ky_pad : kpad - bop->ky_pad;
            g.b_row0 = part == 0 ? 0 : bop->ky_pad;
            g.D = c.d_wzb32.p + (part == 0 ? 0 : bop->ky_pad);
            if (g.N <= 0) continue;
            GemmPlan pl;
            pl.num_sms = c.num_sms;
            pl.tm_b_hi = bop->tm_thi;
            pl.tm_b_lo = bop->tm_tlo;
            const __nv_bfloat16 *ah = part == 0 ? c.d_ybh.p : c.d_obh.p, *al = part == 0 ? c.d_ybl.p : c.d_obl.p;
            if ((e = encode_tmap_2d_bf16(&pl.tm_a_hi, ah, ppad, n, gemm_bk(), gemm_bm())) != cudaSuccess ||
                (e = encode_tmap_2d_bf16(&pl.tm_a_lo, al, ppad, n, gemm_bk(), gemm_bm())) != cudaSuccess) {
                err = msg("cotangent tensor map", e);
                return ST_DATA_MISSING;
            }
            if ((e = run_gemm_bf16x3(pl, g, s)) != cudaSuccess) { err = msg("weights GEMM", e); return ST_DATA_MISSING; }
            ++launches;
        }
        prof_mark(c, 8);
        WzbArgs w;
        w.n_models = n; w.ntz = ntz; w.ldd = kpad; w.D = c.d_wzb32.p; w.col_of = bop->col_of.p;
        w.cscale = c.d_cscale.p; w.mass_bar = mass_bar ? c.d_mass_bar.p : nullptr;
        // (the log-blended L_bol of weights formed on the device has its own cotangent, in the SFH reverse pass)
        w.lbol_bar = (lbol_bar && !dev_blend) ? c.d_lbol_bar.p : nullptr;
        w.sums = c.d_sums.p; w.mass = c.d_mass.p; w.llin = c.d_llin.p;
        // (the AGN's L_bol: the linear sum over ages and metallicities, unless blended on the device, whose
        // log-blended L_bol takes it in the SFH reverse below)
        w.lsum_bar = (c.geom.agn && !dev_blend) ? c.d_lsum_bar.p : nullptr;
        w.wzb = c.d_wzbar.p;
        const size_t tot = (size_t)n * ntz;
        wzbar_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(w);
        if ((e = cudaGetLastError()) != cudaSuccess) { err = msg("weights cotangent kernel", e); return ST_DATA_MISSING; }
        prof_mark(c, 9);
        ++launches;
    }
    // ---- nebular emission's escaping ionizing light (the forward added it at the ionizing pixels)
    if (c.last_ion && !ops) {
        IonRevArgs ia;
        ia.whl = c.whlylim; ia.ntneb = c.nt_neb; ia.nt = c.nt; ia.nz = c.nz; ia.itesc = bop->itesc;
        ia.ppad = (ns + gemm_bk() - 1) / gemm_bk() * gemm_bk(); ia.ntz = ntz;
        ia.ion = c.d_ion.p; ia.wz = c.d_wz.p; ia.par = c.d_params.p; ia.cscale = c.d_cscale.p;
        ia.ybh = c.d_ybh.p; ia.ybl = c.d_ybl.p; ia.obh = c.d_obh.p; ia.obl = c.d_obl.p;
        ia.wzbar = (weights_z_bar || sfh_rev) ? c.d_wzbar.p : nullptr;
        ia.params_bar = c.d_pbar.p;
        const size_t smem = sizeof(float) * 2 * (size_t)c.whlylim;
        if ((e = cudaFuncSetAttribute(ion_rev_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess) {
            err = msg("ionizing light reverse kernel", e);
            return ST_DATA_MISSING;
        }
        ion_rev_kernel<<<n, 256, smem, s>>>(ia);
        if ((e = cudaGetLastError()) != cudaSuccess) { err = msg("ionizing light reverse kernel", e); return ST_DATA_MISSING; }
        ++launches;
    }
    // ---- the nebular continuum (added to the young and old sums by the forward): into the weights' cotangent and
    // the gas_logz, gas_logu and frac_obrun rows
    if (c.geom.neb && !ops) {
        NebContRevArgs na;
        na.n = n; na.nspec = ns; na.nt = c.nt; na.nz = c.nz; na.nt_neb = c.nt_neb; na.cw_ld = c.nt_neb + 2;
        na.itesc = c.geom.itesc; na.ppad = (ns + gemm_bk() - 1) / gemm_bk() * gemm_bk(); na.ntz = ntz;
        // the nebular ages by CLOUDY interval (ascending with the ages)
        for (int k = 0; k < 10; ++k) {
            int t = 0;
            while (t < c.nt_neb && c.neb.ia[t] < k) ++t;
            na.kfirst[k] = t;
        }
        c.neb.h_wa.assign(c.neb.wa.begin(), c.neb.wa.end());
        if ((e = c.neb.d_wa.reserve(std::max<size_t>(c.neb.h_wa.size(), 1))) != cudaSuccess ||
            (e = cudaMemcpyAsync(c.neb.d_wa.p, c.neb.h_wa.data(), sizeof(float) * c.neb.h_wa.size(), cudaMemcpyHostToDevice, s)) != cudaSuccess) {
            err = msg("nebular continuum reverse inputs", e);
            return ST_DATA_MISSING;
        }
        na.dem = c.d_dem.p; na.tab = c.neb.tab[c.geom.neb_table].p; na.off = c.neb.off.p; na.wa = c.neb.d_wa.p;
        na.cw = c.neb.cw.p; na.q0 = c.neb.q0.p; na.q0_exp = c.neb.q0_exp;
        na.ybh = c.d_ybh.p; na.ybl = c.d_ybl.p; na.obh = c.d_obh.p; na.obl = c.d_obl.p; na.cscale = c.d_cscale.p;
        na.wzbar = (weights_z_bar || sfh_rev) ? c.d_wzbar.p : nullptr;
        na.params_bar = c.d_pbar.p; na.rows = NBGRAD;
        na.row_gas_logz = 13; na.row_gas_logu = 14; na.row_frac_obrun = 6;
        if ((e = run_nebular_continuum_reverse(na, s)) != cudaSuccess) {
            err = msg("nebular continuum reverse kernel", e);
            return ST_DATA_MISSING;
        }
        ++launches;
    }
    if (!ops && weights_z_bar &&
        (e = cudaMemcpyAsync(weights_z_bar, c.d_wzbar.p, sizeof(double) * (size_t)n * ntz, cudaMemcpyDeviceToHost, s)) != cudaSuccess) {
        err = msg("weights cotangent copy", e);
        return ST_DATA_MISSING;
    }
    // ---- weights formed on the device: the cotangent of the weights over ages, logzsol's row and the SFH rows
    if (sfh_rev) {
        const int nt = c.nt;
        // (the tabular SFHs have no parameters here: their rows stay zero, sfh_weights_tangent
        // src/physics/opensps_sfh_tangent.f90:61-81)
        const bool tangents = io_in.given_w == nullptr && params_bar != nullptr && io_in.sfh_type != 2 &&
                              io_in.sfh_type != 3;
        if ((e = c.d_wbar.reserve((size_t)nt * n)) != cudaSuccess ||
            (tangents && (e = c.d_dual.reserve((size_t)3 * nt * n * sfh_dual_bytes())) != cudaSuccess)) {
            err = msg("device memory", e);
            return ST_DATA_MISSING;
        }
        SfhRevArgs r;
        r.n = n; r.nt = nt; r.nz = c.nz; r.sfh = io_in.sfh_type; r.rows = NBGRAD; r.has_logzsol = 1;
        r.sfh_tangents = tangents ? 1 : 0;
        r.tf = c.d_logage.p; r.lz = c.d_lz.p; r.lbol = c.d_lbol.p; r.par = c.d_sfhpar.p; r.w = c.d_w.p;
        // (with the operators L_bol is the linear row, whose cotangent the reverse fold took)
        r.lblend = c.d_lblend.p; r.lbol_bar = (lbol_bar && !ops) ? c.d_lbol_bar.p : nullptr; r.wzb = c.d_wzbar.p;
        r.lsum_bar = (c.geom.agn && !ops) ? c.d_lsum_bar.p : nullptr;
        r.weights_bar = c.d_wbar.p; r.scratch = c.d_sfh_scratch.p; r.params_bar = c.d_pbar.p;
        r.dual = tangents ? (void *)c.d_dual.p : nullptr;
        if ((e = run_sfh_reverse(r, s)) != cudaSuccess) { err = msg("SFH reverse kernel", e); return ST_DATA_MISSING; }
        ++launches;
        if (weights_bar &&
            (e = cudaMemcpyAsync(weights_bar, c.d_wbar.p, sizeof(double) * nt * n, cudaMemcpyDeviceToHost, s)) != cudaSuccess) {
            err = msg("weights cotangent copy", e);
            return ST_DATA_MISSING;
        }
    }
    std::vector<double> pb;
    if (params_bar) {
        pb.resize((size_t)NBGRAD * n);
        if ((e = cudaMemcpyAsync(pb.data(), c.d_pbar.p, sizeof(double) * pb.size(), cudaMemcpyDeviceToHost, s)) != cudaSuccess) {
            err = msg("gradient copy", e);
            return ST_DATA_MISSING;
        }
    }
    int kstatus = 0;
    if ((e = cudaMemcpyAsync(&kstatus, c.d_status.p, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess) {
        err = msg("reverse pass", e);
        return ST_DATA_MISSING;
    }
    if (kstatus != 0) {
        char buf[96];
        std::snprintf(buf, sizeof buf, "a device wait gave up in the reverse pass (code 0x%x)", kstatus);
        err = buf;
        return ST_DATA_MISSING;
    }
    if (params_bar)
        for (int m = 0; m < n; ++m)
            std::copy(pb.data() + (size_t)NBGRAD * m, pb.data() + (size_t)NBGRAD * (m + 1),
                      params_bar + (size_t)params_bar_rows * m);
    c.last_launches += launches;
    return 0;
}

}  // namespace sps
