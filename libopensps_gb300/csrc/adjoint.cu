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
// gradients are block reductions. Every cotangent is divided by the model's largest one (cscale) so that the FP32
// arithmetic stays in range; the results are multiplied back in FP64.
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

namespace sps {

constexpr int ADJ_THREADS = 256;
constexpr int ADJ_MAX_BANDS = 256;
constexpr double ADJ_C_KMS = 2.99792458e5;           // C_LIGHT 1e-13: km/s
constexpr double DMAG_DF = -1.0857362047581294;       // -2.5 / ln 10
constexpr int NBGRAD = 44;

// gradient rows of params_bar (opensps.h)
enum { R_DUST1 = 1, R_DUST2 = 2, R_DUST3 = 3, R_DUST_INDEX = 4, R_DUST1_INDEX = 5, R_FRAC_OBRUN = 6,
       R_FRAC_NODUST = 7, R_ZRED = 22, R_SIGMA = 23, R_IGM_FACTOR = 32 };
enum { G_DUST2 = 0, G_DUST_INDEX, G_FNODUST, G_DUST1, G_DUST1_INDEX, G_FOBRUN, G_DUST3, G_ZRED, G_IGMF, G_SIGMA, NG };

__device__ __forceinline__ float adj_ex2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// The forward's per-pixel factors of a model (as the contraction's epilogue forms them).
struct PixFwd {
    float curve, ltab, td, c1, tb, to, D, ssfac_y;
    float tau, dtau;   // IGM optical depth at unit igm_factor and its derivative in z (0 without IGM)
    bool igm;
};

__device__ __forceinline__ PixFwd pix_forward(const AdjointArgs &a, const float *mp, int p, bool igm_model, int jmax,
                                              const float *b, const float *db) {
    PixFwd f;
    const float4 v0 = reinterpret_cast<const float4 *>(a.pix + (size_t)p * PIX_FLOATS)[0];
    const float ltab2 = v0.x;
    f.ltab = ltab2 * 0.6931471805599453f;                        // ln(lambda / 5500)
    f.curve = a.uniform_index ? v0.y : adj_ex2(mp[MP_DUST_INDEX] * ltab2);
    f.td = adj_ex2(mp[MP_KD2] * f.curve);
    f.c1 = adj_ex2(mp[MP_DUST1_INDEX] * ltab2);
    f.tb = (mp[MP_KD1] != 0.f) ? adj_ex2(mp[MP_KD1] * f.c1) : 1.f;
    f.to = (mp[MP_KD3] != 0.f) ? adj_ex2(mp[MP_KD3] * f.curve) : 1.f;
    f.D = fmaf(f.td, mp[MP_ONE_M_FND], mp[MP_FND]);
    f.ssfac_y = f.tb * mp[MP_ONE_M_FO] + mp[MP_FO];
    f.igm = igm_model && p < a.jtop;
    f.tau = 0.f;
    f.dtau = 0.f;
    if (f.igm) {
        // pixels below the one of the largest depth take its depth (apply_igm_z's cap)
        const int jc = (p < jmax) ? jmax - 1 : p;
        const float4 w0 = reinterpret_cast<const float4 *>(a.pix + (size_t)jc * PIX_FLOATS)[0];
        const float4 w1 = reinterpret_cast<const float4 *>(a.pix + (size_t)jc * PIX_FLOATS)[1];
        const float ia[6] = {w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            f.tau = fmaf(ia[k], b[k], f.tau);
            f.dtau = fmaf(ia[k], db[k], f.dtau);
        }
    }
    return f;
}

__global__ void __launch_bounds__(ADJ_THREADS, 2) adjoint_kernel(AdjointArgs a) {
    extern __shared__ float sh[];
    const int ns = a.nspec;
    float *TOT = sh, *S = sh + ns, *SB = sh + 2 * ns, *VB = sh + 3 * ns;   // VB: pixels j0 .. j1
    __shared__ float fbs[ADJ_MAX_BANDS];
    __shared__ float red[NG][ADJ_THREADS / 32];
    __shared__ double cred[ADJ_THREADS / 32];
    __shared__ float b_s[6], db_s[6];
    __shared__ double s_c, s_msum;
    const int m = blockIdx.x, tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const float *mp = a.mpar + (size_t)MODEL_PAR_FLOATS * m;
    const double *pr = a.par + (size_t)PAR_DEVICE * m;
    const float *yv = a.young + (size_t)m * ns, *ov = a.old + (size_t)m * ns;
    const double z = pr[PF_ZRED];
    const bool igm_model = mp[MP_IGM_ON] != 0.f;
    const int jmax = __float_as_int(mp[MP_IGM_JMAX]);
    const double *mb = a.mags_bar ? a.mags_bar + (size_t)m * a.nbands : nullptr;
    const double *fbd = a.fband + (size_t)m * a.nbands;
    const double *sbar = a.spec_bar ? a.spec_bar + (size_t)m * ns : nullptr;

    // ---- the cotangent scale: the largest band-flux cotangent and spectrum cotangent of the model
    double cm = 0.0;
    if (mb)
        for (int b = tid; b < a.nbands; b += ADJ_THREADS) {
            const double f = fbd[b];
            if ((a.do_band == nullptr || a.do_band[b] != 0) && f > 0.0) cm = fmax(cm, fabs(mb[b] * DMAG_DF / f));
        }
    if (sbar)
        for (int p = tid; p < ns; p += ADJ_THREADS) cm = fmax(cm, fabs(sbar[p]));
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) cm = fmax(cm, __shfl_xor_sync(0xffffffffu, cm, off));
    if (lane == 0) cred[warp] = cm;
    if (tid == 0) {
        // the redshift factors b_k = (1 + z)^p_k and d b_k / dz (igm_tau_z_terms, src/physics/opensps_cosmology.f90:
        // 497-522), as the forward forms them
        const double pk[6] = {3.46, 1.68, 3.0 + 0.46, 1.5 + 0.18, 3.0 - 1.32, 1.68};
        const double l1z = igm_model ? log1p(z) : 0.0;
        for (int k = 0; k < 6; ++k) {
            const double bk = igm_model ? exp(pk[k] * l1z) : 0.0;
            b_s[k] = (float)bk;
            db_s[k] = igm_model ? (float)(pk[k] * bk / (1.0 + z)) : 0.f;
        }
    }
    __syncthreads();
    if (tid == 0) {
        double c = 0.0;
        for (int w = 0; w < ADJ_THREADS / 32; ++w) c = fmax(c, cred[w]);
        if (!(c > 0.0) || c > DBL_MAX) c = 1.0;
        s_c = c;
        a.cscale[m] = c;
        // the magnitudes' cotangents over the bands computed (the distance term's share of d / dz)
        double ms = 0.0;
        if (mb)
            for (int b = 0; b < a.nbands; ++b)
                if ((a.do_band == nullptr || a.do_band[b] != 0) && fbd[b] > 0.0) ms += mb[b];
        s_msum = ms;
    }
    __syncthreads();
    const double c = s_c;
    if (mb)
        for (int b = tid; b < a.nbands; b += ADJ_THREADS) {
            const double f = fbd[b];
            fbs[b] = ((a.do_band == nullptr || a.do_band[b] != 0) && f > 0.0) ? (float)(mb[b] * DMAG_DF / f / c) : 0.f;
        }
    float b[6], db[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) { b[k] = b_s[k]; db[k] = db_s[k]; }
    const float f_igm = (float)pr[PF_IGM_FACTOR];
    const float kf = -f_igm * 1.4426950408889634f;

    // ---- pass 0: the pre-smoothing spectrum TOT = ss D T_igm (the forward's epilogue, recomputed)
    for (int p = tid; p < ns; p += ADJ_THREADS) {
        const PixFwd f = pix_forward(a, mp, p, igm_model, jmax, b, db);
        const float ss = yv[p] * f.ssfac_y + ov[p] * f.to;
        float tot = ss * f.D;
        if (f.igm) tot *= adj_ex2(f.tau * kf);
        TOT[p] = tot;
    }
    __syncthreads();
    // ---- pass 1: the smoothed spectrum S (pixels sm_lo .. sm_hi with the model's taps)
    const int R = __float_as_int(mp[MP_SMOOTH_R]);
    float tap[9];
#pragma unroll
    for (int d = 0; d < 9; ++d) tap[d] = mp[MP_TAPS + d];
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
    const float dl2 = (float)(a.dlnl * 1.4426950408889634), inv_em1 = (float)(1.0 / expm1(a.dlnl));
    float gz = 0.f;   // sum of VB_j (S(il + 1) - S(il)) lambda_j / lambda_(il + nsh)
    if (mb) {
        for (int j = a.j0 + tid; j <= a.j1; j += ADJ_THREADS) {
            float fo_bar = 0.f;
            const int e1 = a.bptr[j - a.j0 + 1];
            for (int e = a.bptr[j - a.j0]; e < e1; ++e) fo_bar = fmaf(a.bw[e], fbs[a.bidx[e]], fo_bar);
            float v;
            int cl = j;
            float xf = 1.f;
            if (shifted) {
                const int il = j - nsh;
                cl = min(max(il, 0), ns - 2);
                float t = tin;
                if (cl != il) {
                    // outside the grid: the first / last interval extrapolated
                    t = (adj_ex2(((float)(j - cl) - zi.z) * dl2) - 1.f) * inv_em1;
                    xf = adj_ex2((float)(il - cl) * dl2);
                }
                v = fmaf(t, S[cl + 1] - S[cl], S[cl]);
            } else {
                v = S[j];
            }
            const float vb = (v > 0.f) ? fo_bar * a.wl[j] : 0.f;   // (NaN v: 0, as the forward)
            VB[j - a.j0] = vb;
            if (shifted && vb != 0.f) gz = fmaf(vb * (S[cl + 1] - S[cl]), xf, gz);
        }
    }
    __syncthreads();
    // ---- pass 3: SB = dL / dS: the spectrum's own cotangent and the transpose of the observed-frame interpolation
    for (int p = tid; p < ns; p += ADJ_THREADS) {
        float sb = sbar ? (float)(sbar[p] / c) : 0.f;
        if (mb) {
            if (!shifted) {
                if (p >= a.j0 && p <= a.j1) sb += VB[p - a.j0];
            } else {
                const int ja = p + nsh;        // interval p, weight 1 - t
                const int jb = p - 1 + nsh;    // interval p - 1, weight t
                if (p <= ns - 2 && ja >= a.j0 && ja <= a.j1) sb = fmaf(1.f - tin, VB[ja - a.j0], sb);
                if (p >= 1 && jb >= a.j0 && jb <= a.j1) sb = fmaf(tin, VB[jb - a.j0], sb);
            }
        }
        SB[p] = sb;
    }
    __syncthreads();
    if (tid == 0 && mb && shifted) {
        // observed pixels whose interval lies outside the grid (extrapolated from the first / last interval)
        const int lo_end = min(a.j1, nsh - 1), hi_beg = max(a.j0, ns - 1 + nsh);
        for (int j = a.j0; j <= lo_end; ++j) {
            const float t = (adj_ex2(((float)j - zi.z) * dl2) - 1.f) * inv_em1;
            SB[0] = fmaf(1.f - t, VB[j - a.j0], SB[0]);
            SB[1] = fmaf(t, VB[j - a.j0], SB[1]);
        }
        for (int j = hi_beg; j <= a.j1; ++j) {
            const int cl = ns - 2;
            const float t = (adj_ex2(((float)(j - cl) - zi.z) * dl2) - 1.f) * inv_em1;
            SB[cl] = fmaf(1.f - t, VB[j - a.j0], SB[cl]);
            SB[cl + 1] = fmaf(t, VB[j - a.j0], SB[cl + 1]);
        }
    }
    __syncthreads();
    // ---- pass 4: the smoothing's transpose (dL / dTOT, into S) and d / dsigma of its taps:
    // dc_d / dsigma = c_d (a_d - sum_u c_u a_u), a_d = (ln lambda_i0 - ln lambda_(i0 + d))^2 / (s^3 c), s = sigma / c
    float gs = 0.f;
    float dtap[9];
#pragma unroll
    for (int d = 0; d < 9; ++d) dtap[d] = 0.f;
    {
        const double sig = pr[PF_SIGMA_SMOOTH];
        if (R >= 0 && sig > 0.0) {
            const double sb = sig / ADJ_C_KMS;
            const double inv = 1.0 / (sb * sb * sb * ADJ_C_KMS);
            float av[9], mean = 0.f;
#pragma unroll
            for (int d = -4; d <= 4; ++d) {
                const int j = min(max(a.sm_lo + d, 0), ns - 1);
                const double dd = a.lnlam[a.sm_lo] - a.lnlam[j];
                av[d + 4] = (float)(dd * dd * inv);
                mean = fmaf(tap[d + 4], av[d + 4], mean);
            }
#pragma unroll
            for (int d = 0; d < 9; ++d) dtap[d] = tap[d] * (av[d] - mean);
        }
    }
    // the cotangent of TOT goes to S (S is not read after pass 2)
    for (int p = tid; p < ns; p += ADJ_THREADS) {
        const bool act = R >= 0 && p >= a.sm_lo && p <= a.sm_hi;
        float tb = act ? 0.f : SB[p];
        if (R >= 0) {
#pragma unroll
            for (int d = -4; d <= 4; ++d) {
                const int r = p - d;   // S(r) reads TOT(r + d) = TOT(p)
                if (r >= a.sm_lo && r <= a.sm_hi) tb = fmaf(tap[d + 4], SB[r], tb);
            }
        }
        if (act) {
            float ds = 0.f;
#pragma unroll
            for (int d = -4; d <= 4; ++d) ds = fmaf(dtap[d + 4], TOT[p + d], ds);
            gs = fmaf(SB[p], ds, gs);
        }
        S[p] = tb;
    }
    __syncthreads();
    // ---- pass 5: the IGM and attenuation adjoints; the young / old cotangents (bf16 hi / lo); parameter gradients
    float g[NG];
#pragma unroll
    for (int k = 0; k < NG; ++k) g[k] = 0.f;
    const float d2 = (float)pr[PF_DUST2], d3 = (float)pr[PF_DUST3], d1 = (float)pr[PF_DUST1];
    const float one_m_fnd = mp[MP_ONE_M_FND], one_m_fo = mp[MP_ONE_M_FO];
    float gz_igm = 0.f;
    for (int p = tid; p < a.ppad; p += ADJ_THREADS) {
        float yb = 0.f, ob = 0.f;
        if (p < ns) {
            const PixFwd f = pix_forward(a, mp, p, igm_model, jmax, b, db);
            const float y = yv[p], o = ov[p];
            const float ss = y * f.ssfac_y + o * f.to;
            const float pre = ss * f.D;
            float pb = S[p];
            if (f.igm) {
                // T = exp(-igm_factor tau): dT/dz = -igm_factor T dtau/dz, dT/d igm_factor = -tau T
                const float T = adj_ex2(f.tau * kf);
                const float gT = pb * pre;
                gz_igm = fmaf(gT, -f_igm * T * f.dtau, gz_igm);
                g[G_IGMF] = fmaf(gT, -f.tau * T, g[G_IGMF]);
                pb *= T;
            }
            // pre = ss D, D = T_d (1 - fnd) + fnd, ss = y (T_b (1 - fo) + fo) + o T_o
            const float dcurve = f.curve * f.ltab;   // d curve / d dust_index
            g[G_DUST2] = fmaf(pb * ss * one_m_fnd, -f.td * f.curve, g[G_DUST2]);
            g[G_DUST_INDEX] = fmaf(pb, ss * one_m_fnd * f.td * (-d2 * dcurve) + f.D * o * f.to * (-d3 * dcurve),
                                   g[G_DUST_INDEX]);
            g[G_FNODUST] = fmaf(pb * ss, 1.f - f.td, g[G_FNODUST]);
            const float ybase = pb * f.D * y;
            g[G_DUST1] = fmaf(ybase * one_m_fo, -f.tb * f.c1, g[G_DUST1]);
            g[G_DUST1_INDEX] = fmaf(ybase * one_m_fo, -f.tb * d1 * f.c1 * f.ltab, g[G_DUST1_INDEX]);
            g[G_FOBRUN] = fmaf(ybase, 1.f - f.tb, g[G_FOBRUN]);
            g[G_DUST3] = fmaf(pb * f.D * o, -f.to * f.curve, g[G_DUST3]);
            yb = pb * f.D * f.ssfac_y;
            ob = pb * f.D * f.to;
        }
        const size_t q = (size_t)m * a.ppad + p;
        const __nv_bfloat16 yh = __float2bfloat16_rn(yb), oh = __float2bfloat16_rn(ob);
        a.ybar_hi[q] = yh;
        a.ybar_lo[q] = __float2bfloat16_rn(yb - __bfloat162float(yh));
        a.obar_hi[q] = oh;
        a.obar_lo[q] = __float2bfloat16_rn(ob - __bfloat162float(oh));
    }
    g[G_ZRED] = gz_igm;
    g[G_SIGMA] = gs;
    // the observed frame's d / dz (kept apart: its factor is applied in FP64 below)
    float gobs = gz;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) gobs += __shfl_xor_sync(0xffffffffu, gobs, off);
#pragma unroll
    for (int k = 0; k < NG; ++k) {
        float v = g[k];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
        if (lane == 0) red[k][warp] = v;
    }
    if (lane == 0) cred[warp] = (double)gobs;   // (cred's first use ended before the syncs above)
    __syncthreads();
    if (tid < NBGRAD) {
        const int row_of[NG] = {R_DUST2, R_DUST_INDEX, R_FRAC_NODUST, R_DUST1, R_DUST1_INDEX, R_FRAC_OBRUN,
                                R_DUST3, R_ZRED, R_IGM_FACTOR, R_SIGMA};
        double v = 0.0;
        int k = -1;
#pragma unroll
        for (int i = 0; i < NG; ++i)
            if (row_of[i] == tid) k = i;
        if (k >= 0) {
            for (int w = 0; w < ADJ_THREADS / 32; ++w) v += (double)red[k][w];
            v *= c;
        }
        if (tid == R_ZRED) {
            if (shifted) {
                // dt/dz = -lambda_j / ((1 + z)^2 (lambda_(il+1) - lambda_il)) on the log-uniform grid
                double go = 0.0;
                for (int w = 0; w < ADJ_THREADS / 32; ++w) go += cred[w];
                const double opz = 1.0 + z;
                v += c * go * (-exp((double)nsh * a.dlnl) / (opz * opz * expm1(a.dlnl)));
            }
            if (mb && fabs(z) > SAFE_FLOOR) {
                // the distance term's derivative, d_L linear in the cosmology table
                const int idx = max(0, min(find_interval0(a.zt, 500, z), 498));
                const double slope = (a.dl[idx + 1] - a.dl[idx]) / (a.zt[idx + 1] - a.zt[idx]);
                const double dm = a.dl[idx] + slope * (z - a.zt[idx]);
                if (dm == dm && dm > SAFE_FLOOR)
                    v += s_msum * (5.0 / log(10.0) * slope / dm - 2.5 / (log(10.0) * (1.0 + z)));
            }
        }
        a.params_bar[(size_t)m * NBGRAD + tid] = v;
    }
}

// ---------------------------------------------------------------------------------------------- transposed basis
// t(k, p) = basis(p, k): kpad x ppad from ns x kpad (zero for p >= ns), 32 x 32 tiles through shared memory.
__global__ void transpose_bf16_kernel(const __nv_bfloat16 *__restrict__ src, __nv_bfloat16 *__restrict__ dst, int ns,
                                      int kpad, int ppad) {
    __shared__ __nv_bfloat16 tile[32][33];
    const int k0 = blockIdx.x * 32, p0 = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int p = p0 + r, k = k0 + threadIdx.x;
        tile[r][threadIdx.x] = (p < ns && k < kpad) ? src[(size_t)p * kpad + k] : __float2bfloat16_rn(0.f);
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int k = k0 + r, p = p0 + threadIdx.x;
        if (k < kpad && p < ppad) dst[(size_t)k * ppad + p] = tile[threadIdx.x][r];
    }
}

// ---------------------------------------------------------------------------------------------- weights' cotangent
// wzb(t + nt z, m) = cscale_m D(m, col(t, z)) + mass_bar_m M(t, z) + lsum_bar_m L(t, z), lsum_bar = lbol_bar /
// (ln 10 L_bol) (backward_age_sums_w; the ssp_weights_z branch of compute_csp_batch's reverse pass).
struct WzbArgs {
    int n_models, ntz, ldd;
    const float *D;
    const int *col_of;
    const double *cscale, *mass_bar, *lbol_bar, *sums, *mass, *llin;
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
    a.wzb[i] = v;
}

cudaError_t run_adjoint(const AdjointArgs &a, cudaStream_t st) {
    if (a.n_models <= 0) return cudaSuccess;
    const int nj = a.j1 - a.j0 + 1;
    const size_t smem = sizeof(float) * (3 * (size_t)a.nspec + (size_t)(nj > 0 ? nj : 1));
    cudaError_t e = cudaFuncSetAttribute(adjoint_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    adjoint_kernel<<<a.n_models, ADJ_THREADS, smem, st>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------- the driver
static std::string msg(const char *what, cudaError_t e) { return std::string(what) + ": " + cudaGetErrorString(e); }

int run_grad_batch(Context &c, const BatchIO &io_in, const double *mags_bar, const double *spec_bar,
                   const double *mass_bar, const double *lbol_bar, double *params_bar, int params_bar_rows,
                   double *weights_z_bar, std::string &err) {
    if (!mags_bar && !spec_bar && !mass_bar && !lbol_bar && !params_bar && !weights_z_bar) return run_batch(c, io_in, err);
    const int n = io_in.n, ns = c.nspec, nb = c.nbands, ntz = c.nt * c.nz;
    if (mags_bar && (c.fast_mode || nb == 0)) {
        err = "mags_bar needs the magnitudes (fast mode off, a filter library)";
        return ST_UNSUPPORTED;
    }
    if (nb > ADJ_MAX_BANDS) { err = "more than 256 bands"; return ST_UNSUPPORTED; }
    cudaError_t e;
    // ---- the forward, keeping the young and old sums and the band fluxes on the device
    if ((e = c.d_fband.reserve((size_t)n * std::max(nb, 1))) != cudaSuccess) { err = msg("device memory", e); return ST_DATA_MISSING; }
    BatchIO io = io_in;
    io.keep_parts = true;
    io.fband_dev = nb > 0 ? c.d_fband.p : nullptr;
    int st = run_batch(c, io, err);
    if (st) return st;
    BasisOperand *bop = c.geom.bop;
    if (!bop || c.geom.nacc != 2 || c.geom.n != n) { err = "reverse pass: the forward's state is missing"; return ST_DATA_MISSING; }
    cudaStream_t s = c.stream;
    const int kpad = bop->kpad;

    // ---- the transposed basis (once per operand) and its column map
    if (!bop->thi.p) {
        const int ppad = (ns + gemm_bk() - 1) / gemm_bk() * gemm_bk();
        std::vector<int> kmap(kpad), col_of(ntz, 0);
        if ((e = cudaMemcpy(kmap.data(), bop->kmap.p, sizeof(int) * kpad, cudaMemcpyDeviceToHost)) != cudaSuccess) {
            err = msg("basis map", e);
            return ST_DATA_MISSING;
        }
        for (int k = 0; k < kpad; ++k)
            if (kmap[k] >= 0) col_of[kmap[k] & 0x3fffffff] = k;
        if ((e = bop->thi.reserve((size_t)kpad * ppad)) != cudaSuccess ||
            (e = bop->tlo.reserve((size_t)kpad * ppad)) != cudaSuccess ||
            (e = bop->col_of.reserve(ntz)) != cudaSuccess ||
            (e = cudaMemcpy(bop->col_of.p, col_of.data(), sizeof(int) * ntz, cudaMemcpyHostToDevice)) != cudaSuccess) {
            err = msg("device memory", e);
            bop->thi.release(); bop->tlo.release();
            return ST_DATA_MISSING;
        }
        const dim3 grid((kpad + 31) / 32, (ppad + 31) / 32), block(32, 8);
        transpose_bf16_kernel<<<grid, block, 0, s>>>(bop->hi.p, bop->thi.p, ns, kpad, ppad);
        transpose_bf16_kernel<<<grid, block, 0, s>>>(bop->lo.p, bop->tlo.p, ns, kpad, ppad);
        if ((e = cudaGetLastError()) != cudaSuccess ||
            (e = encode_tmap_2d_bf16(&bop->tm_thi, bop->thi.p, ppad, kpad, gemm_bk(), gemm_bn())) != cudaSuccess ||
            (e = encode_tmap_2d_bf16(&bop->tm_tlo, bop->tlo.p, ppad, kpad, gemm_bk(), gemm_bn())) != cudaSuccess) {
            err = msg("transposed basis", e);
            bop->thi.release(); bop->tlo.release();
            return ST_DATA_MISSING;
        }
        bop->ppad = ppad;
    }
    const int ppad = bop->ppad;

    // ---- cotangents to the device
    auto put = [&](DevBuf<double> &d, const double *h, size_t cnt) -> cudaError_t {
        cudaError_t r = d.reserve(cnt);
        if (r != cudaSuccess) return r;
        return cudaMemcpyAsync(d.p, h, sizeof(double) * cnt, cudaMemcpyHostToDevice, s);
    };
    if ((mags_bar && (e = put(c.d_mags_bar, mags_bar, (size_t)n * nb)) != cudaSuccess) ||
        (spec_bar && (e = put(c.d_spec_bar, spec_bar, (size_t)n * ns)) != cudaSuccess) ||
        (mass_bar && (e = put(c.d_mass_bar, mass_bar, n)) != cudaSuccess) ||
        (lbol_bar && (e = put(c.d_lbol_bar, lbol_bar, n)) != cudaSuccess)) {
        err = msg("cotangent copy", e);
        return ST_DATA_MISSING;
    }
    if ((e = c.d_cscale.reserve(n)) != cudaSuccess || (e = c.d_pbar.reserve((size_t)NBGRAD * n)) != cudaSuccess ||
        (e = c.d_ybh.reserve((size_t)n * ppad)) != cudaSuccess || (e = c.d_ybl.reserve((size_t)n * ppad)) != cudaSuccess ||
        (e = c.d_obh.reserve((size_t)n * ppad)) != cudaSuccess || (e = c.d_obl.reserve((size_t)n * ppad)) != cudaSuccess) {
        err = msg("device memory", e);
        return ST_DATA_MISSING;
    }
    cudaMemsetAsync(c.d_status.p, 0, sizeof(int), s);

    // ---- the per-model adjoint
    AdjointArgs a;
    a.n_models = n; a.nspec = ns; a.ppad = ppad; a.nbands = nb; a.jtop = c.jtop;
    a.j0 = c.band_j0; a.j1 = nb > 0 ? c.band_j1 : c.band_j0 - 1;
    a.sm_lo = c.geom.sm_lo; a.sm_hi = c.geom.sm_hi; a.uniform_index = c.geom.uniform_index;
    a.dlnl = c.dlnl;
    a.young = c.d_young.p; a.old = c.d_old.p; a.mpar = c.d_mpar.p; a.par = c.d_params.p; a.zinfo = c.d_zinfo.p;
    a.fband = c.d_fband.p;
    a.mags_bar = mags_bar ? c.d_mags_bar.p : nullptr;
    a.spec_bar = spec_bar ? c.d_spec_bar.p : nullptr;
    a.do_band = c.mag_mask.empty() ? nullptr : c.d_do_band.p;
    a.pix = c.d_pix.p; a.lam = c.d_lam.p; a.lnlam = c.d_lnlam.p; a.wl = c.d_wl.p;
    a.bptr = c.d_bptr.p; a.bidx = c.d_bidx.p; a.bw = c.d_bw.p; a.zt = c.d_zt.p; a.dl = c.d_dl.p;
    a.ybar_hi = c.d_ybh.p; a.ybar_lo = c.d_ybl.p; a.obar_hi = c.d_obh.p; a.obar_lo = c.d_obl.p;
    a.cscale = c.d_cscale.p; a.params_bar = c.d_pbar.p;
    if ((e = run_adjoint(a, s)) != cudaSuccess) { err = msg("adjoint kernel", e); return ST_DATA_MISSING; }
    int launches = 1;

    // ---- the weights' cotangent: young and old pixel cotangents against the transposed basis
    if (weights_z_bar) {
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
        WzbArgs w;
        w.n_models = n; w.ntz = ntz; w.ldd = kpad; w.D = c.d_wzb32.p; w.col_of = bop->col_of.p;
        w.cscale = c.d_cscale.p; w.mass_bar = mass_bar ? c.d_mass_bar.p : nullptr;
        w.lbol_bar = lbol_bar ? c.d_lbol_bar.p : nullptr; w.sums = c.d_sums.p; w.mass = c.d_mass.p; w.llin = c.d_llin.p;
        w.wzb = c.d_wzbar.p;
        const size_t tot = (size_t)n * ntz;
        wzbar_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(w);
        if ((e = cudaGetLastError()) != cudaSuccess) { err = msg("weights cotangent kernel", e); return ST_DATA_MISSING; }
        ++launches;
        if ((e = cudaMemcpyAsync(weights_z_bar, c.d_wzbar.p, sizeof(double) * tot, cudaMemcpyDeviceToHost, s)) != cudaSuccess) {
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
