// The SSP operator applied to a free IMF per model (OpenSPS opensps_ssp_operator.f90 and opensps_ssp_batch.f90):
// the template weights V = S . (w_IMF x SFH weight) of every model, young and old apart, then spectra = library . V
// as a split-BF16 tcgen05 GEMM.
//
//   IMF bin weights  compute_imf_weights / imf_bin_weights_tab (src/physics/opensps_imf.f90:111-172, 439-559): per
//                    isochrone point the IMF's number of stars over its mass bin, over the IMF's mass between its
//                    limits; inside one power-law segment c lo^e expm1(e ln(hi / lo)) / e (e = 1 - alpha), in FP32
//                    with the segment's constants (FP64) formed once per model, as the reference's FP32 kernels do.
//                    Kroupa (and Salpeter as Kroupa with equal slopes) with its fixed breaks; van Dokkum 2008 (a
//                    lognormal up to 25 vdmc, a power law above) and Dave 2008 (slopes imf1 below mdave, imf2 above)
//                    with breaks per model (imf_integral :206-315).
//   fold             fold_multi (src/physics/opensps_ssp_batch.f90:3095-3188): V(e, m) = sum over points of S(e, p)
//                    w_IMF(p, m) wsfh(age(p), m), young ages and old apart, with the mass and L_bol rows.
//   template product template_columns (:3247-3385): spectra(pixel, m) = sum_e library(pixel, e) V(e, m).
//
// The fold: four models and one metallicity slab per CTA (every point record and entry read once for the four), over
// the slab's grid points any of them weighs; the slabs' template vectors are then summed in slab order. Per grid point the IMF weights of its 1500 points go to shared memory, then its entries, sorted by
// template on the host, are summed in runs of one template per thread and added to the template vectors in shared
// memory (one atomic per run and model). The mass and L_bol rows are summed per grid point in FP32 and over grid
// points in FP64.
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>
#include "context.h"

namespace sps {

constexpr int OPS_THREADS = 256;

__device__ __forceinline__ float ops_ex2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// e^y - 1: the Taylor series to y^6 below |y| = 1/8 (FP32: terms beyond are below its rounding), e^y - 1 above
__device__ __forceinline__ float ops_expm1(float y) {
    if (fabsf(y) < 0.125f) {
        float r = 1.f + y * (1.f / 6.f);
        r = 1.f + y * (1.f / 5.f) * r;
        r = 1.f + y * (1.f / 4.f) * r;
        r = 1.f + y * (1.f / 3.f) * r;
        r = 1.f + y * (1.f / 2.f) * r;
        return y * r;
    }
    return ops_ex2(y * 1.4426950408889634f) - 1.f;
}

// One model's IMF as the fold kernels take it: up to three segments [lo, hi], each a power law c m^-alpha (e = 1 -
// alpha, ce = c / e). Kroupa's breaks are fixed (each point's segment found once, OpsPoint::seg); van Dokkum's and
// Dave's move with the model (generic: every bin split at the model's breaks). For van Dokkum and Chabrier segment 0
// is the lognormal A exp(-z^2) per unit ln m, z = (log10 m - u0) zs (zs = 1 / (sigma sqrt 2)), whose bin integral is
// la int e^(-z^2) dz (la = A ln 10 sigma sqrt 2). For the reverse pass: lnb = ln b of the continuity factor
// c2 = b^(alpha2 - alpha1) (Kroupa b = 0.5, Dave b = mdave) and d3 = d ln c2 / d(third parameter) (Dave:
// (alpha2 - alpha1) / mdave; Kroupa: 0, its third slope acts through segment 3). With custom limits (OpsImfLim)
// the points are gated by initial mass against [glo, ghi] and an age's first bin starts at lb; the user IMF's
// segments (nuser, the table user) replace the three.
struct KroupaSeg {
    float e[3], ce[3], c[3];
    float lo[3], hi[3];
    int generic, logn;
    float la, u0, zs;
    double lnb, d3;
    int custom, nuser;
    float glo, ghi, lb;
    const float *user;
};

// c lo^e expm1(e dl) / e over one segment (e = 0: c dl)
__device__ __forceinline__ float seg_piece(const KroupaSeg &k, int s, float ln_lo, float dl) {
    if (k.e[s] == 0.f) return k.c[s] * dl;
    return k.ce[s] * ops_ex2(k.e[s] * ln_lo * 1.4426950408889634f) * ops_expm1(k.e[s] * dl);
}

// van Dokkum's lognormal over [lo, hi] (integrate_lognormal, src/physics/opensps_imf.f90:677-722, number): la times
// int e^(-z^2) dz, by 3-point Gauss-Legendre on a bin narrower than 0.1 in z (erf's difference would cancel), else
// by the difference of erf (erfc in a tail).
__device__ __forceinline__ float logn_piece(const KroupaSeg &k, float lo, float hi) {
    const float z1 = (log10f(lo) - k.u0) * k.zs, z2 = (log10f(hi) - k.u0) * k.zs;
    if (z2 - z1 < 0.1f) {
        const float zc = 0.5f * (z1 + z2), zh = 0.5f * (z2 - z1), x = 0.7745966692414834f * zh;
        const float q = (8.f / 9.f) * __expf(-zc * zc) +
                        (5.f / 9.f) * (__expf(-(zc - x) * (zc - x)) + __expf(-(zc + x) * (zc + x)));
        return k.la * zh * q;
    }
    const float c = k.la * 0.8862269254527580f;   // sqrt(pi) / 2
    if (z1 >= 0.f) return c * (erfcf(z1) - erfcf(z2));
    if (z2 <= 0.f) return c * (erfcf(-z2) - erfcf(-z1));
    return c * (erff(z2) - erff(z1));
}

// The user IMF over [lo, hi] (imf_integral case 5, src/physics/opensps_imf.f90:287-305): each segment's power law
// c_s m^-alpha_s over its own [lo_s, hi_s] (c_s continuous at each segment's lower mass); overlapping segments add,
// gaps weigh nothing. The table is the same for every lane (broadcast loads).
__device__ __forceinline__ float user_piece(const KroupaSeg &k, float lo, float hi) {
    float v = 0.f;
    for (int s = 0; s < k.nuser; ++s) {
        const float *u = k.user + 5 * s;
        const float a = fmaxf(lo, __ldg(u)), b = fminf(hi, __ldg(u + 1));
        if (b > a) {
            const float e = __ldg(u + 2), dl = logf(b / a);
            v += e == 0.f ? __ldg(u + 4) * dl
                          : __ldg(u + 3) * ops_ex2(e * logf(a) * 1.4426950408889634f) * ops_expm1(e * dl);
        }
    }
    return v;
}

// With custom limits: the bin's lower edge, or a negative value when the point weighs nothing (its initial mass
// outside the limits, or an empty bin).
__device__ __forceinline__ float custom_lo(const KroupaSeg &k, const OpsPoint &q) {
    const float mi = fabsf(q.mini);
    if (mi < k.glo || mi > k.ghi) return -1.f;
    const float lo = q.mini < 0.f ? k.lb : q.lo;
    return q.hi > lo ? lo : -1.f;
}

__device__ __forceinline__ float imf_weight(const KroupaSeg &k, const OpsPoint &q) {
    float qlo = q.lo;
    if (k.custom) {
        qlo = custom_lo(k, q);
        if (qlo < 0.f) return 0.f;
        if (k.nuser) return user_piece(k, qlo, q.hi);
    } else {
        if (q.seg < 0) return 0.f;
        if (q.seg > 0 && !k.generic) return seg_piece(k, q.seg - 1, q.ln_lo, q.dl);
    }
    // a bin across a segment boundary (or any bin with the breaks per model): its pieces in each segment
    float v = 0.f;
#pragma unroll
    for (int s = 0; s < 3; ++s) {
        const float lo = fmaxf(qlo, k.lo[s]), hi = fminf(q.hi, k.hi[s]);
        if (hi > lo) v += (s == 0 && k.logn) ? logn_piece(k, lo, hi) : seg_piece(k, s, logf(lo), logf(hi / lo));
    }
    return v;
}

constexpr double KR_LN2 = 0.6931471805599453;

// g2(x) = int_0^1 s e^(x s) ds = (e^x (x - 1) + 1) / x^2, with its Taylor series sum_k x^k / (k! (k + 2)) near 0
// (FP64 and FP32); g1(x) = (e^x - 1) / x
__device__ inline double kr_g1(double x) { return x == 0.0 ? 1.0 : expm1(x) / x; }
__device__ inline double kr_g2(double x) {
    if (fabs(x) < 0.25) {
        const double cf[11] = {1.0 / 2, 1.0 / 3, 1.0 / 8, 1.0 / 30, 1.0 / 144, 1.0 / 840, 1.0 / 5760, 1.0 / 45360,
                               1.0 / 403200, 1.0 / 3991680, 1.0 / 43545600};
        double r = cf[10];
        for (int k = 9; k >= 0; --k) r = fma(r, x, cf[k]);
        return r;
    }
    return (exp(x) * (x - 1.0) + 1.0) / (x * x);
}
__device__ __forceinline__ float ops_g1(float x) { return x == 0.f ? 1.f : ops_expm1(x) / x; }
__device__ __forceinline__ float ops_g2(float x) {
    if (fabsf(x) < 0.5f) {
        float r = 1.f / 403200.f;
        r = fmaf(r, x, 1.f / 45360.f);
        r = fmaf(r, x, 1.f / 5760.f);
        r = fmaf(r, x, 1.f / 840.f);
        r = fmaf(r, x, 1.f / 144.f);
        r = fmaf(r, x, 1.f / 30.f);
        r = fmaf(r, x, 1.f / 8.f);
        r = fmaf(r, x, 1.f / 3.f);
        return fmaf(r, x, 0.5f);
    }
    return fmaf(ops_ex2(x * 1.4426950408889634f), x - 1.f, 1.f) / (x * x);
}

// One model's Kroupa segments (c = 1, c2, c2 with c2 = 0.5^(alpha2 - alpha1): continuous at 0.5 and 1 Msun; the
// FP32 constants of the bin weights) and 1 / (the IMF's mass between its limits: imf_integral, mass-weighted), in
// FP64. With dlnT non-null also d ln(mass) / d alpha_j, j = 1..3, for the reverse pass: a segment's piece
// P = c lo^em expm1(em dl) / em (em = 2 - alpha, dl = ln(hi / lo)) has dP/dem = c lo^em dl (ln lo g1 + dl g2)(em dl)
// and c2 the factor 2^(alpha1 - alpha2).
__device__ inline void kroupa_setup(const double *al3, double lim_lo, double lim_hi, KroupaSeg &k, float &inv_total,
                                    double *dlnT, double *total_out = nullptr) {
    const double a1 = al3[0], a2 = al3[1], a3 = al3[2];
    const double c2 = pow(0.5, -a1 + a2);
    const double al[3] = {a1, a2, a3}, cs[3] = {1.0, c2, c2};
    const double slo[3] = {0.08, 0.5, 1.0}, shi[3] = {0.5, 1.0, 1.0e30};
    double total = 0.0, t12 = 0.0, dp[3] = {0.0, 0.0, 0.0};
    for (int sg = 0; sg < 3; ++sg) {
        const double e = 1.0 - al[sg];
        k.e[sg] = (float)e;
        k.c[sg] = (float)cs[sg];
        k.ce[sg] = e != 0.0 ? (float)(cs[sg] / e) : 0.f;
        k.lo[sg] = (float)slo[sg];
        k.hi[sg] = (float)shi[sg];
        const double lo = fmax(lim_lo, slo[sg]), hi = fmin(lim_hi, shi[sg]);
        if (hi > lo) {
            const double em = 2.0 - al[sg];   // mass-weighted: int c m^(1 - alpha) dm
            const double piece = (em == 0.0) ? cs[sg] * log(hi / lo) : cs[sg] * pow(lo, em) * expm1(em * log(hi / lo)) / em;
            total += piece;
            if (dlnT) {
                if (sg > 0) t12 += piece;
                const double ll = log(lo), dl = log(hi / lo), x = em * dl;
                dp[sg] = cs[sg] * pow(lo, em) * dl * (ll * kr_g1(x) + dl * kr_g2(x));
            }
        }
    }
    inv_total = total > 0.0 ? (float)(1.0 / total) : 1.f;
    if (total_out) *total_out = total;
    k.generic = 0;
    k.logn = 0;
    k.la = k.u0 = k.zs = 0.f;
    k.lnb = -KR_LN2;
    k.d3 = 0.0;
    if (dlnT) {
        const double it = total > 0.0 ? 1.0 / total : 0.0;
        dlnT[0] = (-dp[0] + KR_LN2 * t12) * it;
        dlnT[1] = (-dp[1] - KR_LN2 * t12) * it;
        dlnT[2] = -dp[2] * it;
    }
}

// Dave 2008 (p = alpha1, alpha2, mdave): m^-alpha1 over [0.08, mdave], mdave^(alpha2 - alpha1) m^-alpha2 above
// (imf_integral case 4); 1 / T and, with dlnT, d ln T / d(alpha1, alpha2, mdave) (imf_integral_dp case 4: the
// moving break's edge terms cancel, the IMF being continuous there).
__device__ inline void dave_setup(const double *p, double lim_lo, double lim_hi, KroupaSeg &k, float &inv_total,
                                  double *dlnT, double *total_out = nullptr) {
    const double a1 = p[0], a2 = p[1], md = p[2];
    const double c2 = pow(md, -a1 + a2);
    const double al[2] = {a1, a2}, cs[2] = {1.0, c2}, slo[2] = {0.08, md}, shi[2] = {md, 1.0e30};
    double total = 0.0, t12 = 0.0, dp[2] = {0.0, 0.0};
    for (int sg = 0; sg < 2; ++sg) {
        const double e = 1.0 - al[sg];
        k.e[sg] = (float)e;
        k.c[sg] = (float)cs[sg];
        k.ce[sg] = e != 0.0 ? (float)(cs[sg] / e) : 0.f;
        k.lo[sg] = (float)slo[sg];
        k.hi[sg] = (float)shi[sg];
        const double lo = fmax(lim_lo, slo[sg]), hi = fmin(lim_hi, shi[sg]);
        if (hi > lo) {
            const double em = 2.0 - al[sg];
            const double piece = (em == 0.0) ? cs[sg] * log(hi / lo) : cs[sg] * pow(lo, em) * expm1(em * log(hi / lo)) / em;
            total += piece;
            if (sg == 1) t12 = piece;
            const double ll = log(lo), dl = log(hi / lo), x = em * dl;
            dp[sg] = cs[sg] * pow(lo, em) * dl * (ll * kr_g1(x) + dl * kr_g2(x));
        }
    }
    k.e[2] = k.c[2] = k.ce[2] = 0.f;
    k.lo[2] = k.hi[2] = 1.0e30f;
    inv_total = total > 0.0 ? (float)(1.0 / total) : 1.f;
    if (total_out) *total_out = total;
    k.generic = 1;
    k.logn = 0;
    k.la = k.u0 = k.zs = 0.f;
    k.lnb = log(md);
    k.d3 = (a2 - a1) / md;
    if (dlnT) {
        const double it = total > 0.0 ? 1.0 / total : 0.0;
        dlnT[0] = (-dp[0] - k.lnb * t12) * it;
        dlnT[1] = (-dp[1] + k.lnb * t12) * it;
        dlnT[2] = k.d3 * t12 * it;
    }
}

// A lognormal A exp(-(log10 m - u0)^2 / (2 0.69^2)) per unit ln m up to the break br, c_hi m^-2.3 above: van Dokkum
// 2008 (imf_integral case 3; A = 0.14 (12.5 vdmc)^-1.3, u0 = log10 vdmc, br = 25 vdmc, c_hi = 0.0443, constants
// src/physics/opensps_imf.f90:39-44) and Chabrier 2003 (case 1: A = 1, u0 = log10 0.08, br = 1 M_sun,
// c_hi = exp(-u0^2 / (2 0.69^2))). 1 / T with the lognormal's mass in closed form (its centre shifted by
// ln 10 sigma^2). No parameters in the reverse pass (imf_integral_dp has none for either): dlnT zero.
__device__ inline void logn_setup(double A, double u0, double br, double c_hi, double lim_lo, double lim_hi,
                                  KroupaSeg &k, float &inv_total, double *dlnT, double *total_out = nullptr) {
    const double s2 = 0.69 * 0.69, sig = 0.69, K = 2.302585092994046;
    double total = 0.0;
    // the lognormal's mass over [lim_lo, min(lim_hi, br)]: A e^(K u0 + K^2 sigma^2 / 2) K sigma sqrt(pi / 2)
    // (erf(z2) - erf(z1)), z about the shifted centre
    double lo = lim_lo, hi = fmin(lim_hi, br);
    if (hi > lo) {
        const double cen = u0 + K * s2, sc = exp(K * u0 + 0.5 * K * K * s2) * K * sig * sqrt(0.5 * 3.141592653589793);
        const double z1 = (log10(lo) - cen) / (sig * 1.4142135623730951), z2 = (log10(hi) - cen) / (sig * 1.4142135623730951);
        const double d = z1 >= 0.0 ? erfc(z1) - erfc(z2) : (z2 <= 0.0 ? erfc(-z2) - erfc(-z1) : erf(z2) - erf(z1));
        total += A * sc * d;
    }
    lo = fmax(lim_lo, br);
    hi = lim_hi;
    if (hi > lo) total += c_hi * pow(lo, -0.3) * expm1(-0.3 * log(hi / lo)) / -0.3;
    k.e[0] = k.c[0] = k.ce[0] = 0.f;
    k.lo[0] = 0.f;
    k.hi[0] = (float)br;
    k.e[1] = -1.3f;
    k.c[1] = (float)c_hi;
    k.ce[1] = (float)(c_hi / -1.3);
    k.lo[1] = (float)br;
    k.hi[1] = 1.0e30f;
    k.e[2] = k.c[2] = k.ce[2] = 0.f;
    k.lo[2] = k.hi[2] = 1.0e30f;
    inv_total = total > 0.0 ? (float)(1.0 / total) : 1.f;
    if (total_out) *total_out = total;
    k.generic = 1;
    k.logn = 1;
    k.la = (float)(A * K * sig * 1.4142135623730951);
    k.u0 = (float)u0;
    k.zs = (float)(1.0 / (sig * 1.4142135623730951));
    k.lnb = 0.0;
    k.d3 = 0.0;
    if (dlnT) dlnT[0] = dlnT[1] = dlnT[2] = 0.0;
}

// The model's IMF by type (0 Salpeter and 2 Kroupa through the Kroupa form, 1 Chabrier, 3 van Dokkum, 4 Dave, 5 the
// user's segments with 1 / T from the host), then the limits and the user table of L.
__device__ inline void imf_setup(int imf_type, const double *p, const OpsImfLim &L, KroupaSeg &k, float &inv_total,
                                 double *dlnT) {
    if (imf_type == 3) {
        const double vdmc = p[0];
        logn_setup(0.14 * pow(12.5 * vdmc, -1.3), log10(vdmc), 25.0 * vdmc, 0.0443, L.lim_lo, L.lim_hi, k, inv_total,
                   dlnT);
    } else if (imf_type == 1) {
        const double u0 = -1.0969100130080565;   // log10 0.08
        logn_setup(1.0, u0, 1.0, exp(-u0 * u0 / (2.0 * 0.69 * 0.69)), L.lim_lo, L.lim_hi, k, inv_total, dlnT);
    } else if (imf_type == 4) {
        dave_setup(p, L.lim_lo, L.lim_hi, k, inv_total, dlnT);
    } else if (imf_type == 5) {
        for (int s = 0; s < 3; ++s) {
            k.e[s] = k.c[s] = k.ce[s] = 0.f;
            k.lo[s] = k.hi[s] = 1.0e30f;
        }
        k.generic = 1;
        k.logn = 0;
        k.la = k.u0 = k.zs = 0.f;
        k.lnb = k.d3 = 0.0;
        inv_total = (float)L.user_inv_total;
        if (dlnT) dlnT[0] = dlnT[1] = dlnT[2] = 0.0;
    } else {
        kroupa_setup(p, L.lim_lo, L.lim_hi, k, inv_total, dlnT);
        if (imf_type == 0) {
            // Salpeter (imf_integral case 0): m^-2.35 with no cut at 0.08 M_sun (the Kroupa form's equal segments,
            // the first opened down to 0); its mass between the limits in closed form
            k.lo[0] = 0.f;
            const double total = (pow(L.lim_hi, -0.35) - pow(L.lim_lo, -0.35)) / -0.35;
            inv_total = L.lim_hi > L.lim_lo ? (float)(1.0 / total) : 1.f;
        }
    }
    k.custom = L.custom;
    k.glo = (float)L.lim_lo;
    k.ghi = (float)L.lim_hi;
    k.lb = L.lb;
    k.user = L.user;
    k.nuser = imf_type == 5 ? L.nuser : 0;
    if (L.custom) k.generic = 1;
}

// A point's IMF bin weight (before the normalisation) and its derivatives: phi = sum of its segments' pieces
// P_s = c_s lo^e dl g1(e dl), D_s = dP_s / de_s = c_s lo^e dl (ln lo g1 + dl g2), and p12 the pieces in segments 2
// and 3 (those scaled by c2). Then dphi/dalpha1 = -D_1 + ln 2 p12, dphi/dalpha2 = -D_2 - ln 2 p12,
// dphi/dalpha3 = -D_3.
struct ImfTan {
    float phi, d0, d1, d2, p12;
};
__device__ __forceinline__ void seg_piece_tan(const KroupaSeg &k, int s, float ln_lo, float dl, float &P, float &D) {
    const float x = k.e[s] * dl;
    const float b = k.c[s] * ops_ex2(k.e[s] * ln_lo * 1.4426950408889634f) * dl;
    const float g1 = ops_g1(x);
    P = b * g1;
    D = b * fmaf(ln_lo, g1, dl * ops_g2(x));
}
__device__ __forceinline__ ImfTan imf_weight_tan(const KroupaSeg &k, const OpsPoint &q) {
    ImfTan r = {0.f, 0.f, 0.f, 0.f, 0.f};
    float qlo = q.lo;
    if (k.custom) {
        qlo = custom_lo(k, q);
        if (qlo < 0.f) return r;
        if (k.nuser) {   // (the user IMF: no parameter of the reverse pass)
            r.phi = user_piece(k, qlo, q.hi);
            return r;
        }
    } else if (q.seg < 0) {
        return r;
    }
    float P, D;
    if (q.seg > 0 && !k.generic) {
        const int s = q.seg - 1;
        seg_piece_tan(k, s, q.ln_lo, q.dl, P, D);
        r.phi = P;
        r.d0 = s == 0 ? D : 0.f;
        r.d1 = s == 1 ? D : 0.f;
        r.d2 = s == 2 ? D : 0.f;
        r.p12 = s > 0 ? P : 0.f;
        return r;
    }
#pragma unroll
    for (int s = 0; s < 3; ++s) {
        const float lo = fmaxf(qlo, k.lo[s]), hi = fminf(q.hi, k.hi[s]);
        if (hi > lo) {
            if (s == 0 && k.logn) {   // (van Dokkum's and Chabrier's lognormal: no parameter of the reverse pass)
                P = logn_piece(k, lo, hi);
                D = 0.f;
            } else {
                seg_piece_tan(k, s, logf(lo), logf(hi / lo), P, D);
            }
            r.phi += P;
            if (s == 0) r.d0 += D;
            else if (s == 1) r.d1 += D;
            else r.d2 += D;
            if (s > 0) r.p12 += P;
        }
    }
    return r;
}

// OPS_K models per CTA: every point record and entry is read once for all of them. A CTA takes one metallicity slab
// (blockIdx.y) of its OPS_K models; the slabs' template weights are summed after (ops_reduce_kernel), in slab order.
constexpr int OPS_K = 4;
constexpr int OPS_PT_PER = 6;     // point records per thread and grid point (npt <= OPS_THREADS x OPS_PT_PER)
constexpr int OPS_ENT_PER = 24;   // entries per thread and grid point (nent <= OPS_THREADS x OPS_ENT_PER)

constexpr int OPS_MAXT = 128;     // ages per slab (nt <= OPS_MAXT)
constexpr int OPS_NBUF = 3;       // IMF-weight buffers (phase A of i + 1 beside phase B of i)

__global__ void __launch_bounds__(OPS_THREADS, 2) ops_fold_kernel(OpsFoldArgs a) {
    extern __shared__ float4 osm4[];
    // OPS_NBUF x npt: the IMF weights of a grid point, one per model. Phase B of grid point i runs beside phase A of
    // i + 1 (no barrier between them), and the barrier after phase A of i + 1 orders phase B of i before phase A of
    // i + 2: three buffers keep the three apart.
    float4 *W4 = osm4;
    float *V = reinterpret_cast<float *>(osm4 + OPS_NBUF * a.npt);   // OPS_K x ntpad: per model, the current part
    __shared__ KroupaSeg kseg[OPS_K];
    __shared__ float inv_total[OPS_K];
    __shared__ float sw_s[OPS_MAXT][OPS_K];           // the models' SFH weights at the slab's ages
    __shared__ int tlist[OPS_MAXT];                   // the ages any model weighs
    __shared__ int n_active;
    __shared__ float gsum[OPS_NBUF][OPS_THREADS / 32][OPS_K][2];   // per warp: sum of w mcur, w L of its points
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int grp = blockIdx.x, z = blockIdx.y;
    const int m0 = grp * OPS_K;
    const int nk = min(OPS_K, a.n - m0);
    const int ngroups = (a.n + OPS_K - 1) / OPS_K;
    const int ng = a.nt * a.nz;
    for (int i = tid; i < OPS_K * a.ntpad; i += OPS_THREADS) V[i] = 0.f;
    for (int i = tid; i < a.nt * OPS_K; i += OPS_THREADS) {
        const int t = i / OPS_K, k = i % OPS_K;
        const double sw = k < nk ? a.wz[(size_t)ng * (m0 + k) + t + (size_t)a.nt * z] : 0.0;
        sw_s[t][k] = (sw > SAFE_FLOOR) ? (float)sw : 0.f;
    }
    if (tid < OPS_K)
        imf_setup(a.imf_type, a.alpha + 3 * min(m0 + tid, a.n - 1), a.lim, kseg[tid], inv_total[tid], nullptr);
    __syncthreads();
    if (tid == 0) {
        int na = 0;
        for (int t = 0; t < a.nt; ++t) {
            bool any = false;
            for (int k = 0; k < OPS_K; ++k) any = any || sw_s[t][k] != 0.f;
            if (any) tlist[na++] = t;
        }
        n_active = na;
    }
    __syncthreads();
    const int na = n_active;
    // threads 0 .. 15: one FP64 accumulator each: (model k, mass / L_bol, young / old)
    double acc = 0.0;
    const int ak = tid >> 2, aq = (tid >> 1) & 1, ap = tid & 1;
    float run[OPS_K];
    // the template vectors hold one part at a time (the ages ascend: young, then old); flushed to this slab's rows
    auto flush = [&](int part) {
        for (int i = tid; i < nk * a.ntpad; i += OPS_THREADS) {
            const int k = i / a.ntpad, e = i % a.ntpad;
            a.vpart[((size_t)z * 2 * a.n + (part == 0 ? m0 + k : a.n + m0 + k)) * a.ntpad + e] = V[i];
            V[i] = 0.f;
        }
    };
    int vpart_of = -1;          // the part V holds (-1: none yet)
    bool flushed[2] = {false, false};
    for (int it = 0; it <= na; ++it) {
        const int buf = it % OPS_NBUF;
        // ---- phase A of grid point it (IMF weights into W4[buf], per-warp mass / L_bol partials into gsum[buf])
        if (it < na) {
            const int t = tlist[it];
            const OpsPoint *pts = a.pts + ((size_t)t + (size_t)a.nt * z) * a.npt;
            float4 *Wb = W4 + buf * a.npt;
            float ma[OPS_K] = {0.f, 0.f, 0.f, 0.f}, la[OPS_K] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 2
            for (int u = 0; u < OPS_PT_PER; ++u) {
                const int p = tid + u * OPS_THREADS;
                if (p >= a.npt) break;
                const OpsPoint q = pts[p];
                float w[OPS_K];
#pragma unroll
                for (int k = 0; k < OPS_K; ++k) {
                    w[k] = imf_weight(kseg[k], q) * inv_total[k];
                    ma[k] = fmaf(w[k], q.mcur, ma[k]);
                    la[k] = fmaf(w[k], q.lum, la[k]);
                }
                Wb[p] = make_float4(w[0], w[1], w[2], w[3]);
            }
#pragma unroll
            for (int k = 0; k < OPS_K; ++k) {
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    ma[k] += __shfl_xor_sync(0xffffffffu, ma[k], off);
                    la[k] += __shfl_xor_sync(0xffffffffu, la[k], off);
                }
            }
            if (lane == 0) {
#pragma unroll
                for (int k = 0; k < OPS_K; ++k) { gsum[buf][warp][k][0] = ma[k]; gsum[buf][warp][k][1] = la[k]; }
            }
        }
        __syncthreads();   // W4[buf] and gsum[buf] of it complete; every thread done with phase B of it - 2
        if (it == 0) continue;
        // ---- phase B of grid point it - 1 (reads W4[(it - 1) % OPS_NBUF], written before the previous barrier)
        const int ip = it - 1, pb = (it - 1) % OPS_NBUF;
        const int t = tlist[ip];
        const int part = t < a.itesc ? 0 : 1;
        if (part != vpart_of) {
            if (vpart_of >= 0) {
                __syncthreads();            // (the previous part's adds are complete; part is the same for all)
                flush(vpart_of);
                flushed[vpart_of] = true;
                __syncthreads();
            }
            vpart_of = part;
        }
        const float sw[OPS_K] = {sw_s[t][0], sw_s[t][1], sw_s[t][2], sw_s[t][3]};
        if (tid < 16 && ap == part) {
            float s = 0.f;
#pragma unroll
            for (int w = 0; w < OPS_THREADS / 32; ++w) s += gsum[pb][w][ak][aq];
            acc += (double)sw[ak] * (double)s;
        }
        const size_t g = (size_t)t + (size_t)a.nt * z;
        const float4 *Wb = W4 + pb * a.npt;
        const int e0 = tid * OPS_ENT_PER;
        const uint32_t *en = a.ent + g * a.nent;
        const float *ec = a.ent_c + g * a.nent;
        uint32_t key[OPS_ENT_PER];
        float cf[OPS_ENT_PER];
        if (e0 + OPS_ENT_PER <= a.nent) {
#pragma unroll
            for (int u = 0; u < OPS_ENT_PER / 4; ++u) {
                const uint4 kk = __ldg(reinterpret_cast<const uint4 *>(en + e0) + u);
                const float4 cc = __ldg(reinterpret_cast<const float4 *>(ec + e0) + u);
                key[4 * u] = kk.x; key[4 * u + 1] = kk.y; key[4 * u + 2] = kk.z; key[4 * u + 3] = kk.w;
                cf[4 * u] = cc.x; cf[4 * u + 1] = cc.y; cf[4 * u + 2] = cc.z; cf[4 * u + 3] = cc.w;
            }
        } else {
#pragma unroll
            for (int u = 0; u < OPS_ENT_PER; ++u) {
                const bool in = e0 + u < a.nent;
                key[u] = in ? __ldg(en + e0 + u) : 0xffffffffu;
                cf[u] = in ? __ldg(ec + e0 + u) : 0.f;
            }
        }
        float *Vp = V;
        int cur = -1;
#pragma unroll
        for (int k = 0; k < OPS_K; ++k) run[k] = 0.f;
#pragma unroll
        for (int u = 0; u < OPS_ENT_PER; ++u) {
            if (key[u] == 0xffffffffu) continue;
            const int te = (int)(key[u] >> 16);
            const float4 w4 = Wb[key[u] & 0xffffu];
            if (te != cur) {
                if (cur >= 0) {
#pragma unroll
                    for (int k = 0; k < OPS_K; ++k)
                        if (run[k] != 0.f) atomicAdd(Vp + (size_t)k * a.ntpad + cur, run[k] * sw[k]);
                }
                cur = te;
                run[0] = w4.x * cf[u]; run[1] = w4.y * cf[u]; run[2] = w4.z * cf[u]; run[3] = w4.w * cf[u];
            } else {
                run[0] = fmaf(w4.x, cf[u], run[0]); run[1] = fmaf(w4.y, cf[u], run[1]);
                run[2] = fmaf(w4.z, cf[u], run[2]); run[3] = fmaf(w4.w, cf[u], run[3]);
            }
        }
        if (cur >= 0) {
#pragma unroll
            for (int k = 0; k < OPS_K; ++k)
                if (run[k] != 0.f) atomicAdd(Vp + (size_t)k * a.ntpad + cur, run[k] * sw[k]);
        }
    }
    __syncthreads();
    // this slab's template weights (each part once: the one held, the other zero if it had no age) and sums, read
    // back in slab order by ops_reduce_kernel
    if (tid == 0) a.flag[(size_t)z * ngroups + grp] = na > 0 ? 1 : 0;
    if (na == 0) return;
    flush(vpart_of);
    flushed[vpart_of] = true;
    for (int part = 0; part < 2; ++part)
        if (!flushed[part]) flush(part);   // (V is zero after the flush above)
    // spart (model, 4): mass young, mass old, L_bol young, L_bol old  <-  accumulator (k, quantity aq, part ap)
    if (tid < 16 && ak < nk) a.spart[((size_t)z * a.n + m0 + ak) * 4 + 2 * aq + ap] = acc;
}

// The slabs' template weights summed in slab order, as the template GEMM's bf16 hi / lo A operand, and the sums.
__global__ void ops_reduce_kernel(OpsFoldArgs a) {
    const int ngroups = (a.n + OPS_K - 1) / OPS_K;
    const size_t total = (size_t)2 * a.n * a.ntpad;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int row = (int)(i / a.ntpad);
        const int m = row < a.n ? row : row - a.n;
        const int grp = m / OPS_K;
        float v = 0.f;
        for (int z = 0; z < a.nz; ++z)
            if (a.flag[(size_t)z * ngroups + grp]) v += a.vpart[(size_t)z * total + i];
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        a.v_hi[i] = h;
        a.v_lo[i] = __float2bfloat16_rn(v - __bfloat162float(h));
        if (i < (size_t)a.n) {
            const int mm = (int)i, gg = mm / OPS_K;
            double s[4] = {0.0, 0.0, 0.0, 0.0};
            for (int z = 0; z < a.nz; ++z)
                if (a.flag[(size_t)z * ngroups + gg])
                    for (int j = 0; j < 4; ++j) s[j] += a.spart[((size_t)z * a.n + mm) * 4 + j];
            double *o = a.sums + (size_t)6 * mm;
            o[0] = s[0] + s[1];
            o[1] = s[2] + s[3];
            o[2] = s[0]; o[3] = s[1]; o[4] = s[2]; o[5] = s[3];
        }
    }
}

cudaError_t run_ops_fold(const OpsFoldArgs &a, cudaStream_t st) {
    if (a.n <= 0) return cudaSuccess;
    if (a.npt > OPS_THREADS * OPS_PT_PER || a.nent > OPS_THREADS * OPS_ENT_PER) return cudaErrorInvalidValue;
    if (a.nt > OPS_MAXT) return cudaErrorInvalidValue;
    const size_t smem = sizeof(float4) * OPS_NBUF * (size_t)a.npt + sizeof(float) * (size_t)OPS_K * a.ntpad;
    cudaError_t e = cudaFuncSetAttribute(ops_fold_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const dim3 grid((a.n + OPS_K - 1) / OPS_K, a.nz);
    ops_fold_kernel<<<grid, OPS_THREADS, smem, st>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    ops_reduce_kernel<<<1024, 256, 0, st>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------- the interpolated fold
// The fold as a GEMM. In x = ln m a bin piece's weight in Kroupa segment s is int e^((1 - alpha_s) x) dx; e^(-alpha_s x)
// interpolated by a degree-9 Lagrange polynomial on equispaced nodes x_j of the segment (the piece in the middle
// interval of its ten nodes) turns it into sum_j L_pj mu_j^-alpha_s, L_pj = int L_j(x) e^x dx over the piece. So
//     V(e, m) = sum_{g, s, j} [sw(g, m) c_s(m) / T(m) mu_j^-alpha_s(m)] B(e, (g, s, j)),
//     B(e, (g, s, j)) = sum over the points p of g and their entries of template e: coef L_pj,
// the bracket (the operand X, one row per model, all entries >= 0) formed per batch and B (the operator basis) once
// per operator: a split-BF16 tcgen05 GEMM over K = (grid point, node), young ages and old apart as two column ranges.
// With the node spacing h_s = 0.44 / |alpha|max_s the interpolation's relative error per bin is below 2e-7 for
// |alpha_1| <= 2.6, |alpha_2| <= 3.0, |alpha_3| <= 3.5; a batch with a slope outside takes the exact fold. The mass
// and L_bol rows go through the same expansion (rows of B over mcur and lum), summed per model in FP64.
constexpr int OPS_IDEG = 9;                          // Lagrange degree (ten nodes per piece)
constexpr double OPS_IH = 0.44;                      // node spacing x the largest |alpha| of the segment
constexpr double OPS_AMAX[3] = {2.6, 3.0, 3.5};      // |alpha_s| of the interpolated fold
constexpr int OPS_IX_THREADS = 256;
constexpr int OPS_IMAXR = 256;                       // nodes per grid point (R <= OPS_IMAXR)

// One model per CTA: its node values c_s / T mu_j^-alpha_s and its SFH weights (as the fold takes them: FP32, zero
// at or below SAFE_FLOOR) in shared memory, then the row of X (bf16 hi / lo) over every grid point, eight columns
// (one grid point) per thread step, and the model's FP64 mass and L_bol sums, young and old. Column group q of grid
// point gp = q / (R / 8) (by a multiply-high with rg_magic = 2^32 / (R / 8) rounded up; exact for q < 2^20).
constexpr int OPS_IMAXG = 4096;                      // grid points (nt nz <= OPS_IMAXG)

// One thread per model: 1 / T (the IMF's mass between its limits, FP64) and c2 = 0.5^(alpha2 - alpha1), for
// ops_interp_x_kernel (formed there by one thread per CTA, the FP64 work ran as one-lane warps).
__global__ void ops_interp_const_kernel(const double *alpha, int n, float lim_lo, float lim_hi, double fixed_inv_total,
                                        double2 *out) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    if (fixed_inv_total > 0.0) {   // an IMF without per-model parameters (Chabrier): its 1 / T, formed on the host
        out[m] = make_double2(fixed_inv_total, 0.0);
        return;
    }
    KroupaSeg ks;
    float itf;
    double total;
    const double *al = alpha + 3 * (size_t)m;
    kroupa_setup(al, lim_lo, lim_hi, ks, itf, nullptr, &total);
    out[m] = make_double2(total > 0.0 ? 1.0 / total : 1.0, pow(0.5, -al[0] + al[1]));
}
// A node's value for the fold: the IMF per unit mass at mu = e^x of segment q, over T (it = 1 / T). Kroupa (and
// Salpeter as Kroupa with equal slopes): c_q mu^-alpha_q (c = 1, c2, c2). Chabrier 2003 (imf_integral case 1,
// src/physics/opensps_imf.f90:234-242): the lognormal exp(-(log10 mu - log10 0.08)^2 / (2 0.69^2)) / mu in segments 0
// and 1 (below 1 M_sun, extended past it at the segment's outer nodes), exp(-(log10 0.08)^2 / (2 0.69^2)) mu^-2.3 in
// segment 2 (continuous at 1 M_sun).
__device__ __forceinline__ double ops_node_value(int imf_type, int q, double x, const double *al, double it, double c2) {
    if (imf_type == 1) {
        const double l0 = -1.0969100130080565, inv2s2 = 1.0 / (2.0 * 0.69 * 0.69);   // log10 0.08
        if (q < 2) {
            const double u = x * 0.43429448190325176 - l0;                          // log10 mu - log10 0.08
            return it * exp(-u * u * inv2s2 - x);
        }
        return it * exp(-l0 * l0 * inv2s2 - 2.3 * x);
    }
    return (q == 0 ? 1.0 : c2) * it * exp(-al[q] * x);
}

__global__ void __launch_bounds__(OPS_IX_THREADS) ops_interp_x_kernel(OpsInterpArgs a) {
    __shared__ __align__(16) float ctk[OPS_IMAXR];
    __shared__ float sws[OPS_IMAXG];
    __shared__ double red[OPS_IX_THREADS / 32][4];
    const int row = blockIdx.x, m = a.m0 + row, tid = threadIdx.x;
    const int ng = a.nt * a.nz;
    const double *al = a.alpha + 3 * (size_t)m;
    const double *wzm = a.wz + (size_t)ng * m;
    for (int g = tid; g < ng; g += OPS_IX_THREADS) {
        const int t = g % a.nt, z = g / a.nt;                 // the weights' order: age fastest
        const double sw = wzm[g];
        sws[t * a.nz + z] = sw > SAFE_FLOOR ? (float)sw : 0.f;   // the columns' order: (t nz + z)
    }
    const double2 kc = a.kconst[m];                  // 1 / T, c2
    const double it = kc.x, c2 = kc.y;
    for (int r = tid; r < a.R; r += OPS_IX_THREADS) {
        float v = 0.f;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const int j = r - a.noff[q];
            if (j >= 0 && j < a.nn[q]) {
                const double x = a.x0[q] + (double)(j - OPS_IDEG / 2) * a.h[q];
                v = (float)ops_node_value(a.imf_type, q, x, al, it, c2);
            }
        }
        ctk[r] = v;
    }
    __syncthreads();
    const int rg = a.R >> 3, ngrp = ng * rg, gyoung = a.itesc * a.nz;
    uint4 *xh = reinterpret_cast<uint4 *>(a.x_hi + (size_t)row * a.ktot);
    uint4 *xl = reinterpret_cast<uint4 *>(a.x_lo + (size_t)row * a.ktot);
    const float4 *mr4 = reinterpret_cast<const float4 *>(a.mrow), *lr4 = reinterpret_cast<const float4 *>(a.lrow);
    const float4 *ct4 = reinterpret_cast<const float4 *>(ctk);
    // mass young, mass old, L_bol young, L_bol old: FP32 over up to 16 thread steps, then FP64 (GB300's FP64 pipe
    // is narrow: one FP64 add per step was a third of the kernel)
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    float fac[4] = {0.f, 0.f, 0.f, 0.f};
    int nstep = 0;
    for (int q = tid; q < ngrp; q += OPS_IX_THREADS) {
        const int gp = (int)__umulhi((unsigned)q, a.rg_magic);
        const int rq = q - gp * rg;
        const float sw = sws[gp];
        const float4 c0 = ct4[2 * rq], c1 = ct4[2 * rq + 1];
        const float4 ma = __ldg(mr4 + 2 * (size_t)q), mb = __ldg(mr4 + 2 * (size_t)q + 1);
        const float4 la = __ldg(lr4 + 2 * (size_t)q), lb = __ldg(lr4 + 2 * (size_t)q + 1);
        const float v[8] = {sw * c0.x, sw * c0.y, sw * c0.z, sw * c0.w, sw * c1.x, sw * c1.y, sw * c1.z, sw * c1.w};
        const float mrv[8] = {ma.x, ma.y, ma.z, ma.w, mb.x, mb.y, mb.z, mb.w};
        const float lrv[8] = {la.x, la.y, la.z, la.w, lb.x, lb.y, lb.z, lb.w};
        uint32_t hw[4], lw[4];
        float ms = 0.f, ls = 0.f;
#pragma unroll
        for (int i = 0; i < 8; i += 2) {
            const __nv_bfloat162 h = __floats2bfloat162_rn(v[i], v[i + 1]);
            const float2 hf = __bfloat1622float2(h);
            const __nv_bfloat162 l = __floats2bfloat162_rn(v[i] - hf.x, v[i + 1] - hf.y);
            hw[i >> 1] = *reinterpret_cast<const uint32_t *>(&h);
            lw[i >> 1] = *reinterpret_cast<const uint32_t *>(&l);
            ms = fmaf(v[i], mrv[i], fmaf(v[i + 1], mrv[i + 1], ms));
            ls = fmaf(v[i], lrv[i], fmaf(v[i + 1], lrv[i + 1], ls));
        }
        xh[q] = make_uint4(hw[0], hw[1], hw[2], hw[3]);
        xl[q] = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        const int part = gp < gyoung ? 0 : 1;
        fac[part] += ms;
        fac[2 + part] += ls;
        if (++nstep == 16) {
#pragma unroll
            for (int i = 0; i < 4; ++i) { acc[i] += (double)fac[i]; fac[i] = 0.f; }
            nstep = 0;
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) acc[i] += (double)fac[i];
    const int warp = tid >> 5, lane = tid & 31;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], off);
        if (lane == 0) red[warp][i] = acc[i];
    }
    __syncthreads();
    if (tid == 0) {
        double s[4] = {0.0, 0.0, 0.0, 0.0};
        for (int w = 0; w < OPS_IX_THREADS / 32; ++w)
            for (int i = 0; i < 4; ++i) s[i] += red[w][i];
        double *o = a.sums + (size_t)6 * m;
        o[0] = s[0] + s[1];
        o[1] = s[2] + s[3];
        o[2] = s[0]; o[3] = s[1]; o[4] = s[2]; o[5] = s[3];
    }
}

// The split-K partial sums of the young and old GEMMs added in split order, as the template GEMM's bf16 hi / lo A
// operand (rows m0 .. m0 + rows - 1 young, n + m0 .. old; columns from ntempl on zero).
__global__ void ops_interp_reduce_kernel(OpsInterpReduceArgs a) {
    const size_t per4 = (size_t)a.rows * a.ntpad / 4;
    const float4 *py = reinterpret_cast<const float4 *>(a.part_young);
    const float4 *po = reinterpret_cast<const float4 *>(a.part_old);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < 2 * per4; i += (size_t)gridDim.x * blockDim.x) {
        const int part = i >= per4 ? 1 : 0;
        const size_t j = i - (size_t)part * per4;
        const int row = (int)(j * 4 / a.ntpad), e = (int)(j * 4 - (size_t)row * a.ntpad);
        const float4 *P = part ? po : py;
        const int ks = part ? a.ks_old : a.ks_young;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (e < a.ntempl)
            for (int s = 0; s < ks; ++s) {
                const float4 p = P[(size_t)s * per4 + j];
                v.x += p.x; v.y += p.y; v.z += p.z; v.w += p.w;
            }
        const float vv[4] = {v.x, v.y, v.z, v.w};
        const size_t o = ((size_t)(part ? a.n : 0) + a.m0 + row) * a.ntpad + e;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float x = e + k < a.ntempl ? vv[k] : 0.f;
            const __nv_bfloat16 h = __float2bfloat16_rn(x);
            a.v_hi[o + k] = h;
            a.v_lo[o + k] = __float2bfloat16_rn(x - __bfloat162float(h));
        }
    }
}

// ---------------------------------------------------------------------------------------------- the reverse fold
// The transpose of the fold for OPS_K models and one metallicity slab per CTA (the layout of ops_fold_kernel), after
// ssp_batch_age_sums_adjoint (src/physics/opensps_ssp_batch.f90:991) and the IMF rows of the batch gradient
// (params_bar(BGRAD_IMF1:, m) = imf_bar cscale, src/physics/opensps_csp_batch.f90:5115). With Vbar the template
// weights' cotangents (the pixel cotangents against the library, divided by cscale), each point p of grid point g
// has the cotangent of its IMF weight
//     q_p = sum over its four entries of coef Vbar(template) + mass_bar / cscale mcur_p
//           + lbol_bar / (ln 10 L_bol cscale) lum_p
// (L_bol with the operators is the linear row of the sums), and then
//     wz_bar(g)  = cscale sum_p w_p q_p                                   (w_p = phi_p / T: the bin weight)
//     alpha_bar_j = cscale sum_g sw(g) sum_p q_p dw_p / dalpha_j,  dw_p / dalpha_j = dphi_p/dalpha_j / T - w_p dlnT_j
// (forward-mode derivatives of the bin weights and of their normalisation T, the IMF's mass). Every grid point of
// the slab is visited when wz_bar is wanted, else only those with weight. Per grid point the threads take its
// points, gather the four models' Vbar of the point's templates from shared memory (one float4 per template), and
// keep per-warp sums of q w (wz_bar) and per-thread sums of sw q dphi (flushed to FP64 every 16 grid points).
__global__ void __launch_bounds__(OPS_THREADS, 2) ops_rev_kernel(OpsRevArgs a) {
    extern __shared__ float4 rsm4[];
    float4 *V4 = rsm4;                                 // ntpad: the four models' Vbar of the current part
    float4 *wpart = rsm4 + a.ntpad;                    // n_active x warps: per warp, sum of q phi
    __shared__ KroupaSeg kseg[OPS_K];
    __shared__ float inv_total[OPS_K], qm_s[OPS_K], ql_s[OPS_K];
    __shared__ double dlnT_s[OPS_K][3];
    __shared__ float sw_s[OPS_MAXT][OPS_K];
    __shared__ int tlist[OPS_MAXT];
    __shared__ int n_active;
    __shared__ double ured[OPS_THREADS / 32][OPS_K][4];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int grp = blockIdx.x, z = blockIdx.y;
    const int m0 = grp * OPS_K;
    const int nk = min(OPS_K, a.n - m0);
    const int ng = a.nt * a.nz;
    const bool all_points = a.wzb != nullptr;
    for (int i = tid; i < a.nt * OPS_K; i += OPS_THREADS) {
        const int t = i / OPS_K, k = i % OPS_K;
        const double sw = k < nk ? a.wz[(size_t)ng * (m0 + k) + t + (size_t)a.nt * z] : 0.0;
        sw_s[t][k] = (sw > SAFE_FLOOR) ? (float)sw : 0.f;
    }
    if (tid < OPS_K) {
        const int k = tid, m = min(m0 + k, a.n - 1);
        double dl[3];
        imf_setup(a.imf_type, a.alpha + 3 * m, a.lim, kseg[k], inv_total[k], dl);
        for (int j = 0; j < 3; ++j) dlnT_s[k][j] = dl[j];
        const double cs = a.cscale[m];
        const double ls = a.sums[(size_t)6 * m + 1];
        qm_s[k] = (k < nk && a.mass_bar) ? (float)(a.mass_bar[m] / cs) : 0.f;
        double qlv = (a.lbol_bar && ls > SAFE_FLOOR) ? a.lbol_bar[m] / (ls * 2.302585092994046) : 0.0;
        if (a.lsum_bar) qlv += a.lsum_bar[m];   // (the AGN's L_bol scale)
        ql_s[k] = k < nk ? (float)(qlv / cs) : 0.f;
    }
    __syncthreads();
    if (tid == 0) {
        int na = 0;
        for (int t = 0; t < a.nt; ++t) {
            bool any = all_points;
            for (int k = 0; k < OPS_K; ++k) any = any || sw_s[t][k] != 0.f;
            if (any) tlist[na++] = t;
        }
        n_active = na;
    }
    __syncthreads();
    const int na = n_active;
    double U[OPS_K][4];
    float G[OPS_K][4];
#pragma unroll
    for (int k = 0; k < OPS_K; ++k)
#pragma unroll
        for (int i = 0; i < 4; ++i) { U[k][i] = 0.0; G[k][i] = 0.f; }
    int vpart_of = -1;
    for (int it = 0; it < na; ++it) {
        const int t = tlist[it];
        const int part = t < a.itesc ? 0 : 1;
        if (part != vpart_of) {
            __syncthreads();                   // every thread done with the previous part's V4 (uniform branch)
            for (int e = tid; e < a.ntpad; e += OPS_THREADS) {
                float v[OPS_K];
#pragma unroll
                for (int k = 0; k < OPS_K; ++k)
                    v[k] = k < nk ? a.vbar[((size_t)part * a.n + m0 + k) * a.ntpad + e] : 0.f;
                V4[e] = make_float4(v[0], v[1], v[2], v[3]);
            }
            __syncthreads();
            vpart_of = part;
        }
        const size_t g = (size_t)t + (size_t)a.nt * z;
        const OpsPoint *pts = a.pts + g * a.npt;
        const ushort4 *pix = a.pidx + g * a.npt;
        const float4 *pco = a.pcoef + g * a.npt;
        float sw[OPS_K], wzp[OPS_K];
#pragma unroll
        for (int k = 0; k < OPS_K; ++k) { sw[k] = sw_s[t][k]; wzp[k] = 0.f; }
#pragma unroll 2
        for (int u = 0; u < OPS_PT_PER; ++u) {
            const int p = tid + u * OPS_THREADS;
            if (p >= a.npt) break;
            const OpsPoint q = pts[p];
            const ushort4 id = __ldg(pix + p);
            const float4 cf = __ldg(pco + p);
            const float4 v0 = V4[id.x], v1 = V4[id.y], v2 = V4[id.z], v3 = V4[id.w];
            const float gq[OPS_K] = {
                fmaf(cf.x, v0.x, fmaf(cf.y, v1.x, fmaf(cf.z, v2.x, cf.w * v3.x))),
                fmaf(cf.x, v0.y, fmaf(cf.y, v1.y, fmaf(cf.z, v2.y, cf.w * v3.y))),
                fmaf(cf.x, v0.z, fmaf(cf.y, v1.z, fmaf(cf.z, v2.z, cf.w * v3.z))),
                fmaf(cf.x, v0.w, fmaf(cf.y, v1.w, fmaf(cf.z, v2.w, cf.w * v3.w)))};
#pragma unroll
            for (int k = 0; k < OPS_K; ++k) {
                const float qk = fmaf(qm_s[k], q.mcur, fmaf(ql_s[k], q.lum, gq[k]));
                const ImfTan r = imf_weight_tan(kseg[k], q);
                wzp[k] = fmaf(qk, r.phi, wzp[k]);
                const float qs = qk * sw[k];
                G[k][0] = fmaf(qs, r.d0, G[k][0]);
                G[k][1] = fmaf(qs, r.d1, G[k][1]);
                G[k][2] = fmaf(qs, r.d2, G[k][2]);
                G[k][3] = fmaf(qs, r.p12, G[k][3]);
            }
        }
#pragma unroll
        for (int k = 0; k < OPS_K; ++k)
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) wzp[k] += __shfl_xor_sync(0xffffffffu, wzp[k], off);
        if (lane == 0) wpart[(size_t)it * (OPS_THREADS / 32) + warp] = make_float4(wzp[0], wzp[1], wzp[2], wzp[3]);
        if ((it & 15) == 15 || it == na - 1) {
#pragma unroll
            for (int k = 0; k < OPS_K; ++k)
#pragma unroll
                for (int i = 0; i < 4; ++i) { U[k][i] += (double)G[k][i]; G[k][i] = 0.f; }
        }
    }
    // the threads' sums of sw q dphi, per warp, then per model
#pragma unroll
    for (int k = 0; k < OPS_K; ++k)
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            double v = U[k][i];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            if (lane == 0) ured[warp][k][i] = v;
        }
    __syncthreads();
    // warp k: model m0 + k's wz_bar over the slab's visited grid points, B = sum_g sw(g) wz_bar(g) / cscale, and the
    // slab's slope cotangents
    if (warp < nk) {
        const int k = warp, m = m0 + k;
        const double cs = a.cscale[m], it_k = (double)inv_total[k];
        double b = 0.0;
        for (int it = lane; it < na; it += 32) {
            const int t = tlist[it];
            double s = 0.0;
            for (int w = 0; w < OPS_THREADS / 32; ++w)
                s += (double)reinterpret_cast<const float *>(wpart + (size_t)it * (OPS_THREADS / 32) + w)[k];
            s *= it_k;
            if (a.wzb) a.wzb[(size_t)ng * m + t + (size_t)a.nt * z] = cs * s;
            b += (double)sw_s[t][k] * s;
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) b += __shfl_xor_sync(0xffffffffu, b, off);
        if (lane == 0) {
            double u[4] = {0.0, 0.0, 0.0, 0.0};
            for (int w = 0; w < OPS_THREADS / 32; ++w)
                for (int i = 0; i < 4; ++i) u[i] += ured[w][k][i];
            // d phi / d(alpha1, alpha2, third) = (-D_1 - ln b p12, -D_2 + ln b p12, -D_3 + d3 p12)
            const double lnb = kseg[k].lnb, d3 = kseg[k].d3;
            const double A[3] = {-u[0] - lnb * u[3], -u[1] + lnb * u[3], -u[2] + d3 * u[3]};
            for (int j = 0; j < 3; ++j)
                a.apart[((size_t)z * a.n + m) * 3 + j] = it_k * A[j] - dlnT_s[k][j] * b;
        }
    }
}

// The slabs' slope cotangents summed in slab order, times cscale, into the params_bar rows.
__global__ void ops_rev_finish_kernel(OpsRevArgs a) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= a.n || !a.params_bar) return;
    double s[3] = {0.0, 0.0, 0.0};
    for (int z = 0; z < a.nz; ++z)
        for (int j = 0; j < 3; ++j) s[j] += a.apart[((size_t)z * a.n + m) * 3 + j];
    // Kroupa: imf1-3; Dave: imf1, imf2 and mdave (row_imf1 + 4); the others (Salpeter as Kroupa with fixed equal
    // slopes, van Dokkum) have none: zero
    double *pb = a.params_bar + (size_t)a.rows * m + a.row_imf1;
    for (int j = 0; j < 5; ++j) pb[j] = 0.0;
    if (a.imf_type == 2)
        for (int j = 0; j < 3; ++j) pb[j] = a.cscale[m] * s[j];
    if (a.imf_type == 4) {
        pb[0] = a.cscale[m] * s[0];
        pb[1] = a.cscale[m] * s[1];
        pb[4] = a.cscale[m] * s[2];
    }
}

cudaError_t run_ops_reverse(const OpsRevArgs &a, cudaStream_t st) {
    if (a.n <= 0) return cudaSuccess;
    if (a.npt > OPS_THREADS * OPS_PT_PER || a.nt > OPS_MAXT || a.ntpad > 65536) return cudaErrorInvalidValue;
    const size_t smem = sizeof(float4) * ((size_t)a.ntpad + (size_t)a.nt * (OPS_THREADS / 32));
    cudaError_t e = cudaFuncSetAttribute(ops_rev_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const dim3 grid((a.n + OPS_K - 1) / OPS_K, a.nz);
    ops_rev_kernel<<<grid, OPS_THREADS, smem, st>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    ops_rev_finish_kernel<<<(a.n + 255) / 256, 256, 0, st>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------- interpolated reverse
// The reverse of the interpolated fold. The forward is V = X B^T with X(m, (g, r)) = sw(g, m) ct_m(r), ct_m(r) =
// c_s / T mu_r^-alpha_s (node r in Kroupa segment s), and the mass and L_bol rows m = X mrow, L = X lrow. With Vbar
// the template weights' cotangents (divided by cscale), the operand's cotangent is Xbar = Vbar B (a split-BF16
// tcgen05 GEMM against the transposed basis, young grid points against the young Vbar and the rest against the old)
// plus mass_bar / cscale mrow + lbol_bar / (ln 10 L_bol cscale) lrow. Then per model
//     wz_bar(g)   = cscale sum_r Xbar(g, r) ct(r)
//     alpha_bar_j = cscale sum_r Y(r) ct(r) d ln ct(r) / d alpha_j,   Y(r) = sum_g sw(g) Xbar(g, r),
//     d ln ct(r) / d alpha_j = -ln mu_r [s = j] + d ln c_s / d alpha_j - d ln T / d alpha_j
// (c_2 = c_3 = 2^(alpha1 - alpha2); T the IMF's mass between its limits), the transposes of the same expansion the
// forward's interpolated fold takes (its interpolation error carries over to the cotangents).
struct OpsInterpRevArgs {
    int m0, nt, nz, R;
    int imf_type;
    size_t ktot;
    int noff[3], nn[3];
    double x0[3], h[3];
    float lim_lo, lim_hi;
    const double *wz, *alpha, *cscale, *mass_bar, *lbol_bar, *lsum_bar, *sums;
    const double2 *kconst;                   // n: 1 / T and c2 (the forward's)
    const float *xbar;                       // rows x ktot: Vbar B of the chunk
    const float *mrow, *lrow;
    double *wzb;                             // n x nt x nz, or null
    double *params_bar;                      // n x rows, or null
    int rows, row_imf1;
};
constexpr int OPS_IR_THREADS = 256, OPS_IR_WARPS = OPS_IR_THREADS / 32, OPS_IR_RI = OPS_IMAXR / 32;

// One model per CTA: the node values and their log-derivatives in shared memory; warp w takes grid points w, w + 8,
// ..., lane l the nodes l + 32 i of each (the row of Xbar read once, coalesced): wz_bar(g) by a warp sum, Y(r) in
// FP32 per lane over 64 grid points at a time (GB300's FP64 pipe is narrow), then FP64; the slopes' sums over the
// nodes by a block reduction.
__global__ void __launch_bounds__(OPS_IR_THREADS) ops_interp_rev_kernel(OpsInterpRevArgs a) {
    __shared__ float ct[OPS_IMAXR];
    __shared__ float dlc[3][OPS_IMAXR];
    __shared__ float sws[OPS_IMAXG];
    __shared__ double ypart[OPS_IR_WARPS][OPS_IMAXR];
    __shared__ double red[OPS_IR_WARPS][3];
    __shared__ double dlnT_s[3];
    __shared__ float qm_s, ql_s;
    const int row = blockIdx.x, m = a.m0 + row, tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ng = a.nt * a.nz;
    const double *al = a.alpha + 3 * (size_t)m;
    const double *wzm = a.wz + (size_t)ng * m;
    for (int g = tid; g < ng; g += OPS_IR_THREADS) {
        const int t = g % a.nt, z = g / a.nt;                 // the weights' order: age fastest
        const double sw = wzm[g];
        sws[t * a.nz + z] = sw > SAFE_FLOOR ? (float)sw : 0.f;   // the columns' order: (t nz + z)
    }
    const double cs = a.cscale[m];
    if (tid == 0) {
        KroupaSeg ks;
        float itf;
        double dl[3];
        kroupa_setup(al, a.lim_lo, a.lim_hi, ks, itf, dl);
        for (int j = 0; j < 3; ++j) dlnT_s[j] = dl[j];
        const double ls = a.sums[(size_t)6 * m + 1];
        qm_s = a.mass_bar ? (float)(a.mass_bar[m] / cs) : 0.f;
        double qlv = (a.lbol_bar && ls > SAFE_FLOOR) ? a.lbol_bar[m] / (ls * 2.302585092994046) : 0.0;
        if (a.lsum_bar) qlv += a.lsum_bar[m];   // (the AGN's L_bol scale)
        ql_s = (float)(qlv / cs);
    }
    __syncthreads();
    const double2 kc = a.kconst[m];                  // 1 / T, c2
    for (int r = tid; r < OPS_IMAXR; r += OPS_IR_THREADS) {
        float v = 0.f, d[3] = {0.f, 0.f, 0.f};
        if (r < a.R) {
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const int j = r - a.noff[q];
                if (j >= 0 && j < a.nn[q]) {
                    const double x = a.x0[q] + (double)(j - OPS_IDEG / 2) * a.h[q];
                    v = (float)ops_node_value(a.imf_type, q, x, al, kc.x, kc.y);
                    if (a.imf_type == 2) {   // (the slopes act with Kroupa only)
                        double g3[3] = {-dlnT_s[0], -dlnT_s[1], -dlnT_s[2]};
                        g3[q] -= x;
                        if (q > 0) { g3[0] += KR_LN2; g3[1] -= KR_LN2; }
                        d[0] = (float)g3[0]; d[1] = (float)g3[1]; d[2] = (float)g3[2];
                    }
                }
            }
        }
        ct[r] = v;
        dlc[0][r] = d[0]; dlc[1][r] = d[1]; dlc[2][r] = d[2];
    }
    __syncthreads();
    const float qm = qm_s, ql = ql_s;
    const float *xr = a.xbar + (size_t)row * a.ktot;
    float y[OPS_IR_RI];
    double yd[OPS_IR_RI];
#pragma unroll
    for (int i = 0; i < OPS_IR_RI; ++i) { y[i] = 0.f; yd[i] = 0.0; }
    int nstep = 0;
    for (int g = warp; g < ng; g += OPS_IR_WARPS) {
        const float sw = sws[g];
        const size_t base = (size_t)g * a.R;
        float ws = 0.f;
#pragma unroll
        for (int i = 0; i < OPS_IR_RI; ++i) {
            const int r = lane + 32 * i;
            if (r < a.R) {
                const float xt = fmaf(qm, __ldg(a.mrow + base + r), fmaf(ql, __ldg(a.lrow + base + r), __ldg(xr + base + r)));
                ws = fmaf(xt, ct[r], ws);
                y[i] = fmaf(sw, xt, y[i]);
            }
        }
        if (a.wzb) {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) ws += __shfl_xor_sync(0xffffffffu, ws, off);
            if (lane == 0) {
                const int t = g / a.nz, z = g - t * a.nz;
                a.wzb[(size_t)ng * m + t + (size_t)a.nt * z] = cs * (double)ws;
            }
        }
        if (++nstep == 64) {
#pragma unroll
            for (int i = 0; i < OPS_IR_RI; ++i) { yd[i] += (double)y[i]; y[i] = 0.f; }
            nstep = 0;
        }
    }
#pragma unroll
    for (int i = 0; i < OPS_IR_RI; ++i) {
        const int r = lane + 32 * i;
        ypart[warp][r] = yd[i] + (double)y[i];
    }
    __syncthreads();
    double s[3] = {0.0, 0.0, 0.0};
    for (int r = tid; r < a.R; r += OPS_IR_THREADS) {
        double yv = 0.0;
        for (int w = 0; w < OPS_IR_WARPS; ++w) yv += ypart[w][r];
        const double yc = yv * (double)ct[r];
#pragma unroll
        for (int j = 0; j < 3; ++j) s[j] += yc * (double)dlc[j][r];
    }
#pragma unroll
    for (int j = 0; j < 3; ++j) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s[j] += __shfl_xor_sync(0xffffffffu, s[j], off);
        if (lane == 0) red[warp][j] = s[j];
    }
    __syncthreads();
    if (tid < 3 && a.params_bar) {
        double v = 0.0;
        for (int w = 0; w < OPS_IR_WARPS; ++w) v += red[w][tid];
        a.params_bar[(size_t)a.rows * m + a.row_imf1 + tid] = cs * v;
    }
}

// FP32 -> bf16 hi / lo, element-wise (count a multiple of 2).
__global__ void split_bf16_kernel(const float *__restrict__ src, __nv_bfloat16 *__restrict__ hi,
                                  __nv_bfloat16 *__restrict__ lo, size_t count) {
    for (size_t i = 2 * ((size_t)blockIdx.x * blockDim.x + threadIdx.x); i < count; i += 2 * (size_t)gridDim.x * blockDim.x) {
        const float2 v = *reinterpret_cast<const float2 *>(src + i);
        const __nv_bfloat162 h = __floats2bfloat162_rn(v.x, v.y);
        const float2 hf = __bfloat1622float2(h);
        *reinterpret_cast<__nv_bfloat162 *>(hi + i) = h;
        *reinterpret_cast<__nv_bfloat162 *>(lo + i) = __floats2bfloat162_rn(v.x - hf.x, v.y - hf.y);
    }
}

static std::string cmsg(const char *what, cudaError_t e);

int run_ops_interp_reverse(Context &c, const OpsRevArgs &r, std::string &err) {
    SspOps &o = c.ops;
    cudaStream_t st = c.stream;
    cudaError_t e;
    const int n = r.n, nt = c.nt, nz = c.nz, R = o.interp_R;
    const size_t ktot = (size_t)nt * nz * R;
    const size_t ky = (size_t)r.itesc * nz * R, ko = ktot - ky;
    if (!o.interp_ready || ktot > (size_t)INT32_MAX) { err = "the interpolated reverse fold needs the interpolated operator"; return ST_UNSUPPORTED; }
    // the transposed basis (once per operator)
    if (!o.ibt_hi.p) {
        if ((e = o.ibt_hi.reserve(ktot * o.ntpad)) != cudaSuccess || (e = o.ibt_lo.reserve(ktot * o.ntpad)) != cudaSuccess ||
            (e = run_transpose_bf16(o.ib_hi.p, o.ibt_hi.p, o.ntempl, ktot, ktot, o.ntpad, st)) != cudaSuccess ||
            (e = run_transpose_bf16(o.ib_lo.p, o.ibt_lo.p, o.ntempl, ktot, ktot, o.ntpad, st)) != cudaSuccess ||
            (e = encode_tmap_2d_bf16(&o.tm_ibt_hi, o.ibt_hi.p, o.ntpad, ktot, gemm_bk(), gemm_bn())) != cudaSuccess ||
            (e = encode_tmap_2d_bf16(&o.tm_ibt_lo, o.ibt_lo.p, o.ntpad, ktot, gemm_bk(), gemm_bn())) != cudaSuccess) {
            err = cmsg("transposed operator basis", e);
            o.ibt_hi.release(); o.ibt_lo.release();
            return ST_DATA_MISSING;
        }
    }
    const size_t nv = (size_t)2 * n * o.ntpad;
    const int chunk = std::min(n, 2048);
    if ((e = c.d_vbh.reserve(nv)) != cudaSuccess || (e = c.d_vbl.reserve(nv)) != cudaSuccess ||
        (e = c.d_xbar.reserve((size_t)chunk * ktot)) != cudaSuccess) {
        err = cmsg("device memory", e);
        return ST_DATA_MISSING;
    }
    split_bf16_kernel<<<(unsigned)std::min<size_t>((nv / 2 + 255) / 256, 8192), 256, 0, st>>>(r.vbar, c.d_vbh.p, c.d_vbl.p, nv);
    if ((e = cudaGetLastError()) != cudaSuccess) { err = cmsg("template cotangent operand kernel", e); return ST_DATA_MISSING; }
    for (int m0 = 0; m0 < n; m0 += chunk) {
        const int rows = std::min(chunk, n - m0);
        for (int part = 0; part < 2; ++part) {
            const size_t N = part ? ko : ky;
            if (N == 0) continue;
            GemmPlan pl;
            pl.num_sms = c.num_sms;
            pl.tm_b_hi = o.tm_ibt_hi;
            pl.tm_b_lo = o.tm_ibt_lo;
            const size_t a0 = ((size_t)(part ? n : 0) + m0) * o.ntpad;
            if ((e = encode_tmap_2d_bf16(&pl.tm_a_hi, c.d_vbh.p + a0, o.ntpad, rows, gemm_bk(), gemm_bm())) != cudaSuccess ||
                (e = encode_tmap_2d_bf16(&pl.tm_a_lo, c.d_vbl.p + a0, o.ntpad, rows, gemm_bk(), gemm_bm())) != cudaSuccess) {
                err = cmsg("template cotangent tensor map", e);
                return ST_DATA_MISSING;
            }
            GemmArgs g;
            g.M = rows; g.N = (int)N; g.K = o.ntpad; g.ldd = (int)ktot; g.b_row0 = part ? (int)ky : 0;
            g.D = c.d_xbar.p + (part ? ky : 0); g.status = c.d_status.p;
            if ((e = run_gemm_bf16x3(pl, g, st)) != cudaSuccess) { err = cmsg("interpolated reverse fold GEMM", e); return ST_DATA_MISSING; }
        }
        OpsInterpRevArgs a;
        a.m0 = m0; a.nt = nt; a.nz = nz; a.R = R; a.ktot = ktot; a.imf_type = r.imf_type;
        for (int s = 0; s < 3; ++s) { a.noff[s] = o.interp_noff[s]; a.nn[s] = o.interp_nn[s]; a.x0[s] = o.interp_x0[s]; a.h[s] = o.interp_h[s]; }
        a.lim_lo = (float)r.lim.lim_lo; a.lim_hi = (float)r.lim.lim_hi;
        a.wz = r.wz; a.alpha = r.alpha; a.cscale = r.cscale; a.mass_bar = r.mass_bar; a.lbol_bar = r.lbol_bar; a.lsum_bar = r.lsum_bar; a.sums = r.sums;
        a.kconst = c.d_ix_const.p; a.xbar = c.d_xbar.p; a.mrow = o.i_mrow.p; a.lrow = o.i_lrow.p;
        a.wzb = r.wzb; a.params_bar = r.params_bar; a.rows = r.rows; a.row_imf1 = r.row_imf1;
        ops_interp_rev_kernel<<<rows, OPS_IR_THREADS, 0, st>>>(a);
        if ((e = cudaGetLastError()) != cudaSuccess) { err = cmsg("interpolated reverse fold kernel", e); return ST_DATA_MISSING; }
    }
    return 0;
}

// ---------------------------------------------------------------------------------------------- the epilogue
// One model per CTA from its young and old sums: the attenuation (attenuate_batch, power law), with dust emission
// the energy balance (dust_emission_reductions / add_dust_emission, src/physics/opensps_csp_batch.f90:3963-4099:
// the light the screens absorb, summed with the grid's frequency trapezoid weights, re-emitted as the Draine & Li
// shape times the diffuse transmission, scaled so that its escaping part carries the absorbed luminosity; dl07_shape
// :4103-4122), then the IGM (apply_igm_z), the AGN torus (add_agn_batch :4342-4433: fagn L_bol times the template
// interpolated in the torus optical depth, through the diffuse dust) and the velocity smoothing.
__device__ __forceinline__ float dl07_shape(const float *tab, int ns, int nq, int i, const DustEmModel &d) {
    const int k0 = 2 * d.iu, k1 = 2 * (d.iu + 1);
    const float *a = tab + (size_t)i;
    auto T = [&](int k, int q) { return __ldg(a + ((size_t)k * nq + q) * ns); };
    const float w00 = (1.f - d.wq) * (1.f - d.wu), w10 = d.wq * (1.f - d.wu), w11 = d.wq * d.wu, w01 = (1.f - d.wq) * d.wu;
    const float lo = w00 * T(k0, d.iq) + w10 * T(k0, d.iq + 1) + w11 * T(k1, d.iq + 1) + w01 * T(k1, d.iq);
    const float hi = w00 * T(k0 + 1, d.iq) + w10 * T(k0 + 1, d.iq + 1) + w11 * T(k1 + 1, d.iq + 1) + w01 * T(k1 + 1, d.iq);
    return fmaxf((1.f - d.gam) * lo + d.gam * hi, FLT_MIN);
}

// The same for the pixel pair (i, i + 1), i even, nspec even (8-byte loads of the eight template rows).
__device__ __forceinline__ float2 dl07_shape2(const float *tab, int ns, int nq, int i, const DustEmModel &d) {
    const int k0 = 2 * d.iu, k1 = 2 * (d.iu + 1);
    const float *a = tab + (size_t)i;
    auto T = [&](int k, int q) { return __ldg(reinterpret_cast<const float2 *>(a + ((size_t)k * nq + q) * ns)); };
    const float w00 = (1.f - d.wq) * (1.f - d.wu), w10 = d.wq * (1.f - d.wu), w11 = d.wq * d.wu, w01 = (1.f - d.wq) * d.wu;
    const float2 a0 = T(k0, d.iq), a1 = T(k0, d.iq + 1), a2 = T(k1, d.iq + 1), a3 = T(k1, d.iq);
    const float2 b0 = T(k0 + 1, d.iq), b1 = T(k0 + 1, d.iq + 1), b2 = T(k1 + 1, d.iq + 1), b3 = T(k1 + 1, d.iq);
    const float lx = w00 * a0.x + w10 * a1.x + w11 * a2.x + w01 * a3.x, ly = w00 * a0.y + w10 * a1.y + w11 * a2.y + w01 * a3.y;
    const float hx = w00 * b0.x + w10 * b1.x + w11 * b2.x + w01 * b3.x, hy = w00 * b0.y + w10 * b1.y + w11 * b2.y + w01 * b3.y;
    return make_float2(fmaxf((1.f - d.gam) * lx + d.gam * hx, FLT_MIN), fmaxf((1.f - d.gam) * ly + d.gam * hy, FLT_MIN));
}

// One CTA per model, two passes over its pixels (the spectrum in shared memory). Pass 1 reads everything from global
// memory: the attenuated sum through the IGM with the AGN added (the AGN does not depend on the energy balance), and
// with dust emission the escaping template through the IGM and the frequency-trapezoid sums of the absorbed and
// escaping light (before the IGM), reduced over the block; the emission scaled by their ratio then joins the
// spectrum. Pass 2 smooths from shared memory. Each thread issues the young and old loads of EPI_U pixel pairs before
// it uses them.
constexpr int EPI_U = 4;

// TAB: the models' curves differ and are tabulated (dust_type other than 0): each from the pixel's T0..T3 and the
// model's scalars (a separate instantiation keeps the others' registers as they were)
template <bool TAB>
__global__ void __launch_bounds__(256, 3) parts_epilogue_kernel(PartsEpilogueArgs a) {
    extern __shared__ float tsm[];         // nspec: the spectrum; with dust emission a second nspec: its emission
    float *esm = tsm + a.nspec;
    __shared__ float red[2][8];
    const int ns = a.nspec, m = blockIdx.x;
    const float *mp = a.mpar + (size_t)MODEL_PAR_FLOATS * m;
    const float *yv = a.young + (size_t)m * ns, *ov = a.old + (size_t)m * ns;
    const float kd2 = mp[MP_KD2], one_m_fnd = mp[MP_ONE_M_FND], fnd = mp[MP_FND], di = mp[MP_DUST_INDEX];
    const float kd1 = mp[MP_KD1], d1i = mp[MP_DUST1_INDEX], one_m_fo = mp[MP_ONE_M_FO], fo = mp[MP_FO];
    const float kd3 = mp[MP_KD3], kcap = mp[MP_IGM_KCAP];
    const int jmax = __float_as_int(mp[MP_IGM_JMAX]);
    const int igm_top = mp[MP_IGM_ON] != 0.f ? a.jtop : 0;     // pixels below carry the IGM
    DustEmModel dm{};
    if (a.dem) dm = a.dem[m];
    const bool emis = a.dem != nullptr && dm.on != 0;
    const bool agn = a.dem != nullptr && dm.agn != 0;
    // the AGN's luminosity: fagn times the model's L_bol (add_agn_batch :4342-4433, the value the batch outputs;
    // 1 when it is not above SAFE_FLOOR, as log10 L_bol is then 0)
    float lagn = 0.f;
    if (agn) {
        const double ls = a.lsum[(size_t)a.lsum_stride * m];
        lagn = (float)((ls > SAFE_FLOOR ? ls : 1.0) * (double)dm.fagn);
    }
    constexpr float LN2 = 0.6931471805599453f;
    float sa = 0.f, se = 0.f;
    // (ln lambda log2 e, the shared diffuse curve) of a pixel
    auto pix0 = [&](int p) { return __ldg(reinterpret_cast<const float2 *>(a.pix + (size_t)p * PIX_FLOATS)); };
    // pass 1 at pixel p: the attenuated young + old sum through the IGM plus the AGN (the torus template between the
    // two bracketing optical depths, through the diffuse dust); with emission the escaping template through the IGM
    // (esc) and the sums
    auto pass1 = [&](int p, float y, float o, float shape, float cn, float t0, float t1, float &esc) -> float {
        const float2 v0 = pix0(p);
        float curve;
        if constexpr (TAB) {
            const float4 t = __ldg(reinterpret_cast<const float4 *>(a.pix + (size_t)p * PIX_FLOATS + PIX_T));
            curve = pix_curve(false, true, 0.f, v0.x, t, make_float4(mp[MP_CS1], mp[MP_CS1 + 1], mp[MP_CS1 + 2], 0.f), di);
        } else {
            curve = a.uniform_index ? v0.y : ops_ex2(di * v0.x);
        }
        const float lb = (kd1 != 0.f) ? kd1 * ops_ex2(d1i * v0.x) : 0.f;   // log2 of the transmissions
        const float lo2 = kd3 * curve, ld2 = kd2 * curve;
        const float tb = (kd1 != 0.f) ? ops_ex2(lb) : 1.f;
        const float to = (kd3 != 0.f) ? ops_ex2(lo2) : 1.f;
        const float td = ops_ex2(ld2);
        const float ss = (y * tb * one_m_fo + y * fo) + o * to;
        float g = 1.f;
        if (p < igm_top) {
            float arg = kcap;
            if (p >= jmax) {
                const float2 va = __ldg(reinterpret_cast<const float2 *>(a.pix + (size_t)p * PIX_FLOATS + PIX_IGM_A));
                const float4 vb = __ldg(reinterpret_cast<const float4 *>(a.pix + (size_t)p * PIX_FLOATS + PIX_IGM_A + 2));
                arg = va.x * mp[MP_IGM_KB] + va.y * mp[MP_IGM_KB + 1] + vb.x * mp[MP_IGM_KB + 2] + vb.y * mp[MP_IGM_KB + 3] +
                      vb.z * mp[MP_IGM_KB + 4] + vb.w * mp[MP_IGM_KB + 5];
            }
            g = ops_ex2(arg);
        }
        if (emis) {
            // 1 - T of each screen from its exponent (no cancellation at small optical depth)
            const float omb = (kd1 != 0.f) ? -ops_expm1(lb * LN2) : 0.f;
            const float omo = (kd3 != 0.f) ? -ops_expm1(lo2 * LN2) : 0.f;
            const float omd = one_m_fnd * -ops_expm1(ld2 * LN2);
            const float ay = tb * one_m_fo + fo;
            const float absorbed = y * (one_m_fo * omb + ay * omd) + o * (omo + to * omd);
            const float e = shape * td;
            sa = fmaf(cn, absorbed, sa);
            se = fmaf(cn, e, se);
            esc = e * g;
        }
        float tot = ss * fmaf(td, one_m_fnd, fnd) * g;
        if (agn) tot = fmaf(lagn * fmaf(dm.wta, t1 - t0, t0), td, tot);
        return tot;
    };
    const int bd = (int)blockDim.x;
    const bool pairs = (ns & 1) == 0;
    if (pairs) {
        const int np2 = ns >> 1;
        const float2 *y2 = reinterpret_cast<const float2 *>(yv), *o2 = reinterpret_cast<const float2 *>(ov);
        const float2 *ga = reinterpret_cast<const float2 *>(a.agn_spec + (size_t)dm.ita * ns);
        const float2 *gb = reinterpret_cast<const float2 *>(a.agn_spec + (size_t)(dm.ita + 1) * ns);
        for (int q0 = threadIdx.x; q0 < np2; q0 += EPI_U * bd) {
            float2 yy[EPI_U], oo[EPI_U];
#pragma unroll
            for (int u = 0; u < EPI_U; ++u) {
                const int q = min(q0 + u * bd, np2 - 1);      // (past the end: the last pair again, not used)
                yy[u] = __ldg(y2 + q);
                oo[u] = __ldg(o2 + q);
            }
#pragma unroll
            for (int u = 0; u < EPI_U; ++u) {
                const int q = q0 + u * bd;
                if (q >= np2) break;
                float2 sh = make_float2(0.f, 0.f), cn = make_float2(0.f, 0.f), g0 = make_float2(0.f, 0.f), g1 = g0;
                if (emis) {
                    sh = dl07_shape2(a.dtab, ns, a.nqpah, 2 * q, dm);
                    cn = __ldg(reinterpret_cast<const float2 *>(a.cnu) + q);
                }
                if (agn) {
                    g0 = __ldg(ga + q);
                    g1 = __ldg(gb + q);
                }
                float e0 = 0.f, e1 = 0.f;
                const float t0 = pass1(2 * q, yy[u].x, oo[u].x, sh.x, cn.x, g0.x, g1.x, e0);
                const float t1 = pass1(2 * q + 1, yy[u].y, oo[u].y, sh.y, cn.y, g0.y, g1.y, e1);
                reinterpret_cast<float2 *>(tsm)[q] = make_float2(t0, t1);
                if (emis) reinterpret_cast<float2 *>(esm)[q] = make_float2(e0, e1);
            }
        }
    } else {
        for (int p = threadIdx.x; p < ns; p += bd) {
            float esc = 0.f, y = __ldg(yv + p), o = __ldg(ov + p);
            tsm[p] = pass1(p, y, o, emis ? dl07_shape(a.dtab, ns, a.nqpah, p, dm) : 0.f,
                           emis ? __ldg(a.cnu + p) : 0.f, agn ? __ldg(a.agn_spec + (size_t)dm.ita * ns + p) : 0.f,
                           agn ? __ldg(a.agn_spec + (size_t)(dm.ita + 1) * ns + p) : 0.f, esc);
            if (emis) esm[p] = esc;
        }
    }
    if (emis) {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            sa += __shfl_xor_sync(0xffffffffu, sa, off);
            se += __shfl_xor_sync(0xffffffffu, se, off);
        }
        if (lane == 0) { red[0][warp] = sa; red[1][warp] = se; }
        __syncthreads();
        float ta = 0.f, te = 0.f;
        for (int w = 0; w < (bd >> 5); ++w) { ta += red[0][w]; te += red[1][w]; }
        const float rn = te > SAFE_FLOOR ? ta / te : 0.f;
        // the emission joins the spectrum (each thread its own pass-1 pixels)
        if (pairs) {
            for (int q = threadIdx.x; q < (ns >> 1); q += bd) {
                const float2 t = reinterpret_cast<const float2 *>(tsm)[q], e = reinterpret_cast<const float2 *>(esm)[q];
                reinterpret_cast<float2 *>(tsm)[q] = make_float2(fmaf(e.x, rn, t.x), fmaf(e.y, rn, t.y));
            }
        } else {
            for (int p = threadIdx.x; p < ns; p += bd) tsm[p] = fmaf(esm[p], rn, tsm[p]);
        }
    }
    __syncthreads();
    const int R = __float_as_int(mp[MP_SMOOTH_R]);
    float tap[9];
#pragma unroll
    for (int d = 0; d < 9; ++d) tap[d] = mp[MP_TAPS + d];
    float *out = a.spec + (size_t)m * ns;
    for (int p = threadIdx.x; p < ns; p += bd) {
        float v = tsm[p];
        if (R >= 0 && p >= a.sm_lo && p <= a.sm_hi) {
            float s = 0.f;
#pragma unroll
            for (int d = -4; d <= 4; ++d) s = fmaf(tap[d + 4], tsm[p + d], s);
            v = s;
        }
        out[p] = v;
    }
}

// ---------------------------------------------------------------------------------------------- nebular continuum
// The CLOUDY-grid nebular continuum (nebular_kernels step 3, src/physics/opensps_csp_batch.f90:2760-2910), added to
// the young and old sums before the per-model epilogue.
//
// neb_weights_kernel, one warp per model: per nebular age t the weight C(t) = |1 - frac_obrun| sum_z w(t, z) q0(t, z)
// (the SFH weight times the ionizing photon rate, over the model's metallicities), normalised by its largest value S;
// log2 S split into an integer part and the rest. Row m of cw: C(t) / S for t < nt_neb, then (S's integer part, the
// rest). In FP32 (the weights rounded on the integer pipes, q0 scaled by 2^q0_exp, which goes into S's integer
// part): the sums of up to a dozen positive terms keep ~1e-7 (the FP64 form held the kernel at GB300's FP64 rate).
__global__ void __launch_bounds__(256) neb_weights_kernel(NebContArgs a) {
    const int m = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (m >= a.n) return;
    const float fabs_m = a.dem[m].neb_fabs;
    const double *w = a.wz + (size_t)m * a.nz * a.nt;
    float cs[(NEB_MAX_AGES + 31) / 32];
    float mx = 0.f;
#pragma unroll
    for (int i = 0; i < (NEB_MAX_AGES + 31) / 32; ++i) {
        const int t = lane + 32 * i;
        float c = 0.f;
        if (t < a.nt_neb) {
            for (int z = 0; z < a.nz; ++z)
                c = fmaf(weight_to_f32(__ldg(w + (size_t)z * a.nt + t)), __ldg(a.q0 + (size_t)t * a.nz + z), c);
            c *= fabs_m;
        }
        cs[i] = c;
        mx = fmaxf(mx, c);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    float *o = a.cw + (size_t)m * a.cw_ld;
#pragma unroll
    for (int i = 0; i < (NEB_MAX_AGES + 31) / 32; ++i) {
        const int t = lane + 32 * i;
        if (t < a.nt_neb) o[t] = mx > 0.f ? cs[i] / mx : 0.f;
    }
    if (lane == 0) {
        // S = mx 2^q0_exp = f 2^(e + q0_exp), f in [0.5, 1): log2 S = (e - 1 + q0_exp) + log2(2 f)
        int e = 0;
        const float f = mx > 0.f ? frexpf(mx, &e) : 0.5f;
        o[a.nt_neb] = mx > 0.f ? (float)(e - 1 + a.q0_exp) : 0.f;
        o[a.nt_neb + 1] = mx > 0.f ? log2f(2.f * f) : 0.f;
    }
}

// neb_cont_kernel: a CTA per (pixel block, group of at most NEB_GROUP models of one (gas_logz, gas_logu) cell, the
// models sorted by cell on the host). Each thread holds its pixel's table at the cell's four corners for the ten
// CLOUDY ages in registers, as the bilinear form L = c + w_z dz + w_u (du + w_z dzu), and takes the group's models four
// at a time (their weights C(t) / S four to a 16-byte shared load). The ages of one CLOUDY interval k are runs in which
// the exponent L_k + wa (L_k+1 - L_k) steps uniformly, so a run's sum is 2^(exponent at its last age) times a
// polynomial in y = 2^(-step dl) in Horner form: one FMA per age and model, two exponentials per run and model. Where
// the run spans more than NEB_STEEP in log2 with the flux falling (y > 1, which could overflow the polynomial) any
// lane of the warp takes the run age by age instead. Sums are relative to 2^(pixel offset + S's integer part), that
// scale applied last as exact powers of two; the young runs (ages below itesc) and the others are added to the young
// and old sums.
constexpr int NEB_PIX = 128;
constexpr float NEB_STEEP = 64.f;

__device__ __forceinline__ float pow2i(int e) {
    e = max(-126, min(e, 127));
    return __int_as_float((e + 127) << 23);
}

static size_t neb_cont_smem(int nt_neb, int nrun) {
    return sizeof(float4) * (size_t)NEB_GROUP + sizeof(float) * (size_t)nt_neb * NEB_GROUP + sizeof(int4) * (size_t)nrun +
           sizeof(int) * (size_t)(NEB_RUN_HEAD + NEB_GROUP);
}

__global__ void __launch_bounds__(NEB_PIX) neb_cont_kernel(NebContArgs a) {
    constexpr int NU = 7, NA = 10, G = NEB_GROUP, G4 = NEB_GROUP / 4;
    static_assert(G % 4 == 0 && (G & (G - 1)) == 0 && G <= NEB_PIX, "groups of a power of two models");
    extern __shared__ float4 nsm[];
    float4 *mp = nsm;                                                  // G: (w_z, w_u, S's fraction, S's integer part)
    float4 *cws = mp + G;                                              // nt_neb x G / 4: C(t) / S, models fastest
    int4 *runs = reinterpret_cast<int4 *>(cws + (size_t)a.nt_neb * G4);
    int *rf = reinterpret_cast<int *>(runs + a.nrun);                  // NEB_RUN_HEAD
    int *mids = rf + NEB_RUN_HEAD;                                     // G
    const int4 g = a.groups[blockIdx.y];                               // (cell z, cell u, first in order, count)
    const int cnt = g.w;
    for (int i = threadIdx.x; i < a.nrun; i += NEB_PIX) runs[i] = __ldg(a.runs + i);
    if (threadIdx.x < NEB_RUN_HEAD) rf[threadIdx.x] = __ldg(a.rfirst + threadIdx.x);
    if (threadIdx.x < G) {
        const int j = threadIdx.x;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        int m = 0;
        if (j < cnt) {
            m = __ldg(a.order + g.z + j);
            const DustEmModel &dm = a.dem[m];
            const float *cw = a.cw + (size_t)m * a.cw_ld;
            v = make_float4(dm.neb_wz, dm.neb_wu, __ldg(cw + a.nt_neb + 1), __ldg(cw + a.nt_neb));
        }
        mp[j] = v;
        mids[j] = m;
    }
    __syncthreads();
    float *cwf = reinterpret_cast<float *>(cws);
    for (int e = threadIdx.x; e < a.nt_neb * G; e += NEB_PIX) {
        const int j = e & (G - 1), t = e / G;
        cwf[e] = j < cnt ? __ldg(a.cw + (size_t)mids[j] * a.cw_ld + t) : 0.f;
    }
    __syncthreads();
    const int p = blockIdx.x * NEB_PIX + threadIdx.x;
    const int pc = min(p, a.nspec - 1);                 // (lanes past the last pixel compute on it and store nothing)
    const size_t plane = (size_t)NA * a.nspec;
    const float *b00 = a.tab + (size_t)(g.x * NU + g.y) * plane + pc, *b01 = b00 + plane;
    const float *b10 = a.tab + (size_t)((g.x + 1) * NU + g.y) * plane + pc, *b11 = b10 + plane;
    float c0[NA], dz[NA], du[NA], dzu[NA];
#pragma unroll
    for (int k = 0; k < NA; ++k) {
        const float t00 = __ldg(b00 + (size_t)k * a.nspec), t01 = __ldg(b01 + (size_t)k * a.nspec);
        const float t10 = __ldg(b10 + (size_t)k * a.nspec), t11 = __ldg(b11 + (size_t)k * a.nspec);
        c0[k] = t00;
        dz[k] = t10 - t00;
        du[k] = t01 - t00;
        dzu[k] = (t11 - t10) - (t01 - t00);
    }
    const int offp = (int)__ldg(a.off + pc);
    for (int j0 = 0; j0 < cnt; j0 += 4) {
        float4 P[4];
        size_t idx[4];
        bool st[4];
        float yv[4], ov[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            P[q] = mp[j0 + q];
            st[q] = p < a.nspec && j0 + q < cnt;
            idx[q] = (size_t)mids[j0 + q] * a.nspec + pc;
            yv[q] = st[q] ? a.young[idx[q]] : 0.f;
            ov[q] = st[q] ? a.old[idx[q]] : 0.f;
        }
        float ys[4] = {0.f, 0.f, 0.f, 0.f}, os[4] = {0.f, 0.f, 0.f, 0.f}, Lk[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) Lk[q] = fmaf(P[q].x, dz[0], fmaf(P[q].y, fmaf(P[q].x, dzu[0], du[0]), c0[0]));
#pragma unroll
        for (int k = 0; k < NA - 1; ++k) {
            float L1[4], dl[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                L1[q] = fmaf(P[q].x, dz[k + 1], fmaf(P[q].y, fmaf(P[q].x, dzu[k + 1], du[k + 1]), c0[k + 1]));
                dl[q] = L1[q] - Lk[q];
            }
            const int r1 = rf[k + 1];
            for (int r = rf[k]; r < r1; ++r) {
                const int4 R = runs[r];
                const int t0 = R.x, nr = R.y & 0xffff;
                const float wtop = __int_as_float(R.z), del = __int_as_float(R.w);
                const float span = (float)(nr - 1) * del;
                bool steep = false;
#pragma unroll
                for (int q = 0; q < 4; ++q) steep |= -dl[q] * span > NEB_STEEP;
                const float4 *cr = cws + (size_t)t0 * G4 + (j0 >> 2);
                float H[4];
                if (__any_sync(0xffffffffu, steep)) {
                    // age by age: each term 2^(S's fraction + L_k + wa dl) <= 2
#pragma unroll
                    for (int q = 0; q < 4; ++q) H[q] = 0.f;
                    for (int t = 0; t < nr; ++t) {
                        const float4 cv = cr[(size_t)t * G4];
                        const float wt = wtop - (float)(nr - 1 - t) * del;
                        H[0] = fmaf(cv.x, ops_ex2(P[0].z + fmaf(wt, dl[0], Lk[0])), H[0]);
                        H[1] = fmaf(cv.y, ops_ex2(P[1].z + fmaf(wt, dl[1], Lk[1])), H[1]);
                        H[2] = fmaf(cv.z, ops_ex2(P[2].z + fmaf(wt, dl[2], Lk[2])), H[2]);
                        H[3] = fmaf(cv.w, ops_ex2(P[3].z + fmaf(wt, dl[3], Lk[3])), H[3]);
                    }
                } else {
                    float y[4] = {1.f, 1.f, 1.f, 1.f};
                    if (nr > 1 && del != 0.f) {
#pragma unroll
                        for (int q = 0; q < 4; ++q) y[q] = ops_ex2(-del * dl[q]);
                    }
                    float4 cv = cr[0];
                    H[0] = cv.x; H[1] = cv.y; H[2] = cv.z; H[3] = cv.w;
                    for (int t = 1; t < nr; ++t) {
                        cv = cr[(size_t)t * G4];
                        H[0] = fmaf(H[0], y[0], cv.x);
                        H[1] = fmaf(H[1], y[1], cv.y);
                        H[2] = fmaf(H[2], y[2], cv.z);
                        H[3] = fmaf(H[3], y[3], cv.w);
                    }
#pragma unroll
                    for (int q = 0; q < 4; ++q) H[q] *= ops_ex2(P[q].z + fmaf(wtop, dl[q], Lk[q]));
                }
                if (R.y >> 16) {
#pragma unroll
                    for (int q = 0; q < 4; ++q) ys[q] += H[q];
                } else {
#pragma unroll
                    for (int q = 0; q < 4; ++q) os[q] += H[q];
                }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) Lk[q] = L1[q];
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (!st[q]) continue;
            const int e = offp + (int)P[q].w, e1 = e >> 1;
            const float s1 = pow2i(e1), s2 = pow2i(e - e1);
            a.young[idx[q]] = fmaf(ys[q] * s1, s2, yv[q]);
            a.old[idx[q]] = fmaf(os[q] * s1, s2, ov[q]);
        }
    }
}

// ---------------------------------------------------------------------------------------------- its reverse pass
// backward_nebular's continuum (src/physics/opensps_csp_batch.f90:5334-5606). With g the young or old sums' cotangent
// (as the forward added age t's term), per model and nebular age t the pixel sums
//     A_t  = sum_j g_j 2^(E + off_j + L_t(j)),     E = log2 S,   L_t = L_k + wa_t (L_k+1 - L_k),
//     Az_t = sum_j g_j 2^(...) dL_t/dw_z (j),      Au_t = sum_j g_j 2^(...) dL_t/dw_u (j),
// (L_k the cell's bilinear form c + w_z dz + w_u (du + w_z dzu) of CLOUDY age k, in log2, as the forward forms it),
// so that dL / dC_t = A_t / S. Then the weights' cotangent gains dL/dC_t |1 - frac_obrun| q0(t, z); the gas_logz and
// gas_logu rows ln 2 sum_t (C_t / S) Az_t (Au_t) times the cell's chain factor; frac_obrun's row sum_t (C_t / S) A_t
// d|1 - fo|/dfo / |1 - fo|. One CTA per model: a thread takes a pixel per step, every age's three sums go over the
// warp's lanes and lane 0 adds them to its warp's row in shared memory.
constexpr int NEB_REV_THREADS = 256;
__global__ void __launch_bounds__(NEB_REV_THREADS) neb_cont_rev_kernel(NebContRevArgs a) {
    constexpr int NU = 7, NA = 10, NW = NEB_REV_THREADS / 32;
    __shared__ float acc[NW][NEB_MAX_AGES][3];
    __shared__ float wa_s[NEB_MAX_AGES];
    __shared__ double red[NW][3];
    const int m = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const DustEmModel dm = a.dem[m];
    if (!(dm.neb_fabs > 0.f)) return;                  // (the forward added no continuum)
    for (int i = tid; i < NW * NEB_MAX_AGES * 3; i += NEB_REV_THREADS) (&acc[0][0][0])[i] = 0.f;
    for (int t = tid; t < a.nt_neb; t += NEB_REV_THREADS) wa_s[t] = __ldg(a.wa + t);
    __syncthreads();
    const float *cw = a.cw + (size_t)m * a.cw_ld;
    const float E = __ldg(cw + a.nt_neb) + __ldg(cw + a.nt_neb + 1);
    const size_t plane = (size_t)NA * a.nspec;
    const float *b00 = a.tab + (size_t)(dm.neb_iz * NU + dm.neb_iu) * plane, *b01 = b00 + plane;
    const float *b10 = a.tab + (size_t)((dm.neb_iz + 1) * NU + dm.neb_iu) * plane, *b11 = b10 + plane;
    const float wz = dm.neb_wz, wu = dm.neb_wu;
    const __nv_bfloat16 *yh = a.ybh + (size_t)m * a.ppad, *yl = a.ybl + (size_t)m * a.ppad;
    const __nv_bfloat16 *oh = a.obh + (size_t)m * a.ppad, *ol = a.obl + (size_t)m * a.ppad;
    for (int p0 = 0; p0 < a.nspec; p0 += NEB_REV_THREADS) {
        const int p = p0 + tid;
        const bool ok = p < a.nspec;
        const int pc = ok ? p : a.nspec - 1;
        const float gy = ok ? __bfloat162float(yh[p]) + __bfloat162float(yl[p]) : 0.f;
        const float go = ok ? __bfloat162float(oh[p]) + __bfloat162float(ol[p]) : 0.f;
        const float base = E + __ldg(a.off + pc);
        float L[NA], Lz[NA], Lu[NA];
#pragma unroll
        for (int k = 0; k < NA; ++k) {
            const float t00 = __ldg(b00 + (size_t)k * a.nspec + pc), t01 = __ldg(b01 + (size_t)k * a.nspec + pc);
            const float t10 = __ldg(b10 + (size_t)k * a.nspec + pc), t11 = __ldg(b11 + (size_t)k * a.nspec + pc);
            const float dz = t10 - t00, du = t01 - t00, dzu = (t11 - t10) - (t01 - t00);
            L[k] = fmaf(wz, dz, fmaf(wu, fmaf(wz, dzu, du), t00));
            Lz[k] = fmaf(wu, dzu, dz);
            Lu[k] = fmaf(wz, dzu, du);
        }
#pragma unroll
        for (int k = 0; k < NA - 1; ++k) {
            const int t1 = a.kfirst[k + 1];
            for (int t = a.kfirst[k]; t < t1; ++t) {
                const float w = wa_s[t];
                const float g = t < a.itesc ? gy : go;
                const float e = ops_ex2(base + fmaf(w, L[k + 1] - L[k], L[k]));
                float v0 = g != 0.f ? g * e : 0.f;
                float v1 = v0 * fmaf(w, Lz[k + 1] - Lz[k], Lz[k]);
                float v2 = v0 * fmaf(w, Lu[k + 1] - Lu[k], Lu[k]);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    v0 += __shfl_xor_sync(0xffffffffu, v0, o);
                    v1 += __shfl_xor_sync(0xffffffffu, v1, o);
                    v2 += __shfl_xor_sync(0xffffffffu, v2, o);
                }
                if (lane == 0) { acc[warp][t][0] += v0; acc[warp][t][1] += v1; acc[warp][t][2] += v2; }
            }
        }
    }
    __syncthreads();
    const double cs = a.cscale[m], fab = (double)dm.neb_fabs;
    const double inv_s = exp2(-(double)E), qs = ldexp(1.0, a.q0_exp);
    double gz = 0.0, gu = 0.0, gfo = 0.0;
    for (int t = tid; t < a.nt_neb; t += NEB_REV_THREADS) {
        double A = 0.0, Az = 0.0, Au = 0.0;
        for (int w = 0; w < NW; ++w) { A += acc[w][t][0]; Az += acc[w][t][1]; Au += acc[w][t][2]; }
        const double ct = (double)__ldg(cw + t);       // C_t / S
        gz += ct * Az;
        gu += ct * Au;
        gfo += ct * A;
        if (a.wzbar) {
            const double dc = A * inv_s * cs * fab * qs;
            for (int z = 0; z < a.nz; ++z)
                a.wzbar[(size_t)m * a.ntz + t + (size_t)a.nt * z] += dc * (double)__ldg(a.q0 + (size_t)t * a.nz + z);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        gz += __shfl_xor_sync(0xffffffffu, gz, o);
        gu += __shfl_xor_sync(0xffffffffu, gu, o);
        gfo += __shfl_xor_sync(0xffffffffu, gfo, o);
    }
    if (lane == 0) { red[warp][0] = gz; red[warp][1] = gu; red[warp][2] = gfo; }
    __syncthreads();
    if (tid == 0) {
        double s[3] = {0.0, 0.0, 0.0};
        for (int w = 0; w < NW; ++w)
            for (int i = 0; i < 3; ++i) s[i] += red[w][i];
        double *pb = a.params_bar + (size_t)a.rows * m;
        const double ln2 = 0.6931471805599453;
        pb[a.row_gas_logz] += cs * ln2 * s[0] * (double)dm.neb_dz;
        pb[a.row_gas_logu] += cs * ln2 * s[1] * (double)dm.neb_du;
        pb[a.row_frac_obrun] += cs * s[2] * (double)dm.neb_dfo / fab;
    }
}

cudaError_t run_nebular_continuum_reverse(const NebContRevArgs &a, cudaStream_t st) {
    if (a.n <= 0 || a.nt_neb <= 0) return cudaSuccess;
    if (a.nt_neb > NEB_MAX_AGES) return cudaErrorInvalidValue;
    neb_cont_rev_kernel<<<a.n, NEB_REV_THREADS, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t run_nebular_continuum(const NebContArgs &a, int ngroups, cudaStream_t st) {
    if (a.n <= 0 || ngroups <= 0) return cudaSuccess;
    neb_weights_kernel<<<(unsigned)((a.n * 32 + 255) / 256), 256, 0, st>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const size_t smem = neb_cont_smem(a.nt_neb, a.nrun);
    if (smem > 48 * 1024 &&
        (e = cudaFuncSetAttribute(neb_cont_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
        return e;
    // (the groups in slices within the grid's y limit)
    for (int g0 = 0; g0 < ngroups; g0 += 65535) {
        NebContArgs b = a;
        b.groups = a.groups + g0;
        const dim3 grid((a.nspec + NEB_PIX - 1) / NEB_PIX, std::min(65535, ngroups - g0));
        neb_cont_kernel<<<grid, NEB_PIX, smem, st>>>(b);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t run_parts_epilogue(const PartsEpilogueArgs &a, cudaStream_t st) {
    if (a.n <= 0) return cudaSuccess;
    const size_t smem = sizeof(float) * (size_t)a.nspec * (a.dem ? 2 : 1);
    const bool tab = !a.uniform_index && a.tab_curve;
    cudaError_t e = tab ? cudaFuncSetAttribute(parts_epilogue_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                        : cudaFuncSetAttribute(parts_epilogue_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (tab) parts_epilogue_kernel<true><<<a.n, 256, smem, st>>>(a);
    else parts_epilogue_kernel<false><<<a.n, 256, smem, st>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------- host side
template <class T>
static bool read_raw(const std::string &path, std::vector<T> &out, size_t count) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    out.resize(count);
    f.read(reinterpret_cast<char *>(out.data()), (std::streamsize)(count * sizeof(T)));
    return (size_t)f.gcount() == count * sizeof(T);
}

static std::string cmsg(const char *what, cudaError_t e) { return std::string(what) + ": " + cudaGetErrorString(e); }

// The interpolated fold's operator basis (ops_interp_x_kernel): per segment equispaced nodes over the x = ln m range
// of its bin pieces (the pieces as imf_weight splits a bin), per piece the Lagrange weights int L_j(x) e^x dx
// (6-point Gauss-Legendre in each node interval the piece meets), summed per grid point in FP64 into B (templates x
// R node columns, then bf16 hi / lo) and into the mass and L_bol rows; uploaded in blocks of grid points. Returns
// false, leaving the exact fold the only one, when memory runs short or the nodes do not fit.
static bool ops_interp_build(Context &c, const std::vector<double> &mini, const std::vector<int> &idx,
                             const std::vector<double> &coef, const std::vector<double> &mcur,
                             const std::vector<double> &lum, int ntempl, int npt, double lower_bound) {
    SspOps &o = c.ops;
    o.interp_ready = false;
    const int nt = c.nt, nz = c.nz, ng = nt * nz;
    if (ng > OPS_IMAXG) return false;
    const double lim_lo = 0.08, lim_hi = 120.0;
    const double slo[3] = {0.08, 0.5, 1.0}, shi[3] = {0.5, 1.0, 1.0e30};
    auto pieces = [&](const double *mi, int i, int *sg, double *lo, double *hi) -> int {
        const double m1 = (i == 0) ? lower_bound : mi[i] - 0.5 * (mi[i] - mi[i - 1]);
        const double m2 = (i == npt - 1) ? mi[i] : mi[i] + 0.5 * (mi[i + 1] - mi[i]);
        if (mi[i] < lim_lo || mi[i] > lim_hi || m2 <= m1) return 0;
        int np = 0;
        for (int s = 0; s < 3; ++s) {
            const double a = std::max(m1, slo[s]), b = std::min(m2, shi[s]);
            if (b > a) { sg[np] = s; lo[np] = a; hi[np] = b; ++np; }
        }
        return np;
    };
    double xlo[3] = {1e300, 1e300, 1e300}, xhi[3] = {-1e300, -1e300, -1e300};
    for (int g = 0; g < ng; ++g) {
        const double *mi = mini.data() + (size_t)g * npt;
        for (int i = 0; i < npt; ++i) {
            int sg[3]; double lo[3], hi[3];
            const int np = pieces(mi, i, sg, lo, hi);
            for (int k = 0; k < np; ++k) {
                xlo[sg[k]] = std::min(xlo[sg[k]], std::log(lo[k]));
                xhi[sg[k]] = std::max(xhi[sg[k]], std::log(hi[k]));
            }
        }
    }
    int R = 0, nint[3];
    for (int s = 0; s < 3; ++s) {
        if (!(xhi[s] > xlo[s])) { o.interp_nn[s] = 0; o.interp_noff[s] = R; nint[s] = 0; o.interp_x0[s] = 0.0; o.interp_h[s] = 1.0; continue; }
        nint[s] = std::max(1, (int)std::ceil((xhi[s] - xlo[s]) * OPS_AMAX[s] / OPS_IH));
        o.interp_h[s] = (xhi[s] - xlo[s]) / nint[s];
        o.interp_x0[s] = xlo[s];
        o.interp_nn[s] = nint[s] + OPS_IDEG;
        o.interp_noff[s] = R;
        R += o.interp_nn[s];
    }
    R = (R + 7) / 8 * 8;
    if (R > OPS_IMAXR || R == 0) return false;
    o.interp_R = R;
    const size_t ktot = (size_t)ng * R;
    if (o.ib_hi.reserve((size_t)ntempl * ktot) != cudaSuccess || o.ib_lo.reserve((size_t)ntempl * ktot) != cudaSuccess ||
        o.i_mrow.reserve(ktot) != cudaSuccess || o.i_lrow.reserve(ktot) != cudaSuccess) {
        o.ib_hi.release(); o.ib_lo.release(); o.i_mrow.release(); o.i_lrow.release();
        cudaGetLastError();
        return false;
    }
    static const double GX[6] = {-0.9324695142031521, -0.6612093864662645, -0.2386191860831969,
                                 0.2386191860831969, 0.6612093864662645, 0.9324695142031521};
    static const double GW[6] = {0.1713244923791704, 0.3607615730481386, 0.4679139345726910,
                                 0.4679139345726910, 0.3607615730481386, 0.1713244923791704};
    double inv_den[OPS_IDEG + 1];
    for (int k = 0; k <= OPS_IDEG; ++k) {
        double d = 1.0;
        for (int l = 0; l <= OPS_IDEG; ++l)
            if (l != k) d *= (double)(k - l);
        inv_den[k] = 1.0 / d;
    }
    std::vector<float> mrow(ktot), lrow(ktot);
    constexpr int BLK = 64;                              // grid points per upload
    std::vector<uint16_t> sh((size_t)ntempl * BLK * R), sl((size_t)ntempl * BLK * R);
    bool ok = true;
    for (int g0 = 0; g0 < ng && ok; g0 += BLK) {
        const int nb = std::min(BLK, ng - g0);
        const size_t w = (size_t)nb * R;                  // staging row length
#pragma omp parallel
        {
            std::vector<double> acc((size_t)ntempl * R), am(R), al(R);
#pragma omp for schedule(dynamic, 1)
            for (int b = 0; b < nb; ++b) {
                const int gp = g0 + b, t = gp / nz, z = gp - t * nz;   // column order (t nz + z)
                const size_t gf = (size_t)t + (size_t)nt * z;         // the files' order (age fastest)
                std::fill(acc.begin(), acc.end(), 0.0);
                std::fill(am.begin(), am.end(), 0.0);
                std::fill(al.begin(), al.end(), 0.0);
                const double *mi = mini.data() + gf * npt;
                for (int i = 0; i < npt; ++i) {
                    int sg[3]; double lo[3], hi[3];
                    const int np = pieces(mi, i, sg, lo, hi);
                    const size_t q = gf * npt + i;
                    for (int k = 0; k < np; ++k) {
                        const int s = sg[k];
                        const double xa = std::log(lo[k]), xb = std::log(hi[k]), h = o.interp_h[s], x0 = o.interp_x0[s];
                        const int ia = std::min(std::max((int)std::floor((xa - x0) / h), 0), nint[s] - 1);
                        const int ib = std::min(std::max((int)std::floor((xb - x0) / h), 0), nint[s] - 1);
                        for (int iv = ia; iv <= ib; ++iv) {
                            const double a = iv == ia ? xa : x0 + iv * h, bb = iv == ib ? xb : x0 + (iv + 1) * h;
                            if (!(bb > a)) continue;
                            const double xs = x0 + (iv - OPS_IDEG / 2) * h;   // the stencil's first node
                            double wl[OPS_IDEG + 1] = {};
                            for (int gq = 0; gq < 6; ++gq) {
                                const double x = 0.5 * (a + bb) + 0.5 * (bb - a) * GX[gq];
                                const double u = (x - xs) / h, ex = std::exp(x) * 0.5 * (bb - a) * GW[gq];
                                for (int kk = 0; kk <= OPS_IDEG; ++kk) {
                                    double p = inv_den[kk];
                                    for (int l = 0; l <= OPS_IDEG; ++l)
                                        if (l != kk) p *= (u - l);
                                    wl[kk] += ex * p;
                                }
                            }
                            const int c0 = o.interp_noff[s] + iv;
                            for (int kk = 0; kk <= OPS_IDEG; ++kk) {
                                am[c0 + kk] += mcur[q] * wl[kk];
                                al[c0 + kk] += lum[q] * wl[kk];
                                for (int j = 0; j < 4; ++j)
                                    acc[(size_t)idx[4 * q + j] * R + c0 + kk] += coef[4 * q + j] * wl[kk];
                            }
                        }
                    }
                }
                for (int r = 0; r < R; ++r) {
                    mrow[(size_t)gp * R + r] = (float)am[r];
                    lrow[(size_t)gp * R + r] = (float)al[r];
                }
                for (int e = 0; e < ntempl; ++e)
                    for (int r = 0; r < R; ++r) {
                        const double v = acc[(size_t)e * R + r];
                        const uint16_t hb = f32_to_bf16_bits((float)v);
                        sh[(size_t)e * w + (size_t)b * R + r] = hb;
                        sl[(size_t)e * w + (size_t)b * R + r] = f32_to_bf16_bits((float)(v - (double)bf16_bits_to_f32(hb)));
                    }
            }
        }
        ok = cudaMemcpy2D(o.ib_hi.p + (size_t)g0 * R, ktot * 2, sh.data(), w * 2, w * 2, ntempl, cudaMemcpyHostToDevice) == cudaSuccess &&
             cudaMemcpy2D(o.ib_lo.p + (size_t)g0 * R, ktot * 2, sl.data(), w * 2, w * 2, ntempl, cudaMemcpyHostToDevice) == cudaSuccess;
    }
    ok = ok && cudaMemcpy(o.i_mrow.p, mrow.data(), sizeof(float) * ktot, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(o.i_lrow.p, lrow.data(), sizeof(float) * ktot, cudaMemcpyHostToDevice) == cudaSuccess;
    if (!ok) {
        o.ib_hi.release(); o.ib_lo.release(); o.i_mrow.release(); o.i_lrow.release();
        cudaGetLastError();
        return false;
    }
    o.interp_ready = true;
    return true;
}

// The operator from the data root's ssp_op dataset (the reference's ssp_operator_build from isochrones and
// libraries; here its synthetic stand-in): points with their bins and Kroupa segments, entries sorted by template per
// grid point, the library transposed to pixels x ntpad in bf16 hi / lo.
int ops_build(Context &c, std::string &err) {
    const std::string dir = data_root() + "/ssp_op/";
    std::ifstream mf(dir + "manifest.json");
    if (!mf) { err = "SSP operator data missing under " + dir; return ST_DATA_MISSING; }
    const int ns = c.nspec, nt = c.nt, nz = c.nz, ng = nt * nz;
    const int npt = 1500, ntempl = 2000;
    std::vector<float> lib;
    std::vector<double> mini, coef, mcur, lum;
    std::vector<int> idx;
    const size_t np = (size_t)ng * npt;
    if (!read_raw(dir + "lib.f32", lib, (size_t)ntempl * ns) || !read_raw(dir + "pt_mini.f64", mini, np) ||
        !read_raw(dir + "pt_idx.i32", idx, np * 4) || !read_raw(dir + "pt_coef.f64", coef, np * 4) ||
        !read_raw(dir + "pt_mcur.f64", mcur, np) || !read_raw(dir + "pt_lum.f64", lum, np)) {
        err = "SSP operator data under " + dir + " does not match the context's grid";
        return ST_DATA_MISSING;
    }
    for (size_t i = 0; i < idx.size(); ++i)
        if (idx[i] < 0 || idx[i] >= ntempl) {
            err = "SSP operator data under " + dir + ": a template index outside the library";
            return ST_DATA_MISSING;
        }
    const double lower_bound = 0.08, lim_lo = 0.08, lim_hi = 120.0;
    // data layout: grid point (z, t) z-major in the files: g_file = z nt + t == t + nt z (age fastest)
    std::vector<OpsPoint> pts(np);
    const int nent = 4 * npt;
    std::vector<uint32_t> ent((size_t)ng * nent);
    std::vector<float> ent_c((size_t)ng * nent);
    std::vector<std::pair<uint32_t, float>> tmp(nent);
    for (int g = 0; g < ng; ++g) {
        const double *mi = mini.data() + (size_t)g * npt;
        for (int i = 0; i < npt; ++i) {
            OpsPoint &q = pts[(size_t)g * npt + i];
            const double m1 = (i == 0) ? lower_bound : mi[i] - 0.5 * (mi[i] - mi[i - 1]);
            const double m2 = (i == npt - 1) ? mi[i] : mi[i] + 0.5 * (mi[i + 1] - mi[i]);
            q.mcur = (float)mcur[(size_t)g * npt + i];
            q.lum = (float)lum[(size_t)g * npt + i];
            q.lo = (float)m1;
            q.hi = (float)m2;
            q.ln_lo = (float)std::log(m1);
            q.dl = (float)std::log1p((m2 - m1) / m1);
            q.mini = (float)(i == 0 ? -mi[i] : mi[i]);
            if (mi[i] < lim_lo || mi[i] > lim_hi || m2 <= m1) q.seg = -1;
            else if (m1 >= 0.08 && m2 <= 0.5) q.seg = 1;
            else if (m1 >= 0.5 && m2 <= 1.0) q.seg = 2;
            else if (m1 >= 1.0) q.seg = 3;
            else q.seg = 0;
        }
        for (int i = 0; i < npt; ++i)
            for (int k = 0; k < 4; ++k) {
                const size_t s = ((size_t)g * npt + i) * 4 + k;
                tmp[4 * i + k] = {((uint32_t)idx[s] << 16) | (uint32_t)i, (float)coef[s]};
            }
        std::sort(tmp.begin(), tmp.end(), [](const std::pair<uint32_t, float> &x, const std::pair<uint32_t, float> &y) {
            return x.first < y.first;
        });
        for (int i = 0; i < nent; ++i) {
            ent[(size_t)g * nent + i] = tmp[i].first;
            ent_c[(size_t)g * nent + i] = tmp[i].second;
        }
    }
    // point-major templates and coefficients (the reverse fold gathers per point)
    std::vector<ushort4> pidx(np);
    std::vector<float4> pcoef(np);
    for (size_t i = 0; i < np; ++i) {
        pidx[i] = make_ushort4((unsigned short)idx[4 * i], (unsigned short)idx[4 * i + 1], (unsigned short)idx[4 * i + 2],
                               (unsigned short)idx[4 * i + 3]);
        pcoef[i] = make_float4((float)coef[4 * i], (float)coef[4 * i + 1], (float)coef[4 * i + 2], (float)coef[4 * i + 3]);
    }
    const int ntpad = (ntempl + 63) / 64 * 64;
    std::vector<uint16_t> lh((size_t)ns * ntpad, 0), ll((size_t)ns * ntpad, 0);
    for (int e = 0; e < ntempl; ++e)
        for (int p = 0; p < ns; ++p) {
            const float f = lib[(size_t)e * ns + p];
            const uint16_t h = f32_to_bf16_bits(f);
            lh[(size_t)p * ntpad + e] = h;
            ll[(size_t)p * ntpad + e] = f32_to_bf16_bits(f - bf16_bits_to_f32(h));
        }
    SspOps &o = c.ops;
    cudaError_t e;
    if ((e = o.pts.reserve(np)) != cudaSuccess || (e = o.ent.reserve(ent.size())) != cudaSuccess ||
        (e = o.ent_c.reserve(ent_c.size())) != cudaSuccess || (e = o.lib_hi.reserve(lh.size())) != cudaSuccess ||
        (e = o.lib_lo.reserve(ll.size())) != cudaSuccess || (e = o.pidx.reserve(np)) != cudaSuccess ||
        (e = o.pcoef.reserve(np)) != cudaSuccess ||
        (e = cudaMemcpy(o.pidx.p, pidx.data(), sizeof(ushort4) * np, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(o.pcoef.p, pcoef.data(), sizeof(float4) * np, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(o.pts.p, pts.data(), sizeof(OpsPoint) * np, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(o.ent.p, ent.data(), sizeof(uint32_t) * ent.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(o.ent_c.p, ent_c.data(), sizeof(float) * ent_c.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(o.lib_hi.p, lh.data(), 2 * lh.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(o.lib_lo.p, ll.data(), 2 * ll.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = encode_tmap_2d_bf16(&o.tm_lib_hi, o.lib_hi.p, ntpad, ns, gemm_bk(), gemm_bn())) != cudaSuccess ||
        (e = encode_tmap_2d_bf16(&o.tm_lib_lo, o.lib_lo.p, ntpad, ns, gemm_bk(), gemm_bn())) != cudaSuccess) {
        err = cmsg("SSP operator upload", e);
        o.release();
        return ST_DATA_MISSING;
    }
    o.ntempl = ntempl;
    o.ntpad = ntpad;
    o.npt = npt;
    o.nent = nent;
    o.lower_bound = lower_bound;
    o.ready = true;
    ops_interp_build(c, mini, idx, coef, mcur, lum, ntempl, npt, lower_bound);
    return 0;
}

// Whether the interpolated fold holds for every model's slopes (and is built and not switched off).
static bool ops_interp_ok(const Context &c, const double *h_alpha, int n) {
    if (!c.ops.interp_ready || c.ops_exact || !h_alpha) return false;
    // (the basis holds the build's mass limits 0.08 - 120 M_sun and the fixed breaks of Kroupa's form)
    if (c.imf_type == 5 || c.imf_lim_lo != 0.08 || c.imf_lim_hi != 120.0) return false;
    if (c.imf_type == 1) return true;   // (Chabrier: no slopes)
    if (c.imf_type == 3 || c.imf_type == 4) return false;   // (breaks per model: the exact fold)
    for (int m = 0; m < n; ++m)
        for (int s = 0; s < 3; ++s)
            if (!(std::fabs(h_alpha[3 * (size_t)m + s]) <= OPS_AMAX[s])) return false;
    return true;
}

// K splits for a GEMM of tiles_mn output tiles over nkb K blocks: the fewest giving at least two waves over the SMs
// with the last wave at least 85% full (else the fullest last wave), each split keeping 8 or more K blocks.
static int choose_ksplit(int tiles_mn, int nkb, int num_sms) {
    int best = 1;
    double best_eff = -1.0;
    const int cap = std::max(1, std::min(64, nkb / 8));
    for (int ks = 1; ks <= cap; ++ks) {
        const long long tiles = (long long)tiles_mn * ks, waves = (tiles + num_sms - 1) / num_sms;
        const double eff = (double)tiles / (double)(waves * num_sms);
        if (tiles >= 2LL * num_sms && eff >= 0.85) return ks;
        if (eff > best_eff + 1e-9) { best_eff = eff; best = ks; }
    }
    return best;
}

// The interpolated fold of n models into the template GEMM's operand (d_vhi / d_vlo) and the sums: per chunk of
// models the operand X, the young and old split-K GEMMs against the operator basis, their reduction.
// Chabrier 2003's mass between m1 and m2 (imf_integral case 1, mass-weighted: src/physics/opensps_imf.f90:234-242):
// the lognormal per unit ln m, exp(-(log10 m - log10 0.08)^2 / (2 sigma^2)) with sigma = 0.69, below 1 M_sun (times m:
// a lognormal of centre log10 0.08 + ln 10 sigma^2, scale exp(ln 10 log10 0.08 + (ln 10 sigma)^2 / 2), in closed form
// with erf), and the power law exp(-(log10 0.08)^2 / (2 sigma^2)) m^-2.3 above. FP64, host.
static double chabrier_mass(double m1, double m2) {
    const double K = std::log(10.0), lmc = std::log10(0.08), s2 = 0.69 * 0.69, sig = 0.69;
    double v = 0.0;
    const double a = m1, b = std::min(m2, 1.0);
    if (b > a) {
        const double centre = lmc + K * s2, scale = std::exp(K * lmc + 0.5 * K * K * s2);
        const double z1 = (std::log10(a) - centre) / (sig * std::sqrt(2.0)), z2 = (std::log10(b) - centre) / (sig * std::sqrt(2.0));
        v += scale * K * sig * std::sqrt(0.5 * M_PI) * (std::erf(z2) - std::erf(z1));
    }
    const double lo = std::max(m1, 1.0);
    if (m2 > lo) v += std::exp(-lmc * lmc / (2.0 * s2)) * (std::pow(m2, -0.3) - std::pow(lo, -0.3)) / -0.3;
    return v;
}

static int run_ops_interp(Context &c, int n, const double *d_wz, const double *d_alpha, int itesc, std::string &err) {
    SspOps &o = c.ops;
    cudaStream_t st = c.stream;
    cudaError_t e;
    const int nt = c.nt, nz = c.nz, R = o.interp_R;
    const size_t ktot = (size_t)nt * nz * R;
    if (nt * nz > OPS_IMAXG || (size_t)nt * nz * (R / 8) >= (1u << 20)) { err = "operator grid too large for the interpolated fold"; return ST_UNSUPPORTED; }
    const int chunk = std::min(n, 4096);
    const int ky = itesc * nz * R, ko = (nt - itesc) * nz * R;
    const int tiles_mn = ((chunk + gemm_bm() - 1) / gemm_bm()) * ((o.ntempl + gemm_bn() - 1) / gemm_bn());
    const int ks_y = ky > 0 ? choose_ksplit(tiles_mn, (ky + gemm_bk() - 1) / gemm_bk(), c.num_sms) : 0;
    const int ks_o = ko > 0 ? choose_ksplit(tiles_mn, (ko + gemm_bk() - 1) / gemm_bk(), c.num_sms) : 0;
    if ((e = c.d_ix_hi.reserve((size_t)chunk * ktot)) != cudaSuccess || (e = c.d_ix_lo.reserve((size_t)chunk * ktot)) != cudaSuccess ||
        (e = c.d_ix_const.reserve((size_t)n)) != cudaSuccess ||
        (e = c.d_ipart.reserve((size_t)std::max(ks_y + ks_o, 1) * chunk * o.ntpad)) != cudaSuccess) {
        err = cmsg("device memory", e);
        return ST_DATA_MISSING;
    }
    const double fixed_it = c.imf_type == 1 ? 1.0 / chabrier_mass(0.08, 120.0) : 0.0;
    ops_interp_const_kernel<<<(n + 127) / 128, 128, 0, st>>>(d_alpha, n, 0.08f, 120.f, fixed_it, c.d_ix_const.p);
    if ((e = cudaGetLastError()) != cudaSuccess) { err = cmsg("interpolated fold constants kernel", e); return ST_DATA_MISSING; }
    c.ops_launches += 1;
    for (int m0 = 0; m0 < n; m0 += chunk) {
        const int rows = std::min(chunk, n - m0);
        OpsInterpArgs xa;
        xa.m0 = m0; xa.nt = nt; xa.nz = nz; xa.R = R; xa.ktot = (int)ktot; xa.itesc = itesc;
        xa.rg_magic = (unsigned)((0x100000000ULL + (unsigned)(R / 8) - 1) / (unsigned)(R / 8));
        for (int s = 0; s < 3; ++s) {
            xa.noff[s] = o.interp_noff[s]; xa.nn[s] = o.interp_nn[s]; xa.x0[s] = o.interp_x0[s]; xa.h[s] = o.interp_h[s];
        }
        xa.lim_lo = 0.08f; xa.lim_hi = 120.f; xa.imf_type = c.imf_type;
        xa.wz = d_wz; xa.alpha = d_alpha; xa.kconst = c.d_ix_const.p; xa.mrow = o.i_mrow.p; xa.lrow = o.i_lrow.p;
        xa.x_hi = c.d_ix_hi.p; xa.x_lo = c.d_ix_lo.p; xa.sums = c.d_sums.p;
        ops_interp_x_kernel<<<rows, OPS_IX_THREADS, 0, st>>>(xa);
        c.ops_launches += 2 + (ky > 0 ? 1 : 0) + (ko > 0 ? 1 : 0);   // operand, GEMMs, reduction
        if ((e = cudaGetLastError()) != cudaSuccess) { err = cmsg("interpolated fold operand kernel", e); return ST_DATA_MISSING; }
        const size_t per = (size_t)rows * o.ntpad;
        for (int part = 0; part < 2; ++part) {
            const int K = part ? ko : ky, ks = part ? ks_o : ks_y;
            if (K <= 0) continue;
            const size_t c0 = part ? (size_t)ky : 0;
            GemmPlan pl;
            pl.num_sms = c.num_sms;
            if ((e = encode_tmap_2d_16s(&pl.tm_a_hi, c.d_ix_hi.p + c0, K, rows, ktot, gemm_bk(), gemm_bm(), false)) != cudaSuccess ||
                (e = encode_tmap_2d_16s(&pl.tm_a_lo, c.d_ix_lo.p + c0, K, rows, ktot, gemm_bk(), gemm_bm(), false)) != cudaSuccess ||
                (e = encode_tmap_2d_16s(&pl.tm_b_hi, o.ib_hi.p + c0, K, o.ntempl, ktot, gemm_bk(), gemm_bn(), false)) != cudaSuccess ||
                (e = encode_tmap_2d_16s(&pl.tm_b_lo, o.ib_lo.p + c0, K, o.ntempl, ktot, gemm_bk(), gemm_bn(), false)) != cudaSuccess) {
                err = cmsg("interpolated fold tensor map", e);
                return ST_DATA_MISSING;
            }
            GemmArgs g;
            g.M = rows; g.N = o.ntempl; g.K = K; g.ldd = o.ntpad; g.b_row0 = 0; g.status = c.d_status.p;
            g.D = c.d_ipart.p + (part ? (size_t)ks_y * per : 0);
            g.ksplit = ks; g.d_split = (long long)per;
            if ((e = run_gemm_bf16x3(pl, g, st)) != cudaSuccess) { err = cmsg("interpolated fold GEMM", e); return ST_DATA_MISSING; }
        }
        OpsInterpReduceArgs ra;
        ra.n = n; ra.m0 = m0; ra.rows = rows; ra.ntpad = o.ntpad; ra.ntempl = o.ntempl;
        ra.ks_young = ks_y; ra.ks_old = ks_o;
        ra.part_young = c.d_ipart.p; ra.part_old = c.d_ipart.p + (size_t)ks_y * per;
        ra.v_hi = c.d_vhi.p; ra.v_lo = c.d_vlo.p;
        const size_t n4 = 2 * per / 4;
        ops_interp_reduce_kernel<<<(unsigned)std::min<size_t>((n4 + 255) / 256, 4096), 256, 0, st>>>(ra);
        if ((e = cudaGetLastError()) != cudaSuccess) { err = cmsg("interpolated fold reduce kernel", e); return ST_DATA_MISSING; }
    }
    return 0;
}

// The young and old sums of n models (d_wz: their SFH weights over ages and metallicities, d_alpha / h_alpha: n x 3
// Kroupa slopes on the device / host) through the operator: the fold (interpolated when every model's slopes allow,
// else exact), then the template GEMM into d_young / d_old (n x nspec each, contiguous: d_old = d_young + n nspec);
// the mass and L_bol sums into the context's sums (n x 6).
int run_ops_parts(Context &c, int n, const double *d_wz, const double *d_alpha, const double *h_alpha, int itesc,
                  float *d_young, float *d_old, std::string &err) {
    SspOps &o = c.ops;
    cudaStream_t st = c.stream;
    cudaError_t e;
    const int ngroups = (n + 3) / 4;
    const bool interp = ops_interp_ok(c, h_alpha, n);
    OpsImfLim lim;
    if (!interp)
        if (int rc = ops_imf_limits(c, c.imf_type, lim, err)) return rc;
    if ((e = c.d_vhi.reserve((size_t)2 * n * o.ntpad)) != cudaSuccess ||
        (e = c.d_vlo.reserve((size_t)2 * n * o.ntpad)) != cudaSuccess || (e = c.d_sums.reserve((size_t)6 * n)) != cudaSuccess ||
        (!interp && (e = c.d_vpart.reserve((size_t)c.nz * 2 * n * o.ntpad)) != cudaSuccess) ||
        (!interp && (e = c.d_spart.reserve((size_t)c.nz * n * 4)) != cudaSuccess) ||
        (!interp && (e = c.d_vflag.reserve((size_t)c.nz * ngroups)) != cudaSuccess)) {
        err = cmsg("device memory", e);
        return ST_DATA_MISSING;
    }
    c.ops_last_interp = interp;
    c.ops_launches = 1;                  // (the template GEMM)
    if (interp) {
        if (int rc = run_ops_interp(c, n, d_wz, d_alpha, itesc, err)) return rc;
    } else {
    c.ops_launches += 2;                 // the fold and its slab reduction
    OpsFoldArgs fa;
    fa.n = n; fa.nt = c.nt; fa.nz = c.nz; fa.npt = o.npt; fa.nent = o.nent; fa.ntpad = o.ntpad; fa.itesc = itesc;
    fa.imf_type = c.imf_type;
    fa.lim = lim;
    fa.wz = d_wz; fa.alpha = d_alpha; fa.pts = o.pts.p; fa.ent = o.ent.p; fa.ent_c = o.ent_c.p;
    fa.v_hi = c.d_vhi.p; fa.v_lo = c.d_vlo.p; fa.sums = c.d_sums.p;
    fa.vpart = c.d_vpart.p; fa.spart = c.d_spart.p; fa.flag = c.d_vflag.p;
    if ((e = run_ops_fold(fa, st)) != cudaSuccess) { err = cmsg("operator fold kernel", e); return ST_DATA_MISSING; }
    }
    GemmPlan pl;
    pl.num_sms = c.num_sms;
    pl.tm_b_hi = o.tm_lib_hi;
    pl.tm_b_lo = o.tm_lib_lo;
    if ((e = encode_tmap_2d_bf16(&pl.tm_a_hi, c.d_vhi.p, o.ntpad, 2 * n, gemm_bk(), gemm_bm())) != cudaSuccess ||
        (e = encode_tmap_2d_bf16(&pl.tm_a_lo, c.d_vlo.p, o.ntpad, 2 * n, gemm_bk(), gemm_bm())) != cudaSuccess) {
        err = cmsg("template tensor map", e);
        return ST_DATA_MISSING;
    }
    GemmArgs g;
    g.M = 2 * n; g.N = c.nspec; g.K = o.ntpad; g.ldd = c.nspec; g.b_row0 = 0; g.D = d_young; g.status = c.d_status.p;
    if (d_old != d_young + (size_t)n * c.nspec) { err = "operator parts: the old sums must follow the young"; return ST_BAD_ARG; }
    if ((e = run_gemm_bf16x3(pl, g, st)) != cudaSuccess) { err = cmsg("template GEMM", e); return ST_DATA_MISSING; }
    return 0;
}

// The operator kernels' three IMF parameters of a model from imf1, imf2, imf3, vdmc, mdave (pv): Kroupa the slopes,
// Salpeter the Kroupa form with the slopes 2.35 (Chabrier: not read), van Dokkum vdmc, Dave imf1, imf2 and mdave.
void imf_pack(int imf_type, const double *pv, double *ap) {
    ap[0] = pv[0]; ap[1] = pv[1]; ap[2] = pv[2];
    if (imf_type == 0 || imf_type == 1) ap[0] = ap[1] = ap[2] = 2.35;
    else if (imf_type == 3) { ap[0] = pv[3]; ap[1] = ap[2] = 0.0; }
    else if (imf_type == 4) ap[2] = pv[4];
}

// The user IMF (imf_type 5) from imf_filename under the data root, imf.dat when none is set (ssp_gen,
// src/physics/opensps_ssp.f90:1756-1808): rows of lower mass, upper mass and slope, read up to the first row that
// does not hold three numbers, at most 100. Read again when the name changes. 0, or ST_IMF_FILE with err.
static int load_user_imf(Context &c, std::string &err) {
    const std::string path = data_root() + "/" + (c.imf_filename.empty() ? std::string("imf.dat") : c.imf_filename);
    if (c.user_imf_file == path && !c.user_imf.empty()) return 0;
    std::ifstream f(path);
    if (!f) { err = "imf_type 5: cannot open the user IMF " + path; return ST_IMF_FILE; }
    std::vector<double> seg;
    std::string line;
    while (seg.size() < 300 && std::getline(f, line)) {
        if (line.find_first_not_of(" \t\r") == std::string::npos) continue;   // (a blank line: the next is read)
        for (char &ch : line)
            if (ch == ',') ch = ' ';
        std::istringstream is(line);
        double lo, hi, al;
        if (!(is >> lo >> hi >> al)) break;
        seg.insert(seg.end(), {lo, hi, al});
    }
    if (seg.empty()) { err = "imf_type 5: the user IMF " + path + " has no segments"; return ST_IMF_FILE; }
    c.user_imf.swap(seg);
    c.user_imf_file = path;
    c.user_imf_dirty = true;
    return 0;
}

int ops_imf_limits(Context &c, int imf_type, OpsImfLim &lim, std::string &err) {
    lim = OpsImfLim();
    lim.lim_lo = c.imf_lim_lo;
    lim.lim_hi = c.imf_lim_hi;
    lim.lb = (float)c.imf_lim_lo;   // (each age's first bin starts at the lower limit: non-Geneva isochrones)
    lim.custom = (c.imf_lim_lo != 0.08 || c.imf_lim_hi != 120.0) ? 1 : 0;
    if (imf_type != 5) return 0;
    if (int rc = load_user_imf(c, err)) return rc;
    const int n = (int)(c.user_imf.size() / 3);
    const double *u = c.user_imf.data();
    // the limits become the first segment's lower and the last one's upper mass (the first bin's edge stays)
    lim.lim_lo = u[0];
    lim.lim_hi = u[3 * (n - 1) + 1];
    std::vector<float> t((size_t)5 * n);
    double cu = 1.0, total = 0.0;
    for (int s = 0; s < n; ++s) {
        const double lo = u[3 * s], hi = u[3 * s + 1], al = u[3 * s + 2];
        if (s > 0) cu *= std::pow(lo, -u[3 * s - 1] + al);   // continuous at the segment's lower mass
        const double e = 1.0 - al;
        t[5 * s] = (float)lo; t[5 * s + 1] = (float)hi; t[5 * s + 2] = (float)e;
        t[5 * s + 3] = e != 0.0 ? (float)(cu / e) : 0.f; t[5 * s + 4] = (float)cu;
        const double a = std::max(lo, lim.lim_lo), b = std::min(hi, lim.lim_hi), em = 2.0 - al;
        if (b > a) total += em == 0.0 ? cu * std::log(b / a) : cu * (std::pow(b, em) - std::pow(a, em)) / em;
    }
    cudaError_t e;
    // (a new table once the stream's earlier work, which may read the old one, is done)
    if (c.user_imf_dirty &&
        ((e = cudaStreamSynchronize(c.stream)) != cudaSuccess || (e = c.d_user_imf.reserve(t.size())) != cudaSuccess ||
         (e = cudaMemcpy(c.d_user_imf.p, t.data(), sizeof(float) * t.size(), cudaMemcpyHostToDevice)) != cudaSuccess)) {
        err = cmsg("user IMF upload", e);
        return ST_DATA_MISSING;
    }
    c.user_imf_dirty = false;
    lim.user = c.d_user_imf.p;
    lim.nuser = n;
    lim.user_inv_total = total > 0.0 ? 1.0 / total : 1.0;
    lim.custom = 1;
    return 0;
}

// One IMF's SSP grid at the context's metallicity zmet: every age as a "model" with a unit weight there.
int ops_evaluate(Context &c, int imf_type, const double *imf_params, double *mass_grid, double *lbol_grid,
                 double *spec_grid, std::string &err) {
    if (!c.ops.ready) { err = "no SSP operators on the context (opensps_context_build_ssp_ops)"; return ST_NO_OPERATOR; }
    if (imf_type < 0 || imf_type > 5) {
        err = "imf_type " + std::to_string(imf_type) + ": the IMF types are 0 to 5";
        return ST_UNSUPPORTED;
    }
    // (the operator batch takes the context's imf_type: this IMF for the call)
    struct ImfTypeScope {
        Context &c;
        int saved;
        ~ImfTypeScope() { c.imf_type = saved; }
    } imf_scope{c, c.imf_type};
    c.imf_type = imf_type;
    const int nt = c.nt, nz = c.nz, ns = c.nspec;
    const int z = std::max(1, std::min(c.zmet, nz)) - 1;
    std::vector<double> wz((size_t)nt * nt * nz, 0.0), alpha((size_t)3 * nt);
    // imf_params: imf1, imf2, imf3, vdmc, mdave
    double pv[5] = {c.pdef[PF_IMF1], c.pdef[PF_IMF2], c.pdef[PF_IMF3], c.pdef[PF_VDMC], c.pdef[PF_MDAVE]};
    if (imf_params)
        for (int j = 0; j < 5; ++j) pv[j] = imf_params[j];
    double ap[3];
    imf_pack(imf_type, pv, ap);
    const double a1 = ap[0], a2 = ap[1], a3 = ap[2];
    for (int t = 0; t < nt; ++t) {
        wz[(size_t)nt * nz * t + t + (size_t)nt * z] = 1.0;
        alpha[3 * t] = a1; alpha[3 * t + 1] = a2; alpha[3 * t + 2] = a3;
    }
    cudaError_t e;
    cudaStream_t st = c.stream;
    if ((e = c.d_wz.reserve(wz.size())) != cudaSuccess || (e = c.d_alpha.reserve(alpha.size())) != cudaSuccess ||
        (e = c.d_yo.reserve((size_t)2 * nt * ns + 4)) != cudaSuccess ||
        (e = cudaMemcpyAsync(c.d_wz.p, wz.data(), sizeof(double) * wz.size(), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(c.d_alpha.p, alpha.data(), sizeof(double) * alpha.size(), cudaMemcpyHostToDevice, st)) != cudaSuccess) {
        err = cmsg("operator inputs", e);
        return ST_DATA_MISSING;
    }
    cudaMemsetAsync(c.d_status.p, 0, sizeof(int), st);
    // every age young (itesc = nt): the spectra are the young sums
    int rc = run_ops_parts(c, nt, c.d_wz.p, c.d_alpha.p, alpha.data(), nt, c.d_yo.p, c.d_yo.p + (size_t)nt * ns, err);
    if (rc) return rc;
    std::vector<float> y((size_t)nt * ns);
    std::vector<double> sums((size_t)6 * nt);
    int kstatus = 0;
    if ((e = cudaMemcpyAsync(y.data(), c.d_yo.p, sizeof(float) * y.size(), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(sums.data(), c.d_sums.p, sizeof(double) * sums.size(), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(&kstatus, c.d_status.p, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess) {
        err = cmsg("operator evaluation", e);
        return ST_DATA_MISSING;
    }
    if (kstatus != 0) {
        char buf[96];
        std::snprintf(buf, sizeof buf, "a device wait gave up (code 0x%x)", kstatus);
        err = buf;
        return ST_DATA_MISSING;
    }
    for (int t = 0; t < nt; ++t) {
        if (mass_grid) mass_grid[t] = sums[(size_t)6 * t];
        if (lbol_grid) lbol_grid[t] = sums[(size_t)6 * t + 1] > SAFE_FLOOR ? std::log10(sums[(size_t)6 * t + 1]) : 0.0;
        if (spec_grid)
            for (int p = 0; p < ns; ++p) spec_grid[(size_t)ns * t + p] = (double)y[(size_t)ns * t + p];
    }
    return 0;
}

}  // namespace sps
