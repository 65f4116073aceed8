/*
 * FP64 CPU oracle of the batched CSP hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker for the GPU path: only the tests, the smoke
 * check and the CPU-baseline leg of the benchmark load it. The product (libopensps_gb300) never
 * links, loads or calls it, and has no CPU fallback.
 *
 * It restates, in plain C with FP64 arithmetic (the reference's FP64 build, KP = WP), the algorithm
 * of OpenSPS's compute_csp_batch for the path it covers. Every function names the reference
 * routine (file:line, paths inside the OpenSPS source tree) that it follows. OpenMP parallelises
 * over models (each model is independent, as in the reference).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

#define SAFE_FLOOR DBL_MIN                 /* src/core/opensps_constants.f90:192 tiny(1.0_wp) */
#define C_LIGHT 2.99792458e18              /* src/core/opensps_constants.f90:41 [A/s] */
#define V_BAND 5500.0                      /* src/physics/opensps_dust.f90:47 */
#define H_PLANCK 6.62607015e-27            /* src/core/opensps_constants.f90:35 [erg s] */
#define L_SUN 3.828e33                     /* src/core/opensps_constants.f90:50 [erg/s] */
#define AB_ZEROPOINT 48.60                 /* src/spectra/opensps_batch_photometry.f90:40 */
#define LINE_PROFILE_CUT 1.0e-14           /* src/physics/opensps_gas.f90:354 */
#define N_SIGMA_RANGE 4.0                  /* src/spectra/opensps_smoothing.f90:28 */

/* Madau (1995) IGM constants as tabulated in src/physics/opensps_cosmology.f90:65-95 (published values). */
#define N_LYMAN 17
static const double LY_WAVE[N_LYMAN] = {1215.67, 1025.72, 972.537, 949.743, 937.803, 930.748, 926.226, 923.150,
                                        920.963, 919.352, 918.129, 917.181, 916.429, 915.824, 915.329, 914.919,
                                        914.576};
static const double LY_COEFF[N_LYMAN] = {0.0036, 0.0017, 0.0011846, 0.0009410, 0.0007960, 0.0006967, 0.0006236,
                                         0.0005665, 0.0005200, 0.0004817, 0.0004487, 0.0004200, 0.0003947,
                                         0.000372, 0.000352, 0.0003334, 0.00031644};
#define LYMAN_LIMIT 911.75
#define A_METAL 0.0017
#define MADAU_C1 0.25
#define MADAU_C2 9.4
#define MADAU_C3 0.7
#define MADAU_C4 0.023
#define MADAU_P1 0.46
#define MADAU_P2 0.18
#define MADAU_P3 1.32
#define MADAU_P4 1.68

/* log10(L_sun / (4 pi (10 pc)^2)), src/core/opensps_constants.f90:87 */
static double abs_mag_zeropoint_log(void) {
    const double pi = acos(-1.0);
    const double pc = (648000.0 / pi) * 1.495978707e13;
    return log10(3.828e33 / (4.0 * pi * (10.0 * pc) * (10.0 * pc)));
}

/* find_interval (src/math/opensps_interpolation.f90:152-197): 1-based i with a(i) <= v < a(i+1)
 * by bisection over 0..n+1, ascending or descending; the legacy end cases v == a(1) -> 1 and
 * v == a(n) -> n-1. Returned 1-based like the reference (0 = below an ascending table). */
int oracle_find_interval(const double *a, int n, double v) {
    if (n < 2) return 1;
    int asc = a[n - 1] >= a[0];
    int lower = 0, upper = n + 1;
    while (upper - lower > 1) {
        int mid = (upper + lower) / 2;
        int ge = v >= a[mid - 1];
        if (asc == ge) lower = mid; else upper = mid;
    }
    if (v == a[0]) return 1;
    if (v == a[n - 1]) return n - 1;
    return lower;
}

/* ------------------------------------------------------------------------------------------ */
/* Nebular lines folded into the young SSPs.                                                  */
/* ------------------------------------------------------------------------------------------ */

/* The line profile table gaussnebarr(:, i) of compute_line_gaussians (src/physics/opensps_gas.f90:303-340)
 * with neb_res_min of compute_nebular_kernels (src/core/opensps_initialization.f90:1377-1385), restricted to the
 * window of add_lines_to_spectrum (src/physics/opensps_gas.f90:364-390; the batch path's nebular_setup uses the
 * same cut, src/physics/opensps_csp_batch.f90:1636-1640). Writes prof (nspec) and the 0-based window [*jlo, *jhi]. */
static void line_profile(int nspec, const double *lam, double line_pos, double sigma_kms, double *prof,
                         int *jlo, int *jhi) {
    int j = oracle_find_interval(lam, nspec, line_pos);
    if (j < 1) j = 1;
    if (j > nspec - 1) j = nspec - 1;
    double res_min = lam[j] - lam[j - 1];
    double sig = line_pos * sigma_kms * (1.0e13 / C_LIGHT);
    if (sig < 2.0 * res_min) sig = 2.0 * res_min;
    double norm = (1.0 / (sqrt(2.0 * acos(-1.0)) * sig)) * (line_pos * line_pos / C_LIGHT);
    for (int i = 0; i < nspec; ++i) {
        double x = (lam[i] - line_pos) / sig;
        prof[i] = norm * exp(-0.5 * x * x);
    }
    int jc = oracle_find_interval(lam, nspec, line_pos);
    if (jc < 1) jc = 1;
    if (jc > nspec) jc = nspec;
    int jh = jc + 1 < nspec ? jc + 1 : nspec;   /* 1-based */
    double pk = prof[jc - 1] > prof[jh - 1] ? prof[jc - 1] : prof[jh - 1];
    double cut = LINE_PROFILE_CUT * pk;
    int jl = jc;
    while (jl > 1 && prof[jl - 2] > cut) jl--;
    while (jh < nspec && prof[jh] > cut) jh++;
    *jlo = jl - 1;
    *jhi = jh - 1;
    if (cut <= 0.0) { *jlo = 0; *jhi = -1; }
}

/* The SSP basis with the nebular lines added to every age that has line luminosity (apply_nebular_emission
 * adds the lines of each young SSP before the age sum; the batch path adds the same sum after it,
 * src/physics/opensps_csp_batch.f90:2565-2610 and line_profiles :3133-3166: linear in the weights, so both are
 * the same sums). ssp_in / ssp_out: nspec x nt x nz (pixel fastest); line_lum: nline x nt x nz. */
/* The nebular ranges of a library: whlylim = find_interval(lambda, 912 A) (the pixels 1..whlylim below the Lyman
 * limit, src/core/opensps_initialization.f90:866) and nt_neb, the ages 1..nt_neb with nebular emission (the nebular
 * grid's age range, opensps_csp_batch.f90:1644-1645; here the ages up to the last one with line luminosity). */
void oracle_neb_ranges(int nspec, int nt, int nz, const double *lam, int nline, const double *line_lum, int *nt_neb,
                       int *whlylim) {
    int w = oracle_find_interval(lam, nspec, 912.0);
    *whlylim = w < 0 ? 0 : w;
    int last = 0;
    for (int z = 0; z < nz; ++z)
        for (int t = 0; t < nt; ++t)
            for (int l = 0; l < nline; ++l)
                if (line_lum[l + (size_t)nline * (t + (size_t)nt * z)] != 0.0 && t + 1 > last) last = t + 1;
    *nt_neb = last;
}

void oracle_line_basis(int nspec, int nt, int nz, const double *lam, int nline, const double *line_pos,
                       const double *line_lum, double sigma_kms, const double *ssp_in, double *ssp_out) {
    memcpy(ssp_out, ssp_in, sizeof(double) * (size_t)nspec * nt * nz);
    /* the gas absorbs the ionizing light of the nebular ages (nebular_kernels step 2, opensps_csp_batch.f90:2726-
     * 2750: the age sums at pixels 1..whlylim with the nebular ages times the escaping fraction; its fesc share is
     * added per model in csp_one) */
    int nt_neb = 0, whlylim = 0;
    oracle_neb_ranges(nspec, nt, nz, lam, nline, line_lum, &nt_neb, &whlylim);
    for (int z = 0; z < nz; ++z)
        for (int t = 0; t < nt_neb; ++t)
            for (int i = 0; i < whlylim && i < nspec; ++i) ssp_out[i + (size_t)nspec * (t + (size_t)nt * z)] = 0.0;
    double *prof = (double *)malloc(sizeof(double) * nspec);
    for (int l = 0; l < nline; ++l) {
        int jlo, jhi;
        line_profile(nspec, lam, line_pos[l], sigma_kms, prof, &jlo, &jhi);
        for (int z = 0; z < nz; ++z)
            for (int t = 0; t < nt; ++t) {
                double L = line_lum[l + (size_t)nline * (t + (size_t)nt * z)];
                if (L == 0.0) continue;
                double *col = ssp_out + (size_t)nspec * (t + (size_t)nt * z);
                for (int j = jlo; j <= jhi; ++j) col[j] += prof[j] * L;
            }
    }
    free(prof);
}

/* ------------------------------------------------------------------------------------------ */
/* Cosmology: distance term of the magnitudes.                                                */
/* ------------------------------------------------------------------------------------------ */

/* get_luminosity_distance (src/physics/opensps_cosmology.f90:244-276): trapezoid over 10000 points, [pc]. */
static double lum_distance_pc(double h0, double om0, double ol0, double z) {
    if (z <= 0.0) return 0.0;
    const int N = 10000;
    double dh = ((C_LIGHT * 1.0e-13) / h0) * 1.0e6;
    double dz = z / (double)(N - 1);
    double prev = 1.0 / sqrt(om0 + ol0), sum = 0.0;
    for (int i = 2; i <= N; ++i) {
        double zc = (double)(i - 1) * dz;
        double now = 1.0 / sqrt(om0 * pow(1.0 + zc, 3) + ol0);
        sum += 0.5 * dz * (prev + now);
        prev = now;
    }
    return (1.0 + z) * dh * sum;
}

/* update_cosmology_table (src/physics/opensps_cosmology.f90:286-300): 500 scale factors; zt decreasing. */
double oracle_lum_distance(double h0, double om0, double ol0, double z) { return lum_distance_pc(h0, om0, ol0, z); }

void oracle_cosmo_table(double h0, double om0, double ol0, double *zt, double *dl) {
    for (int i = 1; i <= 500; ++i) {
        double a = (double)(i - 1) / 499.0 * (1.0 - 1.0 / 1001.0) + 1.0 / 1001.0;
        zt[i - 1] = 1.0 / a - 1.0;
        dl[i - 1] = lum_distance_pc(h0, om0, ol0, zt[i - 1]);
    }
}

/* distance_term (src/spectra/opensps_batch_photometry.f90:784-794) with interpolate_linear_scalar
 * (src/math/opensps_interpolation.f90:45-72). */
double oracle_distance_term(const double *zt, const double *dl, double z) {
    if (fabs(z) <= SAFE_FLOOR) return 0.0;
    int idx = oracle_find_interval(zt, 500, z);
    if (idx < 1) idx = 1;
    if (idx > 499) idx = 499;
    double slope = (dl[idx] - dl[idx - 1]) / (zt[idx] - zt[idx - 1]);
    double dm = dl[idx - 1] + slope * (z - zt[idx - 1]);
    if (dm != dm || dm <= SAFE_FLOOR) return 0.0;
    double mz = 1.0 + z;
    return 5.0 * log10(dm / 10.0) + (mz > 0.0 ? -2.5 * log10(mz) : NAN);
}

/* ------------------------------------------------------------------------------------------ */
/* IGM                                                                                         */
/* ------------------------------------------------------------------------------------------ */

/* igm_tau_pixel_terms (src/physics/opensps_cosmology.f90:466-494) */
void oracle_igm_pixel_terms(double w, double *a) {
    for (int k = 0; k < 6; ++k) a[k] = 0.0;
    if (w < LY_WAVE[0]) {
        double ser = 0.0;
        for (int i = 0; i < N_LYMAN; ++i)
            if (w < LY_WAVE[i]) ser += LY_COEFF[i] * pow(LY_WAVE[i], -3.46);
        a[0] = ser * pow(w, 3.46);
        a[1] = A_METAL * pow(w / LY_WAVE[0], 1.68);
    }
    if (w < LYMAN_LIMIT) {
        double s = w / LYMAN_LIMIT;
        a[2] = MADAU_C1 * pow(s, 3.0) * (1.0 - pow(s, MADAU_P1));
        a[3] = MADAU_C2 * pow(s, 1.5) * (1.0 - pow(s, MADAU_P2));
        a[4] = -MADAU_C3 * pow(s, 3.0) * (pow(s, -MADAU_P3) - 1.0);
        a[5] = -MADAU_C4 * (1.0 - pow(s, MADAU_P4));
    }
}

/* igm_tau_z_terms (src/physics/opensps_cosmology.f90:497-508) */
void oracle_igm_z_terms(double opz, double *b) {
    b[0] = pow(opz, 3.46);
    b[1] = pow(opz, 1.68);
    b[2] = pow(opz, 3.0 + MADAU_P1);
    b[3] = pow(opz, 1.5 + MADAU_P2);
    b[4] = pow(opz, 3.0 - MADAU_P3);
    b[5] = pow(opz, MADAU_P4);
}

/* ------------------------------------------------------------------------------------------ */
/* Velocity smoothing operator                                                                 */
/* ------------------------------------------------------------------------------------------ */

typedef struct {
    int *lo, *hi, *off;   /* 0-based; lo = -1: pixel unchanged */
    double *coef;
} vkernel_t;

/* build_velocity_kernel (src/spectra/opensps_smoothing.f90:553-633) */
static void build_velocity_kernel(int n, const double *lam, double sigma, double minl, double maxl, vkernel_t *k) {
    k->lo = (int *)malloc(sizeof(int) * n);
    k->hi = (int *)malloc(sizeof(int) * n);
    k->off = (int *)malloc(sizeof(int) * n);
    int *wlo = (int *)malloc(sizeof(int) * n), *whi = (int *)malloc(sizeof(int) * n);
    for (int i = 0; i < n; ++i) { k->lo[i] = -1; k->hi[i] = -2; k->off[i] = 0; wlo[i] = -1; whi[i] = -2; }
    k->coef = NULL;
    if (n < 2 || sigma <= SAFE_FLOOR) { free(wlo); free(whi); return; }
    double sb = sigma / (C_LIGHT * 1.0e-13);
    double inv2s2 = 0.5 * (1.0 / sb) * (1.0 / sb);
    double fb = exp(-N_SIGMA_RANGE * sb), fr = exp(N_SIGMA_RANGE * sb);
    int il = 1, ih = 1, ntot = 0;   /* 1-based as the reference */
    for (int i = 1; i <= n; ++i) {
        double li = lam[i - 1];
        if (li < minl || li > maxl) continue;
        double vl = li * fb, vh = li * fr;
        while (il > 1 && lam[il - 1] > vl) il--;
        while (il < n && lam[il - 1] < vl) il++;
        if (il > 1 && lam[il - 1] > vl) il--;
        if (ih < il) ih = il;
        while (ih > il && lam[ih - 1] > vh) ih--;
        while (ih < n && lam[ih - 1] < vh) ih++;
        if (ih - il + 1 < 2) continue;
        wlo[i - 1] = il;
        whi[i - 1] = ih;
        ntot += ih - il + 1;
    }
    k->coef = (double *)malloc(sizeof(double) * (ntot > 0 ? ntot : 1));
    double *w = (double *)malloc(sizeof(double) * n);
    ntot = 0;
    for (int i = 1; i <= n; ++i) {
        if (wlo[i - 1] < 0) continue;
        int l0 = wlo[i - 1], h0 = whi[i - 1], nw = h0 - l0 + 1;
        double lli = log(lam[i - 1]);
        for (int m = 0; m < nw; ++m) {
            double d = lli - log(lam[l0 - 1 + m]);
            w[m] = exp(-inv2s2 * d * d) / lam[l0 - 1 + m];
        }
        double tw = 0.0;
        for (int m = 1; m <= nw; ++m) {
            double dl = 0.0, dr = 0.0;
            if (m > 1) dl = lam[l0 + m - 2] - lam[l0 + m - 3];
            if (m < nw) dr = lam[l0 + m - 1] - lam[l0 + m - 2];
            w[m - 1] = 0.5 * w[m - 1] * (dl + dr);
            tw += w[m - 1];
        }
        if (tw <= SAFE_FLOOR) continue;
        k->lo[i - 1] = l0 - 1;
        k->hi[i - 1] = h0 - 1;
        k->off[i - 1] = ntot;
        for (int m = 0; m < nw; ++m) k->coef[ntot + m] = w[m] / tw;
        ntot += nw;
    }
    free(w); free(wlo); free(whi);
}

static void free_vkernel(vkernel_t *k) { free(k->lo); free(k->hi); free(k->off); free(k->coef); }

/* apply_velocity_kernel: smoothed(i) = sum coef * spec(lo..hi) for active rows, unchanged otherwise. */
static void apply_vkernel(const vkernel_t *k, int n, const double *in, double *out) {
    for (int i = 0; i < n; ++i) {
        if (k->lo[i] < 0) { out[i] = in[i]; continue; }
        double s = 0.0;
        const double *c = k->coef + k->off[i];
        for (int j = k->lo[i]; j <= k->hi[i]; ++j) s += c[j - k->lo[i]] * in[j];
        out[i] = s;
    }
}

/* The smoothing coefficient rows of pixel i for sigma (tests compare the GPU's per-model taps with these). */
int oracle_velocity_row(int n, const double *lam, double sigma, double minl, double maxl, int i, int *lo,
                        double *coef, int maxtaps) {
    vkernel_t k;
    build_velocity_kernel(n, lam, sigma, minl, maxl, &k);
    int nt = 0;
    *lo = k.lo[i];
    if (k.lo[i] >= 0) {
        nt = k.hi[i] - k.lo[i] + 1;
        for (int m = 0; m < nt && m < maxtaps; ++m) coef[m] = k.coef[k.off[i] + m];
    }
    free_vkernel(&k);
    return nt;
}

/* ------------------------------------------------------------------------------------------ */
/* The batch                                                                                   */
/* ------------------------------------------------------------------------------------------ */

/* Per-model parameters, in this order (doubles): */
enum { P_DUST1, P_DUST2, P_DUST3, P_DUST_INDEX, P_DUST1_INDEX, P_FRAC_NODUST, P_FRAC_OBRUN, P_ZRED,
       P_IGM_FACTOR, P_SIGMA_SMOOTH, P_DUST_TESC, P_DUSTE_QPAH, P_DUSTE_UMIN, P_DUSTE_GAMMA, P_FAGN, P_AGN_TAU,
       P_GAS_LOGZ, P_GAS_LOGU, P_MWR, P_UVB, P_NPAR };

typedef struct {
    int nspec, nt, nz, nbands;
    const double *lam;       /* nspec */
    const double *log_age;   /* nt */
    const double *basis;     /* nspec x nt x nz, lines already folded in (oracle_line_basis) */
    const double *mass;      /* nt x nz */
    const double *lbol;      /* nt x nz (log10) */
    const double *bands;     /* nspec x nbands */
    const double *zt, *dl;   /* cosmology table (500) */
    int nline;
    const double *line_lum;  /* nline x nt x nz, or NULL */
    int add_igm;             /* add_igm_absorption */
    int smooth;              /* velocity smoothing on (smooth_velocity = 1, smoothspec_fast = 1) */
    double min_wave_smooth, max_wave_smooth;
    /* dust emission (add_dust_emission; dustem NULL: off): the Draine & Li grid, templates nspec x nqpah x 2 numin
     * (pixel fastest; column 2 u + c, c = 0 the U_min delta function, 1 the power law) */
    int nqpah, numin;
    const double *qpah, *umin, *dustem;
    /* the AGN torus (add_agn_dust; agn_spec NULL: off): ntau templates of nspec over the optical depth agn_tau */
    int ntau;
    const double *agn_tau, *agn_spec;
    /* nebular emission (ssp_ion NULL: off): the library's spectra before the lines and the gas absorption (nspec x
     * nt x nz), the nebular ages 1..nt_neb and the ionizing pixels 1..whlylim */
    const double *ssp_ion;
    int nt_neb, whlylim;
    /* the CLOUDY-grid nebular continuum (neb_cont NULL: off): log10 of the continuum per ionizing photon on the
     * spectral grid, nspec x 11 x 10 x 7 (pixel fastest, then log Z, age, log U: nebem_cont(j, z, a, u)), the grid's
     * log Z, log10 age and log U values */
    const double *neb_cont, *neb_logz, *neb_lage, *neb_logu;
    int dust_type;           /* the diffuse curve (dust_type 0 to 6) */
    const double *att_curve; /* dust_type 3 and 5: the table lookup's curve on the grid (nspec; the dusty
                                environments' chosen curve, or the SMC bar), compute_attenuation_curve_point :256-263 */
} oracle_grid_t;

/* ------------------------------------------------------------------------------------------ */
/* The attenuation curves (compute_attenuation_curve_point, src/physics/opensps_dust.f90:237-269): A_lambda / A_V  */
/* of the power law (0), Cardelli, Clayton & Mathis 1989 with R_V = mwr and the bump scaled by uvb (1), Calzetti   */
/* et al. 2000 (2), Kriek & Conroy 2013 with slope dust_index (4), Reddy et al. 2015 (6); each as those papers'     */
/* published forms, with the extensions beyond their ranges the reference takes (its constants, :47-160).          */
/* ------------------------------------------------------------------------------------------ */

/* CCM89 (get_ccm89_curve_point :424-556) at wavenumber x = 1 / lambda[um], as a + b / R_V in each region: the
 * infrared power law from x = 0.1, the optical polynomial in x - 1.82 (1.1 <= x < 3.3), the ultraviolet's linear
 * term with the 2175 A Drude bump scaled by uvb (3.3 <= x < 8) and its far-UV curvature from x = 5.9, the far-UV
 * cubic in x - 8 (x held at 12 beyond); no extinction below x = 0.1. In the near UV (3.3 <= x < 5.9) the gap
 * between the optical and ultraviolet forms at x = 3.3 is added, fading as (3.3 / x)^6. */
static void ccm89_opt(double y, double *a, double *b) {
    static const double ca[8] = {1.0, 0.17699, -0.50447, -0.02427, 0.72085, 0.01979, -0.77530, 0.32999};
    static const double cb[8] = {0.0, 1.41338, 2.28305, 1.07233, -5.38434, -0.62251, 5.30260, -2.09002};
    double pa = 0.0, pb = 0.0;
    for (int k = 7; k >= 0; --k) { pa = pa * y + ca[k]; pb = pb * y + cb[k]; }
    *a = pa;
    *b = pb;
}
static void ccm89_uv(double x, double uvb, double *a, double *b) {
    *a = 1.752 - 0.316 * x + (-0.104 / ((x - 4.67) * (x - 4.67) + 0.341)) * uvb;
    *b = -3.09 + 1.825 * x + (1.206 / ((x - 4.62) * (x - 4.62) + 0.263)) * uvb;
}
double oracle_ccm89(double lam, double rv, double uvb) {
    const double x = 1.0e4 / lam;
    double a, b;
    if (x >= 8.0) {
        const double t = (x < 12.0 ? x : 12.0) - 8.0;
        a = -1.073 + t * (-0.628 + t * (0.137 + t * -0.070));
        b = 13.67 + t * (4.257 + t * (-0.42 + t * 0.374));
        return a + b / rv;
    }
    if (x >= 3.3) {
        ccm89_uv(x, uvb, &a, &b);
        if (x >= 5.9) {
            const double t = x - 5.9;
            a += -0.04473 * t * t - 0.009779 * t * t * t;
            b += 0.2130 * t * t + 0.1207 * t * t * t;
            return a + b / rv;
        }
        double ao, bo, au, bu;
        ccm89_opt(3.3 - 1.82, &ao, &bo);
        ccm89_uv(3.3, uvb, &au, &bu);
        const double gap = (ao + bo / rv) - (au + bu / rv);
        return a + b / rv + gap * pow(3.3 / x, 6.0);
    }
    if (x >= 1.1) {
        ccm89_opt(x - 1.82, &a, &b);
        return a + b / rv;
    }
    if (x >= 0.1) {
        const double p = pow(x, 1.61);
        return 0.574 * p + (-0.527 * p) / rv;
    }
    return 0.0;
}

/* Calzetti et al. 2000 eq. 4 (get_calzetti_curve_point :567-594): k' = 2.659 (poly(x)) + R_V with R_V = 4.05, the
 * UV-optical cubic below 0.63 um and the linear law above, both extended past 0.12-2.2 um, k' clipped at 0;
 * A / A_V = k' / R_V. */
double oracle_calzetti(double lam) {
    const double x = 1.0e4 / lam;
    const double k = lam > 6300.0 ? 2.659 * (-1.857 + 1.040 * x) + 4.05
                                  : 4.05 + 2.659 * (-2.156 + x * (1.509 + x * (-0.198 + x * 0.011)));
    return (k > 0.0 ? k : 0.0) / 4.05;
}

/* Kriek & Conroy 2013 (get_kriek_conroy_curve_point :598-626): (k'_Calzetti + E_b D(lambda)) / 4.05 times
 * (lambda / 5500)^delta, the Drude bump D at 2175 A of width 350 A with E_b = 0.85 - 1.9 delta. */
double oracle_kc13(double lam, double delta) {
    const double w = lam * 350.0, d = lam * lam - 2175.0 * 2175.0;
    const double drude = (0.85 - 1.9 * delta) * w * w / (d * d + w * w);
    return (oracle_calzetti(lam) * 4.05 + drude) / 4.05 * pow(lam / V_BAND, delta);
}

/* Reddy et al. 2015 (get_reddy_curve_point :630-662): k = poly(x) + 2.505 (the UV cubic below 0.6 um, x held at
 * 1 / 0.15 um shorter; the optical cubic from 0.6 to 2.85 um with the reference's continuity offset -0.036221981;
 * 0 beyond), A / A_V = k / 2.505. */
double oracle_reddy(double lam) {
    const double x = 1.0e4 / lam;
    double k = 0.0;
    if (lam < 6000.0) {
        const double xc = x < 1.0e4 / 1500.0 ? x : 1.0e4 / 1500.0;
        k = -5.726 + xc * (4.004 + xc * (-0.525 + xc * 0.029)) + 2.505;
    } else if (lam < 28500.0) {
        k = -2.672 + x * (-0.010 + x * (1.532 + x * -0.412)) + 2.505 - 0.036221981;
    }
    return k / 2.505;
}

/* The diffuse curve of one model at lambda (dust_type 3 and 5, table lookups, are not restated). */
double oracle_dust_curve(int dust_type, double lam, double dust_index, double mwr, double uvb) {
    switch (dust_type) {
    case 0: return pow(lam / V_BAND, dust_index);
    case 1: return oracle_ccm89(lam, mwr, uvb);
    case 2: return oracle_calzetti(lam);
    case 4: return oracle_kc13(lam, dust_index);
    case 6: return oracle_reddy(lam);
    default: return NAN;
    }
}


#define NEB_NZ 11
#define NEB_NAGE 10
#define NEB_NU 7

/* get_grid_indices_weights (src/physics/opensps_gas.f90:394-412): the 0-based lower node of val's interval, clamped
 * so that the interval lies in the grid, and the weight clamped to [0, 1]. */
static void grid_cell(const double *grid, int n, double val, int *idx, double *w) {
    int i = oracle_find_interval(grid, n, val);    /* 1-based */
    if (i < 1) i = 1;
    if (i > n - 1) i = n - 1;
    double t = (val - grid[i - 1]) / (grid[i] - grid[i - 1]);
    *idx = i - 1;
    *w = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
}

/* The CLOUDY-grid nebular continuum of one model into its young (y) and old (o) sums (compute_csp_batch's nebular
 * stage with add_neb_continuum, src/physics/opensps_csp_batch.f90):
 *   q0(t, z)          nebular_kernels step 1 (:2672-2712): the ionizing photon rate of each nebular age's SSP, the
 *                     frequency trapezoid of L_nu / nu over pixels 1 .. whlylim, / H_PLANCK * L_SOL
 *   ia, wa, dwa, newr batch_nebular_indices (:1651-1686): per nebular age its CLOUDY age interval, the weight in it,
 *                     the weight's step within the interval and where a new step starts
 *   iz, wz, iu, wu    (:1691-1693) the cell in gas_logz and gas_logu; fabs = 1 - frac_obrun (:1697)
 *   C(t)              step 3 (:2781-2828): the weight times |q fabs| (here with weights over ages and metallicities,
 *                     q0 summed against each age's metallicity weights), divided by its largest value S per model
 *   the continuum     (:2839-2905): per pixel sum_t C(t) 10^lg(t), lg = ra + wa (rb - ra) with ra, rb the bilinear
 *                     (log Z, log U) interpolation at the interval's nodes; exp(ra ln10 + wa dl + ln S) at an
 *                     interval's first age, then times exp(dwa dl) per age (recomputed where a new step starts)
 * wz: nt x nz of the model (age fastest); itesc 1-based (ages t <= itesc young). */
static void neb_continuum(const oracle_grid_t *g, const double *wz, const double *par, int itesc, double *y, double *o) {
    const int ns = g->nspec, nt = g->nt, nz = g->nz, nn = g->nt_neb;
    if (nn < 1) return;
    const double LN10 = log(10.0);
    double *cy = (double *)calloc((size_t)nn, sizeof(double)), *co = (double *)calloc((size_t)nn, sizeof(double));
    double *wa = (double *)calloc((size_t)nn, sizeof(double)), *dwa = (double *)calloc((size_t)nn, sizeof(double));
    int *ia = (int *)calloc((size_t)nn, sizeof(int)), *newr = (int *)calloc((size_t)nn, sizeof(int));
    for (int t = 0; t < nn; ++t) grid_cell(g->neb_lage, NEB_NAGE, g->log_age[t], &ia[t], &wa[t]);
    for (int t = 1; t < nn; ++t) {
        if (ia[t] != ia[t - 1]) continue;
        dwa[t] = wa[t] - wa[t - 1];
        newr[t] = ia[t - 1] != ia[t >= 2 ? t - 2 : 0] || t == 1 || dwa[t] != dwa[t - 1];
    }
    int iz, iu;
    double wzg, wug;
    grid_cell(g->neb_logz, NEB_NZ, par[P_GAS_LOGZ], &iz, &wzg);
    grid_cell(g->neb_logu, NEB_NU, par[P_GAS_LOGU], &iu, &wug);
    const double fabs_ = 1.0 - par[P_FRAC_OBRUN];
    double cmax = 0.0;
    for (int t = 0; t < nn; ++t) {
        double c = 0.0;
        for (int z = 0; z < nz; ++z) {
            const double w = wz[t + (size_t)nt * z];
            if (!(w > SAFE_FLOOR)) continue;
            /* step 1: the photon-number trapezoid of this SSP below 912 A */
            const double *b = g->ssp_ion + (size_t)ns * (t + (size_t)nt * z);
            double s = 0.0;
            for (int i = 0; i + 1 < g->whlylim && i + 1 < ns; ++i) {
                const double n0 = C_LIGHT / g->lam[i], n1 = C_LIGHT / g->lam[i + 1];
                s += 0.5 * fabs(n1 - n0) * (b[i] / n0 + b[i + 1] / n1);
            }
            const double q = fabs(s / H_PLANCK * L_SUN * fabs_);
            if (q > SAFE_FLOOR) c += w * q;
        }
        if (t + 1 <= itesc) cy[t] = c; else co[t] = c;
        if (c > cmax) cmax = c;
    }
    if (cmax > 0.0) {
        const double lns = log(cmax);
        for (int t = 0; t < nn; ++t) { cy[t] /= cmax; co[t] /= cmax; }
        const double c00 = (1.0 - wzg) * (1.0 - wug), c01 = (1.0 - wzg) * wug, c10 = wzg * (1.0 - wug), c11 = wzg * wug;
#define NEBC(j, z, a, u) g->neb_cont[(j) + (size_t)ns * ((z) + NEB_NZ * ((a) + (size_t)NEB_NAGE * (u)))]
        for (int j = 0; j < ns; ++j) {
            double ys = 0.0, os = 0.0, sy = 0.0, so = 0.0, ra = 0.0, rb = 0.0, dl = 0.0, f = 0.0, r = 1.0;
            int a_prev = -1;
            for (int t = 0; t < nn; ++t) {
                const int a = ia[t];
                if (a != a_prev) {
                    ys += sy; os += so; sy = 0.0; so = 0.0;
                    if (a_prev >= 0 && a == a_prev + 1)   /* (0-based intervals: the first one has no predecessor) */
                        ra = rb;
                    else
                        ra = c00 * NEBC(j, iz, a, iu) + c01 * NEBC(j, iz, a, iu + 1) + c10 * NEBC(j, iz + 1, a, iu) +
                             c11 * NEBC(j, iz + 1, a, iu + 1);
                    rb = c00 * NEBC(j, iz, a + 1, iu) + c01 * NEBC(j, iz, a + 1, iu + 1) + c10 * NEBC(j, iz + 1, a + 1, iu) +
                         c11 * NEBC(j, iz + 1, a + 1, iu + 1);
                    a_prev = a;
                    dl = (rb - ra) * LN10;
                    f = exp(ra * LN10 + wa[t] * dl + lns);
                } else {
                    if (newr[t]) r = exp(dwa[t] * dl);
                    f = f * r;
                }
                sy += cy[t] * f;
                so += co[t] * f;
            }
            y[j] += ys + sy;
            o[j] += os + so;
        }
#undef NEBC
    }
    free(cy); free(co); free(wa); free(dwa); free(ia); free(newr);
}

/* observed_frame_z (src/spectra/opensps_batch_photometry.f90:819-903) for one model: the rest-frame spectrum fin at
 * lambda / (1 + z) by linear interpolation in the interval find_interval gives (the end intervals extrapolate),
 * NaN to 0, negatives to 0, times 1 / lambda; z with |z| <= SAFE_FLOOR reads the pixel itself. */
void oracle_observed_frame(int ns, const double *lam, double zr, const double *fin, double *fobs) {
    for (int j = 0; j < ns; ++j) {
        double v;
        if (fabs(zr) > SAFE_FLOOR) {
            double target = lam[j] / (1.0 + zr);
            int il = oracle_find_interval(lam, ns, target);
            if (il < 1) il = 1;
            if (il > ns - 1) il = ns - 1;
            double t = (target - lam[il - 1]) / (lam[il] - lam[il - 1]);
            v = fin[il - 1] + t * (fin[il] - fin[il - 1]);
        } else {
            v = fin[j];
        }
        if (v != v) v = 0.0;
        fobs[j] = (v > 0.0 ? v : 0.0) * (lam[j] > DBL_MIN ? 1.0 / lam[j] : 0.0);
    }
}

/* band_fluxes (src/spectra/opensps_batch_photometry.f90:1049-1171) for one model and nb bands: band b (its curve
 * bands + ns b) sums the trapezoid terms wt(j) (fobs(j) T(j) + fobs(j + 1) T(j + 1)) over the 1-based pixels j =
 * jlo[b] .. jhi[b] (pixel j + 1 is read, so jhi <= ns - 1); bands with do_band[b] = 0 are exactly 0. wt: ns weights,
 * or NULL for the trapezoid's 0.5 |lambda(j + 1) - lambda(j)| from lam. */
void oracle_band_fluxes(int ns, int nb, const double *bands, const int *jlo, const int *jhi, const int *do_band,
                        const double *wt, const double *lam, const double *fobs, double *fband) {
    for (int b = 0; b < nb; ++b) {
        double s = 0.0;
        if (do_band[b]) {
            const double *bd = bands + (size_t)ns * b;
            for (int j = jlo[b]; j <= jhi[b]; ++j) {
                double w = wt ? wt[j - 1] : 0.5 * fabs(lam[j] - lam[j - 1]);
                s += w * (fobs[j - 1] * bd[j - 1] + fobs[j] * bd[j]);
            }
        }
        fband[b] = s;
    }
}

/* One model of compute_csp_batch (src/physics/opensps_csp_batch.f90:431-1214) with a weight matrix over
 * ages and metallicities (weights_over_z):
 *   model_sums_zw           :2090-2120   mass, L_bol, weights floored at SAFE_FLOOR, young/old at it_tesc
 *   age_sums_w (CPU order)  :2269-2293   metallicities outer, ages inner
 *   attenuate_batch         :3576-3660 with pixel_transmissions :3765-3818 (the curve of dust_type 0, 1, 2, 4, 6)
 *   apply_igm_z             :4205-4299   Madau terms, the short-wavelength cap, exp(-tau igm_factor)
 *   smooth_columns / apply_velocity_kernel (src/spectra/opensps_smoothing.f90)
 *   compute_magnitudes_columns (src/spectra/opensps_batch_photometry.f90:53-180): observed_frame_z :819-903,
 *   band_fluxes :1049-1171 (trapezoid per band support), magnitudes_from_fluxes :185-232 (AB, distance term).
 * work: 4 * nspec doubles. */
static void post_parts(const oracle_grid_t *g, const double *y, const double *o, const double *par, double lsum,
                       double *spec, double *mags, double *fband_out, double *tot, double *tmp);

static void csp_one(const oracle_grid_t *g, const double *wz, const double *par, double *spec, double *mags,
                    double *mass, double *lbol, double *emlines, double *young, double *old, double *fband_out,
                    double *work, int ab_only) {
    const int ns = g->nspec, nt = g->nt, nz = g->nz;
    double *y = work, *o = work + ns, *tot = work + 2 * ns, *tmp = work + 3 * ns;
    /* it_tesc: batch_model_indices :1554-1560 */
    double dla = par[P_DUST_TESC] > SAFE_FLOOR ? par[P_DUST_TESC] : 7.0;
    int itesc = oracle_find_interval(g->log_age, nt, dla);
    if (itesc < 1) itesc = 1;
    if (itesc > nt) itesc = nt;
    double ms = 0.0, ls = 0.0;
    for (int i = 0; i < ns; ++i) { y[i] = 0.0; o[i] = 0.0; }
    if (emlines) for (int l = 0; l < g->nline; ++l) emlines[l] = 0.0;
    for (int z = 0; z < nz; ++z)
        for (int k = 0; k < nt; ++k) {
            double w = wz[k + (size_t)nt * z];
            if (!(w > SAFE_FLOOR)) continue;
            ms += w * g->mass[k + (size_t)nt * z];
            ls += w * pow(10.0, g->lbol[k + (size_t)nt * z]);
            const double *b = g->basis + (size_t)ns * (k + (size_t)nt * z);
            double *col = (k + 1 <= itesc) ? y : o;
            for (int i = 0; i < ns; ++i) col[i] += w * b[i];
            if (g->ssp_ion && k < g->nt_neb) {
                /* the escaping fraction of the nebular ages' ionizing light, fesc = clamp(frac_obrun, 0, 1)
                 * (batch_nebular_indices :1696) */
                const double fesc = fmax(0.0, fmin(par[P_FRAC_OBRUN], 1.0));
                const double *bi = g->ssp_ion + (size_t)ns * (k + (size_t)nt * z);
                for (int i = 0; i < g->whlylim && i < ns; ++i) col[i] += fesc * w * bi[i];
            }
            if (emlines && g->line_lum)
                for (int l = 0; l < g->nline; ++l) emlines[l] += w * g->line_lum[l + (size_t)g->nline * (k + (size_t)nt * z)];
        }
    if (g->neb_cont) neb_continuum(g, wz, par, itesc, y, o);
    if (mass) *mass = ms;
    if (lbol) *lbol = ls > SAFE_FLOOR ? log10(ls) : 0.0;
    if (young) memcpy(young, y, sizeof(double) * ns);
    if (old) memcpy(old, o, sizeof(double) * ns);
    post_parts(g, y, o, par, ls, spec, mags, fband_out, tot, tmp);
    (void)ab_only;
}

/* dl07_indices (src/physics/opensps_csp_batch.f90:1622-1634): the cell of x in the grid g (n values; the lower
 * corner's 0-based index, clamped so that the cell lies in the grid) and the weight, clamped to [0, 1]. */
static void dl07_cell(const double *gr, int n, double x, int *i, double *w) {
    int k = 0;
    while (k < n && gr[k] <= x) ++k;       /* entries <= x (find_interval) */
    if (k < 1) k = 1;
    if (k > n - 1) k = n - 1;
    *i = k - 1;
    double t = (x - gr[k - 1]) / (gr[k] - gr[k - 1]);
    *w = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
}

/* The diffuse curve of a model at pixel i: the table lookup (types 3, 5), the curve functions (1, 2, 4, 6) or the
 * power law (0). */
static double curve_at(const oracle_grid_t *g, int i, const double *par) {
    if (g->dust_type == 3 || g->dust_type == 5) return g->att_curve[i];
    if (g->dust_type != 0) return oracle_dust_curve(g->dust_type, g->lam[i], par[P_DUST_INDEX], par[P_MWR], par[P_UVB]);
    return par[P_DUST_INDEX] != 0.0 ? exp(par[P_DUST_INDEX] * log(g->lam[i] / V_BAND)) : 1.0;
}

/* From the young and old age sums of a model (and its linear L_bol lsum): attenuation, dust emission, IGM, the AGN
 * torus, smoothing, the spectrum and the magnitudes (the stages of compute_csp_batch after the age sums). tot, tmp:
 * nspec doubles of work. */
static void post_parts(const oracle_grid_t *g, const double *y, const double *o, const double *par, double lsum,
                       double *spec, double *mags, double *fband_out, double *tot, double *tmp) {
    const int ns = g->nspec;
    /* attenuation, dust_type 0 (power law) */
    /* (dust_type 3: the diffuse optical depth is the curve itself, pixel_transmissions :3798-3801) */
    double d1 = par[P_DUST1], d2 = g->dust_type == 3 ? 1.0 : par[P_DUST2], d3 = par[P_DUST3], d1i = par[P_DUST1_INDEX];
    double fnd = par[P_FRAC_NODUST], fo = par[P_FRAC_OBRUN];
    /* dust emission (batch_model_indices :1569-1570): models with dust1 or dust2 above SAFE_FLOOR */
    const int emis = g->dustem != NULL && (d1 > SAFE_FLOOR || d2 > SAFE_FLOOR);
    double s_abs = 0.0, s_esc = 0.0, prev_abs = 0.0, prev_esc = 0.0;
    int iq = 0, iu = 0;
    double wq = 0.0, wu = 0.0, gam = 0.0;
    double *esc = NULL;
    if (emis) {
        dl07_cell(g->qpah, g->nqpah, par[P_DUSTE_QPAH], &iq, &wq);
        dl07_cell(g->umin, g->numin, par[P_DUSTE_UMIN], &iu, &wu);
        gam = par[P_DUSTE_GAMMA] < 0.0 ? 0.0 : (par[P_DUSTE_GAMMA] > 1.0 ? 1.0 : par[P_DUSTE_GAMMA]);
        esc = (double *)malloc(sizeof(double) * (size_t)ns);
    }
    for (int i = 0; i < ns; ++i) {
        double ltab = log(g->lam[i] / V_BAND);
        const double curve = curve_at(g, i, par);
        double tau_d = d2 * curve, td = exp(-tau_d);
        double tb = 1.0, too = 1.0, tau_b = 0.0, tau_o = 0.0;
        if (!(d1 <= SAFE_FLOOR || 1.0 - fo <= SAFE_FLOOR)) { tau_b = d1 * exp(d1i * ltab); tb = exp(-tau_b); }
        if (!(fabs(d3) <= SAFE_FLOOR)) { tau_o = d3 * curve; too = exp(-tau_o); }
        double ss = (y[i] * tb * (1.0 - fo) + y[i] * fo) + o[i] * too;
        tot[i] = (1.0 - fnd <= SAFE_FLOOR) ? ss : ss * (td * (1.0 - fnd) + fnd);
        if (emis) {
            /* attenuate_batch :3640-3655: the absorbed light (1 - T of each screen, here -expm1(-tau)), the
             * dl07_shape template :4103-4122 times the diffuse transmission */
            double omb = -expm1(-tau_b), omo = -expm1(-tau_o);
            double omd = (1.0 - fnd <= SAFE_FLOOR) ? 0.0 : (1.0 - fnd) * -expm1(-tau_d);
            double ay = tb * (1.0 - fo) + fo;
            double absorbed = y[i] * ((1.0 - fo) * omb + ay * omd) + o[i] * (omo + too * omd);
            const double *T = g->dustem;
            const size_t sq = (size_t)ns, su = (size_t)ns * g->nqpah;
            const size_t k0 = (size_t)(2 * iu), k1 = (size_t)(2 * (iu + 1));
            double lo = (1 - wq) * (1 - wu) * T[i + sq * iq + su * k0] + wq * (1 - wu) * T[i + sq * (iq + 1) + su * k0] +
                        wq * wu * T[i + sq * (iq + 1) + su * k1] + (1 - wq) * wu * T[i + sq * iq + su * k1];
            double hi = (1 - wq) * (1 - wu) * T[i + sq * iq + su * (k0 + 1)] +
                        wq * (1 - wu) * T[i + sq * (iq + 1) + su * (k0 + 1)] + wq * wu * T[i + sq * (iq + 1) + su * (k1 + 1)] +
                        (1 - wq) * wu * T[i + sq * iq + su * (k1 + 1)];
            double shape = (1.0 - gam) * lo + gam * hi;
            if (shape < DBL_MIN) shape = DBL_MIN;
            esc[i] = shape * td;
            /* dust_emission_reductions :3963-4042: trapezoids in frequency, wt = |nu(i + 1) - nu(i)| / 2 */
            if (i > 0) {
                double wt = 0.5 * fabs(C_LIGHT / g->lam[i] - C_LIGHT / g->lam[i - 1]);
                s_abs += wt * (prev_abs + absorbed);
                s_esc += wt * (prev_esc + esc[i]);
            }
            prev_abs = absorbed;
            prev_esc = esc[i];
        }
    }
    if (emis) {
        /* add_dust_emission :4045-4099 */
        double rn = s_esc > SAFE_FLOOR ? s_abs / s_esc : 0.0;
        if (rn != 0.0) for (int i = 0; i < ns; ++i) tot[i] += esc[i] * rn;
        free(esc);
    }
    /* IGM per model */
    double zr = par[P_ZRED];
    if (g->add_igm && zr > SAFE_FLOOR) {
        int jtop = 0;
        for (int j = 0; j < ns; ++j) if (g->lam[j] < 1215.67) jtop = j + 1;
        if (jtop > 0) {
            double b[6], a[6];
            oracle_igm_z_terms(1.0 + zr, b);
            double tmax = 0.0;
            int jmax = 1;
            for (int j = 0; j < jtop; ++j) {
                oracle_igm_pixel_terms(g->lam[j], a);
                tmp[j] = a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3] + a[4] * b[4] + a[5] * b[5];
                if (tmp[j] > tmax) { tmax = tmp[j]; jmax = j + 1; }
            }
            if (jmax > 1) for (int j = 0; j < jmax; ++j) tmp[j] = tmax;
            for (int j = 0; j < jtop; ++j) tot[j] *= exp(-tmp[j] * par[P_IGM_FACTOR]);
        }
    }
    /* the AGN torus (add_agn_batch :4342-4433; agn_indices :1575-1589): fagn L_bol times the template interpolated
     * in the torus optical depth, times the diffuse transmission */
    if (g->agn_spec != NULL && par[P_FAGN] > SAFE_FLOOR) {
        int ita;
        double wta;
        dl07_cell(g->agn_tau, g->ntau, par[P_AGN_TAU], &ita, &wta);
        double lagn = (lsum > SAFE_FLOOR ? lsum : 1.0) * par[P_FAGN];
        for (int i = 0; i < ns; ++i) {
            const double curve = curve_at(g, i, par);
            double tmpl = (1.0 - wta) * g->agn_spec[(size_t)ns * ita + i] + wta * g->agn_spec[(size_t)ns * (ita + 1) + i];
            tot[i] += lagn * tmpl * exp(-d2 * curve);
        }
    }
    /* velocity smoothing */
    double *fin = tot;
    if (g->smooth && par[P_SIGMA_SMOOTH] > SAFE_FLOOR) {
        vkernel_t vk;
        build_velocity_kernel(ns, g->lam, par[P_SIGMA_SMOOTH], g->min_wave_smooth, g->max_wave_smooth, &vk);
        apply_vkernel(&vk, ns, tot, tmp);
        free_vkernel(&vk);
        fin = tmp;
    }
    if (spec) memcpy(spec, fin, sizeof(double) * ns);

    /* magnitudes */
    if (mags || fband_out) {
        double *fobs = (fin == tmp) ? tot : tmp;   /* reuse the free buffer */
        oracle_observed_frame(ns, g->lam, zr, fin, fobs);
        double dist = oracle_distance_term(g->zt, g->dl, zr);
        double zp = AB_ZEROPOINT + 2.5 * abs_mag_zeropoint_log();
        for (int b = 0; b < g->nbands; ++b) {
            const double *bd = g->bands + (size_t)ns * b;
            int ilo = ns, ihi = 1;
            for (int j = 1; j <= ns; ++j) if (bd[j - 1] != 0.0) { if (j < ilo) ilo = j; if (j > ihi) ihi = j; }
            int jlo = ilo - 1 > 1 ? ilo - 1 : 1, jhi = ihi < ns - 1 ? ihi : ns - 1;
            if (ilo > ihi) { jlo = 1; jhi = 0; }
            const int on = 1;
            double s;
            oracle_band_fluxes(ns, 1, bd, &jlo, &jhi, &on, NULL, g->lam, fobs, &s);
            if (fband_out) fband_out[b] = s;
            if (mags) mags[b] = (s > 0.0 ? -2.5 * log10(s) : NAN) - zp + dist;
        }
    }
}

/* The batch from given young and old age sums (young, old: nspec x n): spectra, magnitudes, band fluxes. */
void oracle_csp_from_parts(const oracle_grid_t *g, int n, const double *young, const double *old, const double *par,
                           const double *lsum, double *spec, double *mags, double *fband) {
    const int ns = g->nspec;
#pragma omp parallel
    {
        double *work = (double *)malloc(sizeof(double) * 2 * (size_t)ns);
#pragma omp for schedule(dynamic, 4)
        for (int m = 0; m < n; ++m)
            post_parts(g, young + (size_t)ns * m, old + (size_t)ns * m, par + (size_t)P_NPAR * m, lsum ? lsum[m] : 0.0,
                       spec ? spec + (size_t)ns * m : NULL, mags ? mags + (size_t)g->nbands * m : NULL,
                       fband ? fband + (size_t)g->nbands * m : NULL, work, work + ns);
        free(work);
    }
}

/* The batch: n models, wz (nt x nz x n), par (P_NPAR x n). Any output may be NULL. */
void oracle_csp_batch(const oracle_grid_t *g, int n, const double *wz, const double *par, double *spec, double *mags,
                      double *mass, double *lbol, double *emlines, double *young, double *old, double *fband) {
    const int ns = g->nspec;
#pragma omp parallel
    {
        double *work = (double *)malloc(sizeof(double) * 4 * (size_t)ns);
#pragma omp for schedule(dynamic, 4)
        for (int m = 0; m < n; ++m) {
            csp_one(g, wz + (size_t)g->nt * g->nz * m, par + (size_t)P_NPAR * m, spec ? spec + (size_t)ns * m : NULL,
                    mags ? mags + (size_t)g->nbands * m : NULL, mass ? mass + m : NULL, lbol ? lbol + m : NULL,
                    emlines ? emlines + (size_t)g->nline * m : NULL, young ? young + (size_t)ns * m : NULL,
                    old ? old + (size_t)ns * m : NULL, fband ? fband + (size_t)g->nbands * m : NULL, work, 0);
        }
        free(work);
    }
}

int oracle_npar(void) { return P_NPAR; }
double oracle_abs_mag_zeropoint_log(void) { return abs_mag_zeropoint_log(); }

/* ------------------------------------------------------------------------------------------ */
/* IMF bin integrals                                                                           */
/* ------------------------------------------------------------------------------------------ */

/* exp(y) - 1 by the Taylor series to y^13 below |y| = 1/4, exp(y) - 1 above (expm1_series,
 * src/physics/opensps_imf.f90:624-650; the same nested multiply-adds). */
double oracle_expm1_series(double y) {
    if (fabs(y) < 0.25) {
        double r = 1.0 + y * (1.0 / 13);
        r = 1.0 + y * (1.0 / 12) * r;
        r = 1.0 + y * (1.0 / 11) * r;
        r = 1.0 + y * (1.0 / 10) * r;
        r = 1.0 + y * (1.0 / 9) * r;
        r = 1.0 + y * (1.0 / 8) * r;
        r = 1.0 + y * (1.0 / 7) * r;
        r = 1.0 + y * (1.0 / 6) * r;
        r = 1.0 + y * (1.0 / 5) * r;
        r = 1.0 + y * (1.0 / 4) * r;
        r = 1.0 + y * (1.0 / 3) * r;
        r = 1.0 + y * (1.0 / 2) * r;
        return y * r;
    }
    return exp(y) - 1.0;
}

/* ln(m2 / m1) as log1p((m2 - m1) / m1) in Kahan's form (imf_bin_logs, src/physics/opensps_imf.f90:564-580). */
double oracle_bin_dl(double m1, double m2) {
    if (m1 <= 0.0 || m2 <= m1) return 0.0;
    double x = (m2 - m1) / m1, u = 1.0 + x;
    return (u == 1.0) ? x : log(u) * x / (u - 1.0);
}

/* The number of stars of a power-law bin, int_lo^hi c m^-alpha dm, in the table form of imf_bin_weights_tab
 * (src/physics/opensps_imf.f90:519-548, FP64 build): c / e * lo^e * expm1(e dl) with e = 1 - alpha, dl = ln(hi/lo);
 * c dl at e = 0. */
double oracle_powerlaw_bin(double alpha, double c, double lo, double hi) {
    double e = 1.0 - alpha;
    double dl = oracle_bin_dl(lo, hi);
    if (e == 0.0) return c * dl;
    double ce = c / e;
    double plo = exp(e * log(lo));
    return ce * plo * oracle_expm1_series(e * dl);
}
