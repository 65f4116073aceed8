/*
 * FP64 CPU restatement of OpenSPS's SSP operator applied to per-model IMF weights (test infrastructure: the oracle
 * the GPU's operator path is checked against; never part of the product).
 *
 *   compute_imf_weights      src/physics/opensps_imf.f90:111-172  (bin edges halfway between the isochrone masses,
 *                            the first from the IMF's lower bound, the last at the last mass; points outside the
 *                            IMF mass limits weigh nothing; normalised by the IMF's mass over the limits)
 *   imf_integral             src/physics/opensps_imf.f90:206-315: case 2 Kroupa (segments 0.08-0.5-1.0, slopes
 *                            alpha1-3), case 0 Salpeter (slope 2.35, opensps_context_types.f90:120), case 1 Chabrier
 *                            2003 (the lognormal below 1 M_sun, integrate_lognormal :677-722, and the power law above),
 *                            case 3 van Dokkum 2008 (the scaled lognormal up to 25 vdmc, the power law above; constants
 *                            :39-44), case 4 Dave 2008 (slopes alpha1 below mdave and alpha2 above, continuous),
 *                            case 5 the user's segments (:287-305: each a power law over its own mass range, scaled
 *                            to be continuous at its lower mass; the limits the first lower and last upper mass,
 *                            src/physics/opensps_ssp.f90:1756-1808)
 *   integrate_powerlaw       src/physics/opensps_imf.f90:725-748 (the expm1 form: oracle_powerlaw_bin)
 *   ssp_op_model_weights / ssp_op_spmv   src/physics/opensps_ssp_operator.f90:1296-1338: W = S . w_IMF with the
 *                            mass and L_bol rows
 *   fold_multi               src/physics/opensps_ssp_batch.f90:3095-3188: the SFH weights folded in, young / old
 *   template_columns         src/physics/opensps_ssp_batch.f90:3247-3385: spectra = library . V
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define SAFE_FLOOR DBL_MIN

double oracle_powerlaw_bin(double alpha, double c, double lo, double hi);   /* opensps_oracle.c */

typedef struct {
    int nspec, nt, nz, npt, ntempl;
    const float *lib;          /* ntempl x nspec */
    const double *mini;        /* nz x nt x npt */
    const int *idx;            /* nz x nt x npt x 4 */
    const double *coef;        /* nz x nt x npt x 4 */
    const double *mcur, *lum;  /* nz x nt x npt */
    double lower_bound, lim_lo, lim_hi;
    int imf_type;              /* 0 Salpeter, 1 Chabrier, 2 Kroupa (alpha per model: imf1-3), 3 van Dokkum (alpha[0]
                                  = vdmc), 4 Dave (alpha = imf1, imf2, mdave), 5 the user's segments */
    int nuser;
    const double *user;        /* nuser x 3: lower mass, upper mass, slope */
} oracle_ops_t;

/* integrate_powerlaw(lo, hi, alpha, mass_weighted, c) */
static double powerlaw(double lo, double hi, double alpha, int mass_weighted, double c) {
    if (hi <= lo) return 0.0;
    return oracle_powerlaw_bin(mass_weighted ? alpha - 1.0 : alpha, c, lo, hi);
}

/* imf_integral for imf_type 2 (Kroupa): number (mass_weighted 0) or mass over [m1, m2] */
double oracle_kroupa_integral(const double *a, double m1, double m2, int mass_weighted) {
    const double lo = fmin(m1, m2), hi = fmax(m1, m2);
    if (hi <= lo) return 0.0;
    const double c2 = pow(0.5, -a[0] + a[1]);
    double v = 0.0;
    double sl = fmax(lo, 0.08), sh = fmin(hi, 0.5);
    if (sh > sl) v += powerlaw(sl, sh, a[0], mass_weighted, 1.0);
    sl = fmax(lo, 0.5); sh = fmin(hi, 1.0);
    if (sh > sl) v += powerlaw(sl, sh, a[1], mass_weighted, c2);
    sl = fmax(lo, 1.0); sh = hi;
    if (sh > sl) v += powerlaw(sl, sh, a[2], mass_weighted, c2);
    return v;
}

/* The lognormal piece of Chabrier 2003, N(m) = exp(-(log10 m - log10 0.08)^2 / (2 0.69^2)) per unit ln m: its number
 * (or mass) over [m1, m2] in closed form, K sigma sqrt(pi / 2) (erf(z2) - erf(z1)) with z = (log10 m - centre) /
 * (sigma sqrt 2) (the mass-weighted form shifts the centre by K sigma^2 and scales by exp(K log_mc + K^2 sigma^2 / 2),
 * K = ln 10); for a bin narrower than 0.1 in z a 5-point Gauss-Legendre rule on exp(-z^2), and erfc in a tail, against
 * the cancellation of erf near 1 (integrate_lognormal, src/physics/opensps_imf.f90:677-722). */
static double lognormal(double m1, double m2, double log_mc, double sigma2, int mass_weighted) {
    const double K = log(10.0), sig = sqrt(sigma2);
    const double centre = mass_weighted ? log_mc + K * sigma2 : log_mc;
    const double scale = mass_weighted ? exp(K * log_mc + 0.5 * K * K * sigma2) : 1.0;
    const double z1 = (log10(m1) - centre) / (sig * sqrt(2.0)), z2 = (log10(m2) - centre) / (sig * sqrt(2.0));
    if (z2 - z1 < 0.1) {
        static const double x[3] = {0.0, 0.5384693101056831, 0.9061798459386640};
        static const double w[3] = {0.5688888888888889, 0.4786286704993665, 0.2369268850561891};
        const double zc = 0.5 * (z1 + z2), zh = 0.5 * (z2 - z1);
        double q = w[0] * exp(-zc * zc);
        for (int k = 1; k < 3; ++k) {
            const double a = zc - zh * x[k], b = zc + zh * x[k];
            q += w[k] * (exp(-a * a) + exp(-b * b));
        }
        return scale * K * sig * sqrt(2.0) * zh * q;
    }
    const double c = scale * K * sig * sqrt(0.5 * acos(-1.0));
    if (z1 >= 0.0) return c * (erfc(z1) - erfc(z2));
    if (z2 <= 0.0) return c * (erfc(-z2) - erfc(-z1));
    return c * (erf(z2) - erf(z1));
}

/* imf_integral by type: number (mass_weighted 0) or mass over [m1, m2]; a: the Kroupa slopes (type 2), vdmc (a[0],
 * type 3) or the Dave slopes and break mass (type 4). */
double oracle_imf_integral(int imf_type, const double *a, double m1, double m2, int mass_weighted) {
    const double lo = fmin(m1, m2), hi = fmax(m1, m2);
    if (hi <= lo) return 0.0;
    if (imf_type == 2) return oracle_kroupa_integral(a, m1, m2, mass_weighted);
    if (imf_type == 0) return powerlaw(lo, hi, 2.35, mass_weighted, 1.0);
    if (imf_type == 1) {
        const double lmc = log10(0.08), s2 = 0.69 * 0.69;
        double v = 0.0;
        if (fmin(hi, 1.0) > lo) v += lognormal(lo, fmin(hi, 1.0), lmc, s2, mass_weighted);
        if (hi > fmax(lo, 1.0)) v += powerlaw(fmax(lo, 1.0), hi, 2.3, mass_weighted, exp(-lmc * lmc / (2.0 * s2)));
        return v;
    }
    if (imf_type == 3) {
        const double vdmc = a[0], br = 25.0 * vdmc, s2 = 0.69 * 0.69;
        double v = 0.0;
        if (fmin(hi, br) > lo)
            v += 0.14 * pow(0.5 * br, -1.3) * lognormal(lo, fmin(hi, br), log10(vdmc), s2, mass_weighted);
        if (hi > fmax(lo, br)) v += powerlaw(fmax(lo, br), hi, 2.3, mass_weighted, 0.0443);
        return v;
    }
    if (imf_type == 4) {
        const double md = a[2];
        double v = 0.0, sl = fmax(lo, 0.08), sh = fmin(hi, md);
        if (sh > sl) v += powerlaw(sl, sh, a[0], mass_weighted, 1.0);
        sl = fmax(lo, md);
        if (hi > sl) v += powerlaw(sl, hi, a[1], mass_weighted, pow(md, -a[0] + a[1]));
        return v;
    }
    return 0.0;
}

/* imf_integral case 5: the user's segments (n x 3: lower mass, upper mass, slope) over [m1, m2] */
double oracle_user_imf_integral(int n, const double *u, double m1, double m2, int mass_weighted) {
    const double lo = fmin(m1, m2), hi = fmax(m1, m2);
    double v = 0.0, cu = 1.0;
    if (hi <= lo) return 0.0;
    for (int s = 0; s < n; ++s) {
        if (s > 0) cu *= pow(u[3 * s], -u[3 * s - 1] + u[3 * s + 2]);
        const double a = fmax(lo, u[3 * s]), b = fmin(hi, u[3 * s + 1]);
        if (b > a) v += powerlaw(a, b, u[3 * s + 2], mass_weighted, cu);
    }
    return v;
}

static double imf_int(const oracle_ops_t *op, const double *a, double m1, double m2, int mass_weighted) {
    if (op->imf_type == 5) return oracle_user_imf_integral(op->nuser, op->user, m1, m2, mass_weighted);
    return oracle_imf_integral(op->imf_type, a, m1, m2, mass_weighted);
}

/* The IMF weights of one grid point's isochrone points (npt), normalised by the IMF's mass over its limits. */
static void imf_weights(const oracle_ops_t *op, const double *mini, const double *a, double inv_total, double *w) {
    const int n = op->npt;
    for (int i = 0; i < n; ++i) {
        w[i] = 0.0;
        if (mini[i] < op->lim_lo || mini[i] > op->lim_hi) continue;
        const double m1 = (i == 0) ? op->lower_bound : mini[i] - 0.5 * (mini[i] - mini[i - 1]);
        const double m2 = (i == n - 1) ? mini[i] : mini[i] + 0.5 * (mini[i + 1] - mini[i]);
        if (m2 <= m1) continue;
        w[i] = imf_int(op, a, m1, m2, 0) * inv_total;
    }
}

/* Per model: the IMF weights of every point whose grid point has an SFH weight, folded with the SFH weights
 * (wz: nt x nz per model, age fastest; ages t < itesc young) into the young and old template vectors, then the
 * young and old spectra (library . V) and the mass and linear L_bol. Outputs n x nspec, n, n. */
void oracle_ops_csp(const oracle_ops_t *op, int n, const double *alpha, const double *wz, int itesc, double *young,
                    double *old, double *mass, double *lsum) {
    const int ns = op->nspec, nt = op->nt, nz = op->nz, npt = op->npt, ne = op->ntempl;
#pragma omp parallel
    {
        double *w = (double *)malloc(sizeof(double) * npt);
        double *vy = (double *)malloc(sizeof(double) * ne), *vo = (double *)malloc(sizeof(double) * ne);
#pragma omp for schedule(dynamic, 1)
        for (int m = 0; m < n; ++m) {
            const double *a = alpha + 3 * (size_t)m;
            const double total = imf_int(op, a, op->lim_lo, op->lim_hi, 1);
            const double inv = total > 0.0 ? 1.0 / total : 1.0;
            memset(vy, 0, sizeof(double) * ne);
            memset(vo, 0, sizeof(double) * ne);
            double ms = 0.0, ls = 0.0;
            for (int z = 0; z < nz; ++z)
                for (int t = 0; t < nt; ++t) {
                    const double s = wz[(size_t)nt * nz * m + t + (size_t)nt * z];
                    if (!(s > SAFE_FLOOR)) continue;
                    const size_t g = (size_t)t + (size_t)nt * z;
                    imf_weights(op, op->mini + g * npt, a, inv, w);
                    double *v = (t < itesc) ? vy : vo;
                    for (int p = 0; p < npt; ++p) {
                        if (w[p] == 0.0) continue;
                        const size_t q = g * npt + p;
                        for (int k = 0; k < 4; ++k) v[op->idx[4 * q + k]] += s * w[p] * op->coef[4 * q + k];
                        ms += s * w[p] * op->mcur[q];
                        ls += s * w[p] * op->lum[q];
                    }
                }
            double *y = young + (size_t)ns * m, *o = old + (size_t)ns * m;
            for (int i = 0; i < ns; ++i) { y[i] = 0.0; o[i] = 0.0; }
            for (int e = 0; e < ne; ++e) {
                const float *le = op->lib + (size_t)ns * e;
                if (vy[e] != 0.0) for (int i = 0; i < ns; ++i) y[i] += vy[e] * (double)le[i];
                if (vo[e] != 0.0) for (int i = 0; i < ns; ++i) o[i] += vo[e] * (double)le[i];
            }
            mass[m] = ms;
            lsum[m] = ls;
        }
        free(w); free(vy); free(vo);
    }
}
