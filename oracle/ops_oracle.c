/*
 * FP64 CPU restatement of OpenSPS's SSP operator applied to per-model IMF weights (test infrastructure: the oracle
 * the GPU's operator path is checked against; never part of the product).
 *
 *   compute_imf_weights      src/physics/opensps_imf.f90:111-172  (bin edges halfway between the isochrone masses,
 *                            the first from the IMF's lower bound, the last at the last mass; points outside the
 *                            IMF mass limits weigh nothing; normalised by the IMF's mass over the limits)
 *   imf_integral (Kroupa)    src/physics/opensps_imf.f90:206-315, case 2 (segments 0.08-0.5-1.0, slopes alpha1-3)
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

/* The IMF weights of one grid point's isochrone points (npt), normalised by the IMF's mass over its limits. */
static void imf_weights(const oracle_ops_t *op, const double *mini, const double *a, double inv_total, double *w) {
    const int n = op->npt;
    for (int i = 0; i < n; ++i) {
        w[i] = 0.0;
        if (mini[i] < op->lim_lo || mini[i] > op->lim_hi) continue;
        const double m1 = (i == 0) ? op->lower_bound : mini[i] - 0.5 * (mini[i] - mini[i - 1]);
        const double m2 = (i == n - 1) ? mini[i] : mini[i] + 0.5 * (mini[i + 1] - mini[i]);
        if (m2 <= m1) continue;
        w[i] = oracle_kroupa_integral(a, m1, m2, 0) * inv_total;
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
            const double total = oracle_kroupa_integral(a, op->lim_lo, op->lim_hi, 1);
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
