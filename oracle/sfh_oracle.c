/*
 * FP64 CPU restatement of OpenSPS's SFH weights and current SFR (test infrastructure: the oracle the GPU's SFH
 * kernel is checked against; never part of the product).
 *
 *   expi                       src/math/opensps_special_functions.f90:62-122
 *   gammainc (powers 1, 2)     src/math/opensps_special_functions.f90:142-170
 *   convert_sfhparams_pc       src/physics/opensps_sfh.f90:1306-1360
 *   eval_indefinite_moments_log (types 0, 1, 4, 5)  src/physics/opensps_sfh.f90:852-905
 *   compute_ssp_weights        src/physics/opensps_sfh.f90:97-257 (log-age interpolation, interpolation_type 0; the
 *                              Simha window [t0, tq] of clamp_integration_limits :969-1010)
 *   sfh_weights_core_pc        src/physics/opensps_sfh.f90:1077-1212 (sfh 0, 1, 4 with const / burst; sfh 5, the
 *                              delayed tau before the truncation and the linear ramp after it, mixed by the linear
 *                              mass fraction)
 *   get_sfh_properties_at_age_pc  src/physics/opensps_sfh.f90:281-486 (sfh 0, 1, 4, 5), as batch_model_indices
 *                              src/physics/opensps_csp_batch.f90:1558-1567 divides it by the mass fraction
 *
 * Times: time_full = log10(age / yr) of the SSP grid (ascending), tiny_logt = 0 (the context default), years in
 * the weights, Gyr in the parameters.
 */
#include <float.h>
#include <math.h>
#include <string.h>

#define SAFE_FLOOR DBL_MIN
#define EULER_GAMMA 0.57721566490153286060651209008240243104215933593992
#define LOG_E 0.43429448190325182765   /* log10(e) */

int oracle_find_interval(const double *a, int n, double v);   /* opensps_oracle.c */

/* Ei(x): the power series about 0 for x <= 40, the asymptotic series (20 terms) beyond. */
double oracle_expi(double x) {
    if (x == 0.0) return -INFINITY;
    if (x < 0.0) return NAN;
    if (fabs(x) <= 40.0) {
        double res = 1.0, r = 1.0;
        for (int k = 1; k <= 1000; ++k) {
            const double d = (double)k + 1.0;
            r = (r * (double)k * x) / (d * d);
            res += r;
            if (fabs(r) <= 1.0e-20 * fabs(res)) break;
            if (k == 1000) return NAN;
        }
        return EULER_GAMMA + log(x) + x * res;
    }
    double res = 1.0, r = 1.0;
    const double inv = 1.0 / x;
    for (int k = 1; k <= 20; ++k) {
        r *= (double)k * inv;
        res += r;
    }
    return exp(x) * inv * res;
}

/* The regularised lower incomplete gamma function for powers 1 and 2. */
static double gammainc12(int power, double x) {
    if (x < 0.0) return 0.0;
    if (power == 1) return -expm1(-x);
    return -expm1(-x) - x * exp(-x);
}

typedef struct {
    int type;                  /* -1 burst, 0 constant, 1 tau, 4 delayed tau, 5 linear ramp (Simha) */
    double tage, tau, tb, tq;  /* years (lookback) */
    double trunc, slope, t0;   /* the truncation (years after the start), the ramp's slope in lookback time (per
                                  year), the lookback time where the ramp reaches zero (0: none) */
    int simha;                 /* 1: integrate over [t0, tq] (the ramp), else over [tq, tage] */
} sfh_t;

/* Indefinite moments in log10 time: M0 = int SFR dt, M1 = int SFR log10(t) dt. */
static void moments_log(double log_t, const sfh_t *s, double *m0, double *m1) {
    const double t = pow(10.0, log_t);
    switch (s->type) {
    case 0:
        *m0 = t;
        *m1 = t * (log_t - LOG_E);
        return;
    case 1: {
        if (s->tau <= SAFE_FLOOR) { *m0 = 0.0; *m1 = 0.0; return; }
        const double tt = fmax(t / s->tau, SAFE_FLOOR);
        double ei = oracle_expi(tt);
        if (!isfinite(ei)) ei = 0.0;
        *m0 = exp(tt);
        *m1 = log_t * *m0 - LOG_E * ei;
        return;
    }
    case 4: {
        if (s->tau <= SAFE_FLOOR) { *m0 = 0.0; *m1 = 0.0; return; }
        const double tt = fmax(t / s->tau, SAFE_FLOOR);
        double ei = oracle_expi(tt);
        if (!isfinite(ei)) ei = 0.0;
        *m0 = -(t - s->tage - s->tau) * exp(tt);
        *m1 = -((t - s->tage - s->tau) * log_t - s->tau * LOG_E) * exp(tt) - (s->tage + s->tau) * LOG_E * ei;
        return;
    }
    case 5: {
        /* SFR = 1 + slope (t - t'), t' = max(0, tage - trunc): M0 and M1 of the linear function */
        const double tp = fmax(0.0, s->tage - s->trunc), f = 1.0 - s->slope * tp, h = 0.5 * s->slope * t * t;
        *m0 = f * t + h;
        *m1 = f * t * (log_t - LOG_E) + h * (log_t - 0.5 * LOG_E);
        return;
    }
    default:
        *m0 = 0.0;
        *m1 = 0.0;
    }
}

/* compute_ssp_weights: the mass formed against the hat kernel of each grid age (1-based idx_min, idx_max; w has
   nt entries, w[0] for the first age). */
static void ssp_weights(const double *tf, int nt, double tiny_logt, const sfh_t *s, int idx_min, int idx_max,
                        double *w) {
    for (int i = 0; i < nt; ++i) w[i] = 0.0;
    if (s->type == -1) {
        if (s->tb < 0.0) return;
        const double log_tb = log10(fmax(s->tb, pow(10.0, tiny_logt)));
        if (log_tb <= tf[0]) { w[0] = 1.0; return; }
        int j = oracle_find_interval(tf, nt, log_tb);
        j = j < 1 ? 1 : (j > nt - 1 ? nt - 1 : j);
        const double dt = tf[j] - tf[j - 1];
        w[j - 1] = (tf[j] - log_tb) / dt;
        w[j] = (log_tb - tf[j - 1]) / dt;
        return;
    }
    const double lmin = pow(10.0, tiny_logt);
    const double lts = log10(fmax(s->simha ? s->t0 : s->tq, lmin)), lte = log10(fmax(s->simha ? s->tq : s->tage, lmin));
    int js = oracle_find_interval(tf, nt, lts);
    int je = oracle_find_interval(tf, nt, lte) + 1;
    const int lo_bound = idx_min > 1 ? idx_min : 1, hi_bound = idx_max < nt - 1 ? idx_max : nt - 1;
    if (js < lo_bound) js = lo_bound;
    if (je > hi_bound) je = hi_bound;
    double lim_prev = fmin(fmax(tf[js - 1], lts), lte);
    double m0p, m1p;
    moments_log(lim_prev, s, &m0p, &m1p);
    for (int j = js; j <= je; ++j) {
        const double lim2 = fmin(fmax(tf[j], lts), lte);
        if (lim2 <= lim_prev) { lim_prev = lim2; continue; }
        double m0c, m1c;
        moments_log(lim2, s, &m0c, &m1c);
        const double m0 = m0c - m0p, m1 = m1c - m1p;
        m0p = m0c;
        m1p = m1c;
        const double lo = tf[j - 1], hi = tf[j], inv = 1.0 / (hi - lo);
        w[j - 1] += (hi * m0 - m1) * inv;
        w[j] += (m1 - lo * m0) * inv;
        lim_prev = lim2;
    }
    if (idx_min == 0) {
        const double l1 = fmin(fmax(tiny_logt, lts), lte), l2 = fmin(fmax(tf[0], lts), lte);
        if (l1 < l2) {
            double a0, a1, b0, b1;
            moments_log(l2, s, &a0, &a1);
            moments_log(l1, s, &b0, &b1);
            w[0] += a0 - b0;
        }
    }
}

/* compute_ssp_weights alone (tests): SFH type -1 (burst), 0, 1, 4 or 5 with times in years (tage, tau, tq the
 * truncation lookback, tb the burst lookback; for type 5 trunc, slope per year in lookback time, t0 and the window
 * flag simha), the 1-based index range idx_min .. idx_max and tiny_logt; w has nt entries. */
void oracle_ssp_weights_raw(const double *tf, int nt, double tiny_logt, int type, double tage, double tau, double tq,
                            double tb, double trunc, double slope, double t0, int simha, int idx_min, int idx_max,
                            double *w) {
    sfh_t s;
    s.type = type;
    s.tage = tage;
    s.tau = tau;
    s.tq = tq;
    s.tb = tb;
    s.trunc = trunc;
    s.slope = slope;
    s.t0 = t0;
    s.simha = simha;
    ssp_weights(tf, nt, tiny_logt, &s, idx_min, idx_max, w);
}

/* SFH parameters per model, in this order (Gyr where timed): tage, tau, const, fburst, tburst, sf_start, sf_trunc,
   sf_slope (per Gyr). */
enum { SP_TAGE = 0, SP_TAU, SP_CONST, SP_FBURST, SP_TBURST, SP_SF_START, SP_SF_TRUNC, SP_SF_SLOPE, SP_COUNT };

static void convert(int sfh, const double *p, sfh_t *s) {
    const double start = (sfh == 1 || sfh == 4 || sfh == 5) ? p[SP_SF_START] * 1.0e9 : 0.0;
    s->tage = p[SP_TAGE] * 1.0e9 - start;
    const double tburst = p[SP_TBURST] * 1.0e9 - start;
    s->trunc = p[SP_SF_TRUNC] * 1.0e9 - start;
    s->tau = p[SP_TAU] * 1.0e9;
    s->slope = -p[SP_SF_SLOPE] / 1.0e9;
    s->tb = s->tage - tburst;
    s->tq = (s->trunc <= 0.0 || s->trunc > s->tage) ? 0.0 : s->tage - s->trunc;
    s->t0 = s->slope > SAFE_FLOOR ? s->tq - 1.0 / s->slope : 0.0;
    if (s->t0 > s->tq || s->t0 <= 0.0) s->t0 = 0.0;
    s->simha = 0;
}

/* get_sfh_properties_at_age_pc (Gyr): the mass fraction formed by age, the SFR per unit mass formed (per Gyr) and,
   for sfh 5, the fraction of the mass formed by age that formed on the ramp. */
static void sfh_props(const double *tf, int nt, int sfh, const double *p, double age, double *mass_frac,
                      double *sfr, double *frac_linear);

/* sfh_weights_core_pc for one metallicity: w (nt) for SFH type sfh (0, 1 or 4) with the parameters p. */
void oracle_sfh_weights(const double *tf, int nt, int sfh, const double *p, double *w, double *tmp1, double *tmp2) {
    sfh_t s;
    convert(sfh, p, &s);
    int imax = oracle_find_interval(tf, nt, log10(s.tage)) + 2;
    imax = imax < 1 ? 1 : (imax > nt ? nt : imax);
    if (sfh == 0) {
        s.type = -1;
        s.tb = s.tage;
        ssp_weights(tf, nt, 0.0, &s, imax - 2 > 1 ? imax - 2 : 1, imax, w);
        return;
    }
    if (sfh == 5) {
        s.type = 4;
        ssp_weights(tf, nt, 0.0, &s, 0, imax, tmp1);
        s.type = 5;
        s.simha = 1;
        ssp_weights(tf, nt, 0.0, &s, 0, imax, tmp2);
        double mass1 = 0.0, mass2 = 0.0;
        for (int i = 0; i < imax; ++i) { mass1 += tmp1[i]; mass2 += tmp2[i]; }
        if (mass1 < SAFE_FLOOR) mass1 = 1.0;
        if (mass2 < SAFE_FLOOR) mass2 = 1.0;
        double mf, sfr, fl;
        sfh_props(tf, nt, sfh, p, p[SP_TAGE], &mf, &sfr, &fl);
        for (int i = 0; i < nt; ++i) w[i] = tmp1[i] / mass1 * (1.0 - fl) + tmp2[i] / mass2 * fl;
        return;
    }
    s.type = sfh;
    ssp_weights(tf, nt, 0.0, &s, 0, imax, w);
    double mass1 = 0.0;
    for (int i = 0; i < imax; ++i) mass1 += w[i];
    if (mass1 < SAFE_FLOOR) mass1 = 1.0;
    for (int i = 0; i < nt; ++i) w[i] /= mass1;
    const double cst = p[SP_CONST], fb_in = p[SP_FBURST];
    if (cst > 0.0 || fb_in > SAFE_FLOOR) {
        s.type = 0;
        ssp_weights(tf, nt, 0.0, &s, 0, imax, tmp1);
        double m1 = 0.0;
        for (int i = 0; i < imax; ++i) m1 += tmp1[i];
        if (m1 < SAFE_FLOOR) m1 = 1.0;
        for (int i = 0; i < nt; ++i) tmp2[i] = 0.0;
        double fb = 0.0;
        if (s.tb >= 0.0) {
            s.type = -1;
            ssp_weights(tf, nt, 0.0, &s, 0, imax, tmp2);
            fb = fb_in;
        }
        for (int i = 0; i < nt; ++i) w[i] = (1.0 - cst - fb) * w[i] + cst * (tmp1[i] / m1) + fb * tmp2[i];
    }
}

static void sfh_props(const double *tf, int nt, int sfh, const double *p, double age, double *mass_frac,
                      double *sfr_out, double *frac_linear) {
    double mass_frac_v = 1.0, sfr = 0.0, fl = 0.0;
    if (sfh == 1 || sfh == 4 || sfh == 5) {
        const double tau = p[SP_TAU], cst = p[SP_CONST], fburst = p[SP_FBURST];
        const double tburst = p[SP_TBURST], start = p[SP_SF_START], trunc = p[SP_SF_TRUNC];
        const double t_max = pow(10.0, tf[nt - 1] - 9.0) - start;
        const double t_prime = age - start;
        const double t_trunc = (trunc < SAFE_FLOOR || trunc < start) ? t_max : trunc - start;
        const double tau_g = fmax(tau, SAFE_FLOOR);
        const int pw = sfh == 1 ? 1 : 2;
        const double total = tau_g * gammainc12(pw, fmin(t_max, t_trunc) / tau_g);
        double mass_tau = 0.0, sfr_tau = 0.0;
        if (t_prime >= 0.0) {
            const double r = fmin(t_prime, t_trunc) / tau_g;
            mass_tau = tau_g * gammainc12(pw, r);
            sfr_tau = (pw == 1 ? 1.0 : r) * exp(-r);
        }
        if (sfh != 5) {
            const double mfrac_burst = (t_prime > tburst - start) ? 1.0 : 0.0;
            double sfr_const = 0.0, mass_const = 0.0;
            if (t_prime > 0.0) {
                sfr_const = 1.0 / fmin(t_max, t_trunc);
                mass_const = fmax(fmin(t_prime, t_trunc), 0.0) * sfr_const;
            }
            const double norm = 1.0 - cst - fburst;
            mass_frac_v = norm * mass_tau / total + cst * mass_const + fburst * mfrac_burst;
            sfr = (t_prime > t_trunc) ? 0.0 : norm * sfr_tau / total + cst * sfr_const;
        } else {
            /* the ramp after the truncation: SFR = sfr_tr (1 - s (t - t_tr)), s = -sf_slope, from the delayed tau's
               SFR at t_tr, down to its zero t_tr + 1 / s */
            const double s = -p[SP_SF_SLOPE];
            const double t_zero = s > 0.0 ? t_trunc + 1.0 / s : t_max;
            double total_lin = 0.0, mass_lin = 0.0;
            if (t_trunc <= 0.0 || t_trunc > t_max) {
                sfr = sfr_tau / total;
            } else {
                const double sfr_tr = (t_trunc / tau) * exp(-t_trunc / tau);
                double hi = fmin(t_zero, t_max);
                total_lin = sfr_tr * ((hi - t_trunc) - 0.5 * s * (hi * hi + t_trunc * t_trunc) + s * hi * t_trunc);
                if (t_prime <= t_trunc) {
                    sfr = sfr_tau / (total + total_lin);
                } else {
                    hi = fmin(t_zero, t_prime);
                    mass_lin = sfr_tr * ((hi - t_trunc) - 0.5 * s * (hi * hi + t_trunc * t_trunc) + s * hi * t_trunc);
                    sfr = fmax(sfr_tr * (1.0 - s * (t_prime - t_trunc)), 0.0) / (total + total_lin);
                }
            }
            if (t_prime >= 0.0) {
                mass_frac_v = (mass_tau + mass_lin) / (total + total_lin);
                if (mass_lin + mass_tau > SAFE_FLOOR) fl = mass_lin / (mass_lin + mass_tau);
            } else {
                mass_frac_v = 0.0;
                sfr = 0.0;
            }
        }
    }
    *mass_frac = mass_frac_v;
    *sfr_out = sfr;
    *frac_linear = fl;
}

/* get_sfh_properties_at_age_pc alone (tests): age in Gyr, the SFR per Gyr before the unit change. */
void oracle_sfh_props(const double *tf, int nt, int sfh, const double *p, double age, double *out3) {
    sfh_props(tf, nt, sfh, p, age, out3, out3 + 1, out3 + 2);
}

/* The current SFR per unit mass formed, normalised by the mass fraction formed by tage (per yr). */
double oracle_sfh_sfr(const double *tf, int nt, int sfh, const double *p) {
    double mass_frac, sfr, fl;
    sfh_props(tf, nt, sfh, p, p[SP_TAGE], &mass_frac, &sfr, &fl);
    sfr /= 1.0e9;
    if (mass_frac > SAFE_FLOOR) sfr /= mass_frac;
    return sfr;
}

/* sfh_weights_core_pc for the tabular SFHs (sfh 2, 3; src/physics/opensps_sfh.f90:1215-1293) with one metallicity
   (the batch's): each table bin [T_j, T_(j+1)] (years since the start, non-decreasing) is the linear SFR between its
   rows, a type-5 segment of slope -(sfr_(j+1) - sfr_j) / dt / sfr_(j+1) over the lookback window [tage - T_(j+1),
   tage - T_j] clamped to [10^tiny_logt, the grid's oldest age], whose hat-kernel weights (over its own index range)
   are scaled to the bin's mass sfr_(j+1) (1 + slope / 2 (tage' + tq - 2 t1)) (tage' - tq). The weights are masses
   formed (M_sun), not normalised. tage in Gyr; tab_t (years) and tab_sfr have ntab entries. */
void oracle_sfh_tab_weights(const double *tf, int nt, double tage, int ntab, const double *tab_t,
                            const double *tab_sfr, double *w, double *tmp1) {
    for (int i = 0; i < nt; ++i) w[i] = 0.0;
    const double tmin = pow(10.0, 0.0), tmax = pow(10.0, tf[nt - 1]);
    for (int j = 0; j < ntab - 1; ++j) {
        const double t1 = tage * 1.0e9 - tab_t[j + 1], t2 = tage * 1.0e9 - tab_t[j];
        if (t2 < 0.0) continue;
        const double dt = fmax(t2 - t1, SAFE_FLOOR);
        sfh_t s;
        memset(&s, 0, sizeof(s));
        s.type = 5;
        s.slope = -(tab_sfr[j + 1] - tab_sfr[j]) / dt / fmax(tab_sfr[j + 1], SAFE_FLOOR);
        s.tq = fmin(fmax(t1, tmin), tmax);
        s.tage = fmin(fmax(t2, tmin), tmax);
        s.trunc = s.tage - s.tq;
        const double mass2 = tab_sfr[j + 1] * (1.0 + s.slope / 2.0 * (s.tage + s.tq - 2.0 * t1)) * (s.tage - s.tq);
        int imin = oracle_find_interval(tf, nt, log10(fmax(t1, SAFE_FLOOR))) - 1;
        int imax = oracle_find_interval(tf, nt, log10(fmax(t2, SAFE_FLOOR))) + 2;
        imin = imin < 0 ? 0 : (imin > nt ? nt : imin);
        imax = imax < 0 ? 0 : (imax > nt ? nt : imax);
        ssp_weights(tf, nt, 0.0, &s, imin, imax, tmp1);
        double mass1 = 0.0;
        for (int i = 0; i < nt; ++i) mass1 += tmp1[i];
        if (mass1 < SAFE_FLOOR) mass1 = 1.0;
        for (int i = 0; i < nt; ++i) w[i] += tmp1[i] * (mass2 / mass1);
    }
}

/* get_sfh_properties_at_age_pc for the tabular SFHs (:458-480): the table's SFR interpolated linearly at age (Gyr)
   in the interval find_interval_tab_time picks (clamped to the table's first ntab - 1 intervals; the entry past the
   table reads as zero), floored at zero; M_sun / yr, the mass fraction 1. */
double oracle_sfh_tab_sfr(double age, int ntab, const double *tab_t, const double *tab_sfr) {
    int idx = oracle_find_interval(tab_t, ntab, age * 1.0e9);
    idx = idx > ntab - 1 ? ntab - 1 : idx;
    idx = idx < 1 ? 1 : idx;
    const double t0 = tab_t[idx - 1], s0 = tab_sfr[idx - 1];
    const double t1 = idx < ntab ? tab_t[idx] : 0.0, s1 = idx < ntab ? tab_sfr[idx] : 0.0;
    const double v = s0 + (s1 - s0) / (t1 - t0) * (age * 1.0e9 - t0);
    return fmax(v, 0.0);
}

/* Tabular batch form: w (n x nt) and sfr (n) at the models' ages tage (n, Gyr). */
void oracle_sfh_tab_batch(const double *tf, int nt, int n, const double *tage, int ntab, const double *tab_t,
                          const double *tab_sfr, double *w, double *sfr) {
#pragma omp parallel
    {
        double tmp1[512];
#pragma omp for
        for (int m = 0; m < n; ++m) {
            oracle_sfh_tab_weights(tf, nt, tage[m], ntab, tab_t, tab_sfr, w + (size_t)nt * m, tmp1);
            if (sfr) sfr[m] = oracle_sfh_tab_sfr(tage[m], ntab, tab_t, tab_sfr);
        }
    }
}

/* Batch form: w (n x nt) and sfr (n) for the parameter rows p (n x SP_COUNT). */
void oracle_sfh_batch(const double *tf, int nt, int sfh, int n, const double *p, double *w, double *sfr) {
#pragma omp parallel
    {
        double tmp1[512], tmp2[512];
#pragma omp for
        for (int m = 0; m < n; ++m) {
            oracle_sfh_weights(tf, nt, sfh, p + (size_t)SP_COUNT * m, w + (size_t)nt * m, tmp1, tmp2);
            if (sfr) sfr[m] = oracle_sfh_sfr(tf, nt, sfh, p + (size_t)SP_COUNT * m);
        }
    }
}
