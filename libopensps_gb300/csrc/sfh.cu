// SFH weights on the device, one thread per model in FP64 (OpenSPS batch_sfh_weights → sfh_weights_core,
// src/physics/opensps_csp_batch.f90:1865-1917, src/physics/opensps_sfh.f90:1077-1212, compute_ssp_weights :97-257):
// the mass formed against the hat kernel of each grid age for SFH types 0 (SSP), 1 (tau) and 4 (delayed tau), with
// the constant and burst components, normalised to one solar mass formed, and 5 (Simha: the delayed tau up to the
// truncation, then a linear ramp from its SFR there, the two normalised apart and mixed by the ramp's mass fraction).
// Then the models' metallicity blend at logzsol into the weights over ages and metallicities, the log-blended L_bol
// (model_sums MSUMS_BLEND :2129-2176) and the current SFR (get_sfh_properties_at_age :281-486 over the mass fraction,
// batch_model_indices :1558-1567).
//
// The weights are written once as templates over the scalar type: double for the forward, Dual (value and eight
// derivatives: tage, tau, const, fburst, tburst, sf_start, sf_trunc, sf_slope) for the tangents of the reverse pass
// (sfh_weights_tangent, src/physics/opensps_sfh_tangent.f90:61-198, forward mode; d Ei(x)/dx = e^x / x).
#include <cuda_runtime.h>
#include <cmath>
#include <cfloat>
#include <mutex>
#include "context.h"

namespace sps {

constexpr double SFH_LOG_E = 0.43429448190325182765;   // log10(e)
constexpr double SFH_LN10 = 2.302585092994045684;
constexpr double SFH_EULER_GAMMA = 0.57721566490153286060651209008240243104215933593992;

// ---------------------------------------------------------------------------------------------- dual numbers
struct Dual {
    double v;
    double d[SFH_NPAR];
};
__device__ __forceinline__ Dual dconst(double v) {
    Dual r;
    r.v = v;
#pragma unroll
    for (int i = 0; i < SFH_NPAR; ++i) r.d[i] = 0.0;
    return r;
}
__device__ __forceinline__ Dual operator+(const Dual &a, const Dual &b) {
    Dual r; r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < SFH_NPAR; ++i) r.d[i] = a.d[i] + b.d[i];
    return r;
}
__device__ __forceinline__ Dual operator-(const Dual &a, const Dual &b) {
    Dual r; r.v = a.v - b.v;
#pragma unroll
    for (int i = 0; i < SFH_NPAR; ++i) r.d[i] = a.d[i] - b.d[i];
    return r;
}
__device__ __forceinline__ Dual operator-(const Dual &a) {
    Dual r; r.v = -a.v;
#pragma unroll
    for (int i = 0; i < SFH_NPAR; ++i) r.d[i] = -a.d[i];
    return r;
}
__device__ __forceinline__ Dual operator*(const Dual &a, const Dual &b) {
    Dual r; r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < SFH_NPAR; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
__device__ __forceinline__ Dual operator/(const Dual &a, const Dual &b) {
    Dual r; r.v = a.v / b.v;
    const double ib = 1.0 / b.v;
#pragma unroll
    for (int i = 0; i < SFH_NPAR; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
    return r;
}
__device__ __forceinline__ Dual operator+(const Dual &a, double b) { Dual r = a; r.v += b; return r; }
__device__ __forceinline__ Dual operator+(double b, const Dual &a) { return a + b; }
__device__ __forceinline__ Dual operator-(const Dual &a, double b) { Dual r = a; r.v -= b; return r; }
__device__ __forceinline__ Dual operator-(double b, const Dual &a) { return -a + b; }
__device__ __forceinline__ Dual operator*(const Dual &a, double b) {
    Dual r; r.v = a.v * b;
#pragma unroll
    for (int i = 0; i < SFH_NPAR; ++i) r.d[i] = a.d[i] * b;
    return r;
}
__device__ __forceinline__ Dual operator*(double b, const Dual &a) { return a * b; }
__device__ __forceinline__ Dual operator/(const Dual &a, double b) { return a * (1.0 / b); }
__device__ __forceinline__ Dual operator/(double a, const Dual &b) {
    Dual r; r.v = a / b.v;
    const double q = -r.v / b.v;
#pragma unroll
    for (int i = 0; i < SFH_NPAR; ++i) r.d[i] = q * b.d[i];
    return r;
}

__device__ __forceinline__ double val(double x) { return x; }
__device__ __forceinline__ double val(const Dual &x) { return x.v; }
template <class T> __device__ __forceinline__ T lift(double v);
template <> __device__ __forceinline__ double lift<double>(double v) { return v; }
template <> __device__ __forceinline__ Dual lift<Dual>(double v) { return dconst(v); }

// a smooth function f applied to x, with its derivative df at x
__device__ __forceinline__ double chain(double, double f, double) { return f; }
__device__ __forceinline__ Dual chain(const Dual &x, double f, double df) {
    Dual r; r.v = f;
#pragma unroll
    for (int i = 0; i < SFH_NPAR; ++i) r.d[i] = df * x.d[i];
    return r;
}
template <class T> __device__ __forceinline__ T sexp(const T &x) { const double e = exp(val(x)); return chain(x, e, e); }
template <class T> __device__ __forceinline__ T sexpm1(const T &x) { return chain(x, expm1(val(x)), exp(val(x))); }
template <class T> __device__ __forceinline__ T spow10(const T &x) {
    const double e = pow(10.0, val(x));
    return chain(x, e, e * SFH_LN10);
}
template <class T> __device__ __forceinline__ T slog10(const T &x) {
    return chain(x, log10(val(x)), 1.0 / (val(x) * SFH_LN10));
}
template <class T> __device__ __forceinline__ T smax(const T &a, const T &b) { return val(a) >= val(b) ? a : b; }
template <class T> __device__ __forceinline__ T smin(const T &a, const T &b) { return val(a) <= val(b) ? a : b; }

// 1 / (k + 1)^2, k = 0 .. 1000: the power series' term ratio without an FP64 division per term (GB300's FP64 pipe is
// narrow and the series' terms form one dependent chain)
constexpr int SFH_NSER = 1001;
__constant__ double c_inv_sq[SFH_NSER];

// Ei(x) (expi, src/math/opensps_special_functions.f90:62-122): the power series about 0 for x <= 40, the
// asymptotic series (20 terms) beyond; d Ei / dx = e^x / x.
__device__ double expi_d(double x) {
    if (x == 0.0) return -INFINITY;
    if (x < 0.0) return NAN;
    if (fabs(x) <= 40.0) {
        double res = 1.0, r = 1.0;
        for (int k = 1; k <= 1000; ++k) {
            r = (r * (double)k * x) * c_inv_sq[k];
            res += r;
            if (fabs(r) <= 1.0e-20 * fabs(res)) break;
            if (k == 1000) return NAN;
        }
        return SFH_EULER_GAMMA + log(x) + x * res;
    }
    double res = 1.0, r = 1.0;
    const double inv = 1.0 / x;
    for (int k = 1; k <= 20; ++k) {
        r *= (double)k * inv;
        res += r;
    }
    return exp(x) * inv * res;
}
template <class T> __device__ __forceinline__ T sexpi(const T &x, bool &finite) {
    const double e = expi_d(val(x));
    finite = isfinite(e);
    return chain(x, finite ? e : 0.0, finite ? exp(val(x)) / val(x) : 0.0);
}

// ---------------------------------------------------------------------------------------------- the weights
template <class T>
struct SfhT {
    int type;         // -1 burst, 0 constant, 1 tau, 4 delayed tau, 5 linear ramp
    T tage, tau, tb, tq;
    T trunc, slope, t0;   // the truncation (years after the start), the ramp's slope in lookback time (per year), the
                          // lookback time where the ramp reaches zero (0: none)
    int simha;            // 1: the ramp's window [t0, tq], else [tq, tage]
};

// convert_sfhparams_pc (src/physics/opensps_sfh.f90:1306-1360): years, lookback times from the start of star
// formation (sf_start for sfh 1, 4, 5).
template <class T>
__device__ __forceinline__ void sfh_setup(int sfh, const T *p, SfhT<T> &s) {
    const T start = (sfh == 1 || sfh == 4 || sfh == 5) ? p[SFH_SF_START] * 1.0e9 : lift<T>(0.0);
    s.tage = p[SFH_TAGE] * 1.0e9 - start;
    const T tburst = p[SFH_TBURST] * 1.0e9 - start;
    s.trunc = p[SFH_SF_TRUNC] * 1.0e9 - start;
    s.tau = p[SFH_TAU] * 1.0e9;
    s.slope = p[SFH_SF_SLOPE] * -1.0e-9;
    s.tb = s.tage - tburst;
    s.tq = (val(s.trunc) <= 0.0 || val(s.trunc) > val(s.tage)) ? lift<T>(0.0) : s.tage - s.trunc;
    s.t0 = val(s.slope) > SAFE_FLOOR ? s.tq - 1.0 / s.slope : lift<T>(0.0);
    if (val(s.t0) > val(s.tq) || val(s.t0) <= 0.0) s.t0 = lift<T>(0.0);
    s.simha = 0;
}

// The integration window in log10 lookback years (clamp_integration_limits, src/physics/opensps_sfh.f90:969-1010,
// tiny_logt = 0).
template <class T>
__device__ __forceinline__ void sfh_window(const SfhT<T> &s, T &lts, T &lte) {
    const T one = lift<T>(1.0);
    lts = slog10(smax(s.simha ? s.t0 : s.tq, one));
    lte = slog10(smax(s.simha ? s.tq : s.tage, one));
}

// eval_indefinite_moments_log (src/physics/opensps_sfh.f90:852-905): M0 = int SFR dt, M1 = int SFR log10(t) dt
template <class T>
__device__ void moments_log(const T &log_t, const SfhT<T> &s, T &m0, T &m1) {
    const T t = spow10(log_t);
    if (s.type == 0) {
        m0 = t;
        m1 = t * (log_t - SFH_LOG_E);
        return;
    }
    if (s.type == 1 || s.type == 4) {
        if (val(s.tau) <= SAFE_FLOOR) { m0 = lift<T>(0.0); m1 = lift<T>(0.0); return; }
        const T tt = smax(t / s.tau, lift<T>(SAFE_FLOOR));
        bool fin;
        const T ei = sexpi(tt, fin);
        const T e = sexp(tt);
        if (s.type == 1) {
            m0 = e;
            m1 = log_t * m0 - SFH_LOG_E * ei;
        } else {
            const T a = t - s.tage - s.tau;
            m0 = -(a * e);
            m1 = -((a * log_t - s.tau * SFH_LOG_E) * e) - (s.tage + s.tau) * SFH_LOG_E * ei;
        }
        return;
    }
    if (s.type == 5) {   // SFR = 1 + slope (t - t'), t' = max(0, tage - trunc)
        const T f = 1.0 - s.slope * smax(lift<T>(0.0), s.tage - s.trunc);
        const T h = 0.5 * s.slope * t * t;
        m0 = f * t + h;
        m1 = f * t * (log_t - SFH_LOG_E) + h * (log_t - 0.5 * SFH_LOG_E);
        return;
    }
    m0 = lift<T>(0.0);
    m1 = lift<T>(0.0);
}

// compute_ssp_weights (src/physics/opensps_sfh.f90:97-257) with log-age interpolation: w (nt, strided) += the hat
// kernel masses; idx_min / idx_max 1-based as the reference's. w must start at zero.
// The moments at limit lim = the grid age tf[j] clamped to [lts, lte]: from the table when tf[j] lies strictly
// inside (the table's entries are moments_log at tf[j] itself), else formed here.
template <class T>
__device__ __forceinline__ void moments_at(const T &lim, int j, const double *tf, const T &lts, const T &lte,
                                           const SfhT<T> &s, const double2 *mtab, T &m0, T &m1) {
    if (mtab && val(lim) == tf[j] && tf[j] > val(lts) && tf[j] < val(lte)) {
        m0 = lift<T>(mtab[j].x);
        m1 = lift<T>(mtab[j].y);
        return;
    }
    moments_log(lim, s, m0, m1);
}

template <class T>
__device__ __forceinline__ void ssp_weights(const double *tf, int nt, const SfhT<T> &s, int idx_min, int idx_max, T *w, int ws,
                            const double2 *mtab = nullptr) {
    const double tiny_logt = 0.0;
    if (s.type == -1) {
        if (val(s.tb) < 0.0) return;
        const T log_tb = slog10(smax(s.tb, lift<T>(pow(10.0, tiny_logt))));
        if (val(log_tb) <= tf[0]) { w[0] = w[0] + 1.0; return; }
        int j = find_interval0(tf, nt, val(log_tb)) + 1;
        j = j < 1 ? 1 : (j > nt - 1 ? nt - 1 : j);
        const double dt = tf[j] - tf[j - 1];
        w[(j - 1) * ws] = w[(j - 1) * ws] + (tf[j] - log_tb) / dt;
        w[j * ws] = w[j * ws] + (log_tb - tf[j - 1]) / dt;
        return;
    }
    T lts, lte;
    sfh_window(s, lts, lte);
    int js = find_interval0(tf, nt, val(lts)) + 1;
    int je = find_interval0(tf, nt, val(lte)) + 2;
    const int lo_bound = idx_min > 1 ? idx_min : 1, hi_bound = idx_max < nt - 1 ? idx_max : nt - 1;
    if (js < lo_bound) js = lo_bound;
    if (je > hi_bound) je = hi_bound;
    T lim_prev = smin(smax(lift<T>(tf[js - 1]), lts), lte);
    T m0p, m1p;
    moments_at(lim_prev, js - 1, tf, lts, lte, s, mtab, m0p, m1p);
    for (int j = js; j <= je; ++j) {
        const T lim2 = smin(smax(lift<T>(tf[j]), lts), lte);
        if (val(lim2) <= val(lim_prev)) { lim_prev = lim2; continue; }
        T m0c, m1c;
        moments_at(lim2, j, tf, lts, lte, s, mtab, m0c, m1c);
        const T m0 = m0c - m0p, m1 = m1c - m1p;
        m0p = m0c;
        m1p = m1c;
        const double lo = tf[j - 1], hi = tf[j], inv = 1.0 / (hi - lo);
        w[(j - 1) * ws] = w[(j - 1) * ws] + (hi * m0 - m1) * inv;
        w[j * ws] = w[j * ws] + (m1 - lo * m0) * inv;
        lim_prev = lim2;
    }
    if (idx_min == 0) {
        const T l1 = smin(smax(lift<T>(tiny_logt), lts), lte), l2 = smin(smax(lift<T>(tf[0]), lts), lte);
        if (val(l1) < val(l2)) {
            T a0, a1, b0, b1;
            moments_log(l2, s, a0, a1);
            moments_log(l1, s, b0, b1);
            w[0] = w[0] + (a0 - b0);
        }
    }
}

// The regularised lower incomplete gamma function of power 1 or 2 (gammainc, src/math/opensps_special_functions.f90:
// 142-170); 0 below 0.
template <class T>
__device__ __forceinline__ T gammainc12(bool one, const T &x) {
    if (val(x) < 0.0) return lift<T>(0.0);
    const T g = -sexpm1(-x);
    return one ? g : g - x * sexp(-x);
}

// get_sfh_properties_at_age_pc at tage (src/physics/opensps_sfh.f90:281-486, Gyr; sfh 0, 1, 4, 5): the mass fraction
// formed, the normalised SFR (per Gyr) and, for sfh 5, the fraction of the mass formed by tage that formed on the ramp.
template <class T>
__device__ __forceinline__ void sfh_props(const double *tf, int nt, int sfh, const T *p, T &mass_frac, T &sfr, T &frac_linear) {
    mass_frac = lift<T>(1.0);
    sfr = lift<T>(0.0);
    frac_linear = lift<T>(0.0);
    if (sfh != 1 && sfh != 4 && sfh != 5) return;
    const T tau = p[SFH_TAU], start = p[SFH_SF_START], trunc = p[SFH_SF_TRUNC];
    const T t_max = pow(10.0, tf[nt - 1] - 9.0) - start;
    const T t_prime = p[SFH_TAGE] - start;
    const T t_trunc = (val(trunc) < SAFE_FLOOR || val(trunc) < val(start)) ? t_max : trunc - start;
    const T tau_g = smax(tau, lift<T>(SAFE_FLOOR));
    const bool one = sfh == 1;
    const T total = tau_g * gammainc12(one, smin(t_max, t_trunc) / tau_g);
    T mass_tau = lift<T>(0.0), sfr_tau = lift<T>(0.0);
    if (val(t_prime) >= 0.0) {
        const T r = smin(t_prime, t_trunc) / tau_g;
        mass_tau = tau_g * gammainc12(one, r);
        sfr_tau = (one ? lift<T>(1.0) : r) * sexp(-r);
    }
    if (sfh != 5) {
        const T cst = p[SFH_CONST], fburst = p[SFH_FBURST];
        const double mfrac_burst = (val(t_prime) > val(p[SFH_TBURST]) - val(start)) ? 1.0 : 0.0;
        T sfr_const = lift<T>(0.0), mass_const = lift<T>(0.0);
        if (val(t_prime) > 0.0) {
            sfr_const = 1.0 / smin(t_max, t_trunc);
            mass_const = smax(smin(t_prime, t_trunc), lift<T>(0.0)) * sfr_const;
        }
        const T norm = 1.0 - cst - fburst;
        mass_frac = norm * mass_tau / total + cst * mass_const + fburst * mfrac_burst;
        sfr = (val(t_prime) > val(t_trunc)) ? lift<T>(0.0) : norm * sfr_tau / total + cst * sfr_const;
        return;
    }
    // the ramp after the truncation: SFR = sfr_tr (1 - k (t - t_tr)), k = -sf_slope, from the delayed tau's SFR at
    // t_tr, down to its zero t_tr + 1 / k
    const T k = -p[SFH_SF_SLOPE];
    const T t_zero = val(k) > 0.0 ? t_trunc + 1.0 / k : t_max;
    T total_lin = lift<T>(0.0), mass_lin = lift<T>(0.0);
    if (val(t_trunc) <= 0.0 || val(t_trunc) > val(t_max)) {
        sfr = sfr_tau / total;
    } else {
        const T sfr_tr = (t_trunc / tau) * sexp(-(t_trunc / tau));
        T hi = smin(t_zero, t_max);
        total_lin = sfr_tr * ((hi - t_trunc) - 0.5 * k * (hi * hi + t_trunc * t_trunc) + k * hi * t_trunc);
        if (val(t_prime) <= val(t_trunc)) {
            sfr = sfr_tau / (total + total_lin);
        } else {
            hi = smin(t_zero, t_prime);
            mass_lin = sfr_tr * ((hi - t_trunc) - 0.5 * k * (hi * hi + t_trunc * t_trunc) + k * hi * t_trunc);
            sfr = smax(sfr_tr * (1.0 - k * (t_prime - t_trunc)), lift<T>(0.0)) / (total + total_lin);
        }
    }
    if (val(t_prime) >= 0.0) {
        mass_frac = (mass_tau + mass_lin) / (total + total_lin);
        if (val(mass_lin) + val(mass_tau) > SAFE_FLOOR) frac_linear = mass_lin / (mass_lin + mass_tau);
    } else {
        mass_frac = lift<T>(0.0);
        sfr = lift<T>(0.0);
    }
}

// sfh_weights_core_pc for one metallicity (src/physics/opensps_sfh.f90:1077-1212; convert_sfhparams_pc :1306-1360).
// p: tage, tau, const, fburst, tburst, sf_start, sf_trunc (Gyr), sf_slope (per Gyr). w, t1, t2: nt entries at stride
// ws, zeroed here.
template <class T>
__device__ __forceinline__ void sfh_weights_core(const double *tf, int nt, int sfh, const T *p, T *w, T *t1, T *t2, int ws,
                                 const double2 *mtab = nullptr) {
    for (int i = 0; i < nt; ++i) { w[i * ws] = lift<T>(0.0); t1[i * ws] = lift<T>(0.0); t2[i * ws] = lift<T>(0.0); }
    SfhT<T> s;
    sfh_setup(sfh, p, s);
    int imax = find_interval0(tf, nt, log10(val(s.tage))) + 1 + 2;
    imax = imax < 1 ? 1 : (imax > nt ? nt : imax);
    if (sfh == 0) {
        s.type = -1;
        s.tb = s.tage;
        ssp_weights(tf, nt, s, imax - 2 > 1 ? imax - 2 : 1, imax, w, ws);
        return;
    }
    if (sfh == 5) {
        s.type = 4;
        ssp_weights(tf, nt, s, 0, imax, t1, ws, mtab);
        s.type = 5;
        s.simha = 1;
        ssp_weights(tf, nt, s, 0, imax, t2, ws);
        T mass1 = lift<T>(0.0), mass2 = lift<T>(0.0);
        for (int i = 0; i < imax; ++i) { mass1 = mass1 + t1[i * ws]; mass2 = mass2 + t2[i * ws]; }
        if (val(mass1) < SAFE_FLOOR) mass1 = lift<T>(1.0);
        if (val(mass2) < SAFE_FLOOR) mass2 = lift<T>(1.0);
        T mf, sfr, fl;
        sfh_props(tf, nt, sfh, p, mf, sfr, fl);
        const T a = (1.0 - fl) / mass1, b = fl / mass2;
        for (int i = 0; i < nt; ++i) w[i * ws] = t1[i * ws] * a + t2[i * ws] * b;
        return;
    }
    s.type = sfh;
    ssp_weights(tf, nt, s, 0, imax, w, ws, mtab);
    T mass1 = lift<T>(0.0);
    for (int i = 0; i < imax; ++i) mass1 = mass1 + w[i * ws];
    if (val(mass1) < SAFE_FLOOR) mass1 = lift<T>(1.0);
    for (int i = 0; i < nt; ++i) w[i * ws] = w[i * ws] / mass1;
    const T cst = p[SFH_CONST], fb_in = p[SFH_FBURST];
    if (val(cst) > 0.0 || val(fb_in) > SAFE_FLOOR) {
        s.type = 0;
        ssp_weights(tf, nt, s, 0, imax, t1, ws);
        T m1 = lift<T>(0.0);
        for (int i = 0; i < imax; ++i) m1 = m1 + t1[i * ws];
        if (val(m1) < SAFE_FLOOR) m1 = lift<T>(1.0);
        T fb = lift<T>(0.0);
        if (val(s.tb) >= 0.0) {
            s.type = -1;
            ssp_weights(tf, nt, s, 0, imax, t2, ws);
            fb = fb_in;
        }
        for (int i = 0; i < nt; ++i)
            w[i * ws] = (1.0 - cst - fb) * w[i * ws] + cst * (t1[i * ws] / m1) + fb * t2[i * ws];
    }
}

// The current SFR per unit mass formed over the mass fraction formed by tage (per yr).
__device__ double sfh_sfr(const double *tf, int nt, int sfh, const double *p) {
    double mass_frac, sfr, fl;
    sfh_props(tf, nt, sfh, p, mass_frac, sfr, fl);
    sfr /= 1.0e9;
    if (mass_frac > SAFE_FLOOR) sfr /= mass_frac;
    return sfr;
}

// The metallicity interval of logzsol: zlo (0-based) and dz, not clamped (metallicity_interval,
// src/physics/opensps_csp_batch.f90:2071-2085).
__device__ __forceinline__ void zinterval(const double *lz, int nz, double x, int &zlo, double &dz) {
    int idx = find_interval0(lz, nz, x) + 1;
    idx = idx < 1 ? 1 : (idx > nz - 1 ? nz - 1 : idx);
    zlo = idx - 1;
    dz = (x - lz[zlo]) / (lz[zlo + 1] - lz[zlo]);
}

// One thread per (model, grid age): the main component's moments (sfh 1, 4; the delayed tau of sfh 5) at the grid
// ages strictly inside the model's [log t_start, log t_age], the SFH set up as sfh_weights_core sets it, for
// sfh_forward_kernel's table.
__global__ void __launch_bounds__(128) sfh_moments_kernel(SfhArgs a) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)a.n * a.nt) return;
    const int m = (int)(i / a.nt), j = (int)(i % a.nt);
    const double *p = a.par + (size_t)SFH_NCOL * m;
    SfhT<double> s;
    sfh_setup(a.sfh, p, s);
    s.type = a.sfh == 5 ? 4 : a.sfh;
    double lts, lte;
    sfh_window(s, lts, lte);
    const double x = a.tf[j];
    double2 r = make_double2(0.0, 0.0);
    if (x > lts && x < lte) moments_log(x, s, r.x, r.y);
    a.mtab[i] = r;
}

// One component's weights over ages by a warp (ssp_weights for T = double, idx_min 0 or the SSP's window): the
// moments at every boundary of its intervals (the table's, or formed here at the clamped ends), then per age
// w[i] = B_i + A_(i+1), interval j's shares A_j = (hi d0 - d1) / dt to w[j - 1] and B_j = (d1 - lo d0) / dt to w[j]
// (d0, d1 the moments' differences over the interval; intervals of zero width skipped): the sums the serial loop
// forms, in its order. wout[0 .. nt) is written in full; M0s / M1s are the warp's scratch.
__device__ void warp_component(const double *tf, int nt, const SfhT<double> &s, int idx_min, int idx_max,
                               const double2 *mtab, double *M0s, double *M1s, double *wout, int lane) {
    for (int i = lane; i < nt; i += 32) wout[i] = 0.0;
    __syncwarp();
    if (s.type == -1) {
        if (lane == 0 && s.tb >= 0.0) {
            const double log_tb = log10(fmax(s.tb, 1.0));
            if (log_tb <= tf[0]) {
                wout[0] += 1.0;
            } else {
                int j = find_interval0(tf, nt, log_tb) + 1;
                j = j < 1 ? 1 : (j > nt - 1 ? nt - 1 : j);
                const double dt = tf[j] - tf[j - 1];
                wout[j - 1] += (tf[j] - log_tb) / dt;
                wout[j] += (log_tb - tf[j - 1]) / dt;
            }
        }
        __syncwarp();
        return;
    }
    double lts, lte;
    sfh_window(s, lts, lte);
    int js = find_interval0(tf, nt, lts) + 1;
    int je = find_interval0(tf, nt, lte) + 2;
    const int lo_bound = idx_min > 1 ? idx_min : 1, hi_bound = idx_max < nt - 1 ? idx_max : nt - 1;
    if (js < lo_bound) js = lo_bound;
    if (je > hi_bound) je = hi_bound;
    for (int j = lane; j < nt; j += 32)
        if (j >= js - 1 && j <= je) {
            const double lim = fmin(fmax(tf[j], lts), lte);
            double m0, m1;
            moments_at(lim, j, tf, lts, lte, s, mtab, m0, m1);
            M0s[j] = m0;
            M1s[j] = m1;
        }
    __syncwarp();
    for (int i = lane; i < nt; i += 32) {
        double v = 0.0;
        if (i >= js && i <= je) {                          // B_i
            const double lp = fmin(fmax(tf[i - 1], lts), lte), lc = fmin(fmax(tf[i], lts), lte);
            if (lc > lp) {
                const double d0 = M0s[i] - M0s[i - 1], d1 = M1s[i] - M1s[i - 1];
                const double lo = tf[i - 1], hi = tf[i], inv = 1.0 / (hi - lo);
                v = v + (d1 - lo * d0) * inv;
            }
        }
        const int j = i + 1;
        if (j >= js && j <= je && j < nt) {                // A_(i+1)
            const double lp = fmin(fmax(tf[j - 1], lts), lte), lc = fmin(fmax(tf[j], lts), lte);
            if (lc > lp) {
                const double d0 = M0s[j] - M0s[j - 1], d1 = M1s[j] - M1s[j - 1];
                const double lo = tf[j - 1], hi = tf[j], inv = 1.0 / (hi - lo);
                v = v + (hi * d0 - d1) * inv;
            }
        }
        wout[i] = v;
    }
    __syncwarp();
    if (idx_min == 0 && lane == 0) {
        const double l1 = fmin(fmax(0.0, lts), lte), l2 = fmin(fmax(tf[0], lts), lte);
        if (l1 < l2) {
            double a0, a1, b0, b1;
            moments_log(l2, s, a0, a1);
            moments_log(l1, s, b0, b1);
            wout[0] = wout[0] + (a0 - b0);
        }
    }
    __syncwarp();
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// One warp per model (SFH_WARPS models per CTA): the weights over ages (sfh_weights_core: the main component
// normalised to one solar mass formed, then the constant and burst components), the SFR, the blend over
// metallicities (wz, n x nt x nz, age fastest: the other slabs zeroed) and the log-blended L_bol sums (total, young,
// old). The ages are spread over the lanes (GB300's FP64 pipe is narrow: one model per thread left the SMs idle on
// small batches); the warp's weights live in shared memory.
constexpr int SFH_WARPS = 4;
constexpr int SFH_WMAXT = 128;
__global__ void __launch_bounds__(SFH_WARPS * 32) sfh_forward_kernel(SfhArgs a) {
    __shared__ double sm[SFH_WARPS][5][SFH_WMAXT];
    const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
    const int m = blockIdx.x * SFH_WARPS + wi;
    if (m >= a.n) return;
    const double *p = a.par + (size_t)SFH_NCOL * m;
    const int nt = a.nt, nz = a.nz;
    double *w = sm[wi][0], *t1 = sm[wi][1], *t2 = sm[wi][2], *M0s = sm[wi][3], *M1s = sm[wi][4];
    if (a.given) {
        // the caller's weights (SFR NaN), or the tabular SFH's from sfh_tab_kernel (its SFR kept)
        for (int i = lane; i < nt; i += 32) w[i] = a.given[(size_t)nt * m + i];
        if (lane == 0 && a.sfr && a.ntab == 0) a.sfr[m] = NAN;
        __syncwarp();
    } else {
        const int sfh = a.sfh;
        SfhT<double> s;
        sfh_setup(sfh, p, s);
        int imax = find_interval0(a.tf, nt, log10(s.tage)) + 1 + 2;
        imax = imax < 1 ? 1 : (imax > nt ? nt : imax);
        if (sfh == 0) {
            s.type = -1;
            s.tb = s.tage;
            warp_component(a.tf, nt, s, imax - 2 > 1 ? imax - 2 : 1, imax, nullptr, M0s, M1s, w, lane);
        } else if (sfh == 5) {
            // the delayed tau over [tq, tage] and the ramp over [t0, tq], each normalised, mixed by the ramp's
            // mass fraction at tage
            s.type = 4;
            warp_component(a.tf, nt, s, 0, imax, a.mtab ? a.mtab + (size_t)nt * m : nullptr, M0s, M1s, t1, lane);
            s.type = 5;
            s.simha = 1;
            warp_component(a.tf, nt, s, 0, imax, nullptr, M0s, M1s, t2, lane);
            double p1 = 0.0, p2 = 0.0;
            for (int i = lane; i < imax; i += 32) { p1 += t1[i]; p2 += t2[i]; }
            double mass1 = warp_sum(p1), mass2 = warp_sum(p2);
            if (mass1 < SAFE_FLOOR) mass1 = 1.0;
            if (mass2 < SAFE_FLOOR) mass2 = 1.0;
            double mf, sfr, fl;
            sfh_props(a.tf, nt, sfh, p, mf, sfr, fl);
            const double ca = (1.0 - fl) / mass1, cb = fl / mass2;
            for (int i = lane; i < nt; i += 32) w[i] = t1[i] * ca + t2[i] * cb;
            __syncwarp();
        } else {
            s.type = sfh;
            warp_component(a.tf, nt, s, 0, imax, a.mtab ? a.mtab + (size_t)nt * m : nullptr, M0s, M1s, w, lane);
            double part = 0.0;
            for (int i = lane; i < imax; i += 32) part += w[i];
            double mass1 = warp_sum(part);
            if (mass1 < SAFE_FLOOR) mass1 = 1.0;
            for (int i = lane; i < nt; i += 32) w[i] = w[i] / mass1;
            __syncwarp();
            const double cst = p[SFH_CONST], fb_in = p[SFH_FBURST];
            if (cst > 0.0 || fb_in > SAFE_FLOOR) {
                s.type = 0;
                warp_component(a.tf, nt, s, 0, imax, nullptr, M0s, M1s, t1, lane);
                part = 0.0;
                for (int i = lane; i < imax; i += 32) part += t1[i];
                double m1 = warp_sum(part);
                if (m1 < SAFE_FLOOR) m1 = 1.0;
                double fb = 0.0;
                if (s.tb >= 0.0) {
                    s.type = -1;
                    warp_component(a.tf, nt, s, 0, imax, nullptr, M0s, M1s, t2, lane);
                    fb = fb_in;
                } else {
                    for (int i = lane; i < nt; i += 32) t2[i] = 0.0;
                    __syncwarp();
                }
                for (int i = lane; i < nt; i += 32) w[i] = (1.0 - cst - fb) * w[i] + cst * (t1[i] / m1) + fb * t2[i];
                __syncwarp();
            }
        }
        if (lane == 0 && a.sfr) a.sfr[m] = sfh_sfr(a.tf, nt, sfh, p);
    }
    double *wg = a.w + (size_t)nt * m;
    for (int i = lane; i < nt; i += 32) wg[i] = w[i];
    int zlo;
    double dz;
    zinterval(a.lz, nz, p[SFH_LOGZSOL], zlo, dz);
    double *wz = a.wz + (size_t)nt * nz * m;
    for (int k = lane; k < nt * nz; k += 32) {
        const int z = k / nt, t = k - z * nt;
        const double wt = w[t];
        double v = 0.0;
        if (z == zlo) v = (1.0 - dz) * wt;
        else if (z == zlo + 1) v = dz * wt;
        wz[k] = v;
    }
    // log L_bol blended between the slabs, then exponentiated (the SSP's own interpolation); ages <= dust_tesc young
    double ls = 0.0, ly = 0.0, lo = 0.0;
    for (int t = lane; t < nt; t += 32) {
        const double wt = w[t];
        if (!(wt > SAFE_FLOOR)) continue;
        const double lk = wt * pow(10.0, (1.0 - dz) * a.lbol[t + (size_t)nt * zlo] + dz * a.lbol[t + (size_t)nt * (zlo + 1)]);
        ls += lk;
        if (t < a.itesc) ly += lk; else lo += lk;
    }
    ls = warp_sum(ls);
    ly = warp_sum(ly);
    lo = warp_sum(lo);
    if (lane == 0) {
        a.lblend[3 * m] = ls;
        a.lblend[3 * m + 1] = ly;
        a.lblend[3 * m + 2] = lo;
    }
}

// sfh_weights_core_pc for the tabular SFHs (sfh 2, 3; src/physics/opensps_sfh.f90:1215-1293) with one metallicity,
// one warp per model (TAB_WARPS per CTA): each table bin j, rows j and j + 1 (ages T, SFRs S), is the linear SFR
// between them, a type-5 segment over the lookback window [tage - T_(j+1), tage - T_j] clamped to [1 yr, the grid's
// oldest age], with slope -(S_(j+1) - S_j) / dt / S_(j+1); its hat-kernel weights over its own index range (the
// reference's interval loop, the moments carried from one interval to the next, and the youngest edge) are scaled to
// the bin's mass S_(j+1) (1 + slope / 2 (tage' + tq - 2 t1)) (tage' - tq) over their sum. The weights are the masses
// formed (M_sun). Lane l takes bins l, l + 32, ... into its own row of shared memory; the rows are summed per age in
// lane order (deterministic). A bin whose scale is not finite turns every weight to NaN, as the reference's
// w += tmp1 (mass2 / mass1) does. The SFR: the table's, interpolated at tage (get_sfh_properties_at_age_pc
// :458-480; the mass fraction 1). Written: w (n x nt) and sfr.
constexpr int TAB_WARPS = 2;
__global__ void __launch_bounds__(TAB_WARPS * 32) sfh_tab_kernel(SfhArgs a) {
    extern __shared__ double tab_rows[];             // TAB_WARPS x 32 x nt
    const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
    const int m = blockIdx.x * TAB_WARPS + wi;
    if (m >= a.n) return;
    const int nt = a.nt, ntab = a.ntab;
    const double *tf = a.tf, *T = a.tab, *S = a.tab + ntab + 1;
    double *row = tab_rows + ((size_t)wi * 32 + lane) * nt;
    for (int i = 0; i < nt; ++i) row[i] = 0.0;
    const double tage = a.par[(size_t)SFH_NCOL * m + SFH_TAGE] * 1.0e9;
    const double tmax = pow(10.0, tf[nt - 1]);
    bool bad = false;
    for (int b = lane; b < ntab - 1; b += 32) {
        const double t1 = tage - T[b + 1], t2 = tage - T[b];
        if (t2 < 0.0) continue;
        const double dt = fmax(t2 - t1, SAFE_FLOOR);
        SfhT<double> s;
        s.type = 5;
        s.simha = 0;
        s.tau = s.tb = s.t0 = 0.0;
        s.slope = -(S[b + 1] - S[b]) / dt / fmax(S[b + 1], SAFE_FLOOR);
        s.tq = fmin(fmax(t1, 1.0), tmax);
        s.tage = fmin(fmax(t2, 1.0), tmax);
        s.trunc = s.tage - s.tq;
        const double mass2 = S[b + 1] * (1.0 + s.slope / 2.0 * (s.tage + s.tq - 2.0 * t1)) * (s.tage - s.tq);
        int imin = find_interval0(tf, nt, log10(fmax(t1, SAFE_FLOOR)));          // the reference's index - 1
        int imax = find_interval0(tf, nt, log10(fmax(t2, SAFE_FLOOR))) + 3;      // and + 2, 1-based
        imin = imin < 0 ? 0 : (imin > nt ? nt : imin);
        imax = imax < 0 ? 0 : (imax > nt ? nt : imax);
        double lts, lte;
        sfh_window(s, lts, lte);
        int js = find_interval0(tf, nt, lts) + 1, je = find_interval0(tf, nt, lte) + 2;
        const int lo_bound = imin > 1 ? imin : 1, hi_bound = imax < nt - 1 ? imax : nt - 1;
        if (js < lo_bound) js = lo_bound;
        if (je > hi_bound) je = hi_bound;
        // the bin's weights summed: its moments' change over its intervals, and the youngest edge
        double m0s, m1s, m0e, m1e, mass1 = 0.0, edge = 0.0;
        if (js <= je) {
            moments_log(fmin(fmax(tf[je], lts), lte), s, m0e, m1e);
            moments_log(fmin(fmax(tf[js - 1], lts), lte), s, m0s, m1s);
            mass1 = m0e - m0s;
        }
        if (imin == 0) {
            const double l1 = fmin(fmax(0.0, lts), lte), l2 = fmin(fmax(tf[0], lts), lte);
            if (l1 < l2) {
                moments_log(l2, s, m0e, m1e);
                moments_log(l1, s, m0s, m1s);
                edge = m0e - m0s;
            }
        }
        mass1 += edge;
        if (mass1 < SAFE_FLOOR) mass1 = 1.0;
        const double scale = mass2 / mass1;
        if (!isfinite(scale)) { bad = true; continue; }
        if (js <= je) {
            double lim_prev = fmin(fmax(tf[js - 1], lts), lte), m0p, m1p;
            moments_log(lim_prev, s, m0p, m1p);
            for (int j = js; j <= je; ++j) {
                const double lim2 = fmin(fmax(tf[j], lts), lte);
                if (lim2 <= lim_prev) { lim_prev = lim2; continue; }
                double m0c, m1c;
                moments_log(lim2, s, m0c, m1c);
                const double d0 = m0c - m0p, d1 = m1c - m1p;
                m0p = m0c;
                m1p = m1c;
                const double lo = tf[j - 1], hi = tf[j], inv = 1.0 / (hi - lo);
                row[j - 1] += (hi * d0 - d1) * inv * scale;
                row[j] += (d1 - lo * d0) * inv * scale;
                lim_prev = lim2;
            }
        }
        if (imin == 0) row[0] += edge * scale;
    }
    bad = __any_sync(0xffffffffu, bad);
    __syncwarp();
    const double *rows = tab_rows + (size_t)wi * 32 * nt;
    double *wg = a.w + (size_t)nt * m;
    for (int i = lane; i < nt; i += 32) {
        double v = 0.0;
        for (int l = 0; l < 32; ++l) v += rows[(size_t)l * nt + i];
        wg[i] = bad ? NAN : v;
    }
    if (lane == 0 && a.sfr) {
        int idx = find_interval0(T, ntab, tage) + 1;
        idx = idx > ntab - 1 ? ntab - 1 : idx;
        idx = idx < 1 ? 1 : idx;
        const double v = S[idx - 1] + (S[idx] - S[idx - 1]) / (T[idx] - T[idx - 1]) * (tage - T[idx - 1]);
        a.sfr[m] = fmax(v, 0.0);
    }
}

// The series' reciprocal table in constant memory, once per device.
static cudaError_t sfh_init_tables(cudaStream_t st) {
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    if (dev < 64 && done[dev]) return cudaSuccess;
    static double h[SFH_NSER];
    for (int k = 0; k < SFH_NSER; ++k) h[k] = 1.0 / (((double)k + 1.0) * ((double)k + 1.0));
    if ((e = cudaMemcpyToSymbolAsync(c_inv_sq, h, sizeof(h), 0, cudaMemcpyHostToDevice, st)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    if (dev < 64) done[dev] = true;
    return cudaSuccess;
}

cudaError_t run_sfh_forward(const SfhArgs &a, cudaStream_t st) {
    if (a.n <= 0) return cudaSuccess;
    cudaError_t e = sfh_init_tables(st);
    if (e != cudaSuccess) return e;
    SfhArgs b = a;
    if (a.given || (a.sfh != 1 && a.sfh != 4 && a.sfh != 5)) b.mtab = nullptr;
    if (b.mtab) {
        const size_t tot = (size_t)a.n * a.nt;
        sfh_moments_kernel<<<(unsigned)((tot + 127) / 128), 128, 0, st>>>(b);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if (a.nt > SFH_WMAXT) return cudaErrorInvalidValue;
    if ((a.sfh == 2 || a.sfh == 3) && !a.given) {
        if (a.ntab < 1 || !a.tab) return cudaErrorInvalidValue;
        const size_t smem = sizeof(double) * TAB_WARPS * 32 * (size_t)a.nt;
        if (smem > 48 * 1024 &&
            (e = cudaFuncSetAttribute(sfh_tab_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
            return e;
        sfh_tab_kernel<<<(a.n + TAB_WARPS - 1) / TAB_WARPS, TAB_WARPS * 32, smem, st>>>(b);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        b.given = a.w;
    } else {
        b.ntab = 0;
    }
    sfh_forward_kernel<<<(a.n + SFH_WARPS - 1) / SFH_WARPS, SFH_WARPS * 32, 0, st>>>(b);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------- reverse pass
// One thread per model: dL / dw_t = (1 - dz) wzb(t, zlo) + dz wzb(t, zlo + 1) + lbol_bar L~_t / (ln 10 L~) (wzb
// without the linear L_bol term; L~ the log-blended L_bol), the weights' cotangent (weights_bar); the SFH
// parameters' rows sum_t dL/dw_t dw_t/dtheta with the tangents of the weights (batch_sfh_gradients,
// src/physics/opensps_csp_batch.f90:5198-5218); logzsol's row through dz (dchain(7) = 1 / (lz(zlo+1) - lz(zlo))).
__global__ void __launch_bounds__(64) sfh_reverse_kernel(SfhRevArgs a) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= a.n) return;
    const int nt = a.nt, nz = a.nz;
    const double *p = a.par + (size_t)SFH_NCOL * m;
    const double *w = a.w + (size_t)nt * m;
    const double *wzb = a.wzb + (size_t)nt * nz * m;
    int zlo;
    double dz;
    zinterval(a.lz, nz, p[SFH_LOGZSOL], zlo, dz);
    const double ls = a.lblend[3 * m];
    double lbar = (a.lbol_bar && ls > SAFE_FLOOR) ? a.lbol_bar[m] / (ls * SFH_LN10) : 0.0;
    if (a.lsum_bar) lbar += a.lsum_bar[m];   // (the AGN's scale: this log-blended L_bol, linear)
    double gz = 0.0;   // dL / d dz
    double *wb = a.weights_bar ? a.weights_bar + (size_t)nt * m : nullptr;
    for (int t = 0; t < nt; ++t) {
        const double b0 = wzb[t + (size_t)nt * zlo], b1 = wzb[t + (size_t)nt * (zlo + 1)];
        double g = (1.0 - dz) * b0 + dz * b1;
        gz += w[t] * (b1 - b0);
        if (lbar != 0.0 && w[t] > SAFE_FLOOR) {
            const double l0 = a.lbol[t + (size_t)nt * zlo], l1 = a.lbol[t + (size_t)nt * (zlo + 1)];
            const double lt = pow(10.0, (1.0 - dz) * l0 + dz * l1);
            g += lbar * lt;
            gz += lbar * w[t] * lt * SFH_LN10 * (l1 - l0);
        }
        if (wb) wb[t] = g;
        a.scratch[(size_t)nt * m + t] = g;
    }
    double *pb = a.params_bar + (size_t)a.rows * m;
    pb[PB_LOGZSOL] = a.has_logzsol ? gz / (a.lz[zlo + 1] - a.lz[zlo]) : 0.0;
    if (!a.sfh_tangents) return;
    // the tangents of the weights (all eight directions in one pass)
    Dual pd[SFH_NPAR];
#pragma unroll
    for (int i = 0; i < SFH_NPAR; ++i) {
        pd[i] = dconst(p[i]);
        pd[i].d[i] = 1.0;
    }
    Dual *dw = reinterpret_cast<Dual *>(a.dual) + (size_t)3 * nt * m;
    sfh_weights_core<Dual>(a.tf, nt, a.sfh, pd, dw, dw + nt, dw + 2 * nt, 1);
    double acc[SFH_NPAR];
#pragma unroll
    for (int i = 0; i < SFH_NPAR; ++i) acc[i] = 0.0;
    for (int t = 0; t < nt; ++t) {
        const double g = a.scratch[(size_t)nt * m + t];
#pragma unroll
        for (int i = 0; i < SFH_NPAR; ++i) acc[i] += g * dw[t].d[i];
    }
    const int row[SFH_NPAR] = {PB_TAGE, PB_TAU, PB_CONST, PB_FBURST, PB_TBURST, PB_SF_START, PB_SF_TRUNC, PB_SF_SLOPE};
#pragma unroll
    for (int i = 0; i < SFH_NPAR; ++i) pb[row[i]] = acc[i];
}

cudaError_t run_sfh_reverse(const SfhRevArgs &a, cudaStream_t st) {
    if (a.n <= 0) return cudaSuccess;
    cudaError_t e0 = sfh_init_tables(st);
    if (e0 != cudaSuccess) return e0;
    sfh_reverse_kernel<<<(a.n + 63) / 64, 64, 0, st>>>(a);
    return cudaGetLastError();
}

size_t sfh_dual_bytes() { return sizeof(Dual); }

}  // namespace sps
