// The diffuse dust's attenuation curves of the batch (attenuation_tables_cached / attenuation_table_row and
// pixel_transmissions, OpenSPS src/physics/opensps_csp_batch.f90:3494-3560,3765-3818): per pixel up to four FP64
// tables from the curve functions at a few parameter values, and per model up to four scalars, so that
//     curve(pixel, model) = (T0 + s1 T1 + s2 T2 + s3 T3) (lambda / 5500)^ed.
// dust_type 0 (power law): T0 = 1, ed = dust_index. 1 (Cardelli, Clayton & Mathis 1989 with R_V = mwr and the 2175 A
// bump scaled by uvb): the curve is bilinear in 1 / R_V and uvb, s = (1 / mwr, uvb, uvb / mwr). 2 (Calzetti et al.
// 2000) and 6 (Reddy et al. 2015): T0 alone. 4 (Kriek & Conroy 2013): linear in delta once its power law is factored
// out, s1 = ed = dust_index. Types 3 (Witt & Gordon's dusty environments: the optical depth itself, dust2 not applied)
// and 5 (the SMC bar) are table lookups (compute_attenuation_curve_point :237-270) of the data root's
// attenuation/dirty and attenuation/smc_bar libraries on the grid: T0 alone.
//
// The curve functions restate the published forms with the reference's constants and extensions beyond their ranges
// (src/physics/opensps_dust.f90:47-160 constants; get_ccm89_curve_point :424-556, get_calzetti_curve_point :567-594,
// get_kriek_conroy_curve_point :598-626, get_reddy_curve_point :630-662). Host code, FP64.
#include <cmath>
#include <vector>
#include "context.h"
#include "datalib.h"

namespace sps {

namespace {

constexpr double V_BAND = 5500.0;

// CCM89 at wavenumber x = 1 / lambda[um]: a(x) + b(x) / R_V per region.
void ccm_optical(double y, double &a, double &b) {
    // polynomials in y = x - 1.82 (1.1 <= x < 3.3), highest power first
    static const double ca[8] = {0.32999, -0.77530, 0.01979, 0.72085, -0.02427, -0.50447, 0.17699, 1.0};
    static const double cb[8] = {-2.09002, 5.30260, -0.62251, -5.38434, 1.07233, 2.28305, 1.41338, 0.0};
    a = 0.0;
    b = 0.0;
    for (int k = 0; k < 8; ++k) { a = a * y + ca[k]; b = b * y + cb[k]; }
}
void ccm_ultraviolet(double x, double uvb, double &a, double &b) {
    // linear term and the Drude bump (scaled by uvb), 3.3 <= x < 8
    const double da = (x - 4.67) * (x - 4.67) + 0.341, db = (x - 4.62) * (x - 4.62) + 0.263;
    a = 1.752 - 0.316 * x - 0.104 * uvb / da;
    b = -3.09 + 1.825 * x + 1.206 * uvb / db;
}
double ccm89(double lam, double rv, double uvb) {
    const double x = 1.0e4 / lam;
    double a, b;
    if (x < 0.1) return 0.0;                                  // no extinction beyond 10 um
    if (x < 1.1) {                                            // infrared power law, extended from 3.3 to 10 um
        const double p = std::pow(x, 1.61);
        return 0.574 * p - 0.527 * p / rv;
    }
    if (x < 3.3) {
        ccm_optical(x - 1.82, a, b);
        return a + b / rv;
    }
    if (x < 8.0) {
        ccm_ultraviolet(x, uvb, a, b);
        if (x >= 5.9) {                                       // far-UV curvature
            const double t = x - 5.9, t2 = t * t;
            a += -0.04473 * t2 - 0.009779 * t2 * t;
            b += 0.2130 * t2 + 0.1207 * t2 * t;
            return a + b / rv;
        }
        // the near UV closes the gap to the optical form at x = 3.3, the gap fading as (3.3 / x)^6
        double ao, bo, au, bu;
        ccm_optical(3.3 - 1.82, ao, bo);
        ccm_ultraviolet(3.3, uvb, au, bu);
        const double gap = (ao + bo / rv) - (au + bu / rv), r = 3.3 / x, r3 = r * r * r;
        return a + b / rv + gap * r3 * r3;
    }
    const double t = std::min(x, 12.0) - 8.0;                 // far-UV cubic, held at lambda = 833 A below
    a = -1.073 + t * (-0.628 + t * (0.137 - 0.070 * t));
    b = 13.67 + t * (4.257 + t * (-0.42 + 0.374 * t));
    return a + b / rv;
}

// Calzetti et al. 2000 eq. 4 with R_V = 4.05: k' below 0.63 um the cubic in x, above it the linear law, both extended
// beyond 0.12-2.2 um, clipped at zero; A / A_V = k' / R_V.
double calzetti(double lam) {
    const double x = 1.0e4 / lam;
    const double k = (lam > 6300.0) ? 2.659 * (-1.857 + 1.040 * x) + 4.05
                                    : 4.05 + 2.659 * (-2.156 + x * (1.509 + x * (-0.198 + 0.011 * x)));
    return std::max(k, 0.0) / 4.05;
}

// Kriek & Conroy 2013: (k'_Calzetti + E_b D) / 4.05 (lambda / 5500)^delta, the Drude profile D at 2175 A of width
// 350 A, E_b = 0.85 - 1.9 delta.
double kriek_conroy(double lam, double delta) {
    const double w2 = (lam * 350.0) * (lam * 350.0), d = lam * lam - 2175.0 * 2175.0;
    const double bump = (0.85 - 1.9 * delta) * w2 / (d * d + w2);
    return (4.05 * calzetti(lam) + bump) / 4.05 * std::pow(lam / V_BAND, delta);
}

// Reddy et al. 2015 with R_V = 2.505: below 0.6 um the UV cubic (x held at 1 / 0.15 um for shorter wavelengths),
// from 0.6 to 2.85 um the optical cubic with the reference's continuity offset, zero beyond; A / A_V = k / R_V.
double reddy(double lam) {
    const double x = 1.0e4 / lam;
    double k = 0.0;
    if (lam < 6000.0) {
        const double xc = std::min(x, 1.0e4 / 1500.0);
        k = -5.726 + xc * (4.004 + xc * (-0.525 + 0.029 * xc)) + 2.505;
    } else if (lam < 28500.0) {
        k = -2.672 + x * (-0.010 + x * (1.532 - 0.412 * x)) + 2.505 - 0.036221981;
    }
    return k / 2.505;
}

}  // namespace

bool dust_type_supported(int dust_type) { return dust_type >= 0 && dust_type <= 6; }

int attenuation_load(Context &c, std::string &err) {
    const std::string root = data_root();
    const char *name = c.dust_type == 5 ? "smc_bar" : "dirty";
    std::vector<double> &dst = c.dust_type == 5 ? c.att_smc : c.att_wg;
    if (!dst.empty()) return 0;
    if (!datalib_available(root, "attenuation", name)) {
        err = std::string("dust_type ") + std::to_string(c.dust_type) + ": the attenuation/" + name +
              " library is missing under the data root " + root;
        return ST_DATA_MISSING;
    }
    return std_load_attenuation(root, name, c.lam, dst, err);
}

void dust_tables(int dust_type, const std::vector<double> &lam, const double *lookup, std::vector<double> &tab) {
    const size_t ns = lam.size();
    tab.assign(4 * ns, 0.0);
    const double R_BIG = 1.0e30;   // 1 / R_V = 1e-30: the terms without 1 / R_V
    for (size_t i = 0; i < ns; ++i) {
        double *t = tab.data() + 4 * i;
        const double l = lam[i];
        switch (dust_type) {
        case 0: t[0] = 1.0; break;
        case 1: {
            const double f00 = ccm89(l, R_BIG, 0.0), f10 = ccm89(l, 1.0, 0.0);
            const double f01 = ccm89(l, R_BIG, 1.0), f11 = ccm89(l, 1.0, 1.0);
            t[0] = f00; t[1] = f10 - f00; t[2] = f01 - f00; t[3] = f11 - f10 - f01 + f00;
            break;
        }
        case 2: t[0] = calzetti(l); break;
        case 4: {
            const double f0 = kriek_conroy(l, 0.0), f1 = kriek_conroy(l, 1.0) * (V_BAND / l);
            t[0] = f0; t[1] = f1 - f0;
            break;
        }
        case 6: t[0] = reddy(l); break;
        case 3:
        case 5: t[0] = lookup ? lookup[i] : 0.0; break;
        default: break;
        }
    }
}

void dust_scalars(int dust_type, double dust_index, double mwr, double uvb, double s[4]) {
    s[0] = s[1] = s[2] = s[3] = 0.0;
    if (dust_type == 0) {
        s[3] = dust_index;
    } else if (dust_type == 1) {
        s[0] = 1.0 / mwr; s[1] = uvb; s[2] = uvb / mwr;
    } else if (dust_type == 4) {
        s[0] = dust_index; s[3] = dust_index;
    }
}

double dust_curve_value(const double *t, const double s[4], double ltab) {
    const double base = t[0] + s[0] * t[1] + s[1] * t[2] + s[2] * t[3];
    return s[3] != 0.0 ? base * std::exp(s[3] * ltab) : base;
}

}  // namespace sps
