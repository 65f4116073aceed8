// The extern "C" entry points of include/opensps.h and include/opensps_gb300.h: a handle table over contexts, the
// parameter plumbing of the batch calls (names / values -> one parameter row per model, as OpenSPS's batch_handle,
// src/bindings/c/opensps_c_api.f90:663-961) and the status / last-error convention (never abort).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>
#include "context.h"
#include "datalib.h"
#include "../../include/opensps.h"
#include "../../include/opensps_gb300.h"

namespace sps {
void get_error(int *status, std::string *msg);
void clear_error();
void prof_harvest(Context &c, int s);
int run_grad_batch(Context &c, const BatchIO &io, const double *mags_bar, const double *spec_bar,
                   const double *mass_bar, const double *lbol_bar, double *params_bar, int params_bar_rows,
                   double *weights_z_bar, double *weights_bar, std::string &err);
int run_mags_noalloc(Context &c, int n, const float *d_spec, const double *d_zred, double *d_mags, bool sync,
                     std::string &err);
int emu_train(Context &c, long long n_train, int n_val, int epochs, int batch, int seed, const std::string &path,
              std::string &err);
int emu_load(Context &c, const std::string &path, std::string &err);
int emu_predict(Context &c, int n, const double *inputs, int fallback, double *mags, double *pca, double *spread,
                int *source, int *n_fallback, std::string &err);
int emu_infer_device(Context &c, int n, const float *d_x, float *d_mags, float *d_coef, float *d_spread, int *d_flag,
                     int *d_nflag, int *d_flagged, std::string &err);
int emu_init(Context &c, int seed, std::string &err);
int emu_params(Context &c, int set, float *host, std::string &err);
int emu_grads(Context &c, int n, const float *x_std, const float *y_std, const float *lossw, float *loss, float *grads,
              std::string &err);
}  // namespace sps

using namespace sps;

namespace {

std::mutex g_pool_mu;
std::vector<std::unique_ptr<Context>> g_pool;   // handle h -> g_pool[h - 1]

Context *lookup(int handle) {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (handle < 1 || handle > (int)g_pool.size()) return nullptr;
    return g_pool[handle - 1].get();
}

void fail(int *status, int code, const std::string &msg) {
    if (status) *status = code;
    set_error(code, msg);
}

// The gradient rows' names (params_bar rows 0..43), as opensps_get_grad_param_name.
const char *const GRAD_NAMES[OPENSPS_NBGRAD] = {
    "fagn", "dust1", "dust2", "dust3", "dust_index", "dust1_index", "frac_obrun", "frac_nodust", "mwr", "uvb",
    "duste_qpah", "duste_umin", "duste_gamma", "gas_logz", "gas_logu", "logzsol", "tage", "tau", "const", "fburst",
    "tburst", "sf_start", "zred", "sigma_smooth", "sf_trunc", "sf_slope", "imf1", "imf2", "imf3", "vdmc", "mdave",
    "agn_tau", "igm_factor", "gas_logn", "gas_logno", "gas_logco", "afe", "fbhb", "sbss", "agb", "pagb", "redgb",
    "delt", "dell"};

// The tabular SFH from ages [Gyr] and SFRs into the context (years; one zero entry past the table, where the SFR's
// interpolation reads past the last row): 0, or ST_BAD_ARG with err for decreasing ages (the device finds a model's
// bins by bisection).
int store_sfh_tab(Context &c, int ntab, const double *age, const double *sfr, std::string &err) {
    for (int i = 1; i < ntab; ++i)
        if (!(age[i] >= age[i - 1])) {
            err = "the tabular SFH's ages must not decrease on this path (row " + std::to_string(i + 1) + ")";
            return ST_BAD_ARG;
        }
    c.sfh_tab_t.assign((size_t)ntab + 1, 0.0);
    c.sfh_tab_sfr.assign((size_t)ntab + 1, 0.0);
    for (int i = 0; i < ntab; ++i) {
        c.sfh_tab_t[i] = age[i] * 1.0e9;
        c.sfh_tab_sfr[i] = sfr[i];
    }
    c.ntab = ntab;
    c.sfh_tab_dirty = true;
    return 0;
}

// load_tabular_sfh for sfh = 2 (src/io/opensps_io.f90:2375-2491): rows of age [Gyr] and SFR [M_sun / yr] (a third
// column, the metallicity, not read: the batch forms one metallicity's weights) from sfh_filename under the data
// root, at most NTABMAX rows, the SFRs floored at SAFE_FLOOR. Read again when the name changes. 0, or
// ST_TABULAR_SFH with err.
int load_sfh_file(Context &c, std::string &err) {
    const std::string path = data_root() + "/" + c.sfh_filename;
    if (c.sfh_tab_file == path && c.ntab > 0) return 0;
    std::ifstream f(path);
    if (!f) { err = "sfh = 2: cannot open the tabular SFH " + path; return ST_TABULAR_SFH; }
    std::vector<double> age, sfr;
    std::string line;
    int lineno = 0;
    while (std::getline(f, line)) {
        ++lineno;
        for (char &ch : line)
            if (ch == ',') ch = ' ';
        std::istringstream is(line);
        double a, s;
        if (!(is >> a)) {
            if (line.find_first_not_of(" \t\r") == std::string::npos) continue;   // blank
            err = "sfh = 2: cannot read line " + std::to_string(lineno) + " of " + path;
            return ST_TABULAR_SFH;
        }
        if (!(is >> s)) { err = "sfh = 2: line " + std::to_string(lineno) + " of " + path + " has one value"; return ST_TABULAR_SFH; }
        if ((int)age.size() == SFH_NTABMAX) { err = "sfh = 2: " + path + " has more than 20000 rows"; return ST_TABULAR_SFH; }
        age.push_back(a);
        sfr.push_back(s < SAFE_FLOOR ? SAFE_FLOOR : s);
    }
    if (age.empty()) { err = "sfh = 2: " + path + " has no rows"; return ST_TABULAR_SFH; }
    int st = store_sfh_tab(c, (int)age.size(), age.data(), sfr.data(), err);
    if (st) { err = "sfh = 2: " + err; return ST_TABULAR_SFH; }
    c.sfh_tab_file = path;
    return 0;
}

// names / values -> PF_COUNT x n rows (the context's values, with the named ones per model). 0, or a status.
int build_params(Context &c, int n, int n_params, const char *const *names, const double *const *values,
                 std::vector<double> &rows, std::string &err) {
    if (rows.size() < (size_t)PF_COUNT * n) rows.resize((size_t)PF_COUNT * n);
    double *rp = rows.data();
#pragma omp parallel for schedule(static) if (n >= 8192)
    for (int m = 0; m < n; ++m) std::memcpy(rp + (size_t)PF_COUNT * m, c.pdef, sizeof(double) * PF_COUNT);
    if (n_params < 0) { err = "n_params < 0"; return ST_BAD_ARG; }
    if (n_params > 0 && (!names || !values)) { err = "names / values are NULL"; return ST_BAD_ARG; }
    for (int i = 0; i < n_params; ++i) {
        const ParamInfo *pi = find_param(names[i]);
        if (!pi) { err = std::string("compute_csp_batch: unknown parameter ") + (names[i] ? names[i] : "(null)"); return ST_BAD_ARG; }
        if (pi->id < 0) {
            err = std::string("compute_csp_batch: ") + pi->name + " cannot vary per model on this path";
            return ST_UNSUPPORTED;
        }
        if (!values[i]) { err = std::string("compute_csp_batch: no values for ") + pi->name; return ST_BAD_ARG; }
        const double *v = values[i];
        const int id = pi->id;
#pragma omp parallel for schedule(static) if (n >= 8192)
        for (int m = 0; m < n; ++m) rp[(size_t)PF_COUNT * m + id] = v[m];
    }
    return 0;
}


}  // namespace

namespace sps {
// The common body of the batch entry points, on a context the caller has locked: 0 or a status (err).
int batch_core(Context &cref, int n, int n_params, const char *const *names, const double *const *values,
               const double *ssp_weights, const double *ssp_weights_z, const double *zred_mags,
               const double *mags_bar, const double *spec_bar, const double *mass_bar, const double *lbol_bar,
               double *mags, double *spec, double *mass, double *lbol, double *mdust, double *sfr, double *emlines,
               double *indx, double *young, double *old, double *mass_young, double *mass_old, double *lbol_young,
               double *lbol_old, double *params_bar, int params_bar_rows, double *weights_bar,
               double *weights_z_bar, std::string &err) {
    Context *c = &cref;
    if (n <= 0) return 0;
    if (params_bar && params_bar_rows < OPENSPS_NBGRAD) {
        err = "compute_csp_batch_grad: params_bar has " + std::to_string(params_bar_rows) + " rows, the library writes " +
              std::to_string(OPENSPS_NBGRAD) + " (opensps_get_nbgrad)";
        return ST_BAD_ARG;
    }
    if (!c->is_setup) { err = "context not set up"; return ST_NOT_SETUP; }
    if (!mags && !c->fast_mode) { err = "mags is required"; return ST_BAD_ARG; }
    if (indx) { err = "spectral indices are not computed on this path"; return ST_UNSUPPORTED; }
    if (zred_mags) { err = "zred_mags is not supported on this path"; return ST_UNSUPPORTED; }
    std::vector<double> &rows = c->param_rows;     // kept between calls (no fresh pages per batch)
    int st = build_params(*c, n, n_params, names, values, rows, err);
    if (st) return st;
    // weights: the caller's over ages and metallicities, or over ages (blended at logzsol on the device), or the
    // SFH's (formed on the device, then blended)
    std::vector<double> sfhp;
    if (!ssp_weights_z) {
        if (!ssp_weights) {
            if (c->sfh < 0 || c->sfh > 5) {
                err = "sfh = " + std::to_string(c->sfh) + ": the SFH types are 0 to 5";
                return ST_UNSUPPORTED;
            }
            if (c->sfh == 2 && (st = load_sfh_file(*c, err)) != 0) return st;
            if (c->sfh == 3 && c->ntab < 1) {
                err = "sfh = 3 without a tabular SFH (opensps_context_set_sfh_tab)";
                return ST_TABULAR_SFH;
            }
            for (int m = 0; m < n; ++m)
                if (!(rows[(size_t)PF_COUNT * m + PF_TAGE] > 0.0)) {
                    err = "models with tage <= 0 are not supported";
                    return ST_UNSUPPORTED;
                }
        }
        sfhp.resize((size_t)SFH_NCOL * n);
        const int ids[SFH_NCOL] = {PF_TAGE, PF_TAU, PF_CONST, PF_FBURST, PF_TBURST, PF_SF_START, PF_SF_TRUNC,
                                   PF_SF_SLOPE, PF_LOGZSOL};
        for (int m = 0; m < n; ++m)
            for (int k = 0; k < SFH_NCOL; ++k) sfhp[(size_t)SFH_NCOL * m + k] = rows[(size_t)PF_COUNT * m + ids[k]];
    }
    if (emlines) std::fill(emlines, emlines + (size_t)c->nline * n, 0.0);
    BatchIO io;
    io.n = n; io.params = rows.data(); io.wz = ssp_weights_z;
    if (!ssp_weights_z) { io.sfh_par = sfhp.data(); io.given_w = ssp_weights; io.sfh_type = c->sfh; }
    io.mags = mags; io.spec = spec; io.mass = mass; io.lbol = lbol; io.emlines = emlines; io.sfr = sfr;
    io.mdust = mdust; io.young = young; io.old = old; io.mass_young = mass_young; io.mass_old = mass_old;
    io.lbol_young = lbol_young; io.lbol_old = lbol_old;
    const bool grad = mags_bar || spec_bar || mass_bar || lbol_bar || params_bar || weights_bar || weights_z_bar;
    if (grad) {
        // weights over ages and metallicities: weights_bar is zero (the reference's wbl with weights_over_z)
        if (ssp_weights_z && weights_bar) std::fill(weights_bar, weights_bar + (size_t)c->nt * n, 0.0);
        st = run_grad_batch(*c, io, mags_bar, spec_bar, mass_bar, lbol_bar, params_bar, params_bar_rows,
                            ssp_weights_z ? weights_z_bar : nullptr, ssp_weights_z ? nullptr : weights_bar, err);
    } else {
        st = run_batch(*c, io, err);
    }
    return st;
}

// A forward batch with the SFH (or the context's defaults) for magnitudes only; the caller holds the lock.
int csp_batch_mags(Context &c, int n, int n_params, const char *const *names, const double *const *values,
                   double *mags, std::string &err) {
    return batch_core(c, n, n_params, names, values, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                      mags, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                      nullptr, nullptr, nullptr, nullptr, 0, nullptr, nullptr, err);
}
}  // namespace sps

namespace {

void batch_entry(int handle, int n, int n_params, const char *const *names, const double *const *values,
                 const double *ssp_weights, const double *ssp_weights_z, const double *zred_mags,
                 const double *mags_bar, const double *spec_bar, const double *mass_bar, const double *lbol_bar,
                 double *mags, double *spec, double *mass, double *lbol, double *mdust, double *sfr, double *emlines,
                 double *indx, double *young, double *old, double *mass_young, double *mass_old, double *lbol_young,
                 double *lbol_old, double *params_bar, int params_bar_rows, double *weights_bar,
                 double *weights_z_bar, int *status) {
    if (!status) return;
    *status = 0;
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    std::lock_guard<std::mutex> lk(c->mu);
    std::string err;
    const int st = batch_core(*c, n, n_params, names, values, ssp_weights, ssp_weights_z, zred_mags, mags_bar,
                              spec_bar, mass_bar, lbol_bar, mags, spec, mass, lbol, mdust, sfr, emlines, indx, young,
                              old, mass_young, mass_old, lbol_young, lbol_old, params_bar, params_bar_rows,
                              weights_bar, weights_z_bar, err);
    if (st) fail(status, st, err);
}

}  // namespace

extern "C" {

void opensps_clear_error(void) { clear_error(); }

void opensps_get_last_error(int *status, char *message, int message_len) {
    std::string msg;
    int st = 0;
    get_error(&st, &msg);
    if (status) *status = st;
    if (message && message_len > 0) {
        const int k = std::min((int)msg.size(), message_len - 1);
        std::memcpy(message, msg.data(), k);
        message[k] = '\0';
    }
}

void opensps_get_nbgrad(int *nbgrad) { if (nbgrad) *nbgrad = OPENSPS_NBGRAD; }

void opensps_get_grad_param_name(int grad_idx, char *name, int max_len, int *status) {
    if (grad_idx < 0 || grad_idx >= OPENSPS_NBGRAD) { if (status) *status = ST_BAD_ARG; return; }
    if (name && max_len > 0) {
        const int k = std::min((int)std::strlen(GRAD_NAMES[grad_idx]), max_len - 1);
        std::memcpy(name, GRAD_NAMES[grad_idx], k);
        name[k] = '\0';
    }
    if (status) *status = 0;
}

void opensps_context_create(int *handle, int *status) {
    std::unique_ptr<Context> c(new Context());
    for (int i = 0; i < PF_COUNT; ++i) c->pdef[i] = 0.0;
    // the defaults of the parameters this path reads
    const char *names[] = {"dust1", "dust2", "dust3", "dust_index", "dust1_index", "frac_nodust", "frac_obrun",
                           "zred", "igm_factor", "sigma_smooth", "dust_tesc", "logzsol", "tage", "tau",
                           "min_wave_smooth", "max_wave_smooth", "gas_logz", "gas_logu", "mwr", "uvb"};
    for (const char *nm : names) {
        const ParamInfo *p = find_param(nm);
        c->pdef[p->id] = p->def;
    }
    std::lock_guard<std::mutex> lk(g_pool_mu);
    for (size_t i = 0; i < g_pool.size(); ++i)
        if (!g_pool[i]) {
            g_pool[i] = std::move(c);
            if (handle) *handle = (int)i + 1;
            if (status) *status = 0;
            return;
        }
    g_pool.push_back(std::move(c));
    if (handle) *handle = (int)g_pool.size();
    if (status) *status = 0;
}

void opensps_context_destroy(int handle, int *status) {
    std::unique_ptr<Context> victim;
    {
        std::lock_guard<std::mutex> lk(g_pool_mu);
        if (handle < 1 || handle > (int)g_pool.size() || !g_pool[handle - 1]) {
            if (status) *status = ST_BAD_HANDLE;
            return;
        }
        victim = std::move(g_pool[handle - 1]);
    }
    { std::lock_guard<std::mutex> lk(victim->mu); }
    victim.reset();
    if (status) *status = 0;
}

void opensps_context_setup(int zin, const char *isoc_type, const char *spec_type, const char *dust_type, int handle,
                           int *status) {
    (void)zin;
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    std::lock_guard<std::mutex> lk(c->mu);
    std::string err;
    const int st = context_setup(*c, isoc_type, spec_type, dust_type, err);
    if (st) return fail(status, st, err);
    if (status) *status = 0;
}

void opensps_context_set_int(int handle, const char *key, int value, int *status) {
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    if (!key) return fail(status, 101, "NULL key");
    std::lock_guard<std::mutex> lk(c->mu);
    const std::string k(key);
    if (k == "add_neb_emission") c->add_neb_emission = value;
    else if (k == "add_igm_absorption") c->add_igm_absorption = value;
    else if (k == "smooth_velocity") c->smooth_velocity = value;
    else if (k == "dust_type") c->dust_type = value;
    else if (k == "compute_vega_mags") c->compute_vega_mags = value;
    else if (k == "sfh") c->sfh = value;
    else if (k == "nebemlineinspec") c->nebemlineinspec = value;
    else if (k == "zmet") c->zmet = value;
    else if (k == "gb300_fp64") c->fp64 = value;   // extension: the plain FP64 path
    else if (k == "gb300_ops_exact") c->ops_exact = value;   // extension: the operator's exact fold only
    else if (k == "imf_type") c->imf_type = value;
    else if (k == "keep_maggies") c->keep_maggies = value;
    else if (k == "add_dust_emission") c->add_dust_emission = value;
    else if (k == "add_agn_dust") c->add_agn_dust = value;
    else if (k == "add_neb_continuum") c->add_neb_continuum = value;
    else if (k == "cloudy_dust") c->cloudy_dust = value;
    else if (k == "wgp1") c->wgp[0] = value;   // dust_type 3: tau_v, model, structure of the curve
    else if (k == "wgp2") c->wgp[1] = value;
    else if (k == "wgp3") c->wgp[2] = value;
    else if (k == "add_stellar_remnants" ||
             k == "smoothspec_fast" || k == "compute_mags" || k == "compute_indices" ||
             k == "redshift_colors" || k == "add_xrb_emission" || k == "tpagb_norm_type" ||
             k == "vactoair_flag") {
        // known settings this path keeps at the values it implements; other values are refused at batch time
        if ((k == "add_xrb_emission" || k == "redshift_colors") && value != 0)
            return fail(status, 104, k + " = 1 is not supported on this path");
    } else {
        return fail(status, 101, "unknown integer parameter " + k);
    }
    if (status) *status = 0;
}

void opensps_context_set_float(int handle, const char *key, double value, int *status) {
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    if (!key) return fail(status, 102, "NULL key");
    std::lock_guard<std::mutex> lk(c->mu);
    const std::string k(key);
    if (k == "H0") c->h0 = value;
    else if (k == "om0") c->om0 = value;
    else if (k == "ol0") c->ol0 = value;
    else if (k == "imf_lower_limit") c->imf_lim_lo = value;   // (the SSP operators' IMF mass limits)
    else if (k == "imf_upper_limit") c->imf_lim_hi = value;
    else {
        const ParamInfo *p = find_param(key);
        if (!p) return fail(status, 102, "unknown float parameter " + k);
        if (p->id >= 0) c->pdef[p->id] = value;
    }
    if (status) *status = 0;
}

void opensps_context_set_str(int handle, const char *key, const char *value, int *status) {
    (void)value;
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    if (!key) return fail(status, 103, "NULL key");
    const std::string k(key);
    if (k == "sfh_filename") {
        if (!value || !*value) return fail(status, 103, "empty sfh_filename");
        std::lock_guard<std::mutex> lk(c->mu);
        c->sfh_filename = value;
        if (status) *status = 0;
        return;
    }
    if (k == "imf_filename") {   // (the user IMF's file under the data root; read when a batch takes imf_type 5)
        std::lock_guard<std::mutex> lk(c->mu);
        c->imf_filename = value ? value : "";
        if (status) *status = 0;
        return;
    }
    return fail(status, 103, "unknown string parameter " + k);
}

void opensps_context_set_fast_mode(int handle, int fast_mode, int *status) {
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    c->fast_mode = fast_mode;
    if (status) *status = 0;
}

#define GETTER(fn, type, expr)                                                         \
    void fn(int handle, type *out, int *status) {                                      \
        Context *c = lookup(handle);                                                   \
        if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");          \
        if (!c->is_setup) return fail(status, ST_NOT_SETUP, "context not set up");     \
        if (out) *out = (expr);                                                        \
        if (status) *status = 0;                                                       \
    }
GETTER(opensps_context_get_nspec, int, c->nspec)
GETTER(opensps_context_get_ntfull, int, c->nt)
GETTER(opensps_context_get_nbands, int, c->nbands)
GETTER(opensps_context_get_nz, int, c->nz)
GETTER(opensps_context_get_nemline, int, c->nline)
GETTER(opensps_context_get_zsol, double, c->zsol)
#undef GETTER

void opensps_context_get_dims(int handle, int *n_spec, int *n_time, int *status) {
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    if (!c->is_setup) return fail(status, ST_NOT_SETUP, "context not set up");
    if (n_spec) *n_spec = c->nspec;
    if (n_time) *n_time = c->nt;
    if (status) *status = 0;
}

#define ARRAY_GETTER(fn, vec)                                                          \
    void fn(int handle, double *out, int *status) {                                    \
        Context *c = lookup(handle);                                                   \
        if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");          \
        if (!c->is_setup) return fail(status, ST_NOT_SETUP, "context not set up");     \
        if (out) std::copy(c->vec.begin(), c->vec.end(), out);                         \
        if (status) *status = 0;                                                       \
    }
ARRAY_GETTER(opensps_context_get_lambda, lam)
ARRAY_GETTER(opensps_context_get_ages, log_age)
ARRAY_GETTER(opensps_context_get_zlegend, zlegend)
ARRAY_GETTER(opensps_context_get_emlambda, line_lambda)
#undef ARRAY_GETTER

void opensps_context_set_filters_library(int handle, const char *name, int resample, int grid_policy,
                                         int vega_ref_band, int *status) {
    (void)resample; (void)grid_policy; (void)vega_ref_band;
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    std::lock_guard<std::mutex> lk(c->mu);
    if (!c->is_setup) return fail(status, ST_NOT_SETUP, "context not set up");
    std::string err;
    const int st = context_load_filters(*c, name ? name : "", err);
    if (st) return fail(status, st, err);
    if (status) *status = 0;
}

void opensps_context_set_mag_compute(int handle, int n_bands, const int *mask, int *status) {
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    std::lock_guard<std::mutex> lk(c->mu);
    if (!c->is_setup) return fail(status, ST_NOT_SETUP, "context not set up");
    if (!mask) { c->mag_mask.clear(); if (status) *status = 0; return; }
    if (n_bands < 1 || n_bands > c->nbands) return fail(status, ST_BAD_ARG, "n_bands out of range");
    c->mag_mask.assign(c->nbands, 0);
    for (int b = 0; b < n_bands; ++b) c->mag_mask[b] = mask[b] != 0;
    if (status) *status = 0;
}

void opensps_context_set_sfh_tab(int handle, int ntab, const double *age, const double *sfr, const double *met,
                                 int *status) {
    (void)met;
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    if (ntab < 1 || ntab > SFH_NTABMAX) return fail(status, ST_BAD_ARG, "opensps_context_set_sfh_tab: ntab out of range");
    if (!age || !sfr) return fail(status, ST_BAD_ARG, "opensps_context_set_sfh_tab: age and sfr are required");
    std::lock_guard<std::mutex> lk(c->mu);
    std::string err;
    if (store_sfh_tab(*c, ntab, age, sfr, err)) return fail(status, ST_BAD_ARG, "opensps_context_set_sfh_tab: " + err);
    c->sfh_tab_file.clear();
    if (status) *status = 0;
}

void opensps_context_compute_csp_batch(int handle, int n, int n_params, const char *const *names,
                                       const double *const *values, const double *ssp_weights, double *mags,
                                       double *spec, double *mass, double *lbol, double *mdust, double *sfr,
                                       double *emlines, double *indx, int *status) {
    batch_entry(handle, n, n_params, names, values, ssp_weights, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                mags, spec, mass, lbol, mdust, sfr, emlines, indx, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                nullptr, OPENSPS_NBGRAD, nullptr, nullptr, status);
}

void opensps_context_compute_csp_batch_parts(int handle, int n, int n_params, const char *const *names,
                                             const double *const *values, const double *ssp_weights, double *mags,
                                             double *spec, double *mass, double *lbol, double *mdust, double *sfr,
                                             double *emlines, double *indx, double *young, double *old,
                                             double *mass_young, double *mass_old, double *lbol_young,
                                             double *lbol_old, int *status) {
    if (!young || !old) return fail(status, ST_BAD_ARG, "compute_csp_batch_parts: young and old are required");
    batch_entry(handle, n, n_params, names, values, ssp_weights, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                mags, spec, mass, lbol, mdust, sfr, emlines, indx, young, old, mass_young, mass_old, lbol_young,
                lbol_old, nullptr, OPENSPS_NBGRAD, nullptr, nullptr, status);
}

void opensps_context_batch_spec_device(int handle, void **ptr, int *nspec, int *n, int *bytes, int *status) {
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    std::lock_guard<std::mutex> lk(c->mu);
    if (ptr) *ptr = c->last_n > 0 ? (void *)c->d_spec.p : nullptr;
    if (nspec) *nspec = c->nspec;
    if (n) *n = c->last_n;
    if (bytes) *bytes = 4;
    if (status) *status = 0;
}

void opensps_context_batch_spec_host(int handle, void **ptr, int *nspec, int *n, int *bytes, int *status) {
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    std::lock_guard<std::mutex> lk(c->mu);
    if (ptr) *ptr = nullptr;
    if (nspec) *nspec = c->nspec;
    if (n) *n = c->last_n;
    if (bytes) *bytes = 4;
    if (c->last_n <= 0) { if (status) *status = 0; return; }
    const size_t need = sizeof(float) * (size_t)c->nspec * c->last_n;
    if (c->pinned_bytes < need) {
        if (c->pinned_spec) cudaFreeHost(c->pinned_spec);
        c->pinned_spec = nullptr;
        c->pinned_bytes = 0;
        cudaError_t e = cudaMallocHost(&c->pinned_spec, need);
        if (e != cudaSuccess) return fail(status, ST_DATA_MISSING, std::string("pinned buffer: ") + cudaGetErrorString(e));
        c->pinned_bytes = need;
    }
    cudaError_t e = cudaMemcpyAsync(c->pinned_spec, c->d_spec.p, need, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return fail(status, ST_DATA_MISSING, std::string("spectra copy: ") + cudaGetErrorString(e));
    if (ptr) *ptr = c->pinned_spec;
    if (status) *status = 0;
}

void opensps_context_compute_csp_batch_grad(int handle, int n, int n_params, const char *const *names,
                                            const double *const *values, const double *ssp_weights,
                                            const double *ssp_weights_z, const double *zred_mags,
                                            const double *mags_bar, const double *spec_bar, const double *mass_bar,
                                            const double *lbol_bar, double *mags, double *spec, double *mass,
                                            double *lbol, double *mdust, double *sfr, double *emlines, double *indx,
                                            double *params_bar, double *weights_bar, double *weights_z_bar,
                                            int *status) {
    batch_entry(handle, n, n_params, names, values, ssp_weights, ssp_weights_z, zred_mags, mags_bar, spec_bar,
                mass_bar, lbol_bar, mags, spec, mass, lbol, mdust, sfr, emlines, indx, nullptr, nullptr, nullptr,
                nullptr, nullptr, nullptr, params_bar, OPENSPS_NBGRAD, weights_bar, weights_z_bar, status);
}

void opensps_context_compute_csp_batch_grad_rows(int handle, int n, int n_params, const char *const *names,
                                                 const double *const *values, const double *ssp_weights,
                                                 const double *ssp_weights_z, const double *zred_mags,
                                                 const double *mags_bar, const double *spec_bar,
                                                 const double *mass_bar, const double *lbol_bar, double *mags,
                                                 double *spec, double *mass, double *lbol, double *mdust, double *sfr,
                                                 double *emlines, double *indx, double *params_bar,
                                                 int params_bar_rows, double *weights_bar, double *weights_z_bar,
                                                 int *status) {
    batch_entry(handle, n, n_params, names, values, ssp_weights, ssp_weights_z, zred_mags, mags_bar, spec_bar,
                mass_bar, lbol_bar, mags, spec, mass, lbol, mdust, sfr, emlines, indx, nullptr, nullptr, nullptr,
                nullptr, nullptr, nullptr, params_bar, params_bar_rows, weights_bar, weights_z_bar, status);
}

// ---------------------------------------------------------------------------------------------- extensions
void opensps_gb300_batch_device(int handle, int n, const double *d_params, const double *d_wz, double *d_mags,
                                int sync, int *status) {
    if (!status) return;
    *status = 0;
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    std::lock_guard<std::mutex> lk(c->mu);
    if (!c->is_setup) return fail(status, ST_NOT_SETUP, "context not set up");
    if (n <= 0) return;
    // the batch-wide settings come from the context; the per-model table is on the device: a copy is read here for
    // the batch's checks (88 bytes per model, into the page-locked staging buffer, on a stream of its own so that it
    // does not wait for the previous batch's kernels)
    const size_t np = (size_t)PAR_DEVICE * n;
    cudaError_t e = cudaSuccess;
    if (c->pinned_par_n < np) {
        if (c->pinned_par) cudaFreeHost(c->pinned_par);
        c->pinned_par = nullptr;
        c->pinned_par_n = 0;
        if ((e = cudaMallocHost(&c->pinned_par, sizeof(double) * np)) != cudaSuccess)
            return fail(status, ST_DATA_MISSING, std::string("page-locked parameters: ") + cudaGetErrorString(e));
        c->pinned_par_n = np;
    }
    if ((e = cudaMemcpyAsync(c->pinned_par, d_params, sizeof(double) * np, cudaMemcpyDeviceToHost, c->side2)) != cudaSuccess ||
        (e = cudaStreamSynchronize(c->side2)) != cudaSuccess)
        return fail(status, ST_BAD_ARG, std::string("d_params: ") + cudaGetErrorString(e));
    BatchIO io;
    io.n = n; io.params = c->pinned_par; io.params_cols = PAR_DEVICE; io.param_defaults = c->pdef;
    io.wz = d_wz; io.dev_inputs = true; io.dev_params = d_params;
    io.mags = d_mags; io.dev_sync = sync != 0;
    std::string err;
    const int st = run_batch(*c, io, err);
    if (st) return fail(status, st, err);
}

void opensps_context_build_ssp_ops(int handle, int all_metallicities, int *status) {
    (void)all_metallicities;
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    std::lock_guard<std::mutex> lk(c->mu);
    if (!c->is_setup) return fail(status, ST_NOT_SETUP, "context not set up");
    std::string err;
    const int st = ops_build(*c, err);
    if (st) return fail(status, st, err);
    if (status) *status = 0;
}

void opensps_context_build_ssp_ops_free_mods(int handle, int all_metallicities, int *status) {
    (void)all_metallicities;
    if (!lookup(handle)) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    fail(status, ST_UNSUPPORTED, "isochrone modification groups are not supported on this path");
}

void opensps_context_free_ssp_ops(int handle, int *status) {
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    std::lock_guard<std::mutex> lk(c->mu);
    c->ops.release();
    if (status) *status = 0;
}

void opensps_context_has_ssp_ops(int handle, int *has_ops, int *status) {
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    if (has_ops) *has_ops = c->ops.ready ? 1 : 0;
    if (status) *status = 0;
}

void opensps_context_evaluate_ssp_op(int handle, int imf_type, const double *imf_params, double *mass_grid,
                                     double *lbol_grid, double *spec_grid, int *status) {
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    std::lock_guard<std::mutex> lk(c->mu);
    if (!c->is_setup) return fail(status, ST_NOT_SETUP, "context not set up");
    std::string err;
    const int st = ops_evaluate(*c, imf_type, imf_params, mass_grid, lbol_grid, spec_grid, err);
    if (st) return fail(status, st, err);
    if (status) *status = 0;
}

void opensps_gb300_spec_mags_noalloc(int handle, int n, const float *d_spec, const double *d_zred, double *d_mags,
                                     int sync, int *status) {
    if (!status) return;
    *status = 0;
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    std::lock_guard<std::mutex> lk(c->mu);
    if (!c->is_setup) return fail(status, ST_NOT_SETUP, "context not set up");
    std::string err;
    const int st = run_mags_noalloc(*c, n, d_spec, d_zred, d_mags, sync != 0, err);
    if (st) return fail(status, st, err);
}

void opensps_gb300_context_stream(int handle, void **stream, int *device, int *status) {
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    if (stream) *stream = (void *)c->stream;
    if (device) *device = c->device;
    if (status) *status = 0;
}

void opensps_gb300_set_profiling(int handle, int on, int *status) {
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    std::lock_guard<std::mutex> lk(c->mu);
    for (int s = 0; s < 2; ++s) prof_harvest(*c, s);
    c->profile = on;
    c->prof_count = 0;
    c->prof_nstage = 0;
    for (int i = 0; i < Context::NPROF; ++i) c->prof_acc[i] = 0.0;
    if (status) *status = 0;
}

// Mean device time of each stage over the profiled batches since profiling was switched on.
void opensps_gb300_kernel_times(int handle, double *ms, int max_n, int *n, int *status) {
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    std::lock_guard<std::mutex> lk(c->mu);
    for (int s = 0; s < 2; ++s) prof_harvest(*c, s);
    int k = 0;
    for (; k < c->prof_nstage && k < max_n; ++k)
        if (ms) ms[k] = c->prof_count > 0 ? c->prof_acc[k] / c->prof_count : 0.0;
    if (n) *n = k;
    if (status) *status = 0;
}

void opensps_gb300_last_launches(int handle, int *launches, int *status) {
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    if (launches) *launches = c->last_launches;
    if (status) *status = 0;
}

void opensps_gb300_last_input_in_place(int handle, int *in_place, int *status) {
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    if (in_place) *in_place = c->last_direct ? 1 : 0;
    if (status) *status = 0;
}

// A standard-format library of the kinds this path reads, processed as the context's setup processes it (host only;
// no device or context needed): "ssp" -> log L_bol per grid point (nz x nt; lam unused), "dust_emission" -> the
// templates on lam (2 numin x nqpah columns of nspec), "agn_torus" -> ntau x nspec, "filters" -> nb x nspec bands.
void opensps_gb300_data_table(const char *root, const char *kind, const char *name, const double *lam, int nspec,
                              double *out, long long out_cap, long long *n_out, int *status) {
    if (!root || !kind || !name) return fail(status, ST_BAD_ARG, "NULL argument");
    const std::string k(kind);
    std::vector<double> grid;
    if (k != "ssp") {
        if (!lam || nspec < 2) return fail(status, ST_BAD_ARG, "a wavelength grid of at least 2 points is required");
        grid.assign(lam, lam + nspec);
    }
    std::string err;
    std::vector<double> tab, a, b;
    std::vector<std::string> names;
    int rc = 0;
    if (k == "ssp") {
        SspLibrary L;
        rc = std_load_ssp(root, name, L, err);
        tab.swap(L.lbol);
    } else if (k == "dust_emission") {
        rc = std_load_dust_emission(root, name, grid, a, b, tab, err);
    } else if (k == "agn_torus") {
        rc = std_load_agn(root, grid, a, tab, err);
    } else if (k == "filters") {
        rc = std_load_filters(root, name, grid, tab, a, names, err);
    } else if (k == "nebular") {
        std::vector<double> lu;
        rc = std_load_nebular(root, name, grid, a, b, lu, tab, err);
    } else if (k == "attenuation") {
        rc = std_load_attenuation(root, name, grid, tab, err);
    } else {
        return fail(status, ST_BAD_ARG, "kind must be ssp, dust_emission, agn_torus, filters, nebular or attenuation");
    }
    if (rc) return fail(status, rc, err);
    if (n_out) *n_out = (long long)tab.size();
    if (out) {
        if (out_cap < (long long)tab.size()) return fail(status, ST_BAD_ARG, "output buffer too small");
        std::copy(tab.begin(), tab.end(), out);
    }
    if (status) *status = 0;
}

void opensps_gb300_ops_last_fold(int handle, int *interpolated, int *status) {
    Context *c = lookup(handle);
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");
    if (interpolated) *interpolated = c->ops_last_interp ? 1 : 0;
    if (status) *status = 0;
}

// ---------------------------------------------------------------------------------------------- the emulator
#define EMU_ENTRY_PROLOGUE()                                                          \
    Context *c = lookup(handle);                                                      \
    if (!c) return fail(status, ST_BAD_HANDLE, "invalid context handle");             \
    std::lock_guard<std::mutex> lk(c->mu);                                            \
    if (!c->is_setup) return fail(status, ST_NOT_SETUP, "context not set up");        \
    std::string err;                                                                  \
    if (status) *status = 0;

void opensps_gb300_emulator_train(int handle, const char *path, long long n_train, int n_val, int epochs, int batch,
                                  int seed, int *status) {
    EMU_ENTRY_PROLOGUE();
    if (int st = emu_train(*c, n_train, n_val, epochs, batch, seed, path ? path : "", err)) fail(status, st, err);
}

void opensps_gb300_emulator_load(int handle, const char *path, int *status) {
    EMU_ENTRY_PROLOGUE();
    if (!path) return fail(status, ST_BAD_ARG, "NULL path");
    if (int st = emu_load(*c, path, err)) fail(status, st, err);
}

void opensps_gb300_emulator_free(int handle, int *status) {
    EMU_ENTRY_PROLOGUE();
    c->emu.release();
}

void opensps_gb300_emulator_info(int handle, double *info, int max_n, int *n, int *status) {
    EMU_ENTRY_PROLOGUE();
    if (!c->emu.ready) return fail(status, ST_NO_OPERATOR, "no emulator on the context");
    int k = 0;
    for (; k < (int)c->emu.info.size() && k < max_n; ++k)
        if (info) info[k] = c->emu.info[k];
    if (n) *n = k;
}

void opensps_gb300_emulator_predict(int handle, int n, const double *inputs, int fallback, double *mags, double *pca,
                                    double *spread, int *source, int *n_fallback, int *status) {
    EMU_ENTRY_PROLOGUE();
    if (int st = emu_predict(*c, n, inputs, fallback, mags, pca, spread, source, n_fallback, err)) fail(status, st, err);
}

void opensps_gb300_emulator_predict_device(int handle, int n, const float *d_inputs, float *d_mags, float *d_pca,
                                           float *d_spread, int *d_flag, int *d_flagged, int *n_flagged, int sync,
                                           int *status) {
    EMU_ENTRY_PROLOGUE();
    if (n <= 0) { if (n_flagged) *n_flagged = 0; return; }
    if (!d_inputs || !d_mags || !d_flag || !d_flagged) return fail(status, ST_BAD_ARG, "NULL device array");
    if (!c->emu.d_nflag && cudaMalloc(&c->emu.d_nflag, sizeof(int)) != cudaSuccess)
        return fail(status, ST_DATA_MISSING, "device memory");
    if (int st = emu_infer_device(*c, n, d_inputs, d_mags, d_pca, d_spread, d_flag, c->emu.d_nflag, d_flagged, err))
        return fail(status, st, err);
    if (n_flagged || sync) {
        int s = 0, nf = 0;
        cudaMemcpyAsync(&s, c->d_status.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
        cudaMemcpyAsync(&nf, c->emu.d_nflag, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
        const cudaError_t e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return fail(status, ST_DATA_MISSING, std::string("emulator: ") + cudaGetErrorString(e));
        if (s != 0) return fail(status, ST_DATA_MISSING, "emulator kernel gave up waiting");
        if (n_flagged) *n_flagged = nf;
    }
}

void opensps_gb300_emulator_set_threshold(int handle, double spread_max, double faint, int *status) {
    EMU_ENTRY_PROLOGUE();
    if (!(spread_max > 0.0) || !(faint > 0.0)) return fail(status, ST_BAD_ARG, "thresholds must be positive");
    c->emu.spread_max = (float)spread_max;
    c->emu.faint = (float)faint;
}

void opensps_gb300_emulator_init(int handle, int seed, int *status) {
    EMU_ENTRY_PROLOGUE();
    if (int st = emu_init(*c, seed, err)) fail(status, st, err);
}

void opensps_gb300_emulator_param_count(long long *count) {
    if (count) *count = emu_param_count();
}

void opensps_gb300_emulator_params(int handle, int set, float *params, int *status) {
    EMU_ENTRY_PROLOGUE();
    if (!params) return fail(status, ST_BAD_ARG, "NULL params");
    if (int st = emu_params(*c, set, params, err)) fail(status, st, err);
}

void opensps_gb300_emulator_grads(int handle, int n, const float *x_std, const float *y_std,
                                  const float *loss_weights, float *loss, float *grads, int *status) {
    EMU_ENTRY_PROLOGUE();
    if (!x_std || !y_std || !loss_weights || !loss || !grads) return fail(status, ST_BAD_ARG, "NULL argument");
    if (int st = emu_grads(*c, n, x_std, y_std, loss_weights, loss, grads, err)) fail(status, st, err);
}

}  // extern "C"
