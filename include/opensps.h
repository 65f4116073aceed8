/*
 * opensps.h — the C ABI of the GB300 batched SSP/CSP path (libopensps_gb300.so).
 *
 * Each declaration below has the name, argument list and status convention of OpenSPS's public header
 * (include/opensps.h in the OpenSPS tree; the line cited beside each one), so that a C, Fortran (ISO_C_BINDING) or
 * ctypes caller of those entry points links against this library unchanged. Arrays are column-major double, the
 * caller owns every buffer, NULL means "not wanted", and every call reports through *status (0 = success) without
 * aborting; opensps_get_last_error gives the message of the last failure.
 *
 * Status codes: 0 ok; 1 bad handle; 2 unsupported combination; 3 unknown parameter or bad shape; 4 data missing
 * (also: a device failure); 301 context not set up.
 */
#ifndef OPENSPS_H
#define OPENSPS_H

#ifdef __cplusplus
extern "C" {
#endif

/* Rows of params_bar written by the gradient entry points (OpenSPS include/opensps.h:14). */
#define OPENSPS_NBGRAD 44

/* params_bar row indices (OpenSPS include/opensps.h:16-62). */
typedef enum {
    OPENSPS_BGRAD_FAGN = 0, OPENSPS_BGRAD_DUST1 = 1, OPENSPS_BGRAD_DUST2 = 2, OPENSPS_BGRAD_DUST3 = 3,
    OPENSPS_BGRAD_DUST_INDEX = 4, OPENSPS_BGRAD_DUST1_INDEX = 5, OPENSPS_BGRAD_FRAC_OBRUN = 6,
    OPENSPS_BGRAD_FRAC_NODUST = 7, OPENSPS_BGRAD_MWR = 8, OPENSPS_BGRAD_UVB = 9, OPENSPS_BGRAD_DUSTE_QPAH = 10,
    OPENSPS_BGRAD_DUSTE_UMIN = 11, OPENSPS_BGRAD_DUSTE_GAMMA = 12, OPENSPS_BGRAD_GAS_LOGZ = 13,
    OPENSPS_BGRAD_GAS_LOGU = 14, OPENSPS_BGRAD_LOGZSOL = 15, OPENSPS_BGRAD_TAGE = 16, OPENSPS_BGRAD_TAU = 17,
    OPENSPS_BGRAD_CONST = 18, OPENSPS_BGRAD_FBURST = 19, OPENSPS_BGRAD_TBURST = 20, OPENSPS_BGRAD_SF_START = 21,
    OPENSPS_BGRAD_ZRED = 22, OPENSPS_BGRAD_SIGMA_SMOOTH = 23, OPENSPS_BGRAD_SF_TRUNC = 24,
    OPENSPS_BGRAD_SF_SLOPE = 25, OPENSPS_BGRAD_IMF1 = 26, OPENSPS_BGRAD_IMF2 = 27, OPENSPS_BGRAD_IMF3 = 28,
    OPENSPS_BGRAD_VDMC = 29, OPENSPS_BGRAD_MDAVE = 30, OPENSPS_BGRAD_AGN_TAU = 31, OPENSPS_BGRAD_IGM_FACTOR = 32,
    OPENSPS_BGRAD_GAS_LOGN = 33, OPENSPS_BGRAD_GAS_LOGNO = 34, OPENSPS_BGRAD_GAS_LOGCO = 35,
    OPENSPS_BGRAD_AFE = 36, OPENSPS_BGRAD_FBHB = 37, OPENSPS_BGRAD_SBSS = 38, OPENSPS_BGRAD_AGB = 39,
    OPENSPS_BGRAD_PAGB = 40, OPENSPS_BGRAD_REDGB = 41, OPENSPS_BGRAD_DELT = 42, OPENSPS_BGRAD_DELL = 43
} opensps_bgrad_param_t;

#define OPENSPS_STATUS_OK 0
#define OPENSPS_ERR_COMPUTE_UNINIT 301
#define OPENSPS_ERR_SSP_UNINIT 303
#define OPENSPS_ERR_SSP_IMF_FILE 504       /* opensps.h:101: the user IMF file missing, unreadable or empty */
#define OPENSPS_ERR_SSP_TABULAR_SFH 508   /* opensps.h:105: the tabular SFH missing, unreadable or too long */

/* ---- driver utilities ---------------------------------------------------------------------------------- */
void opensps_clear_error(void);                                                   /* opensps.h:113 */
void opensps_get_last_error(int *status, char *message, int message_len);         /* opensps.h:114 */
void opensps_get_nbgrad(int *nbgrad);                                             /* opensps.h:125 */
void opensps_get_grad_param_name(int grad_idx, char *name, int max_len, int *status); /* opensps.h:126 */

/* ---- contexts ------------------------------------------------------------------------------------------- */
void opensps_context_create(int *handle, int *status);                            /* opensps.h:132 */
void opensps_context_destroy(int handle, int *status);                            /* opensps.h:133 */
/* Loads the libraries of the data root ($OPENSPS_DATA_HOME/synthetic): isoc_type and spec_type "synthetic" (or
 * ""), dust_type ignored (no dust emission on this path). */
void opensps_context_setup(int zin, const char *isoc_type, const char *spec_type,
                           const char *dust_type, int handle, int *status);      /* opensps.h:134-135 */
void opensps_context_set_int(int handle, const char *key, int value, int *status);      /* opensps.h:146 */
void opensps_context_set_float(int handle, const char *key, double value, int *status); /* opensps.h:147 */
void opensps_context_set_str(int handle, const char *key, const char *value, int *status); /* opensps.h:148 */
void opensps_context_set_fast_mode(int handle, int fast_mode, int *status);      /* opensps.h:151 */

void opensps_context_get_dims(int handle, int *n_spec, int *n_time, int *status); /* opensps.h:154 */
void opensps_context_get_nspec(int handle, int *n_spec, int *status);            /* opensps.h:155 */
void opensps_context_get_ntfull(int handle, int *n_time, int *status);           /* opensps.h:156 */
void opensps_context_get_nbands(int handle, int *n_bands, int *status);          /* opensps.h:157 */
void opensps_context_get_nz(int handle, int *n_z, int *status);                  /* opensps.h:159 */
void opensps_context_get_nemline(int handle, int *n_line, int *status);          /* opensps.h:160 */
void opensps_context_get_zsol(int handle, double *z_sol, int *status);           /* opensps.h:161 */
void opensps_context_get_lambda(int handle, double *lambda, int *status);        /* opensps.h:168 */
void opensps_context_get_ages(int handle, double *log_age, int *status);         /* opensps.h:169 */
void opensps_context_get_zlegend(int handle, double *z, int *status);            /* opensps.h:170 */
void opensps_context_get_emlambda(int handle, double *emlambda, int *status);    /* opensps.h:171 */

/* The standard-format filter library `name` as the context's filters (opensps.h:211-212). Libraries of the data
 * root: "gauss20", "gauss40". resample, grid_policy and vega_ref_band are accepted and not used. */
void opensps_context_set_filters_library(int handle, const char *name, int resample, int grid_policy,
                                         int vega_ref_band, int *status);
/* The bands a context computes (opensps.h:227). */
void opensps_context_set_mag_compute(int handle, int n_bands, const int *mask, int *status);
/* Tabular SFH for sfh = 3 (opensps.h:229-232): ntab (1 .. 20000) rows of age [Gyr] and SFR [M_sun/yr]; met is
 * accepted and not read (the batch forms one metallicity's weights and blends them at logzsol). status 3: ntab out of
 * range, NULL age or sfr, or ages that decrease (the reference stores those; a bin of negative width gives its
 * segment a slope over SAFE_FLOOR). sfh = 2 reads the same table from $OPENSPS_DATA_HOME/<sfh_filename> (default sfh.dat: rows of age and SFR,
 * a third column not read, the SFRs floored at SAFE_FLOOR) at the first batch after the name is set, status 508
 * when it cannot. */
void opensps_context_set_sfh_tab(int handle, int ntab, const double *age, const double *sfr, const double *met,
                                 int *status);

/* ---- batched CSPs --------------------------------------------------------------------------------------- */
/* opensps.h:266-278. ssp_weights (ntfull x n) blends each model's SSPs at its logzsol; with neither weight matrix
 * the SFH parameters are unsupported on this path (status 2). */
void opensps_context_compute_csp_batch(int handle, int n, int n_params, const char *const *names,
                                       const double *const *values, const double *ssp_weights,
                                       double *mags, double *spec, double *mass, double *lbol,
                                       double *mdust, double *sfr, double *emlines, double *indx,
                                       int *status);

/* opensps.h:291-297 */
void opensps_context_compute_csp_batch_parts(int handle, int n, int n_params, const char *const *names,
                                             const double *const *values, const double *ssp_weights,
                                             double *mags, double *spec, double *mass, double *lbol,
                                             double *mdust, double *sfr, double *emlines, double *indx,
                                             double *young, double *old, double *mass_young,
                                             double *mass_old, double *lbol_young, double *lbol_old,
                                             int *status);

/* The last batch's spectra on the device (opensps.h:315-316): nspec x n FP32 values (bytes = 4). */
void opensps_context_batch_spec_device(int handle, void **ptr, int *nspec, int *n, int *bytes, int *status);
/* The same copied to a page-locked host buffer owned by the context (opensps.h:321-322). */
void opensps_context_batch_spec_host(int handle, void **ptr, int *nspec, int *n, int *bytes, int *status);

/* opensps.h:339-348 */
void opensps_context_compute_csp_batch_grad(
    int handle, int n, int n_params, const char *const *names,
    const double *const *values, const double *ssp_weights,
    const double *ssp_weights_z, const double *zred_mags,
    const double *mags_bar, const double *spec_bar, const double *mass_bar, const double *lbol_bar,
    double *mags, double *spec, double *mass, double *lbol,
    double *mdust, double *sfr, double *emlines, double *indx,
    double *params_bar, double *weights_bar, double *weights_z_bar,
    int *status);

/* opensps.h:355-364 */
void opensps_context_compute_csp_batch_grad_rows(
    int handle, int n, int n_params, const char *const *names,
    const double *const *values, const double *ssp_weights,
    const double *ssp_weights_z, const double *zred_mags,
    const double *mags_bar, const double *spec_bar, const double *mass_bar, const double *lbol_bar,
    double *mags, double *spec, double *mass, double *lbol,
    double *mdust, double *sfr, double *emlines, double *indx,
    double *params_bar, int params_bar_rows, double *weights_bar, double *weights_z_bar,
    int *status);

/* opensps.h:367-398 */
typedef struct {
    int n;
    int n_params;
    const char *const *names;
    const double *const *values;
    const double *ssp_weights;
    const double *ssp_weights_z;
    const double *zred_mags;
    const double *mags_bar;
    const double *spec_bar;
    const double *mass_bar;
    const double *lbol_bar;
    int params_bar_rows;
} opensps_batch_options_t;

typedef struct {
    double *mags;
    double *spec;
    double *mass;
    double *lbol;
    double *mdust;
    double *sfr;
    double *emlines;
    double *indx;
    double *params_bar;
    double *weights_bar;
    double *weights_z_bar;
} opensps_batch_results_t;

/* opensps.h:401-421 */
static inline void opensps_context_compute_csp_batch_ext(int handle, const opensps_batch_options_t *opts,
                                                         opensps_batch_results_t *res, int *status) {
    if (!opts || !res || !status) {
        if (status) *status = 1;
        return;
    }
    opensps_context_compute_csp_batch_grad_rows(
        handle, opts->n, opts->n_params, opts->names, opts->values, opts->ssp_weights, opts->ssp_weights_z,
        opts->zred_mags, opts->mags_bar, opts->spec_bar, opts->mass_bar, opts->lbol_bar, res->mags, res->spec,
        res->mass, res->lbol, res->mdust, res->sfr, res->emlines, res->indx, res->params_bar,
        opts->params_bar_rows > 0 ? opts->params_bar_rows : OPENSPS_NBGRAD, res->weights_bar, res->weights_z_bar,
        status);
}

/* SSP operators (opensps.h:424-455): the SSP as an operator applied to a per-model IMF. With operators on the
 * context, imf1, imf2 and imf3 (Kroupa, imf_type 2) vary per model in the batch calls. all_metallicities: every
 * metallicity of the context is built (logzsol varies per model either way on this path). */
void opensps_context_build_ssp_ops(int handle, int all_metallicities, int *status);            /* opensps.h:430 */
/* The isochrone modification groups as free parameters (opensps.h:440): status 2 on this path. */
void opensps_context_build_ssp_ops_free_mods(int handle, int all_metallicities, int *status);  /* opensps.h:440 */
void opensps_context_free_ssp_ops(int handle, int *status);                                    /* opensps.h:443 */
void opensps_context_has_ssp_ops(int handle, int *has_ops, int *status);                       /* opensps.h:446 */
/* One IMF's SSP grid at the context's metallicity (zmet): imf_params [imf1, imf2, imf3, vdmc, mdave] or NULL
 * (the context's); mass_grid, lbol_grid (log10): ntfull; spec_grid: nspec x ntfull column-major
 * (opensps.h:451-455). */
void opensps_context_evaluate_ssp_op(int handle, int imf_type, const double *imf_params, double *mass_grid,
                                     double *lbol_grid, double *spec_grid, int *status);

#ifdef __cplusplus
}
#endif

#endif /* OPENSPS_H */
