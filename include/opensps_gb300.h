/*
 * opensps_gb300.h — entry points of libopensps_gb300.so that OpenSPS does not have.
 *
 * They serve callers that keep their inputs on the GPU (a fitting loop that draws its weights on the device, the
 * benchmark's device-resident timing). They have no counterpart in OpenSPS's include/opensps.h.
 */
#ifndef OPENSPS_GB300_H
#define OPENSPS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* Number of doubles per model in the device parameter table of opensps_gb300_batch_device, and their order:
 * dust1, dust2, dust3, dust_index, dust1_index, frac_nodust, frac_obrun, zred, igm_factor, sigma_smooth,
 * dust_tesc, mwr, uvb. */
#define OPENSPS_GB300_DEVICE_PARAMS 13

/* A batch of n models whose inputs are already in device memory: d_params (OPENSPS_GB300_DEVICE_PARAMS x n
 * doubles, column-major) and d_wz (ntfull x nz x n doubles, the ssp_weights_z of the C API). The context's
 * settings and its min/max_wave_smooth apply. Outputs stay on the device: the spectra in the context's buffer
 * (opensps_context_batch_spec_device) and, when d_mags is not NULL, the magnitudes (nbands x n doubles) in d_mags.
 * Asynchronous on the context's stream unless sync != 0. Status as opensps_context_compute_csp_batch. */
void opensps_gb300_batch_device(int handle, int n, const double *d_params, const double *d_wz, double *d_mags,
                                int sync, int *status);

/* The context's CUDA stream (cudaStream_t) and the device it runs on. */
void opensps_gb300_context_stream(int handle, void **stream, int *device, int *status);

/* With on != 0, CUDA events are recorded between the kernels of every batch on the handle; afterwards
 * opensps_gb300_kernel_times gives the device time of each stage of the last batch in milliseconds, in order: the
 * per-model parameters, the weight operand, the contraction with its epilogue, the band fluxes and magnitudes, the
 * FP64 mass and L_bol sums; after a gradient call also the forward's output copies with the cotangents' copies
 * (host time included), the per-model adjoint, the weights' GEMMs and the weights' cotangent kernel (mean over the
 * batches since profiling was switched on). At most 9 stages. */
void opensps_gb300_set_profiling(int handle, int on, int *status);
void opensps_gb300_kernel_times(int handle, double *ms, int max_n, int *n, int *status);

/* Kernel launches of the last batch on the handle (for the benchmark's launch count). */
void opensps_gb300_last_launches(int handle, int *launches, int *status);

/* 1 when the last batch through the SSP operator took the interpolated fold (a tcgen05 GEMM against the operator's
 * Lagrange basis in ln m: every model's |imf1| <= 2.6, |imf2| <= 3.0, |imf3| <= 3.5 and the setting "gb300_ops_exact"
 * 0), 0 when it took the exact fold. */
void opensps_gb300_ops_last_fold(int handle, int *interpolated, int *status);

/* 1 when the last batch's weights over ages and metallicities were read in place from the caller's pageable host
 * memory (a chunked batch on a device that reads pageable memory, as Grace systems do over NVLink-C2C), 0 when they
 * were copied. */
void opensps_gb300_last_input_in_place(int handle, int *in_place, int *status);

/* A data library in OpenSPS's standard format (root/libraries/<kind>/<name>/manifest.json plus raw arrays), processed
 * as opensps_context_setup processes it, without a device or a context (replaces nothing in opensps.h: the
 * reference's readers run inside its setup, src/io/opensps_io.f90:991-1318,3131-3155). kind "ssp": log10 L_bol per
 * grid point (nz x nt, the trapezoid integral of each SSP spectrum over frequency; lam unused); "dust_emission": the
 * templates interpolated onto lam (2 numin x nqpah columns of nspec, column (2 u + c) nqpah + q); "agn_torus": the 9
 * templates on lam (9 x nspec); "filters": the bands on lam normalised to int T / lambda = 1 and calibrated where
 * the library says so (nb x nspec); "nebular": log10(continuum + 1e-95) on lam (11 logZ x 10 ages x 7 logU columns of
 * nspec, column z + 11 (a + 10 u), src/io/opensps_io.f90:749-827,910-933); "attenuation": smc_bar's A(lambda) / A(V)
 * on lam (nspec) or dirty's optical depths (2 structures x 18 tau_v x 6 models curves of nspec, in that order;
 * load_attenuation_curves :2079-2234). name may
 * carry axis selections ("name:axis=value"). *n_out receives the table's length; out may be NULL to query it.
 * Status 4 with the message for a missing or malformed library. */
void opensps_gb300_data_table(const char *root, const char *kind, const char *name, const double *lam, int nspec,
                              double *out, long long out_cap, long long *n_out, int *status);

/* Maximum n of opensps_gb300_spec_mags_noalloc. */
#define OPENSPS_GB300_NOALLOC_MAX_MODELS 65536

/* The magnitudes (nbands x n doubles, d_mags) of n rest-frame spectra already on the device (d_spec: nspec x n
 * floats, column-major, as opensps_context_batch_spec_device gives them) at redshifts d_zred (n doubles), through
 * the band GEMM of the batch, with no allocation: the call's scratch (observed-frame shifts, distance terms, band
 * mask, status word) is a fixed 2 MiB device array of the library. No counterpart in OpenSPS: it serves callers that
 * may not allocate device memory (a framework's custom-call handler handed preallocated buffers, where a cudaMalloc
 * can fail and a cudaFree synchronises the device under the framework's stream).
 * n > OPENSPS_GB300_NOALLOC_MAX_MODELS: status 3 and nothing runs.
 * When the array comes into being: opensps_context_setup loads this entry point's kernels on the context's device,
 * which creates the array there (held until the process exits), and looks its address up; the call itself loads and
 * allocates nothing. A context that was not set up gives status 301. Every call shares the array: calls whose kernels
 * overlap on the GPU (other streams, contexts or threads) race. Runs on the context's stream; asynchronous unless
 * sync != 0. With sync = 0 a device wait that gave up (status 4 with sync != 0) is not reported. The context's
 * filter library and magnitude mask apply. */
void opensps_gb300_spec_mags_noalloc(int handle, int n, const float *d_spec, const double *d_zred, double *d_mags,
                                     int sync, int *status);

/* ---- The learned emulator (no counterpart in OpenSPS, whose only network is the cue nebular MLP) ----------------
 * An ensemble of five MLPs, 10 inputs -> 4 x 512 SiLU -> the first 64 PCA coefficients of log10 of the spectrum and
 * the magnitudes less the distance term (f16 weights and activations, f32 accumulation), trained on this
 * library's own CSP through the SSP operators: a Kroupa IMF per model and the delayed-tau SFH (sfh = 4) on the
 * device. Inputs, column-major OPENSPS_GB300_EMU_INPUTS x n doubles, in this order: tau [Gyr], tage [Gyr], logzsol,
 * dust2, dust_index, zred, sigma_smooth [km/s], imf1, imf2, imf3. The training box: log10 tau in [-1, 1], tage in
 * [1, 13.7], logzsol in [-2, 0.5], dust2 in [0, 3], dust_index in [-1, -0.4], zred in [0, 6], sigma_smooth in
 * [50, 300], imf1 in [0.3, 1.8], imf2 in [1.3, 2.8], imf3 in [1.8, 3.3]. A model outside the box, or whose
 * ensemble spread (the members' standard deviation, the largest over the bands less than 15 mag fainter than its
 * brightest) exceeds 0.01 mag, is flagged and, with fallback, computed by the plain CSP. */
#define OPENSPS_GB300_EMU_INPUTS 10
#define OPENSPS_GB300_EMU_NPC 64

/* Generates n_train + n_val models with the context's CSP (SSP operators built, sfh = 4, the context's other
 * settings), fits the PCA and trains the ensemble (epochs over n_train, minibatch `batch`, a multiple of 128, per
 * member), validates on the n_val models, writes the weights to path (unless path is NULL or empty) and leaves the
 * emulator on the context. Progress lines go to stderr. */
void opensps_gb300_emulator_train(int handle, const char *path, long long n_train, int n_val, int epochs, int batch,
                                  int seed, int *status);
/* Loads an emulator written by opensps_gb300_emulator_train (same band set and wavelength grid). */
void opensps_gb300_emulator_load(int handle, const char *path, int *status);
void opensps_gb300_emulator_free(int handle, int *status);
/* Training and validation figures: n_train, n_val, epochs, batch, seed, training-set seconds, training seconds,
 * validation RMS error [mag], maximum error, 99th percentile of the per-model maximum error, flagged fraction,
 * maximum error of the unflagged models, the PCA's explained variance. */
void opensps_gb300_emulator_info(int handle, double *info, int max_n, int *n, int *status);
/* Magnitudes (nbands x n, column-major), optionally the PCA coefficients (64 x n), the spread (n) and the source
 * of each model (0 emulator; 1 outside the box, 2 spread, 3 not finite: computed by the plain CSP when
 * fallback != 0). *n_fallback: the flagged count. */
void opensps_gb300_emulator_predict(int handle, int n, const double *inputs, int fallback, double *mags, double *pca,
                                    double *spread, int *source, int *n_fallback, int *status);
/* The ensemble on device inputs (n x OPENSPS_GB300_EMU_INPUTS floats, row-major): d_mags (n x nbands floats),
 * d_pca (n x 64 floats, or NULL), d_spread (n floats, or NULL), d_flag (n ints), d_flagged (the flagged models'
 * indices, at most n ints); no fallback. With n_flagged not NULL the call waits and returns the flagged count;
 * otherwise it is asynchronous on the context's stream unless sync != 0. */
void opensps_gb300_emulator_predict_device(int handle, int n, const float *d_inputs, float *d_mags, float *d_pca,
                                           float *d_spread, int *d_flag, int *d_flagged, int *n_flagged, int sync,
                                           int *status);
/* The fallback thresholds: spread_max [mag] and the faint-band cut [mag]. */
void opensps_gb300_emulator_set_threshold(int handle, double spread_max, double faint, int *status);
/* An untrained ensemble with random weights (seed), for checks of the training kernels. */
void opensps_gb300_emulator_init(int handle, int seed, int *status);
/* Number of FP32 parameters of the ensemble: weights [w0 | wh | w4] then biases (see libopensps_gb300 docs). */
void opensps_gb300_emulator_param_count(long long *count);
/* Gets (set = 0) or sets (set = 1) the FP32 parameters of a trainable emulator. */
void opensps_gb300_emulator_params(int handle, int set, float *params, int *status);
/* The training kernels' loss (5 floats, one per member) and gradients (param_count floats) on one minibatch given
 * as standardised network features x_std (n x 12 floats: the ten inputs' features, then the two grid clocks) and
 * targets y_std (n x 128 floats) with output weights
 * loss_weights (128 floats); n a multiple of 128. Every member sees the same rows. No update. */
void opensps_gb300_emulator_grads(int handle, int n, const float *x_std, const float *y_std,
                                  const float *loss_weights, float *loss, float *grads, int *status);

#ifdef __cplusplus
}
#endif

#endif /* OPENSPS_GB300_H */
