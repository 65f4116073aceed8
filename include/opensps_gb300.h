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
 * dust_tesc. */
#define OPENSPS_GB300_DEVICE_PARAMS 11

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

/* Maximum n of opensps_gb300_spec_mags_noalloc. */
#define OPENSPS_GB300_NOALLOC_MAX_MODELS 65536

/* The magnitudes (nbands x n doubles, d_mags) of n rest-frame spectra already on the device (d_spec: nspec x n
 * floats, column-major, as opensps_context_batch_spec_device gives them) at redshifts d_zred (n doubles), through
 * the band GEMM of the batch, with no allocation: the call's scratch (observed-frame shifts, distance terms, band
 * mask, status word) is a fixed 2 MiB device array of the library, held on every device that loads the library
 * until the process exits. No counterpart in OpenSPS: it serves callers that may not allocate device memory.
 * n > OPENSPS_GB300_NOALLOC_MAX_MODELS: status 3 and nothing runs. The first call on a device looks the array's
 * address up (cudaGetSymbolAddress) and should come before any stream capture. Every call shares the array:
 * calls whose kernels overlap on the GPU (other streams, contexts or threads) race. Runs on the context's stream;
 * asynchronous unless sync != 0. The context's filter library and magnitude mask apply. */
void opensps_gb300_spec_mags_noalloc(int handle, int n, const float *d_spec, const double *d_zred, double *d_mags,
                                     int sync, int *status);

#ifdef __cplusplus
}
#endif

#endif /* OPENSPS_GB300_H */
