// Device-side data layouts and kernel entry points of the batched CSP path (host-callable launchers).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>

namespace sps {

// Error codes a kernel writes into its status word (0 = ok). A bounded wait that gave up records which role.
enum {
    ERR_TIMEOUT_PRODUCER = 0x101,
    ERR_TIMEOUT_MMA = 0x102,
    ERR_TIMEOUT_EPILOGUE = 0x103,
    ERR_TIMEOUT_BAND = 0x104,
};

// Per-pixel table (floats per pixel): ln(lambda / 5500 A), the six Madau wavelength factors a_k, smoothing on/off.
enum { PIX_LTAB = 0, PIX_IGM_A = 1, PIX_SMOOTH = 7, PIX_FLOATS = 8 };

// Per-model parameter block (floats), written by the model-parameter prologue.
enum {
    MP_DUST2 = 0, MP_ONE_M_FND, MP_FND, MP_DUST_INDEX, MP_DUST1, MP_DUST1_INDEX, MP_ONE_M_FO, MP_FO, MP_DUST3,
    MP_IGM_B,                      // 6 redshift factors b_k(1 + z)
    MP_IGM_FACTOR = MP_IGM_B + 6,  // 15
    MP_IGM_TMAX, MP_IGM_JMAX,      // capped optical depth and the (1-based) pixel of the maximum (int bits)
    MP_IGM_ON,                     // 18
    MP_SMOOTH_R,                   // smoothing half-width in pixels (int bits), -1: none
    MP_TAPS,                       // 9 normalised taps, offsets -4 .. 4 (zero beyond R)
    MODEL_PAR_FLOATS = 32
};

struct ContractArgs {
    int nspec, n_models, n_ptiles, n_mtiles, nkb_young, nkb_old, jtop, ld_spec;
    const float *pix;    // nspec x PIX_FLOATS
    const float *mpar;   // n_models x MODEL_PAR_FLOATS
    float *spec;         // n_models x ld_spec (pixel fastest)
    int *status;
};

struct ContractPlan {
    CUtensorMap tm_a_hi, tm_a_lo, tm_b_hi, tm_b_lo;
    int num_sms;
};

int contract_models_per_tile(int nacc);
int contract_out_rows();
int contract_halo();
int contract_bk();
int contract_bm();
cudaError_t run_contract(int nacc, const ContractPlan &pl, const ContractArgs &a, cudaStream_t st);

// Weights prologue: FP64 weights (ntfull x nz per model) -> bf16 hi / lo in the contraction's K order, and the FP64
// per-model sums (mass, L_bol linear, young and old parts).
struct WeightsArgs {
    int n_models, nt, nz, kpad, nty_young, ky_pad;   // nty_young: ages in the young block (NACC = 2); 0 for NACC = 1
    const double *wz;       // n_models x (nt x nz), age fastest
    const double *mass;     // nt x nz
    const double *llin;     // nt x nz: 10^log L_bol
    __nv_bfloat16 *w_hi, *w_lo;   // n_models x kpad
    double *sums;           // n_models x 6: mass, lsum, mass_young, mass_old, lsum_young, lsum_old
    int itesc;              // ages <= itesc (1-based count) are young
};
cudaError_t run_weights_prep(const WeightsArgs &a, cudaStream_t st);

// Band fluxes (observed frame at each model's redshift, trapezoid filter integrals) and AB magnitudes, as a
// tensor-core GEMM over the pixels any band reaches (band_gemm.cu).
struct BandGemmArgs {
    int n_models, nspec, nbands, npad, nkb, j0, ld_spec;
    const float *spec;      // n_models x ld_spec rest-frame spectra
    const float4 *zinfo;    // n_models: (n0 as int bits, t of the interior interpolation, shift s in pixels, 0 at z = 0)
    const float *wl;        // nspec: 1 / lambda
    double dlnl;            // grid step in ln lambda
    const double *dist;     // n_models: distance term
    double zp;              // 48.60 + 2.5 ABS_MAG_ZEROPOINT_LOG
    const int *do_band;     // nbands
    double *fband;          // n_models x nbands (may be null)
    double *mags;           // n_models x nbands (may be null)
    int *status;
};
int band_gemm_npad(int nbands);
cudaError_t run_band_gemm(const BandGemmArgs &a, const CUtensorMap &tm_hi, const CUtensorMap &tm_lo,
                          cudaStream_t st);

// Casts the FP32 spectra to FP64 (the C API's double outputs), n_models x nspec from ld-strided rows.
cudaError_t run_spec_to_f64(const float *src, int ld, int nspec, int n_models, double *dst, cudaStream_t st);

}  // namespace sps
