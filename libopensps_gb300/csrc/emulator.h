// The learned emulator of the CSP path: an ensemble of five MLPs from ten physical parameters to the PCA
// coefficients of the log spectrum and the magnitudes (without the distance term), trained on spectra and
// magnitudes of this library's own CSP (the SSP operator with a Kroupa IMF per model, the delayed-tau SFH on the
// device, power-law dust, IGM, smoothing). OpenSPS has no emulator of its CSP: its one network is the cue nebular
// MLP (src/physics/opensps_cue.f90; HIP cue_dense_act_kernel / cue_dense_back_kernel), the precedent for the fused
// dense layers here.
//
// Network of each member: 12 features of the 10 inputs (padded to 64) -> 4 x 512 SiLU -> 128 outputs (64 PCA coefficients, the
// magnitudes, zeros); f16 weights and activations, f32 accumulation and biases; the features enter as two f16 parts
// (hi + lo), so that their rounding does not reach the outputs. (f16, not bf16: with bf16 activations and inputs the
// rounding alone moved the magnitudes by 0.009 mag RMS, 0.065 mag at the 99th percentile; with f16 activations and
// split inputs by 0.0005 and 0.003 mag.) The training's reverse pass runs in bf16.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

namespace sps {

constexpr int EMU_NIN = 10;                  // tau [Gyr], tage [Gyr], logzsol, dust2, dust_index, zred,
                                             // sigma_smooth [km/s], imf1, imf2, imf3
constexpr int EMU_NFEAT = 12;                // the network's features: the ten inputs, then two grid clocks
constexpr int EMU_KIN = 64;                  // the input layer's K: features' hi parts at 0..11, lo parts at 16..27
constexpr int EMU_H = 512;                   // hidden width
constexpr int EMU_NOUT = 128;                // output rows (padded)
constexpr int EMU_NPC = 64;                  // PCA coefficients of the log spectrum
constexpr int EMU_MAX_BANDS = 48;            // magnitudes (outputs 64 .. 64 + nb - 1)
constexpr int EMU_MEMBERS = 5;
constexpr int EMU_NBIAS = 4 * EMU_H + EMU_NOUT;     // biases of one member: four hidden layers, then the output
// the parameter block (floats): feature centres and scales, output means and scales, the grid clocks (log-age
// origin and step, log Z origin and step), the cosmology table (z, d_L)
constexpr int EMU_P_INC = 0, EMU_P_INS = EMU_NFEAT, EMU_P_OMU = 2 * EMU_NFEAT, EMU_P_OSIG = EMU_P_OMU + EMU_NOUT;
constexpr int EMU_P_CLK = EMU_P_OSIG + EMU_NOUT, EMU_P_ZT = EMU_P_CLK + 4, EMU_P_DL = EMU_P_ZT + 500;
constexpr int EMU_PAR = EMU_P_DL + 500;
// floats of the inference kernel's scratch per CTA: the members' outputs (5 x 128 rows x 128), then two slots of
// tile inputs (128 rows x 16 words)
constexpr long long EMU_SCRATCH_CTA = (long long)EMU_MEMBERS * 128 * EMU_NOUT + 2 * 128 * 16;
// element counts of one member's weights
constexpr long long EMU_W0 = (long long)EMU_H * EMU_KIN, EMU_WH = (long long)EMU_H * EMU_H,
                    EMU_W4 = (long long)EMU_NOUT * EMU_H;

// The network's feature of input i from its raw value: log10 tau, log10 tage, log10 (1 + zred), the others as they
// are. (In log age the SSP grid's nodes, where short-tau spectra bend, are evenly spaced; the bands move with
// log (1 + z).)
__host__ __device__ inline float emu_feature(int i, float v) {
    if (i == 0 || i == 1) return v > 0.f ? log10f(v) : -INFINITY;
    if (i == 5) return v > -1.f ? log10f(1.f + v) : -INFINITY;
    return v;
}

// The twelve standardised features of one model (raw inputs x): the ten inputs' features, then two grid clocks:
// |sin(pi d)| with d the position, in grid steps, of the SFH's mass-weighted age (tage - 2 tau of the delayed-tau
// SFH, at least tage / 2) on the SSP log-age grid, and of logzsol on the metallicity grid. The CSP interpolates
// linearly between grid nodes, so short-tau magnitudes bend at the nodes, where the clocks bend. Returns false when
// an input is outside the training box (more than 1e-4 beyond its edge) or not finite.
__host__ __device__ inline bool emu_features(const float *x, const float *par, float *s) {
    bool inside = true;
    for (int i = 0; i < EMU_NIN; ++i) {
        s[i] = (emu_feature(i, x[i]) - par[EMU_P_INC + i]) * par[EMU_P_INS + i];
        if (!(fabsf(s[i]) <= 1.0001f)) inside = false;
    }
    const float age = fmaxf(x[1] - 2.f * x[0], 0.5f * x[1]);
    const float da = par[EMU_P_CLK + 1] > 0.f ? (9.f + log10f(age) - par[EMU_P_CLK]) / par[EMU_P_CLK + 1] : 0.f;
    const float dz = par[EMU_P_CLK + 3] > 0.f ? (x[2] - par[EMU_P_CLK + 2]) / par[EMU_P_CLK + 3] : 0.f;
    const float ca = fabsf(sinf(3.14159265358979f * da)), cz = fabsf(sinf(3.14159265358979f * dz));
    s[10] = (ca - par[EMU_P_INC + 10]) * par[EMU_P_INS + 10];
    s[11] = (cz - par[EMU_P_INC + 11]) * par[EMU_P_INS + 11];
    return inside;
}

struct EmuInferArgs {
    int n, nb;
    const float *x;              // n x EMU_NIN raw inputs (tau, not log tau)
    const float *bias;           // EMU_MEMBERS x EMU_NBIAS
    const float *par;            // EMU_PAR
    float spread_max, faint;     // flag models whose ensemble spread exceeds spread_max [mag], over the bands
                                 // less than `faint` mag fainter than the model's brightest band
    float *mags;                 // n x nb (AB, with the distance term)
    float *coef;                 // n x EMU_NPC, or null
    float *spread;               // n, or null
    int *flag;                   // n: 0 emulated, 1 outside the training box, 2 spread, 3 not finite
    int *nflag, *flagged;        // count and indices of the flagged models
    float *scratch;              // grid x EMU_SCRATCH_CTA: each CTA's members' outputs and tile inputs
    int *status;
};

// Device and host state of a context's emulator.
struct Emulator {
    bool ready = false;          // weights loaded or trained
    bool trainable = false;      // FP32 masters and Adam moments present
    int nb = 0, ns = 0;
    double box_lo[EMU_NIN] = {}, box_hi[EMU_NIN] = {};   // the training box (raw values)
    float par[EMU_PAR] = {};     // in_c, in_s, out_mu, out_sig, clocks, zt, dl
    float spread_max = 0.01f, faint = 15.f;
    std::vector<float> pca_mean, pca_basis;     // ns, EMU_NPC x ns
    std::vector<double> info;                   // training and validation figures
    // f16 weights of the forward pass, members stacked: w0 [5][512][64] (columns 16..27 repeat 0..11: the
    // features' lo parts), wh [3][5][512][512], w4 [5][128][512]; bf16 transposes for the training's input cotangents:
    // wht [3][5][512][512], w4t [5][512][128]
    __half *w0 = nullptr, *wh = nullptr, *w4 = nullptr;
    __nv_bfloat16 *wht = nullptr, *w4t = nullptr;
    float *bias = nullptr, *d_par = nullptr;
    float *d_pca_mean = nullptr, *d_pca_basis = nullptr;
    // FP32 masters and Adam moments (training): [w0 | wh | w4 | bias] each
    float *master = nullptr, *adam_m = nullptr, *adam_v = nullptr;
    long long adam_t = 0;
    CUtensorMap tm_w0, tm_wh, tm_w4;
    // predict scratch
    float *d_x = nullptr, *d_mags = nullptr, *d_coef = nullptr, *d_spread = nullptr;
    int *d_flag = nullptr, *d_nflag = nullptr, *d_flagged = nullptr;
    float *d_scratch = nullptr;                  // the inference kernel's per-CTA member outputs
    int cap = 0;
    void release();
};

long long emu_param_count();                 // FP32 parameters of the ensemble (weights and biases)

}  // namespace sps
