// Device-side data layouts and kernel entry points of the batched CSP path (host-callable launchers).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>

namespace sps {

// 0-based index i with a[i] <= v < a[i + 1] for ascending or descending a (bisection over 0..n+1 as the reference's
// find_interval, src/math/opensps_interpolation.f90:152-197, with its end cases), as the reference's 1-based
// result minus one (so -1 below an ascending table).
__host__ __device__ inline int find_interval0(const double *a, int n, double v) {
    if (n < 2) return 0;
    const bool asc = a[n - 1] >= a[0];
    int lower = 0, upper = n + 1;
    while (upper - lower > 1) {
        const int mid = (upper + lower) / 2;
        const bool ge = v >= a[mid - 1];
        if (asc == ge) lower = mid; else upper = mid;
    }
    if (v == a[0]) return 0;
    if (v == a[n - 1]) return n - 2;
    return lower - 1;
}

// Error codes a kernel writes into its status word (0 = ok). A bounded wait that gave up records which role.
enum {
    ERR_TIMEOUT_PRODUCER = 0x101,
    ERR_TIMEOUT_MMA = 0x102,
    ERR_TIMEOUT_EPILOGUE = 0x103,
    ERR_TIMEOUT_BAND = 0x104,
    ERR_TIMEOUT_ADJOINT = 0x105,
};

// Per-pixel table (floats per pixel): ln(lambda / 5500 A) log2(e), the batch's shared diffuse curve (used when
// uniform_index), the six Madau wavelength factors a_k, the curve tables T0..T3 (a model's curve is
// (T0 + s1 T1 + s2 T2 + s3 T3) exp2(ed ln(lambda / 5500) log2 e) with its scalars MP_CS1.. and MP_DUST_INDEX).
enum { PIX_LTAB2 = 0, PIX_CURVE = 1, PIX_IGM_A = 2, PIX_T = 8, PIX_FLOATS = 12 };

// The weight as an FP32 value, 0 unless it is above SAFE_FLOOR (model_sums_zw's floor): the FP64 -> FP32 rounding
// done on the integer pipes (round to nearest even on the 29 dropped mantissa bits) so that the cast keeps off the
// FP64 unit, which GB300 has little of. Weights below FP32's smallest normal also give 0.
__device__ __forceinline__ float weight_to_f32(double w) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(w);
    const uint32_t hi32 = (uint32_t)(b >> 32), lo32 = (uint32_t)b;
    if (b <= 0x0010000000000000ull || (hi32 >> 31)) return 0.f;       // <= DBL_MIN, or negative
    const int fe = (int)((hi32 >> 20) & 0x7ff) - 896;                  // FP32 biased exponent
    if (fe < 1) return 0.f;
    if (fe > 254) return __int_as_float(0x7f800000);
    uint32_t m = ((hi32 & 0xfffffu) << 3) | (lo32 >> 29);
    const uint32_t rem = lo32 & 0x1fffffffu;
    m += (rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) ? 1u : 0u;
    return __uint_as_float(((uint32_t)fe << 23) + m);                  // a mantissa carry moves into the exponent
}

// A model's diffuse curve at a pixel: the batch's shared one (uniform), its tabulated form (tab: the pixel's
// T0..T3 with the model's s1..s3 = cs and power ed), or the power law exp2(ed ltab2). ex2: the SFU's 2^x.
__device__ __forceinline__ float pix_curve(bool uniform, bool tab, float curve_u, float ltab2, float4 t, float4 cs,
                                           float ed) {
    if (uniform) return curve_u;
    float pl;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(pl) : "f"(ed * ltab2));
    if (!tab) return pl;
    return fmaf(cs.x, t.y, fmaf(cs.y, t.z, fmaf(cs.z, t.w, t.x))) * (ed != 0.f ? pl : 1.f);
}

// Per-model parameter block (floats), written by the model-parameter prologue; exponents are pre-scaled by
// log2(e) so that every transmission is one exp2. Groups of four start on 16-byte boundaries (vector loads).
enum {
    MP_KD2 = 0,          // -dust2 log2(e):            T_diffuse = exp2(MP_KD2 curve)
    MP_ONE_M_FND = 1,    // 1 - frac_nodust (0 when frac_nodust = 1)
    MP_FND = 2,          // frac_nodust (1 when frac_nodust = 1)
    MP_DUST_INDEX = 3,   // the curve's power ed (dust_index with dust_type 0 and 4, else 0)
    MP_KD1 = 4,          // -dust1 log2(e) (0: no birth-cloud screen)
    MP_DUST1_INDEX = 5,
    MP_ONE_M_FO = 6,     // 1 - frac_obrun
    MP_FO = 7,           // frac_obrun
    MP_IGM_ON = 8,       // 1: IGM for this model
    MP_IGM_JMAX = 9,     // (1-based) pixel of the maximum optical depth (int bits): pixels below are capped
    MP_IGM_KCAP = 10,    // -tmax igm_factor log2(e)
    MP_KD3 = 11,         // -dust3 log2(e) (0: no old-star screen)
    MP_IGM_KB = 12,      // 6 redshift factors b_k(1 + z) times -igm_factor log2(e) (12..17)
    MP_SMOOTH_R = 18,    // smoothing half-width in pixels (int bits), -1: none
    MP_TAPS = 20,        // 9 normalised taps, offsets -4 .. 4 (zero beyond R)
    MP_CS1 = 29,         // the curve's scalars s1, s2, s3 (29..31; the tables' weights)
    MODEL_PAR_FLOATS = 32
};

// The operand's column map (BasisOperand::kmap, WeightsArgs::kmap): per K column the source index t + nt z of the
// weights, with flag bits; -1: padding.
constexpr int KMAP_YOUNG = 0x40000000;   // a young age (t < itesc)
constexpr int KMAP_ION = 0x20000000;     // an escaping-light column: the weight times the model's clamp(frac_obrun, 0, 1)
constexpr int KMAP_SRC = 0x1fffffff;     // the source index

struct ContractArgs {
    int nspec, n_models, n_ptiles, n_mtiles, nkb_young, nkb_old, jtop, ld_spec;
    // nebular emission's escaping ionizing light: K blocks after the young and old ones (ion young blocks into the
    // young accumulator, then ion old blocks into the old one), run only by the pixel tiles that reach a pixel below
    // ion_pix (the ionizing pixels; the basis holds those columns' unabsorbed spectra there and zeros above)
    int nkb_ion_young = 0, nkb_ion_old = 0, ion_pix = 0;
    int sm_lo, sm_hi;    // pixels smoothed (lambda within [min_wave_smooth, max_wave_smooth]); sm_lo > sm_hi: none
    int uniform_index;   // every model has the pixel table's curve
    int tab_curve = 0;   // not uniform: each model's curve from the pixel table's T0..T3 (else its power law)
    const float *pix;    // nspec x PIX_FLOATS
    const float *mpar;   // n_models x MODEL_PAR_FLOATS
    float *spec;         // n_models x ld_spec (pixel fastest); null: not written (NACC = 2 with the parts)
    float *young, *old;  // NACC = 2 only, may be null: the age sums before dust (n_models x ld_spec)
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
    int n_models, nt, nz, kpad;
    const int *kmap;        // kpad: source index t + nt z of operand column k with the KMAP_ flags, -1: padding
    const float *mpar = nullptr;   // n_models x MODEL_PAR_FLOATS: frac_obrun of the KMAP_ION columns (null: none)
    const double *wz;       // n_models x (nt x nz), age fastest
    const double *mass;     // nt x nz
    const double *llin;     // nt x nz: 10^log L_bol
    __nv_bfloat16 *w_hi, *w_lo;   // n_models x kpad
    double *sums;           // n_models x 6: mass, lsum, mass_young, mass_old, lsum_young, lsum_old
    int parts;              // also the young and old sums
    int itesc;              // ages t < itesc (0-based) are young
    int grid;               // blocks of the FP64 sums kernel (0: one warp per model)
};
// the bf16 hi / lo operand with the FP64 sums in one pass over the weights; the FP64 sums alone (the FP64 path)
cudaError_t run_weights_convert_sums(const WeightsArgs &a, cudaStream_t st);
cudaError_t run_weights_prep(const WeightsArgs &a, cudaStream_t st);

// Band fluxes (observed frame at each model's redshift, trapezoid filter integrals) and AB magnitudes, as a
// tensor-core GEMM over the pixels any band reaches (band_gemm.cu).
struct BandGemmArgs {
    int n_models, nspec, nbands, npad, nkb, j0, ld_spec;
    const float *spec;      // n_models x ld_spec rest-frame spectra
    const float4 *zinfo;    // n_models: (n0 as int bits, t of the interior interpolation, shift s in pixels, 0 at z = 0)
    double dlnl;            // grid step in ln lambda
    const double *dist;     // n_models: distance term
    double zp;              // 48.60 + 2.5 ABS_MAG_ZEROPOINT_LOG
    const int *do_band;     // nbands
    double *fband;          // n_models x nbands (may be null)
    double *mags;           // n_models x nbands (may be null)
    int *status;
    // with few models, the pixels split over CTAs: partial band fluxes (ksplit x n_models x npad floats, at most
    // fpart_cap) summed by a second kernel that forms the magnitudes (fpart null: no split)
    float *fpart = nullptr;
    size_t fpart_cap = 0;
    int num_sms = 148;
    int ksplit = 1;         // set by run_band_gemm
};
int band_gemm_npad(int nbands);
// The pixel splits run_band_gemm takes for n_models (1: none).
int band_gemm_ksplit(int n_models, int nkb, int num_sms);
cudaError_t run_band_gemm(const BandGemmArgs &a, const CUtensorMap &tm_hi, const CUtensorMap &tm_lo,
                          cudaStream_t st);
// Loads the band GEMM's module on the current device (no launch).
cudaError_t band_gemm_load();
// Loads the no-allocation entry point's modules on `device` (current) and records its scratch's device address.
cudaError_t noalloc_prepare(int device);

// Emission-line luminosities: eml(l, m) = sum_k w(k, m) L(l, k) over the (age, metallicity) entries with lines.
struct EmlineArgs {
    int n_models, nline, ntz, nnz;
    const double *wz;       // n_models x ntz
    const int *kidx;        // nnz source indices k with line luminosity
    const float *lum;       // nnz x nline: L(l, kidx[i])
    float *eml;             // n_models x nline
};
cudaError_t run_emlines(const EmlineArgs &a, cudaStream_t st);

// Split-BF16 GEMM D(M x N) = A(M x K) B(N x K)^T, f32 out (gemm_bf16x3.cu). B's rows start at b_row0.
struct GemmArgs {
    int M, N, K, ldd, b_row0;
    float *D;
    int *status;
    int groups = 1, ksplit = 1;                  // see gemm_bf16x3.cu: groups of rows, partial sums over K splits
    long long a_grp = 0, b_grp = 0;              // rows between the groups' A / B operands
    long long d_grp = 0, d_split = 0;            // elements between the groups' / splits' D
    int f16 = 0;                                 // one-product kind: operands f16 (else bf16)
};
struct GemmPlan {
    CUtensorMap tm_a_hi, tm_a_lo, tm_b_hi, tm_b_lo;
    int num_sms;
};
int gemm_bk();
int gemm_bm();
int gemm_bn();
cudaError_t run_gemm_bf16x3(const GemmPlan &pl, const GemmArgs &g, cudaStream_t st);   // three products (hi / lo)
cudaError_t run_gemm_bf16(const GemmPlan &pl, const GemmArgs &g, cudaStream_t st);     // one product (hi only)

// The reverse pass per model (adjoint.cu): from the forward's young / old sums, band fluxes and the cotangents, the
// cotangents of the young and old sums (bf16 hi / lo operands of the weight GEMM) and the parameter gradients.
struct AdjointPrepArgs {
    int n_models, nspec, sm_lo;
    double dlnl, em1;                // grid step in ln lambda, e^dlnl - 1
    const double *par;               // n_models x PAR_DEVICE
    const float *mpar;               // n_models x MODEL_PAR_FLOATS
    const float4 *zinfo;
    const double *lnlam;             // nspec
    const double *zt, *dl;           // cosmology table (500)
    float *apar;                     // n_models x 32: the per-model block of the reverse pass
};
struct DustEmModel {
    int on, iq, iu;
    float wq, wu, gam;
    int agn, ita;
    float wta, fagn;
    // the nebular continuum's CLOUDY cell: the lower corner (0-based, clamped so that the cell lies in the grid) and
    // the weights (clamped to [0, 1]) in gas_logz and gas_logu, and |1 - frac_obrun|
    int neb_iz, neb_iu;
    float neb_wz, neb_wu, neb_fabs;
    // for the reverse pass: d w_z / d gas_logz and d w_u / d gas_logu (zero where the weight is clamped), and
    // d |1 - frac_obrun| / d frac_obrun
    float neb_dz, neb_du, neb_dfo;
};
struct AdjointArgs {
    int n_models, nspec, ppad, nbands, jtop, j0, j1, sm_lo, sm_hi, uniform_index;
    int dust_type = 0;               // the diffuse curve (0: the power law; else from the pixel table's T0..T3)
    float dl2, inv_em1;              // dlnl log2(e), 1 / (e^dlnl - 1)
    const float *young, *old;        // n_models x nspec (+ 4 floats of padding): the forward's age sums before dust
    const float *mpar;               // n_models x MODEL_PAR_FLOATS
    const float *apar;               // n_models x 32 (AdjointPrepArgs::apar)
    const double *par;               // n_models x PAR_DEVICE (dust1 .. dust_tesc)
    const float4 *zinfo;             // n_models: the observed-frame shift
    const double *fband;             // n_models x nbands
    const double *mags_bar;          // n_models x nbands, or null
    const double *spec_bar;          // n_models x nspec, or null
    const int *do_band;              // nbands, or null: every band
    const float *pix;                // nspec x PIX_FLOATS
    const float *wl;                 // nspec: 1 / lambda
    const float *bc;                 // the band matrix C(j, b) by band: band b's pixels lo .. hi at bc + off
    const int4 *bmeta;               // nbands: (lo, hi, off, 0)
    const int2 *bchunk;              // per 32 pixels from j0: the first and last band reaching them
    float lt_base, lt_step;          // ln(lambda_p / 5500) log2(e) = lt_base + p lt_step (the log-uniform grid)
    __nv_bfloat16 *ybar_hi, *ybar_lo, *obar_hi, *obar_lo;   // n_models x ppad (zero beyond nspec)
    double *cscale;                  // n_models: the cotangent scale (the A operands are divided by it)
    double *params_bar;              // n_models x 44
    int *status;
    // dust emission and the AGN torus (dem null: neither): per model the cells (DustEmModel), the Draine & Li
    // templates and the frequency trapezoid weights (as PartsEpilogueArgs), the AGN templates, each model's linear
    // L_bol (lsum at lsum_stride m: the AGN's scale), the chain factors (d wq / d q_PAH, d wu / d U_min, d gam / d gamma,
    // d wta / d agn_tau) and the AGN's cotangent of the linear L_bol (lsum_bar, n_models, unscaled; null: not wanted)
    const DustEmModel *dem = nullptr;
    const float *dtab = nullptr, *cnu = nullptr;
    int nqpah = 0;
    const float *agn_spec = nullptr;
    const double *lsum = nullptr;
    int lsum_stride = 6;
    const float4 *dchain = nullptr;
    double *lsum_bar = nullptr;
};
cudaError_t run_adjoint(const AdjointPrepArgs &pa, const AdjointArgs &a, cudaStream_t st);

// SFH weights (sfh.cu). Per-model FP64 columns: tage, tau, const, fburst, tburst, sf_start, sf_trunc (Gyr),
// sf_slope (per Gyr), logzsol.
enum { SFH_TAGE = 0, SFH_TAU, SFH_CONST, SFH_FBURST, SFH_TBURST, SFH_SF_START, SFH_SF_TRUNC, SFH_SF_SLOPE,
       SFH_NPAR = 8, SFH_LOGZSOL = 8, SFH_NCOL = 9 };
// their params_bar rows (opensps.h)
enum { PB_LOGZSOL = 15, PB_TAGE = 16, PB_TAU = 17, PB_CONST = 18, PB_FBURST = 19, PB_TBURST = 20, PB_SF_START = 21,
       PB_SF_TRUNC = 24, PB_SF_SLOPE = 25, PB_IMF1 = 26 };
struct SfhArgs {
    int n, nt, nz, sfh, itesc;
    const double *tf;        // nt: log10(age / yr) of the grid
    const double *lz;        // nz: log10(Z / Zsun)
    const double *lbol;      // nz x nt: log10 L_bol of the SSPs (age fastest)
    const double *par;       // n x SFH_NCOL
    const double *given;     // n x nt weights over ages given by the caller, or null: the SFH's
    double *w;               // n x nt: the weights over ages
    double *scratch;         // n x 2 nt
    double *wz;              // n x nt x nz: the weights over ages and metallicities
    double *lblend;          // n x 3: log-blended L_bol (total, young, old)
    double *sfr;             // n, or null
    double2 *mtab = nullptr; // n x nt: the main component's moments at the grid ages (sfh 1, 4, and 5's delayed
                             // tau; null: formed serially per model)
    int ntab = 0;            // the tabular SFH (sfh 2, 3): ntab rows, tab = ages (years since the start,
    const double *tab = nullptr;   // non-decreasing) then SFRs, each with one zero entry past the table
};
cudaError_t run_sfh_forward(const SfhArgs &a, cudaStream_t st);
struct SfhRevArgs {
    int n, nt, nz, sfh, rows, has_logzsol, sfh_tangents;
    const double *tf, *lz, *lbol, *par, *w, *lblend, *lbol_bar;
    const double *lsum_bar = nullptr;   // n: the AGN's cotangent of the log-blended L_bol (linear, absolute), or null
    const double *wzb;       // n x nt x nz: dL / dwz without the L_bol term
    double *weights_bar;     // n x nt, or null
    double *scratch;         // n x nt
    double *params_bar;      // n x rows
    void *dual;              // n x 3 nt dual numbers (sfh_dual_bytes() each)
};
cudaError_t run_sfh_reverse(const SfhRevArgs &a, cudaStream_t st);
size_t sfh_dual_bytes();

// The SSP operator applied to per-model IMFs (ssp_op.cu). A point of the isochrones of one grid point: the IMF bin
// [lo, hi] (ln lo and ln(hi / lo) for the bins inside one power-law segment of the IMF), the Kroupa segment (1 .. 3,
// 0: the bin crosses a segment boundary, -1: no stars within the mass limits 0.08 - 120 M_sun the operator is built
// with), the star's current mass and L_bol, and its initial mass (negative for the first point of its age, whose bin
// starts at the IMF's lower edge).
struct OpsPoint {
    float ln_lo, dl, mcur, lum, lo, hi;
    int seg;
    float mini;
};
// The IMF's mass limits and the user IMF as the exact fold and its reverse take them. custom: limits or a lower edge
// other than the build's (0.08, 120, 0.08 M_sun), or the user IMF: every bin then takes the generic path, gated by
// its point's initial mass (compute_imf_weights, src/physics/opensps_imf.f90:111-172).
struct OpsImfLim {
    double lim_lo = 0.08, lim_hi = 120.0;    // the normalisation's mass range and the points' gate
    float lb = 0.08f;                        // the lower edge of each age's first bin
    int custom = 0;
    const float *user = nullptr;             // nuser x 5: lo, hi, e = 1 - alpha, c / e (0 for e = 0), c
    int nuser = 0;
    double user_inv_total = 1.0;             // 1 / (the user IMF's mass between the limits), FP64 on the host
};
struct OpsFoldArgs {
    int n, nt, nz, npt, nent, ntpad, itesc;
    int imf_type = 2;         // 0 Salpeter, 1 Chabrier, 2 Kroupa, 3 van Dokkum, 4 Dave, 5 the user's segments
    OpsImfLim lim;
    const double *wz;         // n x nt x nz SFH weights (age fastest)
    const double *alpha;      // n x 3: the IMF's parameters (Kroupa: imf1-3; van Dokkum: vdmc; Dave: imf1, imf2,
                              // mdave)
    const OpsPoint *pts;      // (nt x nz) x npt
    const uint32_t *ent;      // (nt x nz) x nent: template << 16 | point, sorted by template within a grid point
    const float *ent_c;       // the entries' coefficients
    __nv_bfloat16 *v_hi, *v_lo;   // 2n x ntpad template weights: rows 0 .. n-1 young, n .. 2n-1 old
    double *sums;             // n x 6: mass, L_bol, young mass, old mass, young L_bol, old L_bol
    float *vpart;             // nz x 2n x ntpad: each metallicity slab's template weights
    double *spart;            // nz x n x 4: each slab's mass and L_bol rows (young, old)
    int *flag;                // nz x ceil(n / 4): the slab has weight for some model of the group
};
cudaError_t run_ops_fold(const OpsFoldArgs &a, cudaStream_t st);
// The interpolated fold's operand (one row per model of a chunk) and its GEMM's reduction.
struct OpsInterpArgs {
    int m0, nt, nz, R, ktot, itesc;          // models m0 .. m0 + gridDim.x - 1; ktot = nt nz R columns
    int imf_type = 2;                        // 2 Kroupa (slopes per model; 0 Salpeter as Kroupa), 1 Chabrier
    unsigned rg_magic;                       // 2^32 / (R / 8), rounded up
    int noff[3], nn[3];                      // the segments' node columns: noff[s] .. noff[s] + nn[s] - 1
    double x0[3], h[3];                      // node j of segment s at ln m = x0[s] + (j - 4) h[s]
    float lim_lo, lim_hi;
    const double *wz, *alpha;                // n x nt x nz SFH weights; n x 3 slopes
    const double2 *kconst;                   // n: 1 / T and c2 of each model
    const float *mrow, *lrow;                // ktot: the operator basis's mass and L_bol rows
    __nv_bfloat16 *x_hi, *x_lo;              // chunk rows x ktot
    double *sums;                            // n x 6
};
struct OpsInterpReduceArgs {
    int n, m0, rows, ntpad, ntempl, ks_young, ks_old;
    const float *part_young, *part_old;      // ks x rows x ntpad split-K partial sums
    __nv_bfloat16 *v_hi, *v_lo;              // 2n x ntpad
};
// The operator's reverse pass: from the template cotangents, the cotangents of the SFH weights over ages and
// metallicities and of the three Kroupa slopes.
struct OpsRevArgs {
    int n, nt, nz, npt, ntpad, itesc;
    int imf_type = 2;         // the IMF's rows: Kroupa (2) imf1-3, Dave (4) imf1, imf2, mdave; zero otherwise
    OpsImfLim lim;
    const double *wz;         // n x nt x nz SFH weights (age fastest)
    const double *alpha;      // n x 3: the IMF's parameters (as OpsFoldArgs)
    const OpsPoint *pts;      // (nt x nz) x npt
    const ushort4 *pidx;      // (nt x nz) x npt: each point's four templates
    const float4 *pcoef;      // and their coefficients
    const float *vbar;        // 2n x ntpad: the template weights' cotangents / cscale (young rows, then old)
    const double *cscale;     // n: the reverse pass's cotangent scale
    const double *mass_bar, *lbol_bar;   // n each, or null
    const double *lsum_bar = nullptr;    // n: the AGN's cotangent of the linear L_bol row (absolute), or null
    const double *sums;       // n x 6: the forward's mass and linear L_bol
    double *wzb;              // n x nt x nz: the weights' cotangent (every grid point), or null (slopes only)
    double *apart;            // nz x n x 3: each slab's slope cotangents / cscale
    double *params_bar;       // n x rows: the IMF's rows from row_imf1 (imf1-3, vdmc, mdave; written), or null
    int rows, row_imf1;
};
cudaError_t run_ops_reverse(const OpsRevArgs &a, cudaStream_t st);
// dst(k, p) = src(p, k) (adjoint.cu): kpad x ppad from the first kpad columns of ns rows of ld, zero for p >= ns
cudaError_t run_transpose_bf16(const __nv_bfloat16 *src, __nv_bfloat16 *dst, int ns, size_t kpad, size_t ld, int ppad,
                               cudaStream_t st);
// The spectrum from the young and old sums (the contraction epilogue's attenuation, IGM and smoothing).
// A model's emission terms of the per-model epilogue: dust emission (on, the Draine & Li grid cell iq, iu: 0-based
// lower corner, with its weights and gamma: dl07_indices, src/physics/opensps_csp_batch.f90:1622-1634) and the AGN
// torus (agn, the template interval ita with its weight and fagn: agn_indices :1575-1589).

struct PartsEpilogueArgs {
    int n, nspec, jtop, sm_lo, sm_hi, uniform_index;
    int tab_curve = 0;            // not uniform: each model's curve from the pixel table's T0..T3 (else its power law)
    const float *pix, *mpar;
    const float *young, *old;     // n x nspec
    float *spec;                  // n x nspec
    // dust emission (dem null: none): per model its cell; the templates (nspec x nqpah x 2 numin) and the frequency
    // trapezoid weights per pixel
    const DustEmModel *dem = nullptr;
    const float *dtab = nullptr, *cnu = nullptr;
    int nqpah = 0;
    // the AGN torus: the templates (ntau x nspec) and each model's L_bol as the batch outputs it (linear), at
    // lsum[lsum_stride m]: the FP64 sums' L_bol, or with weights blended at logzsol on the device the log-blended one
    const float *agn_spec = nullptr;
    const double *lsum = nullptr;
    int lsum_stride = 6;
};
cudaError_t run_parts_epilogue(const PartsEpilogueArgs &a, cudaStream_t st);

// The CLOUDY-grid nebular continuum added to the young and old sums (ssp_op.cu): n models, their cells in dem, the
// table (log2 less the pixel's integer offset, [logZ][logU][age][pixel]) and offsets, q0 (nt_neb x nz), the FP64
// weights (n x nz x nt); the nebular ages as runs of one CLOUDY interval, one side of itesc and a uniform step in the
// interval's weight wa: runs[r] = (first age, age count | young << 16, wa of the run's last age, the step), as int
// bits; rfirst[k] = interval k's first run (k = 0 .. NEB_NAGE - 2), rfirst[NEB_NAGE - 1] = nrun; groups: (cell z,
// cell u, first index into order, count <= NEB_GROUP), order: the models sorted by cell; cw: scratch, n x cw_ld floats
// (cw_ld >= nt_neb + 2).
constexpr int NEB_MAX_AGES = 128;         // nebular ages the continuum takes
constexpr int NEB_GROUP = 64;             // models per group of one cell
constexpr int NEB_MAX_RUNS = NEB_MAX_AGES + 16;
constexpr int NEB_RUN_HEAD = 12;          // ints before the runs: the intervals' first runs, the run count
struct NebContArgs {
    int n, nspec, nt, nz, nt_neb, cw_ld, nrun;
    const DustEmModel *dem;
    const float *tab, *off;
    const int4 *runs;
    const int *rfirst;
    const float *q0;          // nt_neb x nz, times 2^q0_exp
    int q0_exp;
    const double *wz;
    const int4 *groups;
    const int *order;
    float *cw;
    float *young, *old;       // n x nspec
};
cudaError_t run_nebular_continuum(const NebContArgs &a, int ngroups, cudaStream_t st);
// The continuum's reverse pass (ssp_op.cu): the young and old sums' cotangents (bf16 hi / lo, scaled by 1 / cscale)
// against the forward's terms, into the weights' cotangent and the gas_logz, gas_logu and frac_obrun rows.
struct NebContRevArgs {
    int n, nspec, nt, nz, nt_neb, cw_ld, itesc, ppad, ntz;
    int kfirst[10];           // the nebular ages in CLOUDY interval k: kfirst[k] .. kfirst[k + 1] - 1 (k < 9)
    const DustEmModel *dem;
    const float *tab, *off;   // the forward's table (log2, relative to the pixel offsets off)
    const float *wa;          // nt_neb: each nebular age's weight in its CLOUDY interval
    const float *cw;          // n x cw_ld: the forward's C(t) / S, then log2 S (integer part, rest)
    const float *q0;          // nt_neb x nz, times 2^q0_exp
    int q0_exp;
    const __nv_bfloat16 *ybh, *ybl, *obh, *obl;   // n x ppad
    const double *cscale;
    double *wzbar;            // n x ntz (age t + nt z), or null
    double *params_bar;       // n x rows
    int rows, row_gas_logz, row_gas_logu, row_frac_obrun;
};
cudaError_t run_nebular_continuum_reverse(const NebContRevArgs &a, cudaStream_t st);

// Casts the FP32 spectra to FP64 (the C API's double outputs), n_models x nspec from ld-strided rows.
cudaError_t run_spec_to_f64(const float *src, int ld, int nspec, int n_models, double *dst, cudaStream_t st);

}  // namespace sps
