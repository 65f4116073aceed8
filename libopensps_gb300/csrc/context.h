// Host-side state of a context: the libraries read at setup, their device copies, the per-model parameter table
// and the scratch of the batch calls.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <vector>
#include "csp_kernels.h"
#include "emulator.h"

namespace sps {

constexpr double SAFE_FLOOR = 2.2250738585072014e-308;   // tiny(1.0_wp)
constexpr double C_LIGHT = 2.99792458e18;                 // A / s

// The float parameters of a model that this path reads, in the order of the per-model table handed to the device
// (the first PAR_DEVICE of them), with the defaults of OpenSPS's PARAMS_CORE (src/core/opensps_types.f90:32-45).
enum ParamId {
    PF_DUST1 = 0, PF_DUST2, PF_DUST3, PF_DUST_INDEX, PF_DUST1_INDEX, PF_FRAC_NODUST, PF_FRAC_OBRUN, PF_ZRED,
    PF_IGM_FACTOR, PF_SIGMA_SMOOTH, PF_DUST_TESC, PF_MWR, PF_UVB,
    PAR_DEVICE,                  // = 13: the per-model table of the device kernels stops here
    PF_LOGZSOL = PAR_DEVICE, PF_TAGE, PF_TAU, PF_MIN_WAVE_SMOOTH, PF_MAX_WAVE_SMOOTH, PF_CONST, PF_FBURST,
    PF_TBURST, PF_SF_START, PF_SF_TRUNC, PF_IMF1, PF_IMF2, PF_IMF3, PF_DUSTE_QPAH, PF_DUSTE_UMIN, PF_DUSTE_GAMMA,
    PF_FAGN, PF_AGN_TAU, PF_GAS_LOGZ, PF_GAS_LOGU, PF_SF_SLOPE, PF_VDMC, PF_MDAVE,
    PF_COUNT
};

struct ParamInfo {
    const char *name;
    int id;           // ParamId, or -1: a parameter of the reference that this path does not vary per model
    double def;
};
const ParamInfo *find_param(const char *name);
extern const char *const REFERENCE_FLOAT_PARAMS[];

template <class T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    cudaError_t reserve(size_t count) {
        if (count <= n && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr; n = 0;
        cudaError_t e = cudaMalloc(&p, sizeof(T) * (count > 0 ? count : 1));
        if (e == cudaSuccess) n = count;
        return e;
    }
    void release() { if (p) cudaFree(p); p = nullptr; n = 0; }
};

// The contraction's basis operand for one K order (bf16 hi and lo, pixels x kpad).
struct BasisOperand {
    // K columns: [young block (ky_pad) | old block | escaping-light young block (kion_y) | escaping-light old block
    // (kion_o)]; kmain = the young and old blocks, kpad = all (the blocks padded to the contraction's K step)
    int nacc = 0, itesc = 0, kpad = 0, ky_pad = 0, nty = 0, kmain = 0, kion_y = 0, kion_o = 0;
    bool ion = false;
    DevBuf<__nv_bfloat16> hi, lo;
    DevBuf<int> kmap;            // operand column -> source (age, metallicity) of the weights with the KMAP_ flags
    CUtensorMap tm_hi, tm_lo;
    bool neb = false;
    double line_sigma = 0.0;
    // the plain FP64 path's copy (nspec x kpad, column-major, the same K order), made on first use
    DevBuf<double> b64;
    // the reverse pass's copy, transposed (kpad x ppad, pixels padded to ppad with zeros), made on first use
    int ppad = 0;
    DevBuf<__nv_bfloat16> thi, tlo;
    DevBuf<int> col_of;          // source index t + nt z -> operand column
    CUtensorMap tm_thi, tm_tlo;
    void release() {
        hi.release(); lo.release(); kmap.release(); thi.release(); tlo.release(); col_of.release(); b64.release();
    }
};

// The SSP operator on the device (opensps_context_build_ssp_ops): points, sorted entries, the library as the
// template GEMM's B operand (pixels x ntpad, bf16 hi / lo).
struct SspOps {
    bool ready = false;
    int ntempl = 0, ntpad = 0, npt = 0, nent = 0;
    double lower_bound = 0.08;
    DevBuf<OpsPoint> pts;
    DevBuf<uint32_t> ent;
    DevBuf<float> ent_c;
    DevBuf<__nv_bfloat16> lib_hi, lib_lo;
    CUtensorMap tm_lib_hi, tm_lib_lo;
    // the reverse pass: each point's four templates and coefficients (point-major), and the library transposed
    // (ntpad x ppad, bf16 hi / lo: the B operand of the template cotangents' GEMM, built on first use)
    DevBuf<ushort4> pidx;
    DevBuf<float4> pcoef;
    DevBuf<__nv_bfloat16> lib_thi, lib_tlo;
    CUtensorMap tm_lib_thi, tm_lib_tlo;
    int ppad = 0;
    // the interpolated fold: each bin weight as Lagrange weights (degree 9 in ln m) on fixed mass nodes of its
    // Kroupa segment, so that a model's IMF enters only through the node values mu^-alpha; the fold is then a
    // tcgen05 GEMM of the models' node values x SFH weights against this operator basis (ntempl x nt nz R, columns
    // (t nz + z) R + r), with the mass and L_bol rows beside it
    bool interp_ready = false;
    int interp_R = 0, interp_noff[3] = {}, interp_nn[3] = {};
    double interp_x0[3] = {}, interp_h[3] = {};
    DevBuf<__nv_bfloat16> ib_hi, ib_lo;
    DevBuf<float> i_mrow, i_lrow;
    // the reverse of the interpolated fold: the basis transposed (nt nz R x ntpad, bf16 hi / lo, built on first use)
    DevBuf<__nv_bfloat16> ibt_hi, ibt_lo;
    CUtensorMap tm_ibt_hi, tm_ibt_lo;
    void release() {
        pts.release(); ent.release(); ent_c.release(); lib_hi.release(); lib_lo.release();
        pidx.release(); pcoef.release(); lib_thi.release(); lib_tlo.release();
        ib_hi.release(); ib_lo.release(); i_mrow.release(); i_lrow.release(); ibt_hi.release(); ibt_lo.release();
        ppad = 0;
        interp_ready = false;
        ready = false;
    }
};

// The dust emission's template grid (dust_emission_reductions / add_dust_emission / dl07_shape of OpenSPS): on
// the device nspec x nqpah x 2 numin FP32 templates (pixel fastest; column 2 u + c, c = 0 the U_min
// delta-function, 1 the power law) and per pixel the trapezoid weight in frequency of the energy sums, c(p) =
// wt(p) + wt(p - 1), wt(i) = |nu(i + 1) - nu(i)| / 2 (wt beyond the last pixel 0).
struct DustEmission {
    bool ready = false;
    int nqpah = 0, numin = 0;
    std::vector<double> qpah, umin;
    DevBuf<float> tab, cnu;
    void release() { tab.release(); cnu.release(); ready = false; }
};

// The AGN torus templates over the torus optical depth (add_agn_batch's agndust_spec(i, ita) over agndust_tau): on
// the device ntau x nspec FP32 (a template per row).
struct AgnTorus {
    bool ready = false;
    std::vector<double> tau;
    DevBuf<float> spec;
    void release() { spec.release(); ready = false; }
};

// The CLOUDY-grid nebular continuum (nebular/<isoc>_<nodust|dust>, nebular_kernels step 3 of OpenSPS,
// src/physics/opensps_csp_batch.f90:2760-2910): the continuum per ionizing photon over 11 gas metallicities x 10 ages
// x 7 ionization parameters at each pixel, with per nebular age of the SSP grid its CLOUDY age interval and the
// ionizing photon rate of each (age, metallicity) SSP. On the device, per table (0: nodust, 1: dust) the log2 of
// the continuum less a per-pixel offset (off: the largest log2 value of the pixel over the grid, rounded up to an
// integer) as FP32, [logZ][logU][age][pixel]; q0 (nt_neb x nz, metallicity fastest; FP32 times 2^q0_exp); per nebular age its
// interval and weight as batch_nebular_indices forms them (:1651-1686).
struct NebularGrid {
    bool have[2] = {false, false};
    std::vector<double> logz, lage, logu;
    DevBuf<float> tab[2], off;
    DevBuf<float> q0;            // the ionizing photon rates scaled by 2^-q0_exp (FP32; their largest in [0.5, 1))
    int q0_exp = 0;
    // per nebular age its CLOUDY interval (lower node, 0-based) and weight wa in it (clamped to [0, 1]); the ages as
    // runs for the last itesc (NEB_RUN_HEAD ints: each interval's first run and the run count, then the runs as int4)
    std::vector<int> ia;
    std::vector<double> wa;
    std::vector<int> h_runs;
    int runs_itesc = -1, nrun = 0;
    DevBuf<int> runs;
    // a batch's continuum: the models sorted by cell and their groups (host staging and device copies), the per-model
    // weights (scratch)
    std::vector<int> h_order;
    std::vector<int4> h_groups;
    DevBuf<int> order;
    DevBuf<int4> groups;
    DevBuf<float> cw;
    std::vector<float> h_wa;     // wa in FP32 (the reverse pass's copy, d_wa)
    DevBuf<float> d_wa;
    void release() {
        tab[0].release(); tab[1].release(); off.release(); q0.release(); runs.release();
        ia.clear(); wa.clear(); h_runs.clear(); runs_itesc = -1; nrun = 0;
        order.release(); groups.release(); cw.release(); d_wa.release(); h_wa.clear();
        have[0] = have[1] = false;
    }
};

// What the reverse pass needs of the forward batch it follows.
struct BatchGeom {
    BasisOperand *bop = nullptr;
    int nacc = 0, sm_lo = 0, sm_hi = -1, uniform_index = 0, n = 0;
    int tab_curve = 0;           // the models' diffuse curves from the pixel table's T0..T3 (dust_type other than 0)
    int itesc = 0;               // the first old age
    const double *wz = nullptr;  // the weights over ages and metallicities on the device (with the operators)
    bool emis = false, agn = false;   // the batch had dust emission / the AGN torus (cells in d_dem, chains in d_dchain)
    bool neb = false;                 // the batch had the nebular continuum (cells in d_dem, C(t) / S in neb.cw)
    int neb_table = 0;                // its table (nebular/<isoc>_nodust or _dust)
};

struct Context {
    std::mutex mu;
    bool is_setup = false;
    // settings (set_int / set_float)
    int add_neb_emission = 0, add_igm_absorption = 0, smooth_velocity = 1, dust_type = 0, compute_vega_mags = 0;
    int sfh = 0, nebemlineinspec = 1, fast_mode = 0, zmet = 1, imf_type = 2;
    // the tabular SFH (sfh 2, 3): ages in years since the start (non-decreasing) and SFRs [M_sun / yr], ntab entries
    // and one zero entry past them; the file it came from (sfh 2; empty: the caller's arrays, sfh 3)
    std::vector<double> sfh_tab_t, sfh_tab_sfr;
    int ntab = 0;
    std::string sfh_filename = "sfh.dat", sfh_tab_file;
    bool sfh_tab_dirty = true;       // the device copy is stale
    // the IMF's mass limits (imf_lower_limit, imf_upper_limit) and the user IMF (imf_type 5): its file under the data
    // root (imf.dat when no name is set) and its segments as read (lower mass, upper mass, slope)
    double imf_lim_lo = 0.08, imf_lim_hi = 120.0;
    std::string imf_filename, user_imf_file;
    std::vector<double> user_imf;
    DevBuf<float> d_user_imf;        // nuser x 5: lo, hi, 1 - alpha, c / (1 - alpha), c
    bool user_imf_dirty = true;      // the device table is stale
    int fp64 = 0;                // the plain FP64 path (an extension setting, "gb300_fp64")
    int ops_exact = 0;           // the SSP operator's exact fold only ("gb300_ops_exact"), never the interpolated one
    int add_dust_emission = 0;   // the energy-balance dust emission (Draine & Li templates)
    int add_agn_dust = 0;        // the AGN torus emission
    int add_neb_continuum = 1;   // the CLOUDY-grid nebular continuum (with add_neb_emission, when the grid exists)
    int cloudy_dust = 0;         // the continuum table with dust in the ionized gas (nebular/<isoc>_dust)
    bool ops_last_interp = false;   // the last operator batch took the interpolated fold
    int ops_launches = 0;        // kernels the last run_ops_parts launched
    int pageable_access = -1;    // the device reads pageable host memory (-1: not asked yet)
    bool last_direct = false;    // the last batch read the caller's pageable weights in place
    void *cublas = nullptr;      // cublasHandle_t of the FP64 path
    double h0 = 72.0, om0 = 0.27, ol0 = 0.73;
    double pdef[PF_COUNT];
    std::string filter_set = "gauss40";
    std::string dust_emission_lib = "DL07";   // dust_emission/<name> of a standard-format data root
    // nebular emission's gas absorption: ages 0..nt_neb-1 carry nebular emission, pixels 0..whlylim-1 are ionizing
    // (below 912 A); d_ion holds those ages' ionizing pixels of the library, (z nt_neb + t) x whlylim FP32
    int nt_neb = 0, whlylim = 0;
    DevBuf<float> d_ion;
    bool last_ion = false;           // the last batch added the escaping ionizing light (its reverse pass follows)
    std::vector<int> mag_mask;   // empty: all bands

    // libraries (host, FP64)
    int nspec = 0, nt = 0, nz = 0, nline = 0, nbands = 0;
    double zsol = 0.0142, dlnl = 0.0;
    std::vector<double> lam, log_age, zlegend, ssp, mass, lbol, line_lambda, line_lum, bands, band_center;
    std::vector<double> llin;    // 10^lbol
    std::vector<double> zt, dl;  // cosmology table (500)
    std::vector<float> igm_a;    // jtop x 6 Madau wavelength factors
    int jtop = 0;

    // device copies
    int device = 0, num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;                 // the per-model parameters run here
    cudaStream_t side2 = nullptr;                // the FP64 sums run here (after the contraction)
    cudaStream_t side3 = nullptr;                // a reverse pass's cotangents go up here, beside its forward
    cudaStream_t side4 = nullptr;                // the weight operand, beside the per-model parameters
    cudaEvent_t ev_cot = nullptr, ev_w0 = nullptr, ev_w1 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_params = nullptr, ev_contract = nullptr, ev_sums = nullptr;
    DevBuf<float> d_pix, d_wl, d_igm_a;
    DevBuf<int> d_do_band;
    // band matrix of the band GEMM: bf16 hi / lo, band_npad rows x 64 band_nkb pixels from pixel band_j0
    DevBuf<__nv_bfloat16> d_cb_hi, d_cb_lo;
    CUtensorMap tm_cb_hi, tm_cb_lo;
    int band_j0 = 0, band_nkb = 0, band_npad = 0;
    DevBuf<double> d_lam, d_lnlam, d_mass, d_llin, d_zt, d_dl;
    std::map<long long, BasisOperand *> basis_cache;   // key: nacc, itesc, line-width key
    double pix_key[6] = {-1e300, 0.0, 0.0, 0.0, 0.0, 0.0};   // the device pixel table's curve: dust_type, its 4
                                                               // scalars, the dusty environments' curve (type 3)
    // dust types 3 and 5 (attenuation/dirty and attenuation/smc_bar of the data root, on the grid): wgp1 (tau_v),
    // wgp2 (model), wgp3 (structure) choose the dirty curve
    int wgp[3] = {1, 1, 1};
    std::vector<double> att_smc, att_wg;

    // batch scratch
    DevBuf<double> d_wz, d_params, d_sums, d_dist, d_fband, d_mags, d_spec64;
    DevBuf<float4> d_zinfo;
    DevBuf<__nv_bfloat16> d_whi, d_wlo;
    DevBuf<float> d_mpar, d_spec, d_young, d_old, d_eml, d_eml_lum;
    DevBuf<int> d_eml_kidx;
    int eml_nnz = -1;            // entries of the line table (-1: not built)
    BatchGeom geom;              // of the last batch
    // reverse pass: the band matrix by band (band b's nonzero pixels lo .. hi as a dense row at off), the bands
    // reaching each 32-pixel chunk from band_j0 (first, last), cotangents and results
    int band_j1 = -1;
    DevBuf<float> d_bc;
    DevBuf<int4> d_bmeta;        // (lo, hi, off, 0) per band
    DevBuf<int2> d_bchunk;       // (first, last) band per chunk; first > last: none
    DevBuf<double> d_mags_bar, d_spec_bar, d_mass_bar, d_lbol_bar, d_cscale, d_pbar, d_wzbar;
    DevBuf<__nv_bfloat16> d_ybh, d_ybl, d_obh, d_obl;
    DevBuf<float> d_wzb32, d_apar;
    // SFH weights: grid tables, per-model parameters, weights over ages, log-blended L_bol, SFR; reverse-pass scratch
    DevBuf<double> d_logage, d_lz, d_lbol;
    DevBuf<double> d_sfhpar, d_wgiven, d_w, d_sfh_scratch, d_lblend, d_sfr, d_wbar;
    DevBuf<double> d_sfhtab;         // the tabular SFH: 2 (ntab + 1) doubles, ages then SFRs
    DevBuf<double2> d_sfh_mtab;  // the SFH's moments at the grid ages (n x nt)
    DevBuf<unsigned char> d_dual;
    // the dust emission templates (Draine & Li shapes) and the frequency trapezoid weights of the grid; the AGN torus
    // templates
    DustEmission dustem;
    AgnTorus agn;
    // the reverse pass with dust emission / AGN: per model the chain factors (d wq / d q_PAH, d wu / d U_min,
    // d gam / d gamma, d wta / d agn_tau) and the AGN's cotangent of the linear L_bol
    std::vector<float4> h_dchain;
    DevBuf<float4> d_dchain;
    DevBuf<double> d_lsum_bar;
    NebularGrid neb;
    std::string isoc = "synthetic";   // the isochrone set of the setup (names the nebular libraries)
    SspOps ops;
    Emulator emu;                // the learned emulator (emulator.cu, emulator_train.cu)
    DevBuf<double> d_w64, d_y64, d_bc64, d_igm_a64;
    DevBuf<double> d_alpha;
    DevBuf<__nv_bfloat16> d_vhi, d_vlo;
    DevBuf<float> d_yo, d_vpart;
    DevBuf<double> d_spart;
    DevBuf<__nv_bfloat16> d_ix_hi, d_ix_lo;   // the interpolated fold's operand: node values x SFH weights
    DevBuf<float> d_ipart;       // and its GEMM's split-K partial sums
    DevBuf<double2> d_ix_const;  // and each model's 1 / T and c2
    DevBuf<DustEmModel> d_dem;   // the batch's dust emission cells (one per model)
    DevBuf<float> d_bpart;       // the band GEMM's partial fluxes when it splits the pixels (few models)
    DevBuf<float> d_vbar;        // reverse pass with operators: 2n x ntpad template cotangents (young, old)
    DevBuf<__nv_bfloat16> d_vbh, d_vbl;   // and as bf16 hi / lo (the interpolated reverse fold's A operand)
    DevBuf<float> d_xbar;        // the interpolated reverse fold: a chunk's cotangents of the operand X
    DevBuf<double> d_apart;      // and nz x n x 3 IMF-slope cotangents per metallicity slab
    DevBuf<int> d_vflag;
    DevBuf<int> d_status;
    int last_n = 0;              // models of the last batch (device spectra valid for these)
    int last_launches = 0;       // kernels launched by the last batch
    // profiling: events recorded between the kernels of a batch (opensps_gb300_set_profiling)
    static constexpr int NPROF = 10;
    int profile = 0, prof_set = 0, prof_used[2] = {0, 0}, prof_count = 0, prof_nstage = 0;
    bool prof_pending[2] = {false, false};
    double prof_acc[NPROF] = {};
    cudaEvent_t prof_ev[2][NPROF] = {};
    void *pinned_spec = nullptr; size_t pinned_bytes = 0;
    double *pinned_par = nullptr; size_t pinned_par_n = 0;   // page-locked staging of the per-model parameter table
    DustEmModel *pinned_dem = nullptr; size_t pinned_dem_n = 0;   // page-locked staging of the dust emission / AGN cells
    double *pinned_sums = nullptr; size_t pinned_sums_n = 0; // page-locked copy of the mass and L_bol sums
    std::vector<int> do_band_h;                               // the band mask last uploaded to d_do_band
    double *pinned_mags = nullptr; size_t pinned_mags_n = 0; // page-locked staging of the chunked batch's magnitudes
    std::vector<double> param_rows;                          // the batch's parameter rows (PF_COUNT x n)
    static constexpr int NCHUNK_EV = 64;
    cudaEvent_t chunk_ev[NCHUNK_EV] = {};                    // the chunked batch's weight copies
    cudaEvent_t par_ev = nullptr;                            // and its parameter table's copy
    cudaEvent_t mag_ev[NCHUNK_EV] = {};                      // and its chunks' band kernels (magnitude copies)
    std::vector<double> last_maggies;
    int keep_maggies = 0;

    ~Context();
};

// status codes of opensps.h
enum { ST_OK = 0, ST_BAD_HANDLE = 1, ST_UNSUPPORTED = 2, ST_BAD_ARG = 3, ST_DATA_MISSING = 4,
       ST_NOT_SETUP = 301, ST_NO_OPERATOR = 303, ST_IMF_FILE = 504, ST_TABULAR_SFH = 508 };
constexpr int SFH_NTABMAX = 20000;   // the tabular SFH's rows at most (NTABMAX, src/core/opensps_constants.f90:147)

void set_error(int status, const std::string &msg);
int context_setup(Context &c, const char *isoc, const char *spec, const char *dust, std::string &err);
int context_setup_grid(Context &c, std::string &err);
int context_load_filters(Context &c, const std::string &name, std::string &err);
std::string data_root();

// Host-side bf16 conversion, round to nearest even (the device's __float2bfloat16_rn).
uint16_t f32_to_bf16_bits(float f);
float bf16_bits_to_f32(uint16_t b);

// The batch driver (batch.cu). Inputs are host pointers (the C API) unless dev_inputs, in which case wz and params
// are device pointers and the spectra stay on the device.
struct BatchIO {
    int n = 0;
    // per-model parameters (host): params_cols x n, the first params_cols of the ParamId order, the others the
    // context's defaults (param_defaults, PF_COUNT; with params_cols = PF_COUNT none)
    const double *params = nullptr;
    int params_cols = PF_COUNT;
    const double *param_defaults = nullptr;
    const double *wz = nullptr;      // nt x nz x n
    bool dev_inputs = false;         // wz, dev_params and mags are device pointers; outputs stay on the device
    const double *dev_params = nullptr;   // PAR_DEVICE x n on the device (dev_inputs)
    bool dev_sync = true;            // dev_inputs: wait for the batch before returning
    double *fband_dev = nullptr;     // device n x nbands band fluxes (the reverse pass), or null
    bool keep_parts = false;         // the reverse pass: the young and old sums kept on the device (d_young, d_old)
    // weights formed on the device (wz unused): per-model SFH columns (SFH_NCOL x n, host) with the SFH type, or the
    // caller's weights over ages (nt x n, host) blended at logzsol
    const double *sfh_par = nullptr;
    const double *given_w = nullptr;
    int sfh_type = 0;
    // outputs (host, may be null)
    double *mags = nullptr, *spec = nullptr, *mass = nullptr, *lbol = nullptr, *emlines = nullptr;
    double *young = nullptr, *old = nullptr, *mass_young = nullptr, *mass_old = nullptr, *lbol_young = nullptr,
           *lbol_old = nullptr, *sfr = nullptr, *mdust = nullptr;
};
int run_batch(Context &c, const BatchIO &io, std::string &err);
// The SSP operator (ssp_op.cu): build from the data root, the young / old sums of a batch, one IMF's SSP grid.
int ops_build(Context &c, std::string &err);
int dustem_load(Context &c, std::string &err);
int agn_load(Context &c, std::string &err);
// the diffuse dust curves (dust_curves.cu): per pixel the tables T0..T3 (4 x nspec, pixel-major) of dust_type, per
// model its scalars (s1, s2, s3, ed); a pixel's curve (T0 + s1 T1 + s2 T2 + s3 T3) exp(ed ltab)
// (types 3 and 5: T0 the table lookup's curve on the grid, lookup)
bool dust_type_supported(int dust_type);
void dust_tables(int dust_type, const std::vector<double> &lam, const double *lookup, std::vector<double> &tab);
// the curves of dust types 3 and 5 from the data root (once per context): 0 or a status with err
int attenuation_load(Context &c, std::string &err);
void dust_scalars(int dust_type, double dust_index, double mwr, double uvb, double s[4]);
double dust_curve_value(const double *t, const double s[4], double ltab);
// the nebular ages as the continuum kernel's runs for this itesc (context.cu; rebuilt when itesc changes)
int nebular_runs(Context &c, int itesc, std::string &err);
// The plain FP64 path (fp64_path.cu): the age sums by DGEMM and the rest in FP64, into the host outputs of io.
void line_basis_host(const Context &c, bool neb, double line_sigma, std::vector<double> &b);
int run_fp64_tail(Context &c, const BatchIO &io, BasisOperand *bop, const double *d_wz, const double *d_par, int nacc,
                  int sm_lo, int sm_hi, int i0, std::string &err);
void fp64_release(Context &c);
// the reverse of the interpolated fold (ssp_op.cu): r as for run_ops_reverse, the template cotangents in r.vbar
int run_ops_interp_reverse(Context &c, const OpsRevArgs &r, std::string &err);
int run_ops_parts(Context &c, int n, const double *d_wz, const double *d_alpha, const double *h_alpha, int itesc,
                  float *d_young, float *d_old, std::string &err);
void imf_pack(int imf_type, const double *pv, double *ap);
// The IMF's limits and user segments for the operator kernels (the user IMF read and uploaded when imf_type is 5): 0,
// or ST_IMF_FILE / ST_DATA_MISSING with err.
int ops_imf_limits(Context &c, int imf_type, OpsImfLim &lim, std::string &err);
int ops_evaluate(Context &c, int imf_type, const double *imf_params, double *mass_grid, double *lbol_grid,
                 double *spec_grid, std::string &err);
// With profiling on: records event k on the context's stream (0 starts a batch's set).
void prof_mark(Context &c, int k);

cudaError_t encode_tmap_2d_bf16(CUtensorMap *m, const void *ptr, uint64_t inner, uint64_t outer, uint32_t box_inner,
                                uint32_t box_outer);
cudaError_t encode_tmap_2d_16(CUtensorMap *m, const void *ptr, uint64_t inner, uint64_t outer, uint32_t box_inner,
                              uint32_t box_outer, bool f16);
cudaError_t encode_tmap_2d_16s(CUtensorMap *m, const void *ptr, uint64_t inner, uint64_t outer, uint64_t row_elems,
                               uint32_t box_inner, uint32_t box_outer, bool f16);

}  // namespace sps
