// Magnitudes of spectra already on the device, through the band GEMM, with no allocation in the call: the band GEMM's
// per-model scratch (the observed-frame shift, the distance term), the band mask and the status word live in one
// file-scope device array of fixed size instead of the context's device buffers.
//
// The scratch (SCRATCH_BYTES = 2 MiB, held on every device that loads the library until the process exits):
//   [0, 16 MAX_MODELS)                   float4 zinfo per model (the band GEMM's observed-frame shift)
//   [16 MAX_MODELS, 24 MAX_MODELS)       double dist per model (distance modulus and (1 + z) term)
//   [24 MAX_MODELS, + 4 MAX_BANDS)       int do_band per band
//   [.., + 4)                            int status (cleared by every call)
// Every call on a device shares the array and leaves its contents behind; two calls whose kernels overlap on the
// GPU (other streams, other contexts, other threads) race on it.
//
// When the array comes into being: the library's kernels sit in separately compiled modules that CUDA loads lazily,
// on a module's first use on a device. Loading this file's module creates the array (and its code) in device memory,
// and loading the band GEMM's module creates its code. So that a call of the entry point never does either, every
// context set-up (opensps_context_setup) loads both modules on the context's device and looks the array's device
// address up there with cudaGetSymbolAddress (noalloc_prepare); the call only reads that address. A set-up after a
// device reset looks it up again.
#include <cuda_runtime.h>
#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>
#include "context.h"

namespace sps {

constexpr int NOALLOC_MAX_MODELS = 65536;
constexpr int NOALLOC_MAX_BANDS = 256;
constexpr size_t NOALLOC_ZINFO_OFF = 0;
constexpr size_t NOALLOC_DIST_OFF = NOALLOC_ZINFO_OFF + 16 * (size_t)NOALLOC_MAX_MODELS;
constexpr size_t NOALLOC_BAND_OFF = NOALLOC_DIST_OFF + 8 * (size_t)NOALLOC_MAX_MODELS;
constexpr size_t NOALLOC_STATUS_OFF = NOALLOC_BAND_OFF + 4 * (size_t)NOALLOC_MAX_BANDS;
constexpr size_t NOALLOC_SCRATCH_BYTES = 2u << 20;
static_assert(NOALLOC_STATUS_OFF + 4 <= NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the array");

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

int noalloc_max_models() { return NOALLOC_MAX_MODELS; }

struct ObsFrameArgs {
    int n, nbands;
    const double *zred;      // n
    const double *zt, *dl;   // cosmology table (500)
    double dlnl;
    uint32_t band_mask[NOALLOC_MAX_BANDS / 32];   // bit b: band b computed
    float4 *zinfo;
    double *dist;
    int *do_band;
};

// Per model: the observed-frame shift on the log-uniform grid and the distance term, as the batch's model-parameter
// kernel forms them (compute_magnitudes_columns' observed_frame_z and distance_term,
// src/spectra/opensps_batch_photometry.f90:784-903); thread 0 of block 0 also writes the band mask.
__global__ void obs_frame_kernel(ObsFrameArgs a) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m == 0)
        for (int b = 0; b < a.nbands; ++b) a.do_band[b] = (a.band_mask[b >> 5] >> (b & 31)) & 1u;
    if (m >= a.n) return;
    const double z = a.zred[m];
    float4 zi = make_float4(__int_as_float(0), 0.f, 0.f, 0.f);
    double dd = 0.0;
    if (fabs(z) > SAFE_FLOOR) {
        const double s = log1p(z) / a.dlnl;
        const double n0 = floor(s), phi = s - n0;
        zi.x = __int_as_float((int)n0);
        zi.y = phi > 0.0 ? (float)(expm1((1.0 - phi) * a.dlnl) / expm1(a.dlnl)) : 0.f;
        zi.z = (float)s;
        zi.w = 1.f;
        const int idx = max(0, min(find_interval0(a.zt, 500, z), 498));
        const double slope = (a.dl[idx + 1] - a.dl[idx]) / (a.zt[idx + 1] - a.zt[idx]);
        const double dm = a.dl[idx] + slope * (z - a.zt[idx]);
        if (dm == dm && dm > SAFE_FLOOR) dd = 5.0 * log10(dm / 10.0) - 2.5 * log10(1.0 + z);
    }
    a.zinfo[m] = zi;
    a.dist[m] = dd;
}

// The scratch's device address on each device, looked up by noalloc_prepare at every context set-up there.
static std::mutex g_noalloc_mu;
static unsigned char *g_noalloc_ptr[256] = {};

// With `device` current: loads this file's module and the band GEMM's on it (the array is created then), and records
// the array's device address. Called by the context's set-up, so that the entry point itself allocates nothing.
cudaError_t noalloc_prepare(int device) {
    if (device < 0 || device >= 256) return cudaErrorInvalidDevice;
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, obs_frame_kernel);
    if (e == cudaSuccess) e = band_gemm_load();
    void *p = nullptr;
    if (e == cudaSuccess) e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    g_noalloc_ptr[device] = static_cast<unsigned char *>(p);
    return cudaSuccess;
}

static cudaError_t noalloc_scratch(int device, unsigned char **out) {
    if (device < 0 || device >= 256) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[device]) return cudaErrorNotReady;   // the context was not set up on this device
    *out = g_noalloc_ptr[device];
    return cudaSuccess;
}

int run_mags_noalloc(Context &c, int n, const float *d_spec, const double *d_zred, double *d_mags, bool sync,
                     std::string &err) {
    if (n < 0 || n > NOALLOC_MAX_MODELS) {
        err = "spec_mags_noalloc: n = " + std::to_string(n) + " is beyond the scratch's maximum of " +
              std::to_string(NOALLOC_MAX_MODELS) + " models";
        return ST_BAD_ARG;
    }
    if (c.nbands <= 0 || c.nbands > NOALLOC_MAX_BANDS || c.band_nkb <= 0) {
        err = "spec_mags_noalloc: no filter library of 1 .. 256 bands is loaded";
        return ST_BAD_ARG;
    }
    if (n == 0) return 0;
    if (!d_spec || !d_zred || !d_mags) { err = "spec_mags_noalloc: a device pointer is NULL"; return ST_BAD_ARG; }
    int prev = -1;
    cudaError_t e = cudaGetDevice(&prev);
    if (e == cudaSuccess && prev != c.device) e = cudaSetDevice(c.device);
    unsigned char *base = nullptr;
    if (e == cudaSuccess && noalloc_scratch(c.device, &base) != cudaSuccess) {
        err = "spec_mags_noalloc: the context was not set up on its device";
        if (prev >= 0 && prev != c.device) cudaSetDevice(prev);
        return ST_NOT_SETUP;
    }
    int rc = 0;
    if (e == cudaSuccess) {
        float4 *zinfo = reinterpret_cast<float4 *>(base + NOALLOC_ZINFO_OFF);
        double *dist = reinterpret_cast<double *>(base + NOALLOC_DIST_OFF);
        int *do_band = reinterpret_cast<int *>(base + NOALLOC_BAND_OFF);
        int *status = reinterpret_cast<int *>(base + NOALLOC_STATUS_OFF);
        cudaStream_t st = c.stream;
        ObsFrameArgs oa;
        oa.n = n; oa.nbands = c.nbands; oa.zred = d_zred; oa.zt = c.d_zt.p; oa.dl = c.d_dl.p; oa.dlnl = c.dlnl;
        for (int i = 0; i < NOALLOC_MAX_BANDS / 32; ++i) oa.band_mask[i] = 0u;
        for (int b = 0; b < c.nbands; ++b)
            if (b >= (int)c.mag_mask.size() || c.mag_mask[b] != 0) oa.band_mask[b >> 5] |= 1u << (b & 31);
        oa.zinfo = zinfo; oa.dist = dist; oa.do_band = do_band;
        e = cudaMemsetAsync(status, 0, sizeof(int), st);
        if (e == cudaSuccess) {
            obs_frame_kernel<<<(n + 255) / 256, 256, 0, st>>>(oa);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) {
            BandGemmArgs ba{};
            ba.n_models = n; ba.nspec = c.nspec; ba.nbands = c.nbands; ba.npad = c.band_npad; ba.nkb = c.band_nkb;
            ba.j0 = c.band_j0; ba.ld_spec = c.nspec; ba.spec = d_spec; ba.zinfo = zinfo;
            ba.dlnl = c.dlnl; ba.dist = dist;
            ba.zp = 48.60 + 2.5 * std::log10(3.828e33 / (4.0 * M_PI * std::pow(10.0 * (648000.0 / M_PI) * 1.495978707e13, 2)));
            ba.do_band = do_band; ba.fband = nullptr; ba.mags = d_mags; ba.status = status;
            e = run_band_gemm(ba, c.tm_cb_hi, c.tm_cb_lo, st);
        }
        if (e == cudaSuccess && sync) {
            int kstatus = 0;
            e = cudaMemcpyAsync(&kstatus, status, sizeof(int), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e == cudaSuccess && kstatus != 0) {
                err = "spec_mags_noalloc: a device wait gave up (code " + std::to_string(kstatus) + ")";
                rc = ST_DATA_MISSING;
            }
        }
    }
    if (e != cudaSuccess) {
        err = std::string("spec_mags_noalloc: ") + cudaGetErrorString(e);
        rc = ST_DATA_MISSING;
    }
    if (prev >= 0 && prev != c.device) cudaSetDevice(prev);
    return rc;
}

}  // namespace sps
