// The plain FP64 path on the GPU (the "gb300_fp64" setting): the same batch as the mixed-precision path with every
// stage in FP64, the denominator of the mixed path's speed-up. The age sums are two FP64 GEMMs (cuBLAS DGEMM: a plain
// library GEMM) over the basis in the contraction's K order (young ages, then old); the rest is one CTA per model in
// FP64: attenuation (attenuate_batch, src/physics/opensps_csp_batch.f90:3576-3660), the IGM (apply_igm_z :4205-4299),
// velocity smoothing (build_velocity_kernel, src/spectra/opensps_smoothing.f90:553-633), the observed frame
// (observed_frame_z, src/spectra/opensps_batch_photometry.f90:819-903), the band integrals and magnitudes (:185-232,
// :1049-1171) with libm's exp / log in FP64.
#include <cuda_runtime.h>
#include <cublas_v2.h>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>
#include "context.h"

namespace sps {

constexpr int F64_THREADS = 256;
constexpr double F64_C_KMS = 2.99792458e5;

__global__ void gather_w64_kernel(int n, int kpad, int ntz, const int *kmap, const double *wz, double *w64) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)n * kpad) return;
    const int m = (int)(i / kpad), k = (int)(i % kpad);
    const int code = kmap[k];
    double v = 0.0;
    if (code >= 0) {
        const double w = wz[(size_t)m * ntz + (code & KMAP_SRC)];
        v = (w > SAFE_FLOOR) ? w : 0.0;   // (model_sums_zw: weights at or below SAFE_FLOOR are skipped)
    }
    w64[i] = v;
}

struct F64Args {
    int n, ns, nb, jtop, sm_lo, sm_hi, i0, smooth, j0, j1;
    const double *par;          // n x PAR_DEVICE
    const double *y, *o;        // ns x n (column per model)
    const double *lam, *lnlam;  // ns
    const double *igm_a;        // jtop x 6
    const double *zt, *dl;
    const double *bc;           // the band matrix by band, FP64 (band b's pixels lo .. hi at off)
    const int4 *bmeta;          // (lo, hi, off, 0)
    const int *do_band;
    double zp;
    double *spec;               // n x ns
    double *mags;               // n x nb
};

__global__ void __launch_bounds__(F64_THREADS) fp64_tail_kernel(F64Args a) {
    extern __shared__ double dsm[];
    const int ns = a.ns, m = blockIdx.x, tid = threadIdx.x;
    double *TOT = dsm, *S = dsm + ns;            // then TOT holds the observed frame / lambda
    __shared__ double tap[9];
    __shared__ int s_R;
    __shared__ double b_s[6];
    __shared__ double red_v[F64_THREADS / 32];
    __shared__ int red_j[F64_THREADS / 32];
    __shared__ double s_tmax;
    __shared__ int s_jmax;
    const double *p = a.par + (size_t)PAR_DEVICE * m;
    const double d1 = p[PF_DUST1], d2 = p[PF_DUST2], d3 = p[PF_DUST3], di = p[PF_DUST_INDEX], d1i = p[PF_DUST1_INDEX];
    const double fnd = p[PF_FRAC_NODUST], fo = p[PF_FRAC_OBRUN], z = p[PF_ZRED], fi = p[PF_IGM_FACTOR];
    const double *y = a.y + (size_t)ns * m, *o = a.o + (size_t)ns * m;
    const bool igm = a.jtop > 0 && z > SAFE_FLOOR && a.igm_a != nullptr;
    if (tid == 0) {
        const double l1z = log1p(z);
        const double pk[6] = {3.46, 1.68, 3.0 + 0.46, 1.5 + 0.18, 3.0 - 1.32, 1.68};
        for (int k = 0; k < 6; ++k) b_s[k] = igm ? exp(pk[k] * l1z) : 0.0;
        // the smoothing row of pixel i0 (its taps serve every pixel of the log-uniform grid)
        s_R = -1;
        for (int d = 0; d < 9; ++d) tap[d] = 0.0;
        const double sig = p[PF_SIGMA_SMOOTH];
        if (a.smooth && sig > SAFE_FLOOR && a.i0 >= 0) {
            const int i = a.i0;
            const double sb = sig / F64_C_KMS, inv2s2 = 0.5 / (sb * sb);
            const double vl = a.lnlam[i] - 4.0 * sb, vh = a.lnlam[i] + 4.0 * sb;
            int lo = 0, hi = ns;
            while (lo < hi) { const int md = (lo + hi) / 2; if (a.lnlam[md] < vl) lo = md + 1; else hi = md; }
            int il = lo < ns ? lo : ns - 1;
            if (il > 0 && a.lnlam[il] > vl) il--;
            lo = il; hi = ns;
            while (lo < hi) { const int md = (lo + hi) / 2; if (a.lnlam[md] < vh) lo = md + 1; else hi = md; }
            int ih = lo < ns ? lo : ns - 1;
            if (ih < il) ih = il;
            if (ih - il + 1 >= 2 && i - il <= 4 && ih - i <= 4) {
                double w[9], tw = 0.0;
                for (int u = 0; u < 9; ++u) {
                    const int j = il + u;
                    double wj = 0.0;
                    if (j <= ih) {
                        const double dd = a.lnlam[i] - a.lnlam[j];
                        const double dlft = (j > il) ? a.lam[j] - a.lam[j - 1] : 0.0;
                        const double drgt = (j < ih) ? a.lam[j + 1] - a.lam[j] : 0.0;
                        wj = exp(-inv2s2 * dd * dd) / a.lam[j] * 0.5 * (dlft + drgt);
                    }
                    w[u] = wj;
                    tw += wj;
                }
                if (tw > 0.0) {
                    for (int d = -4; d <= 4; ++d) {
                        const int u = i + d - il;
                        tap[4 + d] = (u >= 0 && u <= ih - il && u < 9) ? w[u] / tw : 0.0;
                    }
                    s_R = max(i - il, ih - i);
                }
            }
        }
    }
    __syncthreads();
    // ---- the IGM cap: the first pixel of the largest optical depth below Lyman alpha
    if (igm) {
        double tmax = 0.0;
        int jmax = 1 << 30;
        for (int j = tid; j < a.jtop; j += F64_THREADS) {
            const double *ia = a.igm_a + 6 * (size_t)j;
            double t = 0.0;
            for (int k = 0; k < 6; ++k) t += ia[k] * b_s[k];
            if (t > tmax || (t == tmax && j < jmax && t > 0.0)) { tmax = t; jmax = j; }
        }
        for (int off = 16; off > 0; off >>= 1) {
            const double t2 = __shfl_xor_sync(0xffffffffu, tmax, off);
            const int j2 = __shfl_xor_sync(0xffffffffu, jmax, off);
            if (t2 > tmax || (t2 == tmax && j2 < jmax)) { tmax = t2; jmax = j2; }
        }
        if ((tid & 31) == 0) { red_v[tid >> 5] = tmax; red_j[tid >> 5] = jmax; }
        __syncthreads();
        if (tid == 0) {
            double tm = 0.0;
            int jm = 1 << 30;
            for (int w = 0; w < F64_THREADS / 32; ++w)
                if (red_v[w] > tm || (red_v[w] == tm && red_j[w] < jm)) { tm = red_v[w]; jm = red_j[w]; }
            s_tmax = tm;
            s_jmax = (tm > 0.0) ? jm + 1 : 1;   // 1-based; pixels below it take its depth
        }
        __syncthreads();
    }
    // ---- attenuation and IGM: TOT
    for (int j = tid; j < ns; j += F64_THREADS) {
        const double ltab = a.lnlam[j] - 8.612503371220562;   // ln(lambda / 5500)
        const double curve = (di != 0.0) ? exp(di * ltab) : 1.0;
        const double td = exp(-d2 * curve);
        const double tb = (d1 <= SAFE_FLOOR || 1.0 - fo <= SAFE_FLOOR) ? 1.0 : exp(-(d1 * exp(d1i * ltab)));
        const double too = (fabs(d3) <= SAFE_FLOOR) ? 1.0 : exp(-(d3 * curve));
        const double ss = (y[j] * tb * (1.0 - fo) + y[j] * fo) + o[j] * too;
        double tot = (1.0 - fnd <= SAFE_FLOOR) ? ss : ss * (td * (1.0 - fnd) + fnd);
        if (igm && j < a.jtop) {
            double tau;
            if (j < s_jmax - 1 && s_jmax > 1) {
                tau = s_tmax;
            } else {
                const double *ia = a.igm_a + 6 * (size_t)j;
                tau = 0.0;
                for (int k = 0; k < 6; ++k) tau += ia[k] * b_s[k];
            }
            tot *= exp(-tau * fi);
        }
        TOT[j] = tot;
    }
    __syncthreads();
    // ---- smoothing
    const int R = s_R;
    double *spec = a.spec + (size_t)ns * m;
    for (int j = tid; j < ns; j += F64_THREADS) {
        double v = TOT[j];
        if (R >= 0 && j >= a.sm_lo && j <= a.sm_hi) {
            double s = 0.0;
            for (int d = -4; d <= 4; ++d) s += tap[d + 4] * TOT[j + d];
            v = s;
        }
        S[j] = v;
        spec[j] = v;
    }
    __syncthreads();
    if (!a.mags) return;
    // ---- observed frame / lambda over the pixels the bands reach (into TOT)
    const bool shifted = fabs(z) > SAFE_FLOOR;
    for (int j = a.j0 + tid; j <= a.j1; j += F64_THREADS) {
        double v;
        if (shifted) {
            const double target = a.lam[j] / (1.0 + z);
            int il = find_interval0(a.lam, ns, target) + 1;
            il = il < 1 ? 1 : (il > ns - 1 ? ns - 1 : il);
            const double t = (target - a.lam[il - 1]) / (a.lam[il] - a.lam[il - 1]);
            v = S[il - 1] + t * (S[il] - S[il - 1]);
        } else {
            v = S[j];
        }
        if (v != v) v = 0.0;
        TOT[j] = (v > 0.0 ? v : 0.0) / a.lam[j];
    }
    __syncthreads();
    // ---- band fluxes (warp per band) and magnitudes
    double dist = 0.0;
    if (shifted) {
        const int idx = max(0, min(find_interval0(a.zt, 500, z), 498));
        const double slope = (a.dl[idx + 1] - a.dl[idx]) / (a.zt[idx + 1] - a.zt[idx]);
        const double dm = a.dl[idx] + slope * (z - a.zt[idx]);
        if (dm == dm && dm > SAFE_FLOOR) dist = 5.0 * log10(dm / 10.0) - 2.5 * log10(1.0 + z);
    }
    const int warp = tid >> 5, lane = tid & 31;
    for (int b = warp; b < a.nb; b += F64_THREADS / 32) {
        const int4 bm = a.bmeta[b];
        double s = 0.0;
        for (int j = bm.x + lane; j <= bm.y; j += 32) s += a.bc[bm.z + (j - bm.x)] * TOT[j];
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (lane == 0) {
            double mg = __longlong_as_double(0x7ff8000000000000LL);
            if ((a.do_band == nullptr || a.do_band[b] != 0) && s > 0.0) mg = -2.5 * log10(s) - a.zp + dist;
            a.mags[(size_t)a.nb * m + b] = mg;
        }
    }
}

void fp64_release(Context &c) {
    if (c.cublas) cublasDestroy(static_cast<cublasHandle_t>(c.cublas));
    c.cublas = nullptr;
}

static std::string fmsg(const char *what, cudaError_t e) { return std::string(what) + ": " + cudaGetErrorString(e); }

int run_fp64_tail(Context &c, const BatchIO &io, BasisOperand *bop, const double *d_wz, const double *d_par, int nacc,
                  int sm_lo, int sm_hi, int i0, std::string &err) {
    const int n = io.n, ns = c.nspec, nt = c.nt, nz = c.nz, nb = c.nbands, kpad = bop->kpad;
    cudaStream_t st = c.stream;
    cudaError_t e;
    // the basis in FP64 (once per operand), in the operand's K order
    if (!bop->b64.p) {
        std::vector<double> b, kb((size_t)ns * kpad, 0.0);
        line_basis_host(c, bop->neb, bop->line_sigma, b);
        std::vector<int> kmap(kpad);
        if ((e = cudaMemcpy(kmap.data(), bop->kmap.p, sizeof(int) * kpad, cudaMemcpyDeviceToHost)) != cudaSuccess) {
            err = fmsg("basis map", e);
            return ST_DATA_MISSING;
        }
        for (int k = 0; k < kpad; ++k)
            if (kmap[k] >= 0)
                std::copy(b.data() + (size_t)ns * (kmap[k] & KMAP_SRC), b.data() + (size_t)ns * ((kmap[k] & KMAP_SRC) + 1),
                          kb.data() + (size_t)ns * k);
        if ((e = bop->b64.reserve(kb.size())) != cudaSuccess ||
            (e = cudaMemcpy(bop->b64.p, kb.data(), sizeof(double) * kb.size(), cudaMemcpyHostToDevice)) != cudaSuccess) {
            err = fmsg("FP64 basis", e);
            bop->b64.release();
            return ST_DATA_MISSING;
        }
    }
    if (!c.cublas) {
        cublasHandle_t h;
        if (cublasCreate(&h) != CUBLAS_STATUS_SUCCESS) { err = "cuBLAS could not be initialised"; return ST_DATA_MISSING; }
        c.cublas = h;
    }
    cublasHandle_t h = static_cast<cublasHandle_t>(c.cublas);
    cublasSetStream(h, st);
    if ((e = c.d_w64.reserve((size_t)n * kpad)) != cudaSuccess || (e = c.d_y64.reserve((size_t)2 * ns * n)) != cudaSuccess ||
        (e = c.d_spec64.reserve((size_t)n * ns)) != cudaSuccess || (e = c.d_mags.reserve((size_t)n * std::max(nb, 1))) != cudaSuccess) {
        err = fmsg("device memory", e);
        return ST_DATA_MISSING;
    }
    gather_w64_kernel<<<(unsigned)(((size_t)n * kpad + 255) / 256), 256, 0, st>>>(n, kpad, nt * nz, bop->kmap.p, d_wz,
                                                                                    c.d_w64.p);
    if ((e = cudaGetLastError()) != cudaSuccess) { err = fmsg("FP64 weights", e); return ST_DATA_MISSING; }
    double *Y = c.d_y64.p, *O = c.d_y64.p + (size_t)ns * n;
    const double one = 1.0, zero = 0.0;
    const int ky = (nacc == 1) ? kpad : bop->ky_pad;
    if (cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, ns, n, ky, &one, bop->b64.p, ns, c.d_w64.p, kpad, &zero, Y, ns) !=
        CUBLAS_STATUS_SUCCESS) {
        err = "DGEMM (young) failed";
        return ST_DATA_MISSING;
    }
    if (kpad - ky > 0) {
        if (cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_N, ns, n, kpad - ky, &one, bop->b64.p + (size_t)ns * ky, ns,
                        c.d_w64.p + ky, kpad, &zero, O, ns) != CUBLAS_STATUS_SUCCESS) {
            err = "DGEMM (old) failed";
            return ST_DATA_MISSING;
        }
    } else if ((e = cudaMemsetAsync(O, 0, sizeof(double) * ns * n, st)) != cudaSuccess) {
        err = fmsg("FP64 old sums", e);
        return ST_DATA_MISSING;
    }
    F64Args a;
    a.n = n; a.ns = ns; a.nb = nb; a.jtop = c.add_igm_absorption == 1 ? c.jtop : 0;
    a.sm_lo = sm_lo; a.sm_hi = sm_hi; a.i0 = i0; a.smooth = sm_hi >= sm_lo ? 1 : 0;
    a.j0 = c.band_j0; a.j1 = nb > 0 ? c.band_j1 : c.band_j0 - 1;
    a.par = d_par; a.y = Y; a.o = O; a.lam = c.d_lam.p; a.lnlam = c.d_lnlam.p; a.igm_a = c.d_igm_a64.p;
    a.zt = c.d_zt.p; a.dl = c.d_dl.p; a.bc = c.d_bc64.p; a.bmeta = c.d_bmeta.p;
    a.do_band = c.mag_mask.empty() ? nullptr : c.d_do_band.p;
    a.zp = 48.60 + 2.5 * std::log10(3.828e33 / (4.0 * M_PI * std::pow(10.0 * (648000.0 / M_PI) * 1.495978707e13, 2)));
    a.spec = c.d_spec64.p;
    a.mags = (io.mags && !c.fast_mode && nb > 0) ? c.d_mags.p : nullptr;
    const size_t smem = sizeof(double) * 2 * (size_t)ns;
    if ((e = cudaFuncSetAttribute(fp64_tail_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess) {
        err = fmsg("FP64 kernel", e);
        return ST_DATA_MISSING;
    }
    fp64_tail_kernel<<<n, F64_THREADS, smem, st>>>(a);
    if ((e = cudaGetLastError()) != cudaSuccess) { err = fmsg("FP64 kernel", e); return ST_DATA_MISSING; }
    return 0;
}

}  // namespace sps
