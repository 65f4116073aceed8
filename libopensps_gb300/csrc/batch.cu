// The batch driver: per-model parameters and checks on the host, then the device pipeline
//   weights_prep -> model_params -> contraction (+ fused epilogue) -> bands / magnitudes
// on the context's stream (OpenSPS compute_csp_batch, src/physics/opensps_csp_batch.f90:431-1214).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include "context.h"
#include "datalib.h"

namespace sps {

// ---------------------------------------------------------------------------------------------- model params
struct ModelParamArgs {
    int n, nspec, jtop, add_igm, smooth, i0;   // i0: the pixel whose smoothing row gives the model's taps
    int mpw = 32;            // models per warp (1 .. 32)
    int dust_type = 0;       // the diffuse curve's scalars (MP_DUST_INDEX: its power, MP_CS1..: the tables' weights)
    const double *par;       // PAR_DEVICE x n
    const float *igm_a;      // jtop x 6
    const double *lam;       // nspec
    const double *lnlam;     // nspec: ln lambda
    const double *zt, *dl;   // 500
    double dlnl;
    float *mpar;             // n x MODEL_PAR_FLOATS
    float4 *zinfo;           // n: the observed-frame shift (band_gemm.cu)
    double *dist;            // n
};

// One thread per model for the FP64 scalars (GB300's FP64 rate is low: a warp instruction serves 32 models); the IGM
// cap's search for the largest optical depth over the pixels below Lyman alpha is shared by the warp's lanes, model
// after model.
__global__ void __launch_bounds__(256) model_params_kernel(ModelParamArgs a) {
    // a.mpw models per warp (lanes 0 .. mpw - 1): fewer than 32 when the batch is small, so that more warps share
    // the cap searches
    const int lane = threadIdx.x & 31;
    const int m = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * a.mpw + lane;
    const bool live = lane < a.mpw && m < a.n;
    const double LOG2E = 1.4426950408889634;
    const double *p = a.par + (size_t)PAR_DEVICE * (live ? m : 0);
    const double z = live ? p[PF_ZRED] : 0.0;
    const bool igm = live && a.add_igm && z > SAFE_FLOOR && a.jtop > 0;
    // redshift factors b_k = (1 + z)^p_k (igm_tau_z_terms, src/physics/opensps_cosmology.f90:497-508)
    float b[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const double l1z = live ? log1p(z) : 0.0;   // (also the observed frame's shift below)
    if (igm) {
        // (1 + z)^p = 2^(p ln(1 + z) log2 e): the exponent formed and split in FP64 (x = n + r, |r| <= 1/2), 2^r
        // by the SFU and 2^n exactly (the reference's exp_kp: FP64 argument, exponential at kernel precision; the
        // factors are stored as FP32)
        auto pw = [&](double pexp) {
            const double x = pexp * l1z * LOG2E, n = rint(x);
            float r;
            asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"((float)(x - n)));
            const int ni = (int)n;
            return (ni > -126 && ni < 128) ? r * __int_as_float((ni + 127) << 23) : (float)exp(pexp * l1z);
        };
        b[0] = pw(3.46);
        b[1] = pw(1.68);
        b[2] = pw(3.0 + 0.46);
        b[3] = pw(1.5 + 0.18);
        b[4] = pw(3.0 - 1.32);
        b[5] = b[1];
    }
    // the cap (apply_igm_z :4272-4299): the first pixel of the largest optical depth, searched by the whole warp for
    // each of its models in turn, over the wavelength factors staged in shared memory (one array per factor)
    extern __shared__ float4 sa4[];  // jtop float4 (factors 0..3), then jtop float2 (factors 4, 5)
    const int nj = a.add_igm ? a.jtop : 0;
    float2 *sa2 = reinterpret_cast<float2 *>(sa4 + nj);
    for (int j = threadIdx.x; j < nj; j += blockDim.x) {
        const float *g = a.igm_a + 6 * (size_t)j;
        sa4[j] = make_float4(g[0], g[1], g[2], g[3]);
        sa2[j] = make_float2(g[4], g[5]);
    }
    __syncthreads();
    float my_tmax = 0.f;
    int my_jmax = 1;
    const unsigned todo = __ballot_sync(0xffffffffu, igm);
    for (int i = 0; i < a.mpw; ++i) {
        if (!((todo >> i) & 1u)) continue;
        float bb[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) bb[k] = __shfl_sync(0xffffffffu, b[k], i);
        float tmax = 0.f;
        int jmax = 1;
        for (int j = lane; j < nj; j += 32) {
            const float4 f = sa4[j];
            const float2 g = sa2[j];
            const float t = f.x * bb[0] + f.y * bb[1] + f.z * bb[2] + f.w * bb[3] + g.x * bb[4] + g.y * bb[5];
            if (t > tmax) { tmax = t; jmax = j + 1; }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const float t2 = __shfl_xor_sync(0xffffffffu, tmax, off);
            const int j2 = __shfl_xor_sync(0xffffffffu, jmax, off);
            if (t2 > tmax || (t2 == tmax && j2 < jmax)) { tmax = t2; jmax = j2; }
        }
        if (lane == i) { my_tmax = tmax; my_jmax = tmax > 0.f ? jmax : 1; }
    }
    if (!live) return;

    float *o = a.mpar + (size_t)MODEL_PAR_FLOATS * m;
    float blk[MODEL_PAR_FLOATS];
#pragma unroll
    for (int i = 0; i < MODEL_PAR_FLOATS; ++i) blk[i] = 0.f;
    // (dust_type 3: the diffuse optical depth is the curve itself, pixel_transmissions :3798-3801)
    const double d1 = p[PF_DUST1], d2 = a.dust_type == 3 ? 1.0 : p[PF_DUST2], d3 = p[PF_DUST3];
    const double fnd = p[PF_FRAC_NODUST], fo = p[PF_FRAC_OBRUN];
    // attenuate_batch / pixel_transmissions (src/physics/opensps_csp_batch.f90:3576-3660, 3765-3818)
    blk[MP_KD2] = (float)(-d2 * LOG2E);
    if (1.0 - fnd <= SAFE_FLOOR) { blk[MP_ONE_M_FND] = 0.f; blk[MP_FND] = 1.f; }
    else { blk[MP_ONE_M_FND] = (float)(1.0 - fnd); blk[MP_FND] = (float)fnd; }
    // the diffuse curve (T0 + s1 T1 + s2 T2 + s3 T3) (lambda / 5500)^ed (pixel_transmissions :3765-3818): power law
    // (0) ed = dust_index; CCM89 (1) s = (1 / mwr, uvb, uvb / mwr); Kriek & Conroy (4) s1 = ed = dust_index
    {
        const double di = p[PF_DUST_INDEX];
        float ed = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
        if (a.dust_type == 0) ed = (float)di;
        else if (a.dust_type == 4) { ed = (float)di; s1 = (float)di; }
        else if (a.dust_type == 1) { const double ir = 1.0 / p[PF_MWR], u = p[PF_UVB]; s1 = (float)ir; s2 = (float)u; s3 = (float)(u * ir); }
        blk[MP_DUST_INDEX] = ed;
        blk[MP_CS1] = s1; blk[MP_CS1 + 1] = s2; blk[MP_CS1 + 2] = s3;
    }
    blk[MP_KD1] = (d1 <= SAFE_FLOOR || 1.0 - fo <= SAFE_FLOOR) ? 0.f : (float)(-d1 * LOG2E);
    blk[MP_DUST1_INDEX] = (float)p[PF_DUST1_INDEX];
    blk[MP_ONE_M_FO] = (float)(1.0 - fo);
    blk[MP_FO] = (float)fo;
    blk[MP_KD3] = (fabs(d3) <= SAFE_FLOOR) ? 0.f : (float)(-d3 * LOG2E);
    blk[MP_IGM_JMAX] = __int_as_float(0);
    if (igm) {
        const double kf = -p[PF_IGM_FACTOR] * LOG2E;
#pragma unroll
        for (int k = 0; k < 6; ++k) blk[MP_IGM_KB + k] = (float)((double)b[k] * kf);
        blk[MP_IGM_KCAP] = (float)((double)my_tmax * kf);
        blk[MP_IGM_JMAX] = __int_as_float(my_jmax);
        blk[MP_IGM_ON] = 1.f;
    }
    // velocity smoothing taps: row i0 of build_velocity_kernel (src/spectra/opensps_smoothing.f90:553-633)
    blk[MP_SMOOTH_R] = __int_as_float(-1);
    const double sig = p[PF_SIGMA_SMOOTH];
    if (a.smooth && sig > SAFE_FLOOR && a.i0 >= 0) {
        const int n = a.nspec, i = a.i0;
        const double sb = sig / (C_LIGHT * 1.0e-13);
        const double inv2s2 = 0.5 * (1.0 / sb) * (1.0 / sb);
        // the window in ln lambda: lambda_j vs lambda_i exp(-+4 sigma / c) compared as logarithms
        const double vl = a.lnlam[i] - 4.0 * sb, vh = a.lnlam[i] + 4.0 * sb;
        // il: first pixel >= vl, one lower when it lies above vl; ih: first pixel >= vh
        int lo = 0, hi = n;
        while (lo < hi) { const int md = (lo + hi) / 2; if (a.lnlam[md] < vl) lo = md + 1; else hi = md; }
        int il = lo < n ? lo : n - 1;
        if (il > 0 && a.lnlam[il] > vl) il--;
        lo = il; hi = n;
        while (lo < hi) { const int md = (lo + hi) / 2; if (a.lnlam[md] < vh) lo = md + 1; else hi = md; }
        int ih = lo < n ? lo : n - 1;
        if (ih < il) ih = il;
        if (ih - il + 1 >= 2 && i - il <= 4 && ih - i <= 4) {
            // Gaussian weights / lambda_j times the trapezoid widths, normalised: the exponent is formed in FP64
            // (differences of ln lambda), the exponential and the normalisation in FP32 (the taps are stored so)
            float w[9], tw = 0.f;
            const double lli = a.lnlam[i];
#pragma unroll
            for (int u = 0; u < 9; ++u) {
                const int j = il + u;
                float wj = 0.f;
                if (j <= ih) {
                    const double d = lli - a.lnlam[j];
                    const float dlft = (j > il) ? (float)(a.lam[j] - a.lam[j - 1]) : 0.f;
                    const float drgt = (j < ih) ? (float)(a.lam[j + 1] - a.lam[j]) : 0.f;
                    wj = expf((float)(-inv2s2 * d * d)) / (float)a.lam[j] * 0.5f * (dlft + drgt);
                }
                w[u] = wj;
                tw += wj;
            }
            if (tw > 0.f) {
                const float inv = 1.f / tw;
#pragma unroll
                for (int d = -4; d <= 4; ++d) {
                    const int u = i + d - il;
                    blk[MP_TAPS + 4 + d] = (u >= 0 && u <= ih - il && u < 9) ? w[u] * inv : 0.f;
                }
                blk[MP_SMOOTH_R] = __int_as_float(max(i - il, ih - i));
            }
        }
    }
#pragma unroll
    for (int i = 0; i < MODEL_PAR_FLOATS; i += 4)
        reinterpret_cast<float4 *>(o)[i / 4] = make_float4(blk[i], blk[i + 1], blk[i + 2], blk[i + 3]);
    // observed frame: the shift of lambda / (1 + z) on the log-uniform grid, in pixels
    // (observed pixel j reads rest pixels j - n0 - 1 and j - n0 at t, the same t for every interior pixel)
    float4 zi = make_float4(__int_as_float(0), 0.f, 0.f, 0.f);
    double dd = 0.0;
    if (fabs(z) > SAFE_FLOOR) {
        const double s = l1z / a.dlnl;
        const double n0 = floor(s), phi = s - n0;
        zi.x = __int_as_float((int)n0);
        zi.y = phi > 0.0 ? (float)(expm1((1.0 - phi) * a.dlnl) / expm1(a.dlnl)) : 0.f;
        zi.z = (float)s;
        zi.w = 1.f;
        // distance term (distance_term, src/spectra/opensps_batch_photometry.f90:784-794)
        int idx = find_interval0(a.zt, 500, z);
        idx = max(0, min(idx, 498));
        const double slope = (a.dl[idx + 1] - a.dl[idx]) / (a.zt[idx + 1] - a.zt[idx]);
        const double dm = a.dl[idx] + slope * (z - a.zt[idx]);
        if (dm == dm && dm > SAFE_FLOOR) dd = 5.0 * log10(dm / 10.0) - 2.5 * log10(1.0 + z);
    }
    a.zinfo[m] = zi;
    a.dist[m] = dd;
}

// ---------------------------------------------------------------------------------------------- basis operand
// The line profile of one line (compute_line_gaussians src/physics/opensps_gas.f90:303-340, windowed as
// add_lines_to_spectrum :364-390): prof[j] for j in [jlo, jhi].
static void line_profile(const Context &c, double pos, double sigma_kms, std::vector<double> &prof, int &jlo,
                         int &jhi) {
    const int n = c.nspec;
    int j = find_interval0(c.lam.data(), n, pos) + 1;   // 1-based as the reference
    j = std::max(1, std::min(j, n - 1));
    const double res_min = c.lam[j] - c.lam[j - 1];
    double sig = pos * sigma_kms * (1.0e13 / C_LIGHT);
    sig = std::max(sig, 2.0 * res_min);
    const double norm = (1.0 / (std::sqrt(2.0 * M_PI) * sig)) * (pos * pos / C_LIGHT);
    prof.assign(n, 0.0);
    for (int i = 0; i < n; ++i) {
        const double x = (c.lam[i] - pos) / sig;
        prof[i] = norm * std::exp(-0.5 * x * x);
    }
    int jc = find_interval0(c.lam.data(), n, pos) + 1;
    jc = std::max(1, std::min(jc, n));
    int jh = std::min(jc + 1, n);
    const double cut = 1.0e-14 * std::max(prof[jc - 1], prof[jh - 1]);
    int jl = jc;
    while (jl > 1 && prof[jl - 2] > cut) jl--;
    while (jh < n && prof[jh] > cut) jh++;
    jlo = jl - 1;
    jhi = jh - 1;
    if (cut <= 0.0) { jlo = 0; jhi = -1; }
}

// True when every line's width at sigma_kms is the grid floor (2 pixels' width at the line).
static bool lines_floor_limited(const Context &c, double sigma_kms) {
    for (int l = 0; l < c.nline; ++l) {
        const double pos = c.line_lambda[l];
        int j = find_interval0(c.lam.data(), c.nspec, pos) + 1;
        j = std::max(1, std::min(j, c.nspec - 1));
        const double res_min = c.lam[j] - c.lam[j - 1];
        if (pos * sigma_kms * (1.0e13 / C_LIGHT) > 2.0 * res_min) return false;
    }
    return true;
}

// The SSP basis (nspec x nt x nz, FP64) with the nebular lines folded into the young SSPs.
void line_basis_host(const Context &c, bool neb, double line_sigma, std::vector<double> &b) {
    const int ns = c.nspec, nt = c.nt, nz = c.nz;
    b = c.ssp;
    if (neb) {
        // the young SSPs with their lines (add_neb_emission: linear in the weights, so part of the basis)
        std::vector<double> prof;
        for (int l = 0; l < c.nline; ++l) {
            int jlo, jhi;
            line_profile(c, c.line_lambda[l], line_sigma, prof, jlo, jhi);
            for (int z = 0; z < nz; ++z)
                for (int t = 0; t < nt; ++t) {
                    const double L = c.line_lum[l + (size_t)c.nline * (t + (size_t)nt * z)];
                    if (L == 0.0) continue;
                    double *col = b.data() + (size_t)ns * (t + (size_t)nt * z);
                    for (int j = jlo; j <= jhi; ++j) col[j] += prof[j] * L;
                }
        }
        // the gas absorbs the nebular ages' ionizing light (nebular_kernels step 2, opensps_csp_batch.f90:2726-2750:
        // the age sums at pixels 1..whlylim with the nebular ages times the escaping fraction; that fraction's share
        // is added per model by the epilogue when frac_obrun > 0)
        for (int z = 0; z < nz; ++z)
            for (int t = 0; t < c.nt_neb; ++t) {
                double *col = b.data() + (size_t)ns * (t + (size_t)nt * z);
                for (int i = 0; i < c.whlylim && i < ns; ++i) col[i] = 0.0;
            }
    }
}

// The contraction's basis operand for a K order (accumulators, dust_tesc's age, nebular lines at a line width), cached
// on the context. With ion (nebular emission and some model's frac_obrun above 0) two more K blocks follow the young
// and old ones: the nebular ages' unabsorbed ionizing spectra (the library's spectra at pixels below whlylim, zero
// above), ages below itesc then the rest, against the weights times each model's escaping fraction.
static BasisOperand *get_basis(Context &c, int nacc, int itesc, bool neb, double line_sigma, bool ion,
                               std::string &err) {
    union { double d; long long i; } u;
    u.d = neb ? line_sigma : -1.0;
    ion = ion && neb && c.nt_neb > 0 && c.whlylim > 0;
    const long long key = ((u.i * 31 + (long long)nacc) * 1009 + itesc) * 2 + (ion ? 1 : 0);
    auto it = c.basis_cache.find(key);
    if (it != c.basis_cache.end()) return it->second;
    const int ns = c.nspec, nt = c.nt, nz = c.nz;
    std::vector<double> b;
    line_basis_host(c, neb, line_sigma, b);
    BasisOperand *op = new BasisOperand();
    op->neb = neb;
    op->line_sigma = line_sigma;
    op->nacc = nacc;
    op->itesc = itesc;
    const int BK = contract_bk();
    auto pad = [BK](int k) { return (k + BK - 1) / BK * BK; };
    if (nacc == 1) {
        op->nty = 0;
        op->ky_pad = 0;
        op->kmain = pad(nt * nz);
    } else {
        op->nty = itesc;
        op->ky_pad = pad(itesc * nz);
        op->kmain = op->ky_pad + pad((nt - itesc) * nz);
    }
    // the escaping light's blocks: nebular ages below itesc (ty_end of them), then the other nebular ages
    const int ty_end = ion ? std::min(c.nt_neb, itesc) : 0, n_ion_old = ion ? c.nt_neb - ty_end : 0;
    op->ion = ion;
    op->kion_y = pad(ty_end * nz);
    op->kion_o = pad(n_ion_old * nz);
    op->kpad = op->kmain + op->kion_y + op->kion_o;
    const int kpad = op->kpad;
    std::vector<uint16_t> hi((size_t)ns * kpad, 0), lo((size_t)ns * kpad, 0);
    std::vector<int> kmap(kpad, -1);   // operand column -> source index t + nt z with the KMAP_ flags
    auto put = [&](int k, const double *col, int jn) {
        for (int j = 0; j < jn; ++j) {
            const float f = (float)col[j];
            const uint16_t h = f32_to_bf16_bits(f);
            hi[(size_t)j * kpad + k] = h;
            lo[(size_t)j * kpad + k] = f32_to_bf16_bits(f - bf16_bits_to_f32(h));
        }
    };
    for (int k = 0; k < op->kmain; ++k) {
        int t = -1, z = -1;
        if (nacc == 1) {
            if (k < nt * nz) { t = k % nt; z = k / nt; }
        } else if (k < op->ky_pad) {
            if (itesc > 0 && k < itesc * nz) { t = k % itesc; z = k / itesc; }
        } else {
            const int kk = k - op->ky_pad, nto = nt - itesc;
            if (nto > 0 && kk < nto * nz) { t = itesc + kk % nto; z = kk / nto; }
        }
        if (t < 0) continue;
        kmap[k] = (t + nt * z) | ((t < itesc) ? KMAP_YOUNG : 0);
        put(k, b.data() + (size_t)ns * (t + (size_t)nt * z), ns);
    }
    // (the library's own spectra at the ionizing pixels: the lines lie above 912 A, and b has these pixels zeroed)
    const int jion = std::min(c.whlylim, ns);
    for (int kk = 0; kk < op->kion_y + op->kion_o; ++kk) {
        int t = -1, z = -1;
        if (kk < op->kion_y) {
            if (kk < ty_end * nz) { t = kk % ty_end; z = kk / ty_end; }
        } else {
            const int j = kk - op->kion_y;
            if (j < n_ion_old * nz) { t = ty_end + j % n_ion_old; z = j / n_ion_old; }
        }
        if (t < 0) continue;
        const int k = op->kmain + kk;
        kmap[k] = (t + nt * z) | ((t < itesc) ? KMAP_YOUNG : 0) | KMAP_ION;
        put(k, c.ssp.data() + (size_t)ns * (t + (size_t)nt * z), jion);
    }
    cudaError_t e;
    if ((e = op->hi.reserve(hi.size())) != cudaSuccess || (e = op->lo.reserve(lo.size())) != cudaSuccess ||
        (e = cudaMemcpy(op->hi.p, hi.data(), hi.size() * 2, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(op->lo.p, lo.data(), lo.size() * 2, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = op->kmap.reserve(kpad)) != cudaSuccess ||
        (e = cudaMemcpy(op->kmap.p, kmap.data(), sizeof(int) * kpad, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = encode_tmap_2d_bf16(&op->tm_hi, op->hi.p, kpad, ns, BK, contract_bm())) != cudaSuccess ||
        (e = encode_tmap_2d_bf16(&op->tm_lo, op->lo.p, kpad, ns, BK, contract_bm())) != cudaSuccess) {
        err = std::string("basis operand: ") + cudaGetErrorString(e);
        op->hi.release(); op->lo.release(); op->kmap.release();
        delete op;
        return nullptr;
    }
    c.basis_cache[key] = op;
    return op;
}

// ---------------------------------------------------------------------------------------------- the batch
// Profiling marks: with profiling on, event k is recorded on the stream after stage k (0 = before the first kernel),
// so that the kernels' device times can be read back after the batch (opensps_gb300_kernel_times).
// Two event sets alternate between batches; a set is read back (and its times added to the running sums) when it
// is about to be reused, so that up to two profiled batches can be in flight.
void prof_harvest(Context &c, int s) {
    if (!c.prof_pending[s]) return;
    cudaEventSynchronize(c.prof_ev[s][c.prof_used[s] - 1]);
    for (int i = 1; i < c.prof_used[s]; ++i) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, c.prof_ev[s][i - 1], c.prof_ev[s][i]) == cudaSuccess) c.prof_acc[i - 1] += t;
    }
    c.prof_nstage = std::max(c.prof_nstage, c.prof_used[s] - 1);
    c.prof_count += 1;
    c.prof_pending[s] = false;
}

void prof_mark(Context &c, int k) {
    if (!c.profile || k >= Context::NPROF) return;
    if (k == 0) {
        c.prof_set ^= 1;
        prof_harvest(c, c.prof_set);
    }
    const int s = c.prof_set;
    if (!c.prof_ev[s][k]) cudaEventCreate(&c.prof_ev[s][k]);
    cudaEventRecord(c.prof_ev[s][k], c.stream);
    c.prof_used[s] = k + 1;
    c.prof_pending[s] = k > 0;
}

static std::string cuda_msg(const char *what, cudaError_t e) { return std::string(what) + ": " + cudaGetErrorString(e); }

int run_batch(Context &c, const BatchIO &io, std::string &err) {
    const int n = io.n, ns = c.nspec, nt = c.nt, nz = c.nz, nb = c.nbands;
    if (n <= 0) return 0;
    const double *P = io.params;   // params_cols x n
    const int pc = io.params_cols;
    auto par = [&](int m, int id) { return id < pc ? P[(size_t)pc * m + id] : io.param_defaults[id]; };

    // host weights over ages and metallicities on the mixed path go up in chunks on the side stream, each chunk's
    // kernels running while the next chunk's weights are copied. The first chunk's copy starts here, under the
    // host's checks and parameter staging; the parameter table follows it on the same stream, then the other chunks
    // (the first kernels need the table)
    constexpr int CHUNK = 16384;
    // dust emission (add_dust_emission, for models with dust1 or dust2 above SAFE_FLOOR: batch_model_indices
    // :1569-1570): the per-model epilogue forms it from the young and old sums
    bool any_emis = false, any_agn = false;
    if (c.add_dust_emission == 1)
        for (int m = 0; m < n && !any_emis; ++m)
            any_emis = par(m, PF_DUST1) > SAFE_FLOOR || par(m, PF_DUST2) > SAFE_FLOOR || c.dust_type == 3;
    // the AGN torus (add_agn_dust, for models with fagn above SAFE_FLOOR: agn_indices :1575-1589), in the same epilogue
    if (c.add_agn_dust == 1)
        for (int m = 0; m < n && !any_agn; ++m) any_agn = par(m, PF_FAGN) > SAFE_FLOOR;
    // nebular emission's escaping ionizing light (frac_obrun above zero: nebular_kernels step 2,
    // opensps_csp_batch.f90:2726-2750, the basis holding the absorbed case): extra K blocks of the contraction
    bool ion_terms = false;
    if (c.add_neb_emission == 1 && c.nebemlineinspec == 1 && c.nline > 0 && c.nt_neb > 0 && c.whlylim > 0)
        for (int m = 0; m < n && !ion_terms; ++m) ion_terms = par(m, PF_FRAC_OBRUN) > 0.0;
    // the CLOUDY-grid nebular continuum (nb%cont = neb .and. add_neb_continuum, :1646; nebular_kernels step 3): in the
    // per-model epilogue, when the data root has the grid of the setup's isochrones (nebular/<isoc>_<nodust|dust>)
    const int neb_table = c.cloudy_dust == 1 ? 1 : 0;
    const bool neb_cont = c.add_neb_emission == 1 && c.add_neb_continuum == 1 && c.nt_neb > 0 &&
                          (c.neb.have[0] || c.neb.have[1]);
    if (neb_cont && !c.neb.have[neb_table]) {
        err = "nebular/" + c.isoc + (neb_table ? "_dust" : "_nodust") + " is missing (cloudy_dust = " +
              std::to_string(c.cloudy_dust) + ")";
        return ST_DATA_MISSING;
    }
    if (neb_cont && c.nt_neb > NEB_MAX_AGES) {
        err = "the nebular continuum takes at most " + std::to_string(NEB_MAX_AGES) + " nebular ages";
        return ST_UNSUPPORTED;
    }
    const bool epi_terms = any_emis || any_agn || neb_cont;
    const bool epi = epi_terms;                      // spectra from the per-model epilogue
    const bool parts_kept = ((io.young || io.old) && !io.dev_inputs) || io.keep_parts;   // the caller wants the parts
    const bool parts = parts_kept || epi;
    const bool chunked = !io.dev_inputs && !io.sfh_par && io.wz && c.fp64 == 0 && !c.ops.ready && !parts_kept &&
                         n >= 2 * CHUNK;
    // chunk k's models (a smaller first chunk, to start the kernels earlier, measured slower: the kernels lose
    // more on the small chunk than its shorter copy saves)
    const int nch = chunked ? (n + CHUNK - 1) / CHUNK : 1;
    auto chunk_off = [&](int k) { return k * CHUNK; };
    auto chunk_len = [&](int k) { return std::min(CHUNK, n - k * CHUNK); };
    // pageable host weights on a device that reads pageable memory (Grace's address translation over NVLink-C2C):
    // the operand kernel reads each chunk in place (the link's rate, against about a fifth of it for a copy from
    // pageable memory); page-locked weights still go up by copies, which overlap the kernels on the copy engine
    bool direct = false;
    if (chunked) {
        if (c.pageable_access < 0) {
            int dev = 0, v = 0;
            c.pageable_access = (cudaGetDevice(&dev) == cudaSuccess &&
                                 cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess && v == 1) ? 1 : 0;
        }
        cudaPointerAttributes pa;
        if (c.pageable_access == 1 && cudaPointerGetAttributes(&pa, io.wz) == cudaSuccess &&
            pa.type == cudaMemoryTypeUnregistered)
            direct = true;
        cudaGetLastError();
    }
    c.last_direct = direct;
    auto chunk_copy = [&](int k) -> cudaError_t {
        const int off = chunk_off(k), nk = chunk_len(k);
        cudaEvent_t &ev = c.chunk_ev[k % Context::NCHUNK_EV];
        cudaError_t r = cudaSuccess;
        if (!ev) r = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (r == cudaSuccess)
            r = cudaMemcpyAsync(c.d_wz.p + (size_t)nt * nz * off, io.wz + (size_t)nt * nz * off,
                                sizeof(double) * nt * nz * nk, cudaMemcpyHostToDevice, c.side);
        if (r == cudaSuccess) r = cudaEventRecord(ev, c.side);
        return r;
    };
    // the band mask on the device (when it changed; before any weight copy, which would queue it)
    if (nb > 0) {
        std::vector<int> do_band(nb, 1);
        for (int b = 0; b < nb && b < (int)c.mag_mask.size(); ++b) do_band[b] = c.mag_mask[b];
        if (do_band != c.do_band_h || !c.d_do_band.p) {
            cudaError_t e1 = c.d_do_band.reserve(nb);
            if (e1 == cudaSuccess)
                e1 = cudaMemcpyAsync(c.d_do_band.p, do_band.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, c.stream);
            if (e1 == cudaSuccess) e1 = cudaStreamSynchronize(c.stream);
            if (e1 != cudaSuccess) { err = cuda_msg("band mask", e1); return ST_DATA_MISSING; }
            c.do_band_h = do_band;
        }
    }
    if (chunked && !direct) {
        cudaError_t e0 = c.d_wz.reserve((size_t)n * nt * nz);
        if (e0 == cudaSuccess) e0 = chunk_copy(0);
        if (e0 != cudaSuccess) { err = cuda_msg("weights copy", e0); return ST_DATA_MISSING; }
    }

    // ---- checks shared by the batch (the reference's batch_check_models / plan_smoothing rules)
    if (!dust_type_supported(c.dust_type)) {
        err = "dust_type " + std::to_string(c.dust_type) + ": the types are 0 to 6";
        return ST_UNSUPPORTED;
    }
    if (c.dust_type == 3 && (c.wgp[0] < 1 || c.wgp[0] > WG_NTAU || c.wgp[1] < 1 || c.wgp[1] > WG_NMODEL || c.wgp[2] < 1 ||
                             c.wgp[2] > WG_NSTRUCT)) {
        err = "dust_type 3: wgp1 (1-18), wgp2 (1-6) and wgp3 (1-2) select the curve";
        return ST_BAD_ARG;
    }
    if (c.dust_type == 3 || c.dust_type == 5)
        if (int rc = attenuation_load(c, err)) return rc;
    if (c.compute_vega_mags != 0) { err = "compute_vega_mags = 1 is not supported on this path"; return ST_UNSUPPORTED; }
    if (c.smooth_velocity != 1) { err = "smooth_velocity = 0 is not supported on this path"; return ST_UNSUPPORTED; }
    const double minl = par(0, PF_MIN_WAVE_SMOOTH), maxl = par(0, PF_MAX_WAVE_SMOOTH);
    int itesc = -1;
    bool nacc2 = false, any_smooth = false;
    double last_tesc = std::nan("");
    for (int m = 0; m < n; ++m) {
        const double tesc = par(m, PF_DUST_TESC);
        if (!(tesc == last_tesc)) {        // the age search once per distinct dust_tesc
            last_tesc = tesc;
            const double dla = tesc > SAFE_FLOOR ? tesc : 7.0;
            int it = find_interval0(c.log_age.data(), nt, dla) + 1;
            it = std::max(1, std::min(it, nt));
            if (itesc < 0) itesc = it;
            else if (it != itesc) { err = "dust_tesc must select the same age for every model of a batch on this path"; return ST_UNSUPPORTED; }
        }
        if (par(m, PF_MIN_WAVE_SMOOTH) != minl || par(m, PF_MAX_WAVE_SMOOTH) != maxl) {
            err = "models must share min_wave_smooth and max_wave_smooth";
            return ST_UNSUPPORTED;
        }
        const double d1 = par(m, PF_DUST1), fo = par(m, PF_FRAC_OBRUN), d3 = par(m, PF_DUST3);
        if ((d1 > SAFE_FLOOR && 1.0 - fo > SAFE_FLOOR) || std::fabs(d3) > SAFE_FLOOR) nacc2 = true;
        if (io.young || io.old || io.keep_parts || epi) nacc2 = true;   // the parts need the young and old sums apart
        const double sig = par(m, PF_SIGMA_SMOOTH);
        if (sig > SAFE_FLOOR) {
            any_smooth = true;
            const double x = 4.0 * (sig / (C_LIGHT * 1.0e-13)) / c.dlnl;
            if (x > 4.0 - 1e-9) {
                err = "sigma_smooth above ~350 km/s (a window wider than +-4 pixels) is not supported on this path";
                return ST_UNSUPPORTED;
            }
        }
    }
    // smoothing rows must keep their whole window inside the grid
    int i0 = -1;
    if (any_smooth) {
        for (int j = 0; j < ns; ++j)
            if (c.lam[j] >= minl && c.lam[j] <= maxl) { i0 = j; break; }
        if (i0 >= 0 && (minl <= c.lam[contract_halo()] || maxl >= c.lam[ns - 1 - contract_halo()])) {
            err = "the smoothing range must lie inside the wavelength grid's interior";
            return ST_UNSUPPORTED;
        }
    }
    // nebular lines: one profile table per batch, from the first model's sigma (prepare_line_gaussians(ctx,
    // psets(1)), src/physics/opensps_csp_batch.f90:1733); a model whose own sigma would give other widths is
    // unsupported, as in the reference (:747-751)
    const bool neb = c.add_neb_emission == 1 && c.nebemlineinspec == 1 && c.nline > 0;
    double line_sigma = 0.0;
    if (neb) {
        const double s1 = par(0, PF_SIGMA_SMOOTH);
        const bool f1 = lines_floor_limited(c, s1);
        line_sigma = f1 ? 0.0 : s1;
        // below 0.999 of the smallest line's threshold every line is at the floor (no per-line test needed)
        double thr = 1e300;
        for (int l = 0; l < c.nline; ++l) {
            const double pos = c.line_lambda[l];
            int j = find_interval0(c.lam.data(), c.nspec, pos) + 1;
            j = std::max(1, std::min(j, c.nspec - 1));
            thr = std::min(thr, 2.0 * (c.lam[j] - c.lam[j - 1]) / (pos * (1.0e13 / C_LIGHT)));
        }
        for (int m = 1; m < n; ++m) {
            const double sm = par(m, PF_SIGMA_SMOOTH);
            if (sm == s1) continue;
            if (f1 && sm < 0.999 * thr) continue;
            if (!(f1 && lines_floor_limited(c, sm))) {
                err = "nebular lines with a sigma_smooth of each model's own (above the grid's line width) are unsupported";
                return ST_UNSUPPORTED;
            }
        }
    }
    // with SSP operators on the context (opensps_context_build_ssp_ops) the age sums come from the operator applied
    // to each model's IMF; else from the resident basis, whose IMF is fixed
    const bool ops = c.ops.ready;
    const bool fp64 = c.fp64 != 0 && !ops;
    if (fp64 && (io.dev_inputs || io.keep_parts || io.young || io.old)) {
        err = "the plain FP64 path computes host-input batches' outputs only (no parts, device inputs or gradients)";
        return ST_UNSUPPORTED;
    }
    if (ion_terms && c.fp64 != 0) {
        err = "nebular emission with frac_obrun above zero is supported by the mixed batch only";
        return ST_UNSUPPORTED;
    }
    c.last_ion = ion_terms;
    DustEmModel *dem = nullptr;            // the per-model cells, page-locked (uploaded beside the parameter table)
    std::vector<int2> neb_chunk_groups;    // the nebular continuum: per chunk its first group and group count
    if (epi_terms) {
        if (fp64) { err = "dust emission, AGN and the nebular continuum are not supported on the plain FP64 path"; return ST_UNSUPPORTED; }
        if (io.dev_inputs) { err = "dust emission, AGN and the nebular continuum need host inputs on this path"; return ST_UNSUPPORTED; }
        if (neb_cont && c.ops.ready) { err = "the nebular continuum with the SSP operators is not supported on this path"; return ST_UNSUPPORTED; }
        if (any_emis) { if (int rc = dustem_load(c, err)) return rc; }
        if (any_agn) { if (int rc = agn_load(c, err)) return rc; }
        // dl07_indices (src/physics/opensps_csp_batch.f90:1622-1634): the grid cell in q_PAH and U_min (clamped to
        // the grid) and the weights, clamped to [0, 1]; gamma clamped to [0, 1]
        const DustEmission &d = c.dustem;
        auto cell = [](const std::vector<double> &g, double x, int &i, float &w) {
            int k = (int)(std::upper_bound(g.begin(), g.end(), x) - g.begin());   // entries <= x (find_interval)
            k = std::max(1, std::min(k, (int)g.size() - 1));
            i = k - 1;
            w = (float)std::max(0.0, std::min((x - g[i]) / (g[i + 1] - g[i]), 1.0));
        };
        if (c.pinned_dem_n < (size_t)n) {
            if (c.pinned_dem) cudaFreeHost(c.pinned_dem);
            c.pinned_dem = nullptr;
            c.pinned_dem_n = 0;
            if (cudaMallocHost(&c.pinned_dem, sizeof(DustEmModel) * n) != cudaSuccess) {
                cudaGetLastError();
                err = "page-locked dust emission inputs: out of memory";
                return ST_DATA_MISSING;
            }
            c.pinned_dem_n = (size_t)n;
        }
        dem = c.pinned_dem;
        if (io.keep_parts) c.h_dchain.assign((size_t)n, make_float4(0.f, 0.f, 0.f, 0.f));
        for (int m = 0; m < n; ++m) {
            DustEmModel &q = dem[m];
            q = DustEmModel{};
            q.on = (any_emis && (par(m, PF_DUST1) > SAFE_FLOOR || par(m, PF_DUST2) > SAFE_FLOOR || c.dust_type == 3)) ? 1 : 0;
            if (q.on) {
                cell(d.qpah, par(m, PF_DUSTE_QPAH), q.iq, q.wq);
                cell(d.umin, par(m, PF_DUSTE_UMIN), q.iu, q.wu);
                q.gam = (float)std::max(0.0, std::min(par(m, PF_DUSTE_GAMMA), 1.0));
            }
            q.agn = (any_agn && par(m, PF_FAGN) > SAFE_FLOOR) ? 1 : 0;
            if (q.agn) {
                cell(c.agn.tau, par(m, PF_AGN_TAU), q.ita, q.wta);
                q.fagn = (float)par(m, PF_FAGN);
            }
            if (io.keep_parts) {
                // the reverse pass's chain factors (batch_chain_derivatives, opensps_csp_batch.f90:4701-4706; agn_tau_slope
                // :1598-1608): 1 / the cell's width where the parameter lies in the cell (its ends included), gamma within
                // [0, 1]; agn_tau within [tau_1, tau_n)
                float4 dc = make_float4(0.f, 0.f, 0.f, 0.f);
                if (q.on) {
                    const double xq = par(m, PF_DUSTE_QPAH), xu = par(m, PF_DUSTE_UMIN), xg = par(m, PF_DUSTE_GAMMA);
                    if (xq >= d.qpah[q.iq] && xq <= d.qpah[q.iq + 1]) dc.x = (float)(1.0 / (d.qpah[q.iq + 1] - d.qpah[q.iq]));
                    if (xu >= d.umin[q.iu] && xu <= d.umin[q.iu + 1]) dc.y = (float)(1.0 / (d.umin[q.iu + 1] - d.umin[q.iu]));
                    if (xg >= 0.0 && xg <= 1.0) dc.z = 1.f;
                }
                if (q.agn) {
                    const std::vector<double> &ta = c.agn.tau;
                    const double xt = par(m, PF_AGN_TAU);
                    if (ta.size() >= 2 && xt >= ta.front() && xt < ta.back())
                        dc.w = (float)(1.0 / (ta[q.ita + 1] - ta[q.ita]));
                }
                c.h_dchain[m] = dc;
            }
            if (neb_cont) {
                // get_grid_indices_weights (opensps_gas.f90:394-412) in gas_logz and gas_logu; fabs = 1 - frac_obrun
                // (:1697), its magnitude as the continuum's q = |q0 fabs| takes it (:2795)
                cell(c.neb.logz, par(m, PF_GAS_LOGZ), q.neb_iz, q.neb_wz);
                cell(c.neb.logu, par(m, PF_GAS_LOGU), q.neb_iu, q.neb_wu);
                q.neb_fabs = (float)std::fabs(1.0 - par(m, PF_FRAC_OBRUN));
                // the reverse pass's chain factors (batch_chain_derivatives :4686-4697: inside the cell, its
                // inverse width; zero where the weight is clamped) and d|1 - fo| / dfo
                auto chain = [](const std::vector<double> &g, double x, int i) {
                    return (x >= g[i] && x <= g[i + 1]) ? (float)(1.0 / (g[i + 1] - g[i])) : 0.f;
                };
                q.neb_dz = chain(c.neb.logz, par(m, PF_GAS_LOGZ), q.neb_iz);
                q.neb_du = chain(c.neb.logu, par(m, PF_GAS_LOGU), q.neb_iu);
                const double om = 1.0 - par(m, PF_FRAC_OBRUN);
                q.neb_dfo = om > 0.0 ? -1.f : (om < 0.0 ? 1.f : 0.f);
            }
        }
        if (neb_cont) {
            if (int rc = nebular_runs(c, itesc, err)) return rc;
            // per chunk, its models with a continuum sorted by their (gas_logz, gas_logu) cell (chunk-relative
            // indices) and cut into groups of at most NEB_GROUP (cell z, cell u, first index into the order, count)
            c.neb.h_order.clear();
            c.neb.h_groups.clear();
            const int ncell = (NEB_NZ - 1) * (NEB_NU - 1);
            std::vector<int> cnt(ncell + 1);
            for (int k = 0; k < nch; ++k) {
                const int off = chunk_off(k), nk = chunk_len(k);
                std::fill(cnt.begin(), cnt.end(), 0);
                for (int i = 0; i < nk; ++i) {
                    const DustEmModel &q = dem[off + i];
                    if (q.neb_fabs > 0.f) ++cnt[q.neb_iz * (NEB_NU - 1) + q.neb_iu + 1];
                }
                for (int cc = 0; cc < ncell; ++cc) cnt[cc + 1] += cnt[cc];
                const size_t base = c.neb.h_order.size();
                c.neb.h_order.resize(base + (size_t)cnt[ncell]);
                std::vector<int> pos(cnt.begin(), cnt.end() - 1);
                for (int i = 0; i < nk; ++i) {
                    const DustEmModel &q = dem[off + i];
                    if (q.neb_fabs > 0.f) c.neb.h_order[base + pos[q.neb_iz * (NEB_NU - 1) + q.neb_iu]++] = i;
                }
                const int g0 = (int)c.neb.h_groups.size();
                for (int cc = 0; cc < ncell; ++cc)
                    for (int j = cnt[cc]; j < cnt[cc + 1]; j += NEB_GROUP)
                        c.neb.h_groups.push_back(make_int4(cc / (NEB_NU - 1), cc % (NEB_NU - 1), (int)base + j,
                                                           std::min(NEB_GROUP, cnt[cc + 1] - j)));
                neb_chunk_groups.push_back(make_int2(g0, (int)c.neb.h_groups.size() - g0));
            }
        }
    }
    if (ops) {
        if (neb) { err = "nebular emission with the SSP operators is not supported on this path"; return ST_UNSUPPORTED; }
        if (c.imf_type < 0 || c.imf_type > 5) {
            err = "imf_type " + std::to_string(c.imf_type) + ": the IMF types are 0 to 5";
            return ST_UNSUPPORTED;
        }
        if (!(c.imf_lim_lo > 0.0 && c.imf_lim_hi > c.imf_lim_lo)) {
            err = "the IMF's mass limits must satisfy 0 < imf_lower_limit < imf_upper_limit";
            return ST_BAD_ARG;
        }
        nacc2 = true;
    } else {
        if (c.imf_lim_lo != 0.08 || c.imf_lim_hi != 120.0) {
            err = "IMF mass limits other than 0.08 - 120 M_sun need the SSP operators (opensps_context_build_ssp_ops)";
            return ST_UNSUPPORTED;
        }
        for (int m = 0; m < n; ++m)
            for (int id : {PF_IMF1, PF_IMF2, PF_IMF3, PF_VDMC, PF_MDAVE})
                if (par(m, id) != c.pdef[id]) {
                    err = "an IMF per model needs the SSP operators (opensps_context_build_ssp_ops)";
                    return ST_UNSUPPORTED;
                }
    }
    const int nacc = nacc2 ? 2 : 1;
    BasisOperand *bop = nullptr;
    if (!ops) {
        bop = get_basis(c, nacc, itesc, neb, line_sigma, ion_terms, err);
        if (!bop) return ST_DATA_MISSING;
    }

    // ---- per-pixel table (rebuilt when the batch's shared curve changes): ln(lambda / 5500) log2(e), the diffuse
    // curve shared by the batch's models in FP64 (the reference's tables, attenuation_tables_cached :3494-3560, times
    // exp_kp of the power law: the argument formed in FP64), the Madau wavelength factors, the curve tables T0..T3
    // (FP32: the kernels form a model's own curve from them when the models' curves differ)
    double sc0[4];
    dust_scalars(c.dust_type, par(0, PF_DUST_INDEX), par(0, PF_MWR), par(0, PF_UVB), sc0);
    bool uniform_index = true;
    for (int m = 1; m < n && uniform_index; ++m) {
        double sc[4];
        dust_scalars(c.dust_type, par(m, PF_DUST_INDEX), par(m, PF_MWR), par(m, PF_UVB), sc);
        uniform_index = sc[0] == sc0[0] && sc[1] == sc0[1] && sc[2] == sc0[2] && sc[3] == sc0[3];
    }
    if (c.dust_type != 0 && fp64) {
        err = "dust_type " + std::to_string(c.dust_type) + " is not supported on the plain FP64 path";
        return ST_UNSUPPORTED;
    }
    // (the dusty environments' curve: structure wgp3, tau_v wgp1, model wgp2)
    const double *lookup = c.dust_type == 5 ? c.att_smc.data()
                         : (c.dust_type == 3 ? c.att_wg.data() + (size_t)ns * (((c.wgp[2] - 1) * WG_NTAU + (c.wgp[0] - 1)) *
                                                                              WG_NMODEL + (c.wgp[1] - 1))
                                             : nullptr);
    const double key[6] = {(double)c.dust_type, sc0[0], sc0[1], sc0[2], sc0[3],
                           c.dust_type == 3 ? (double)(c.wgp[0] + 100 * c.wgp[1] + 10000 * c.wgp[2]) : 0.0};
    bool same_key = true;
    for (int k = 0; k < 6; ++k) same_key = same_key && c.pix_key[k] == key[k];
    if (!c.d_pix.p || c.pix_key[0] != key[0] || c.pix_key[5] != key[5] || (uniform_index && !same_key)) {
        std::vector<double> tab;
        dust_tables(c.dust_type, c.lam, lookup, tab);
        std::vector<float> pix((size_t)ns * PIX_FLOATS, 0.f);
        for (int j = 0; j < ns; ++j) {
            float *px = pix.data() + (size_t)j * PIX_FLOATS;
            const double ltab = std::log(c.lam[j] / 5500.0);
            px[PIX_LTAB2] = (float)(ltab * 1.4426950408889634);
            px[PIX_CURVE] = (float)dust_curve_value(tab.data() + 4 * (size_t)j, sc0, ltab);
            if (j < c.jtop)
                for (int k = 0; k < 6; ++k) px[PIX_IGM_A + k] = c.igm_a[(size_t)j * 6 + k];
            for (int k = 0; k < 4; ++k) px[PIX_T + k] = (float)tab[4 * (size_t)j + k];
        }
        cudaError_t e;
        if ((e = c.d_pix.reserve(pix.size())) != cudaSuccess ||
            (e = cudaMemcpy(c.d_pix.p, pix.data(), sizeof(float) * pix.size(), cudaMemcpyHostToDevice)) != cudaSuccess) {
            err = cuda_msg("pixel table", e);
            return ST_DATA_MISSING;
        }
        for (int k = 0; k < 6; ++k) c.pix_key[k] = key[k];
    }
    const int tab_curve = c.dust_type != 0 ? 1 : 0;   // (models' own curves from the tables, else the power law)
    // the smoothed pixels: lambda within [min_wave_smooth, max_wave_smooth]
    int sm_lo = ns, sm_hi = -1;
    for (int j = 0; j < ns; ++j)
        if (c.lam[j] >= minl && c.lam[j] <= maxl) { sm_lo = std::min(sm_lo, j); sm_hi = std::max(sm_hi, j); }

    c.geom.bop = bop;
    c.geom.nacc = nacc;
    c.geom.sm_lo = any_smooth ? sm_lo : ns;
    c.geom.sm_hi = any_smooth ? sm_hi : -1;
    c.geom.uniform_index = uniform_index ? 1 : 0;
    c.geom.tab_curve = tab_curve;
    c.geom.itesc = itesc;
    c.geom.wz = nullptr;
    c.geom.n = 0;
    c.geom.emis = epi_terms && any_emis;
    c.geom.agn = epi_terms && any_agn;
    c.geom.neb = neb_cont;
    c.geom.neb_table = neb_table;

    // ---- scratch
    const int bn = contract_models_per_tile(nacc);
    const int n_mtiles = (n + bn - 1) / bn;
    const int kpad = ops ? 64 : bop->kpad;
    cudaError_t e;
    const size_t nwz = (size_t)n * nt * nz;
    if ((!io.dev_inputs && (e = c.d_wz.reserve(nwz)) != cudaSuccess) ||
        (e = c.d_params.reserve((size_t)PAR_DEVICE * n)) != cudaSuccess ||
        (e = c.d_whi.reserve((size_t)n * kpad)) != cudaSuccess || (e = c.d_wlo.reserve((size_t)n * kpad)) != cudaSuccess ||
        (e = c.d_sums.reserve((size_t)6 * n)) != cudaSuccess || (e = c.d_mpar.reserve((size_t)MODEL_PAR_FLOATS * n)) != cudaSuccess ||
        (e = c.d_zinfo.reserve((size_t)n)) != cudaSuccess || (e = c.d_dist.reserve(n)) != cudaSuccess ||
        (e = c.d_spec.reserve((size_t)n * ns)) != cudaSuccess || (e = c.d_mags.reserve((size_t)n * nb)) != cudaSuccess) {
        err = cuda_msg("device memory", e);
        return ST_DATA_MISSING;
    }
    cudaStream_t st = c.stream;
    const double *d_wz = io.wz;
    const double *d_par = nullptr;
    std::vector<double> hp;
    if (io.dev_inputs) {
        d_par = io.dev_params;   // already PAR_DEVICE x n on the device
    } else if (io.sfh_par) {
        // the weights over ages (the SFH's, or the caller's) and their blend at logzsol, formed on the device
        if ((e = c.d_sfhpar.reserve((size_t)SFH_NCOL * n)) != cudaSuccess || (e = c.d_w.reserve((size_t)nt * n)) != cudaSuccess ||
            (e = c.d_sfh_scratch.reserve((size_t)2 * nt * n)) != cudaSuccess ||
            (e = c.d_sfh_mtab.reserve((size_t)nt * n)) != cudaSuccess ||
            (e = c.d_lblend.reserve((size_t)3 * n)) != cudaSuccess || (e = c.d_sfr.reserve(n)) != cudaSuccess ||
            (io.given_w && (e = c.d_wgiven.reserve((size_t)nt * n)) != cudaSuccess) ||
            (e = cudaMemcpyAsync(c.d_sfhpar.p, io.sfh_par, sizeof(double) * SFH_NCOL * n, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
            (io.given_w && (e = cudaMemcpyAsync(c.d_wgiven.p, io.given_w, sizeof(double) * nt * n, cudaMemcpyHostToDevice, st)) != cudaSuccess)) {
            err = cuda_msg("SFH inputs", e);
            return ST_DATA_MISSING;
        }
        SfhArgs sa;
        sa.n = n; sa.nt = nt; sa.nz = nz; sa.sfh = io.sfh_type; sa.itesc = itesc;
        sa.tf = c.d_logage.p; sa.lz = c.d_lz.p; sa.lbol = c.d_lbol.p; sa.par = c.d_sfhpar.p;
        sa.given = io.given_w ? c.d_wgiven.p : nullptr;
        sa.w = c.d_w.p; sa.scratch = c.d_sfh_scratch.p; sa.wz = c.d_wz.p; sa.lblend = c.d_lblend.p; sa.sfr = c.d_sfr.p;
        sa.mtab = c.d_sfh_mtab.p;
        if ((io.sfh_type == 2 || io.sfh_type == 3) && !io.given_w) {
            // the tabular SFH: ages then SFRs, each with its zero entry past the table
            const size_t nt1 = (size_t)c.ntab + 1;
            if (c.sfh_tab_dirty || c.d_sfhtab.n < 2 * nt1) {
                if ((e = c.d_sfhtab.reserve(2 * nt1)) != cudaSuccess ||
                    (e = cudaMemcpyAsync(c.d_sfhtab.p, c.sfh_tab_t.data(), sizeof(double) * nt1, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
                    (e = cudaMemcpyAsync(c.d_sfhtab.p + nt1, c.sfh_tab_sfr.data(), sizeof(double) * nt1, cudaMemcpyHostToDevice, st)) != cudaSuccess) {
                    err = cuda_msg("tabular SFH copy", e);
                    return ST_DATA_MISSING;
                }
                c.sfh_tab_dirty = false;
            }
            sa.ntab = c.ntab;
            sa.tab = c.d_sfhtab.p;
        }
        if ((e = run_sfh_forward(sa, st)) != cudaSuccess) { err = cuda_msg("SFH weights kernel", e); return ST_DATA_MISSING; }
        d_wz = c.d_wz.p;
    } else {
        if (!chunked && (e = cudaMemcpyAsync(c.d_wz.p, io.wz, sizeof(double) * nwz, cudaMemcpyHostToDevice, st)) != cudaSuccess) {
            err = cuda_msg("weights copy", e);
            return ST_DATA_MISSING;
        }
        d_wz = direct ? io.wz : c.d_wz.p;
    }
    if (!io.dev_inputs) {
        // the device table from the parameter rows, through a page-locked staging buffer
        const size_t np = (size_t)PAR_DEVICE * n;
        if (c.pinned_par_n < np) {
            if (c.pinned_par) cudaFreeHost(c.pinned_par);
            c.pinned_par = nullptr;
            c.pinned_par_n = 0;
            if ((e = cudaMallocHost(&c.pinned_par, sizeof(double) * np)) != cudaSuccess) {
                err = cuda_msg("page-locked parameters", e);
                return ST_DATA_MISSING;
            }
            c.pinned_par_n = np;
        }
        double *hpp = c.pinned_par;
#pragma omp parallel for schedule(static) if (n >= 8192)
        for (int m = 0; m < n; ++m)
            for (int k = 0; k < PAR_DEVICE; ++k) hpp[(size_t)PAR_DEVICE * m + k] = par(m, k);
        // (with the weights in chunks the table goes up on the side stream between the first chunk and the others:
        // a copy on the batch's stream was served only after all the side stream's copies)
        cudaStream_t cs = chunked ? c.side : st;
        if ((e = cudaMemcpyAsync(c.d_params.p, hpp, sizeof(double) * np, cudaMemcpyHostToDevice, cs)) != cudaSuccess) {
            err = cuda_msg("parameter copy", e);
            return ST_DATA_MISSING;
        }
        if (neb_cont && ((e = c.neb.order.reserve(std::max<size_t>(c.neb.h_order.size(), 1))) != cudaSuccess ||
                         (e = c.neb.groups.reserve(std::max<size_t>(c.neb.h_groups.size(), 1))) != cudaSuccess ||
                         (!c.neb.h_order.empty() &&
                          (e = cudaMemcpyAsync(c.neb.order.p, c.neb.h_order.data(), sizeof(int) * c.neb.h_order.size(),
                                               cudaMemcpyHostToDevice, cs)) != cudaSuccess) ||
                         (!c.neb.h_groups.empty() &&
                          (e = cudaMemcpyAsync(c.neb.groups.p, c.neb.h_groups.data(), sizeof(int4) * c.neb.h_groups.size(),
                                               cudaMemcpyHostToDevice, cs)) != cudaSuccess))) {
            err = cuda_msg("nebular continuum groups", e);
            return ST_DATA_MISSING;
        }
        if (dem && ((e = c.d_dem.reserve(n)) != cudaSuccess ||
                    (e = cudaMemcpyAsync(c.d_dem.p, dem, sizeof(DustEmModel) * n, cudaMemcpyHostToDevice, cs)) != cudaSuccess)) {
            err = cuda_msg("dust emission inputs", e);
            return ST_DATA_MISSING;
        }
        if (dem && io.keep_parts &&
            ((e = c.d_dchain.reserve(n)) != cudaSuccess ||
             (e = cudaMemcpyAsync(c.d_dchain.p, c.h_dchain.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, cs)) != cudaSuccess)) {
            err = cuda_msg("dust emission chain factors", e);
            return ST_DATA_MISSING;
        }
        if (chunked) {
            if ((!c.par_ev && (e = cudaEventCreateWithFlags(&c.par_ev, cudaEventDisableTiming)) != cudaSuccess) ||
                (e = cudaEventRecord(c.par_ev, c.side)) != cudaSuccess || (e = cudaStreamWaitEvent(st, c.par_ev, 0)) != cudaSuccess) {
                err = cuda_msg("parameter copy", e);
                return ST_DATA_MISSING;
            }
        }
        d_par = c.d_params.p;
    }
    if (chunked && !direct)
        for (int k = 1; k < nch; ++k)
            if ((e = chunk_copy(k)) != cudaSuccess) { err = cuda_msg("weights copy", e); return ST_DATA_MISSING; }
    cudaMemsetAsync(c.d_status.p, 0, sizeof(int), st);

    // ---- the per-model parameters, then the weight operand (one stream: run side by side they took longer than in
    // turn)
    prof_mark(c, 0);
    const int smem_mp = (c.add_igm_absorption == 1 ? c.jtop : 0) * 6 * (int)sizeof(float);
    if (smem_mp > 48 * 1024 &&
        (e = cudaFuncSetAttribute(model_params_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_mp)) != cudaSuccess) {
        err = cuda_msg("model parameter kernel", e);
        return ST_DATA_MISSING;
    }
    // per-model parameters of models [off, off + nk)
    auto model_params = [&](int off, int nk) -> cudaError_t {
        ModelParamArgs ma;
        ma.n = nk; ma.nspec = ns; ma.jtop = c.jtop; ma.add_igm = c.add_igm_absorption == 1; ma.smooth = any_smooth ? 1 : 0;
        ma.i0 = i0; ma.dust_type = c.dust_type; ma.par = d_par + (size_t)PAR_DEVICE * off; ma.igm_a = c.d_igm_a.p; ma.lam = c.d_lam.p;
        ma.zt = c.d_zt.p; ma.dl = c.d_dl.p; ma.dlnl = c.dlnl; ma.mpar = c.d_mpar.p + (size_t)MODEL_PAR_FLOATS * off;
        ma.zinfo = c.d_zinfo.p + off; ma.dist = c.d_dist.p + off; ma.lnlam = c.d_lnlam.p;
        int mpw = 32;
        while (mpw > 4 && (nk + mpw - 1) / mpw < 8 * c.num_sms) mpw >>= 1;
        ma.mpw = mpw;
        const long long warps = (nk + mpw - 1) / mpw;
        model_params_kernel<<<(unsigned)((warps * 32 + 255) / 256), 256, smem_mp, st>>>(ma);
        return cudaGetLastError();
    };
    int launches = 0;
    WeightsArgs wa;
    wa.n_models = n; wa.nt = nt; wa.nz = nz; wa.kpad = kpad; wa.kmap = bop ? bop->kmap.p : nullptr;
    wa.wz = d_wz; wa.mass = c.d_mass.p; wa.llin = c.d_llin.p; wa.w_hi = c.d_whi.p; wa.w_lo = c.d_wlo.p;
    wa.sums = c.d_sums.p;
    wa.parts = (io.mass_young || io.mass_old || io.lbol_young || io.lbol_old) ? 1 : 0;
    wa.itesc = itesc;
    wa.grid = 0;
    wa.mpar = (bop && bop->ion) ? c.d_mpar.p : nullptr;   // (the escaping fraction of the escaping-light columns)
    float *d_y = c.d_young.p, *d_o = c.d_old.p;
    const bool want_mags = io.mags != nullptr && !c.fast_mode && nb > 0;
    // bands and magnitudes of models [off, off + nk)
    auto bands = [&](int off, int nk) -> cudaError_t {
        BandGemmArgs ba;
        ba.n_models = nk; ba.nspec = ns; ba.nbands = nb; ba.npad = c.band_npad; ba.nkb = c.band_nkb; ba.j0 = c.band_j0;
        ba.ld_spec = ns; ba.spec = c.d_spec.p + (size_t)ns * off; ba.zinfo = c.d_zinfo.p + off;
        ba.dlnl = c.dlnl; ba.dist = c.d_dist.p + off;
        ba.zp = 48.60 + 2.5 * std::log10(3.828e33 / (4.0 * M_PI * std::pow(10.0 * (648000.0 / M_PI) * 1.495978707e13, 2)));
        ba.do_band = c.d_do_band.p; ba.fband = io.fband_dev ? io.fband_dev + (size_t)nb * off : nullptr;
        ba.mags = (io.dev_inputs ? io.mags : c.d_mags.p) + (size_t)nb * off;
        ba.status = c.d_status.p;
        ba.num_sms = c.num_sms;
        const int ks = band_gemm_ksplit(nk, c.band_nkb, c.num_sms);
        if (ks > 1) {
            const size_t cap = (size_t)ks * nk * c.band_npad;
            if (c.d_bpart.reserve(cap) == cudaSuccess) { ba.fpart = c.d_bpart.p; ba.fpart_cap = cap; }
            else cudaGetLastError();
        }
        return run_band_gemm(ba, c.tm_cb_hi, c.tm_cb_lo, st);
    };
    // the per-model epilogue from the young and old sums (the operator's path, and any batch with dust emission)
    const DustEmModel *d_dem = epi_terms ? c.d_dem.p : nullptr;
    // (models [off, off + nk))
    auto epilogue = [&](const float *y, const float *o, int off, int nk) -> cudaError_t {
        PartsEpilogueArgs pe;
        pe.n = nk; pe.nspec = ns; pe.jtop = c.jtop; pe.sm_lo = any_smooth ? sm_lo : ns; pe.sm_hi = any_smooth ? sm_hi : -1;
        pe.uniform_index = uniform_index ? 1 : 0; pe.tab_curve = tab_curve; pe.pix = c.d_pix.p; pe.mpar = c.d_mpar.p + (size_t)MODEL_PAR_FLOATS * off;
        pe.young = y + (size_t)ns * off; pe.old = o + (size_t)ns * off;
        pe.spec = c.d_spec.p + (size_t)ns * off;
        pe.dem = d_dem ? d_dem + off : nullptr;
        pe.dtab = c.dustem.tab.p; pe.cnu = c.dustem.cnu.p; pe.nqpah = c.dustem.nqpah;
        pe.agn_spec = c.agn.spec.p;
        if (neb_cont) {
            // the CLOUDY-grid continuum into the young and old sums of models [off, off + nk) (their groups by cell)
            const int2 cg = neb_chunk_groups[chunked ? off / CHUNK : 0];
            NebContArgs na;
            na.n = nk; na.nspec = ns; na.nt = nt; na.nz = nz; na.nt_neb = c.nt_neb;
            na.cw_ld = c.nt_neb + 2; na.nrun = c.neb.nrun;
            na.dem = d_dem + off; na.tab = c.neb.tab[neb_table].p; na.off = c.neb.off.p;
            na.rfirst = c.neb.runs.p; na.runs = reinterpret_cast<const int4 *>(c.neb.runs.p + NEB_RUN_HEAD);
            na.q0 = c.neb.q0.p; na.q0_exp = c.neb.q0_exp;
            na.wz = d_wz + (size_t)nt * nz * off;
            na.groups = c.neb.groups.p + cg.x; na.order = c.neb.order.p;
            cudaError_t r = c.neb.cw.reserve((size_t)nk * na.cw_ld);
            if (r != cudaSuccess) return r;
            na.cw = c.neb.cw.p;
            na.young = const_cast<float *>(y) + (size_t)ns * off;
            na.old = const_cast<float *>(o) + (size_t)ns * off;
            if ((r = run_nebular_continuum(na, cg.y, st)) != cudaSuccess) return r;
            launches += 2;
        }
        // (the model's L_bol output: log-blended between the slabs for weights formed on the device, except with
        // the operators, whose L_bol is their linear row)
        const bool blend = io.sfh_par != nullptr && !ops;
        pe.lsum = (blend ? c.d_lblend.p : c.d_sums.p + 1) + (size_t)(blend ? 3 : 6) * off;
        pe.lsum_stride = blend ? 3 : 6;
        return run_parts_epilogue(pe, st);
    };
    if (!fp64 && !ops) {
        // ---- the mixed path over models [off, off + nk): weight operand, contraction with its epilogue, bands,
        // FP64 sums (stage marks on the first range)
        auto run_range = [&](int off, int nk, bool marks) -> int {
            WeightsArgs w = wa;
            w.n_models = nk; w.wz = d_wz + (size_t)nt * nz * off; w.w_hi = c.d_whi.p + (size_t)kpad * off;
            w.w_lo = c.d_wlo.p + (size_t)kpad * off; w.sums = c.d_sums.p + (size_t)6 * off;
            if (w.mpar) w.mpar = c.d_mpar.p + (size_t)MODEL_PAR_FLOATS * off;
            // the operand (which does not read the model parameters unless it forms escaping-light columns) on its
            // own stream beside the model parameters, forked from the batch's stream and joined before the
            // contraction
            const bool fork_w = !direct && !w.mpar;
            if (fork_w && ((e = cudaEventRecord(c.ev_w0, st)) != cudaSuccess || (e = cudaStreamWaitEvent(c.side4, c.ev_w0, 0)) != cudaSuccess ||
                           (e = run_weights_convert_sums(w, c.side4)) != cudaSuccess || (e = cudaEventRecord(c.ev_w1, c.side4)) != cudaSuccess)) {
                err = cuda_msg("weights kernel", e);
                return ST_DATA_MISSING;
            }
            if ((e = model_params(off, nk)) != cudaSuccess) { err = cuda_msg("model parameter kernel", e); return ST_DATA_MISSING; }
            if (marks) prof_mark(c, 1);
            // (the operand and, in the same pass over the FP64 weights, the FP64 mass and L_bol sums; reading the
            // caller's pageable weights in place, on the side stream beside the previous chunk's kernels)
            if (direct) {
                cudaEvent_t &ev = c.chunk_ev[(off / CHUNK) % Context::NCHUNK_EV];
                // (escaping-light columns read the chunk's model parameters, formed on the batch's stream)
                if (w.mpar && ((e = cudaEventRecord(c.ev_params, st)) != cudaSuccess ||
                               (e = cudaStreamWaitEvent(c.side, c.ev_params, 0)) != cudaSuccess)) {
                    err = cuda_msg("weights kernel", e);
                    return ST_DATA_MISSING;
                }
                if ((!ev && (e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) ||
                    (e = run_weights_convert_sums(w, c.side)) != cudaSuccess || (e = cudaEventRecord(ev, c.side)) != cudaSuccess ||
                    (e = cudaStreamWaitEvent(st, ev, 0)) != cudaSuccess) {
                    err = cuda_msg("weights kernel", e);
                    return ST_DATA_MISSING;
                }
            } else if (fork_w) {
                if ((e = cudaStreamWaitEvent(st, c.ev_w1, 0)) != cudaSuccess) { err = cuda_msg("weights kernel", e); return ST_DATA_MISSING; }
            } else if ((e = run_weights_convert_sums(w, st)) != cudaSuccess) {
                err = cuda_msg("weights kernel", e);
                return ST_DATA_MISSING;
            }
            if (marks) prof_mark(c, 2);
            ContractPlan pl;
            pl.tm_a_hi = bop->tm_hi;
            pl.tm_a_lo = bop->tm_lo;
            pl.num_sms = c.num_sms;
            if ((e = encode_tmap_2d_bf16(&pl.tm_b_hi, w.w_hi, kpad, nk, contract_bk(), bn)) != cudaSuccess ||
                (e = encode_tmap_2d_bf16(&pl.tm_b_lo, w.w_lo, kpad, nk, contract_bk(), bn)) != cudaSuccess) {
                err = cuda_msg("weights tensor map", e);
                return ST_DATA_MISSING;
            }
            ContractArgs ca;
            ca.nspec = ns; ca.n_models = nk;
            ca.n_ptiles = (ns + contract_out_rows() - 1) / contract_out_rows();
            ca.n_mtiles = (nk + bn - 1) / bn;
            ca.nkb_young = (nacc == 1) ? bop->kmain / contract_bk() : bop->ky_pad / contract_bk();
            ca.nkb_old = (nacc == 1) ? 0 : (bop->kmain - bop->ky_pad) / contract_bk();
            ca.nkb_ion_young = bop->kion_y / contract_bk();
            ca.nkb_ion_old = bop->kion_o / contract_bk();
            ca.ion_pix = bop->ion ? c.whlylim : 0;
            ca.jtop = c.jtop; ca.ld_spec = ns; ca.pix = c.d_pix.p; ca.mpar = c.d_mpar.p + (size_t)MODEL_PAR_FLOATS * off;
            // (with dust emission or AGN the per-model epilogue forms the spectra from the young and old sums)
            ca.spec = epi ? nullptr : c.d_spec.p + (size_t)ns * off;
            ca.sm_lo = any_smooth ? sm_lo : ns; ca.sm_hi = any_smooth ? sm_hi : -1; ca.uniform_index = uniform_index ? 1 : 0; ca.tab_curve = tab_curve;
            ca.young = ca.old = nullptr;
            if (parts) {
                ca.young = d_y + (size_t)ns * off;
                ca.old = d_o + (size_t)ns * off;
            }
            ca.status = c.d_status.p;
            if ((e = run_contract(nacc, pl, ca, st)) != cudaSuccess) { err = cuda_msg("contraction kernel", e); return ST_DATA_MISSING; }
            if (marks) prof_mark(c, 3);
            launches += 3;
            if (epi) {
                if ((e = epilogue(d_y, d_o, off, nk)) != cudaSuccess) { err = cuda_msg("epilogue kernel", e); return ST_DATA_MISSING; }
                ++launches;
                if (marks) prof_mark(c, 4);
            }
            if (want_mags) {
                if ((e = bands(off, nk)) != cudaSuccess) { err = cuda_msg("band kernel", e); return ST_DATA_MISSING; }
                ++launches;
                if (chunked) {
                    // this chunk's magnitudes to the page-locked staging buffer on the third stream, beside the next
                    // chunk's kernels (the end of the batch then copies only into the caller's array on the host)
                    cudaEvent_t &ev = c.mag_ev[(off / CHUNK) % Context::NCHUNK_EV];
                    if ((!ev && (e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) ||
                        (e = cudaEventRecord(ev, st)) != cudaSuccess || (e = cudaStreamWaitEvent(c.side2, ev, 0)) != cudaSuccess ||
                        (e = cudaMemcpyAsync(c.pinned_mags + (size_t)nb * off, c.d_mags.p + (size_t)nb * off,
                                             sizeof(double) * nb * nk, cudaMemcpyDeviceToHost, c.side2)) != cudaSuccess) {
                        err = cuda_msg("magnitudes copy", e);
                        return ST_DATA_MISSING;
                    }
                }
            }
            if (marks && !epi) prof_mark(c, 4);
            return 0;
        };
        if (parts) {
            // (4 floats of padding: the reverse pass copies whole 16-byte units of each row)
            if ((e = c.d_young.reserve((size_t)n * ns + 4)) != cudaSuccess || (e = c.d_old.reserve((size_t)n * ns + 4)) != cudaSuccess) {
                err = cuda_msg("device memory", e);
                return ST_DATA_MISSING;
            }
            d_y = c.d_young.p;
            d_o = c.d_old.p;
        }
        if (chunked && want_mags && c.pinned_mags_n < (size_t)n * nb) {
            if (c.pinned_mags) cudaFreeHost(c.pinned_mags);
            c.pinned_mags = nullptr;
            c.pinned_mags_n = 0;
            if ((e = cudaMallocHost(&c.pinned_mags, sizeof(double) * n * nb)) != cudaSuccess) {
                err = cuda_msg("page-locked magnitudes", e);
                return ST_DATA_MISSING;
            }
            c.pinned_mags_n = (size_t)n * nb;
        }
        if (!chunked) {
            if (int rc = run_range(0, n, true)) return rc;
        } else {
            // chunks: each chunk's weight operand, contraction, bands and FP64 sums run while the next chunk's
            // weights are copied (the copies are the longer part: the kernels hide under them)
            for (int k = 0; k < nch; ++k) {
                const int off = chunk_off(k), nk = chunk_len(k);
                // (the copies were enqueued above; beyond NCHUNK_EV chunks a slot's event was recorded again by a
                // later chunk's copy, and waiting for that later copy is waiting for this one too)
                if (!direct && (e = cudaStreamWaitEvent(st, c.chunk_ev[k % Context::NCHUNK_EV], 0)) != cudaSuccess) {
                    err = cuda_msg("weights copy", e);
                    return ST_DATA_MISSING;
                }
                if (int rc = run_range(off, nk, k == 0)) return rc;
            }
        }
        prof_mark(c, 5);
    } else {
        if ((e = model_params(0, n)) != cudaSuccess) { err = cuda_msg("model parameter kernel", e); return ST_DATA_MISSING; }
        prof_mark(c, 1);
        if (fp64) {
            // ---- the plain FP64 path: DGEMM age sums, then the rest in FP64 (spectra into d_spec64, magnitudes)
            const int rc = run_fp64_tail(c, io, bop, d_wz, d_par, nacc, any_smooth ? sm_lo : ns, any_smooth ? sm_hi : -1,
                                         i0, err);
            if (rc) return rc;
            prof_mark(c, 2);
            prof_mark(c, 3);
            launches = 5;   // model parameters, weights gather, two DGEMMs, the FP64 tail
        } else if (ops) {
            // ---- the operator: the IMF weights folded with the SFH weights, the template GEMM, then the epilogue
            std::vector<double> al((size_t)3 * n);
            for (int m = 0; m < n; ++m) {
                const double pv[5] = {par(m, PF_IMF1), par(m, PF_IMF2), par(m, PF_IMF3), par(m, PF_VDMC), par(m, PF_MDAVE)};
                imf_pack(c.imf_type, pv, al.data() + 3 * m);
            }
            if ((e = c.d_alpha.reserve(al.size())) != cudaSuccess || (e = c.d_yo.reserve((size_t)2 * n * ns + 4)) != cudaSuccess ||
                (e = cudaMemcpyAsync(c.d_alpha.p, al.data(), sizeof(double) * al.size(), cudaMemcpyHostToDevice, st)) != cudaSuccess) {
                err = cuda_msg("operator inputs", e);
                return ST_DATA_MISSING;
            }
            d_y = c.d_yo.p;
            d_o = c.d_yo.p + (size_t)n * ns;
            c.geom.wz = d_wz;
            const int rc = run_ops_parts(c, n, d_wz, c.d_alpha.p, al.data(), itesc, d_y, d_o, err);
            if (rc) return rc;
            prof_mark(c, 2);
            if ((e = epilogue(d_y, d_o, 0, n)) != cudaSuccess) { err = cuda_msg("epilogue kernel", e); return ST_DATA_MISSING; }
            prof_mark(c, 3);
            launches = 2 + c.ops_launches;   // model parameters, the operator's kernels, the epilogue
        }
        if (want_mags && !fp64) {
            if ((e = bands(0, n)) != cudaSuccess) { err = cuda_msg("band kernel", e); return ST_DATA_MISSING; }
            launches += band_gemm_ksplit(n, c.band_nkb, c.num_sms) > 1 ? 2 : 1;
        }
        prof_mark(c, 4);
        // the FP64 mass and L_bol sums (the operator's fold forms its own)
        if (fp64) {
            if ((e = run_weights_prep(wa, st)) != cudaSuccess) { err = cuda_msg("weights sums kernel", e); return ST_DATA_MISSING; }
            ++launches;
        }
        prof_mark(c, 5);
    }
    c.last_launches = launches + ((io.spec && !io.dev_inputs) ? 1 : 0);
    if (io.dev_inputs) {
        c.last_n = n;
        c.geom.n = n;
        if (!io.dev_sync) return 0;
        int kstatus = 0;
        if ((e = cudaMemcpyAsync(&kstatus, c.d_status.p, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess) {
            err = cuda_msg("batch", e);
            return ST_DATA_MISSING;
        }
        if (kstatus != 0) {
            char buf[96];
            std::snprintf(buf, sizeof buf, "a device wait gave up (code 0x%x)", kstatus);
            err = buf;
            return ST_DATA_MISSING;
        }
        return 0;
    }

    // ---- emission-line luminosities (with nebular emission)
    const bool want_eml = io.emlines && neb && !io.dev_inputs;
    if (want_eml) {
        if (c.eml_nnz < 0) {
            // the (age, metallicity) entries with lines, and their luminosities as FP32 (once per context)
            std::vector<int> kidx;
            std::vector<float> lum;
            for (int k = 0; k < nt * nz; ++k) {
                bool any = false;
                for (int l = 0; l < c.nline; ++l) any = any || c.line_lum[l + (size_t)c.nline * k] != 0.0;
                if (!any) continue;
                kidx.push_back(k);
                for (int l = 0; l < c.nline; ++l) lum.push_back((float)c.line_lum[l + (size_t)c.nline * k]);
            }
            if ((e = c.d_eml_kidx.reserve(std::max<size_t>(kidx.size(), 1))) != cudaSuccess ||
                (e = c.d_eml_lum.reserve(std::max<size_t>(lum.size(), 1))) != cudaSuccess ||
                (!kidx.empty() && (e = cudaMemcpy(c.d_eml_kidx.p, kidx.data(), sizeof(int) * kidx.size(), cudaMemcpyHostToDevice)) != cudaSuccess) ||
                (!lum.empty() && (e = cudaMemcpy(c.d_eml_lum.p, lum.data(), sizeof(float) * lum.size(), cudaMemcpyHostToDevice)) != cudaSuccess)) {
                err = cuda_msg("line table", e);
                return ST_DATA_MISSING;
            }
            c.eml_nnz = (int)kidx.size();
        }
        EmlineArgs ea;
        ea.n_models = n; ea.nline = c.nline; ea.ntz = nt * nz; ea.nnz = c.eml_nnz; ea.wz = d_wz;
        ea.kidx = c.d_eml_kidx.p; ea.lum = c.d_eml_lum.p;
        if ((e = c.d_eml.reserve((size_t)n * c.nline)) != cudaSuccess) { err = cuda_msg("device memory", e); return ST_DATA_MISSING; }
        ea.eml = c.d_eml.p;
        if ((e = run_emlines(ea, st)) != cudaSuccess) { err = cuda_msg("line kernel", e); return ST_DATA_MISSING; }
        ++c.last_launches;
    }
    std::vector<float> eml_h, young_h, old_h;
    if (want_eml) {
        eml_h.resize((size_t)n * c.nline);
        if ((e = cudaMemcpyAsync(eml_h.data(), c.d_eml.p, sizeof(float) * eml_h.size(), cudaMemcpyDeviceToHost, st)) != cudaSuccess) {
            err = cuda_msg("line copy", e);
            return ST_DATA_MISSING;
        }
    }
    const bool parts_out = (io.young || io.old) && !io.dev_inputs;
    if (parts_out) {
        young_h.resize((size_t)n * ns);
        old_h.resize((size_t)n * ns);
        if ((e = cudaMemcpyAsync(young_h.data(), d_y, sizeof(float) * young_h.size(), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(old_h.data(), d_o, sizeof(float) * old_h.size(), cudaMemcpyDeviceToHost, st)) != cudaSuccess) {
            err = cuda_msg("parts copy", e);
            return ST_DATA_MISSING;
        }
    }

    // ---- outputs
    if (io.spec && !io.dev_inputs) {
        if ((e = c.d_spec64.reserve((size_t)n * ns)) != cudaSuccess ||
            (!fp64 && (e = run_spec_to_f64(c.d_spec.p, ns, ns, n, c.d_spec64.p, st)) != cudaSuccess) ||
            (e = cudaMemcpyAsync(io.spec, c.d_spec64.p, sizeof(double) * n * ns, cudaMemcpyDeviceToHost, st)) != cudaSuccess) {
            err = cuda_msg("spectra copy", e);
            return ST_DATA_MISSING;
        }
    }
    if (want_mags && !io.dev_inputs && !chunked) {
        if ((e = cudaMemcpyAsync(io.mags, c.d_mags.p, sizeof(double) * n * nb, cudaMemcpyDeviceToHost, st)) != cudaSuccess) {
            err = cuda_msg("magnitudes copy", e);
            return ST_DATA_MISSING;
        }
    }
    const bool want_sums = io.mass || io.lbol || io.mass_young || io.mass_old || io.lbol_young || io.lbol_old;
    const double *sums = nullptr;
    if (want_sums && !io.dev_inputs) {
        // through a page-locked buffer kept by the context
        const size_t ns6 = (size_t)6 * n;
        if (c.pinned_sums_n < ns6) {
            if (c.pinned_sums) cudaFreeHost(c.pinned_sums);
            c.pinned_sums = nullptr;
            c.pinned_sums_n = 0;
            if ((e = cudaMallocHost(&c.pinned_sums, sizeof(double) * ns6)) != cudaSuccess) {
                err = cuda_msg("page-locked sums", e);
                return ST_DATA_MISSING;
            }
            c.pinned_sums_n = ns6;
        }
        sums = c.pinned_sums;
        if ((e = cudaMemcpyAsync(c.pinned_sums, c.d_sums.p, sizeof(double) * ns6, cudaMemcpyDeviceToHost, st)) != cudaSuccess) {
            err = cuda_msg("sums copy", e);
            return ST_DATA_MISSING;
        }
    }
    // weights formed on the device: L_bol blended in log between the slabs (model_sums MSUMS_BLEND,
    // src/physics/opensps_csp_batch.f90:2129-2176), not the sum over the two slabs' linear L_bol (with the operators
    // L_bol is their linear L_bol row); the SFH's SFR
    std::vector<double> lblend, sfr_h;
    if (io.sfh_par && !io.dev_inputs) {
        sfr_h.resize(n);
        if (!ops) lblend.resize((size_t)3 * n);
        if ((!ops && (e = cudaMemcpyAsync(lblend.data(), c.d_lblend.p, sizeof(double) * lblend.size(), cudaMemcpyDeviceToHost, st)) != cudaSuccess) ||
            (e = cudaMemcpyAsync(sfr_h.data(), c.d_sfr.p, sizeof(double) * n, cudaMemcpyDeviceToHost, st)) != cudaSuccess) {
            err = cuda_msg("SFH outputs copy", e);
            return ST_DATA_MISSING;
        }
    }
    int kstatus = 0;
    if ((e = cudaMemcpyAsync(&kstatus, c.d_status.p, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess) {
        err = cuda_msg("batch", e);
        return ST_DATA_MISSING;
    }
    if (kstatus != 0) {
        char buf[96];
        std::snprintf(buf, sizeof buf, "a device wait gave up (code 0x%x)", kstatus);
        err = buf;
        return ST_DATA_MISSING;
    }
    c.last_n = n;
    c.geom.n = n;
    if (want_mags && chunked) {
        // (the chunks' magnitude copies on the third stream: waited for, then spread over the host threads)
        if ((e = cudaStreamSynchronize(c.side2)) != cudaSuccess) { err = cuda_msg("magnitudes copy", e); return ST_DATA_MISSING; }
        const double *src = c.pinned_mags;
#pragma omp parallel for schedule(static)
        for (int m = 0; m < n; ++m) std::memcpy(io.mags + (size_t)nb * m, src + (size_t)nb * m, sizeof(double) * nb);
    }
    if (want_sums && !io.dev_inputs) {
#pragma omp parallel for schedule(static) if (n >= 8192)
        for (int m = 0; m < n; ++m) {
            const double *s = sums + (size_t)6 * m;
            if (io.mass) io.mass[m] = s[0];
            if (io.lbol) io.lbol[m] = s[1] > SAFE_FLOOR ? std::log10(s[1]) : 0.0;
            if (io.mass_young) io.mass_young[m] = s[2];
            if (io.mass_old) io.mass_old[m] = s[3];
            if (io.lbol_young) io.lbol_young[m] = std::log10(std::max(s[4], SAFE_FLOOR));
            if (io.lbol_old) io.lbol_old[m] = std::log10(std::max(s[5], SAFE_FLOOR));
        }
    }
    if (want_eml)
        for (size_t i = 0; i < eml_h.size(); ++i) io.emlines[i] = (double)eml_h[i];
    if (parts_out) {
        for (size_t i = 0; i < young_h.size(); ++i) {
            if (io.young) io.young[i] = (double)young_h[i];
            if (io.old) io.old[i] = (double)old_h[i];
        }
    }
    if (!lblend.empty()) {
        for (int m = 0; m < n; ++m) {
            const double *l = lblend.data() + (size_t)3 * m;
            if (io.lbol) io.lbol[m] = l[0] > SAFE_FLOOR ? std::log10(l[0]) : 0.0;
            if (io.lbol_young) io.lbol_young[m] = std::log10(std::max(l[1], SAFE_FLOOR));
            if (io.lbol_old) io.lbol_old[m] = std::log10(std::max(l[2], SAFE_FLOOR));
        }
    }
    if (io.sfr) for (int m = 0; m < n; ++m) io.sfr[m] = sfr_h.empty() ? std::nan("") : sfr_h[m];
    if (io.mdust) for (int m = 0; m < n; ++m) io.mdust[m] = SAFE_FLOOR;
    return 0;
}

}  // namespace sps
