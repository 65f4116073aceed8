// Band fluxes and AB magnitudes as a tensor-core GEMM: fband(m, b) = sum_j Fobs(m, j) C(j, b); with, beside them,
// the FP64 mass and L_bol sums of the same models.
//
// compute_magnitudes_columns (OpenSPS src/spectra/opensps_batch_photometry.f90:53-180): each model's rest-frame
// spectrum resampled to the observed frame at its redshift, divided by lambda (observed_frame_z :819-903), then the
// trapezoid filter integrals regrouped by pixel, C(j, b) = band(j, b) (wtl(j - 1) + wtl(j)) (the split-K product
// :1002-1044, prepare_batch_grid :375-392), then magnitudes_from_fluxes :185-232 (AB, distance term, NaN for bands
// not computed).
//
// Per CTA: 128 models (MMA M). K = the pixels that any band reaches, 64 per stage. The A operand (observed frame
// of 128 models x 64 pixels) is built by warps 0..7 in shared memory from the spectra, in the 128-byte swizzled
// K-major layout, split into bf16 hi and lo; the B operand (band matrix, hi and lo, bands x pixels) comes by TMA.
// fband = A_hi B_hi + A_hi B_lo + A_lo B_hi in f32 in tensor memory; the epilogue forms the magnitudes. Two stages:
// the builders fill stage s + 1 while the tensor core works on stage s.
//
// With args.sums set, warps 8 and 9 form the FP64 sums of model_sums_zw (src/physics/opensps_csp_batch.f90:2090-2120)
// for the CTA's 128 models (measured slower than the separate sums kernel; the batch does not set it).
#include <cuda_runtime.h>
#include <algorithm>
#include <cuda_bf16.h>
#include <cfloat>
#include <cstdint>
#include "sm103_ptx.cuh"
#include "csp_kernels.h"

namespace sps {

constexpr int BG_M = 128;
constexpr int BG_K = 64;
constexpr int BG_BUILD_WARPS = 8;
constexpr int BG_BUILD_THREADS = BG_BUILD_WARPS * 32;
constexpr int BG_SUM_WARPS = 2;
constexpr int BG_THREADS = BG_BUILD_THREADS + BG_SUM_WARPS * 32;
constexpr int BG_A_BYTES = BG_M * BG_K * 2;   // 16 KB

struct BandGemmSmem {
    static int b_bytes(int npad) { return npad * BG_K * 2; }
    static int total(int npad) { return 2 * (2 * BG_A_BYTES + 2 * b_bytes(npad)) + 256 + 1024; }
};

// 2^x by the SFU
__device__ __forceinline__ float bg_ex2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// The FP64 sums of one model (one warp): mass and L_bol over the weights above SAFE_FLOOR (the comparison on the
// bit pattern: positive doubles order as their bits), young and old apart with parts.
__device__ __forceinline__ void model_sums_warp(const BandGemmArgs &a, int m, int lane) {
    const double *w = a.wz + (size_t)m * a.ntz;
    double ms = 0.0, ls = 0.0, msy = 0.0, lsy = 0.0, mso = 0.0, lso = 0.0;
    int t = lane % a.nt;
#pragma unroll 4
    for (int k = lane; k < a.ntz; k += 32) {
        const double wv = __ldg(w + k);
        if (__double_as_longlong(wv) > 0x0010000000000000LL) {   // wv > DBL_MIN (and not negative)
            const double mk = wv * __ldg(a.mass + k), lk = wv * __ldg(a.llin + k);
            ms += mk;
            ls += lk;
            if (a.parts) {
                if (t < a.itesc) { msy += mk; lsy += lk; } else { mso += mk; lso += lk; }
            }
        }
        if (a.parts) { t += 32; while (t >= a.nt) t -= a.nt; }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        ms += __shfl_xor_sync(0xffffffffu, ms, off);
        ls += __shfl_xor_sync(0xffffffffu, ls, off);
        if (a.parts) {
            msy += __shfl_xor_sync(0xffffffffu, msy, off);
            lsy += __shfl_xor_sync(0xffffffffu, lsy, off);
            mso += __shfl_xor_sync(0xffffffffu, mso, off);
            lso += __shfl_xor_sync(0xffffffffu, lso, off);
        }
    }
    if (lane == 0) {
        double *o = a.sums + (size_t)m * 6;
        o[0] = ms; o[1] = ls;
        if (a.parts) { o[2] = msy; o[3] = mso; o[4] = lsy; o[5] = lso; }
    }
}

// AB magnitude of an FP32 band flux (NaN when not positive): -2.5 log10 f in FP32 (the flux carries FP32's precision
// already; an FP64 logarithm per band was most of the epilogue's time on GB300's narrow FP64 pipe), then the zero
// point and the model's distance term in FP64.
__device__ __forceinline__ double band_mag(float f, double zp, double dist) {
    if (!(f > 0.f)) return __longlong_as_double(0x7ff8000000000000LL);
    return (double)(-2.5f * log10f(f)) - zp + dist;
}

__global__ void __launch_bounds__(BG_THREADS, 2)
band_gemm_kernel(const __grid_constant__ CUtensorMap tm_c_hi, const __grid_constant__ CUtensorMap tm_c_lo,
                 BandGemmArgs a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int npad = a.npad;
    const int b_bytes = npad * BG_K * 2;
    const int stage_bytes = 2 * BG_A_BYTES + 2 * b_bytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + 2 * stage_bytes);
    uint64_t *bar_tma = bars;        // [2]
    uint64_t *bar_mma = bars + 2;    // [2]
    uint64_t *bar_done = bars + 4;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 5);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * BG_M;
    // this CTA's pixel blocks: split blockIdx.y of gridDim.y
    const int kb0 = (int)((long long)blockIdx.y * a.nkb / gridDim.y), kb1 = (int)((long long)(blockIdx.y + 1) * a.nkb / gridDim.y);
    const bool split = gridDim.y > 1;
    int *status = a.status;
    const uint32_t tcols = npad <= 32 ? 32 : (npad <= 64 ? 64 : (npad <= 128 ? 128 : 256));
    __shared__ float4 zsm[BG_M];     // the observed-frame shift of the CTA's models (w = 2: no model in this row)

    if (tid == 0) {
        for (int s = 0; s < 2; ++s) { mbar_init(&bar_tma[s], 1); mbar_init(&bar_mma[s], 1); }
        mbar_init(bar_done, 1);
        fence_mbar_init();
        tma_prefetch_desc(&tm_c_hi);
        tma_prefetch_desc(&tm_c_lo);
    }
    if (warp == 0) { tmem_alloc(tmem_slot, tcols); tmem_relinquish(); }
    for (int i = tid; i < BG_M; i += BG_THREADS)
        zsm[i] = (m0 + i < a.n_models) ? a.zinfo[m0 + i] : make_float4(0.f, 0.f, 0.f, 2.f);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp >= BG_BUILD_WARPS) {
        // ---------------------------------------------------------------- FP64 sums of the CTA's models
        if (a.sums && blockIdx.y == 0) {
            for (int r = warp - BG_BUILD_WARPS; r < BG_M; r += BG_SUM_WARPS)
                if (m0 + r < a.n_models) model_sums_warp(a, m0 + r, lane);
        }
    } else {
        // ---------------------------------------------------------------- band GEMM (warps 0..7)
        const uint32_t idesc = idesc_bf16_f32(BG_M, npad);
        const float dl2 = (float)(a.dlnl * 1.4426950408889634);   // grid step in log2 units
        const float inv_em1 = (float)(1.0 / expm1(a.dlnl));
        // each warp builds 16 model rows; lane l takes pixels 2l, 2l + 1 of the stage
        for (int kb = kb0; kb < kb1; ++kb) {
            const int li = kb - kb0;                          // this CTA's stage count
            const int s = li & 1;
            uint8_t *st = smem + s * stage_bytes;
            if (li >= 2) mbar_wait(&bar_mma[s], ((li - 2) >> 1) & 1, status, ERR_TIMEOUT_BAND, false);
            if (tid == 0) {
                mbar_arrive_expect_tx(&bar_tma[s], 2 * b_bytes);
                tma_load_2d(st + 2 * BG_A_BYTES, &tm_c_hi, kb * BG_K, 0, &bar_tma[s]);
                tma_load_2d(st + 2 * BG_A_BYTES + b_bytes, &tm_c_lo, kb * BG_K, 0, &bar_tma[s]);
            }
            const int j = a.j0 + kb * BG_K + 2 * lane;       // observed pixel of this lane (and j + 1)
            float wl0 = 0.f, wl1 = 0.f;
            if (j < a.nspec) wl0 = __ldg(a.wl + j);
            if (j + 1 < a.nspec) wl1 = __ldg(a.wl + j + 1);
            // rows in two halves of 8: each half's loads are all issued before any is used
#pragma unroll 1
            for (int h = 0; h < 2; ++h) {
            float s00[8], s01[8], s10[8], s11[8], t0v[8], t1v[8];
#pragma unroll
            for (int rr = 0; rr < 8; ++rr) {
                const int r = warp * 16 + h * 8 + rr;
                const float4 zs = zsm[r];                     // n0, t, s, (0: rest frame, 2: no model)
                const float *sp = a.spec + (size_t)(m0 + r) * a.ld_spec;
                s00[rr] = s01[rr] = s10[rr] = s11[rr] = 0.f;
                t0v[rr] = t1v[rr] = 0.f;
                if (zs.w == 1.f) {
                    const int n0 = __float_as_int(zs.x);
                    const int sub = (zs.y > 0.f) ? 1 : 0;
                    const int il0 = j - n0 - sub, il1 = il0 + 1;
                    // intervals outside the grid extrapolate from the first / last one (the reference's clamped
                    // find_interval): position t = (e^(x dlnl) - 1) / (e^dlnl - 1), x pixels from the interval start
                    const int c0 = min(max(il0, 0), a.nspec - 2), c1 = min(max(il1, 0), a.nspec - 2);
                    const float t0 = (c0 == il0) ? zs.y : (bg_ex2(((float)(j - c0) - zs.z) * dl2) - 1.f) * inv_em1;
                    const float t1 = (c1 == il1) ? zs.y : (bg_ex2(((float)(j + 1 - c1) - zs.z) * dl2) - 1.f) * inv_em1;
                    s00[rr] = __ldg(sp + c0); s01[rr] = __ldg(sp + c0 + 1);
                    s10[rr] = __ldg(sp + c1); s11[rr] = __ldg(sp + c1 + 1);
                    t0v[rr] = t0; t1v[rr] = t1;
                } else if (zs.w == 0.f) {
                    // rest frame: v = s00 (t = 0)
                    if (j < a.nspec) s00[rr] = __ldg(sp + j);
                    if (j + 1 < a.nspec) s10[rr] = __ldg(sp + j + 1);
                }
            }
#pragma unroll
            for (int rr = 0; rr < 8; ++rr) {
                const int r = warp * 16 + h * 8 + rr;
                float v0 = fmaf(t0v[rr], s01[rr] - s00[rr], s00[rr]);
                float v1 = fmaf(t1v[rr], s11[rr] - s10[rr], s10[rr]);
                if (v0 != v0) v0 = 0.f;
                if (v1 != v1) v1 = 0.f;
                const float f0 = fmaxf(v0, 0.f) * wl0;
                const float f1 = fmaxf(v1, 0.f) * wl1;
                const __nv_bfloat16 h0 = __float2bfloat16_rn(f0), h1 = __float2bfloat16_rn(f1);
                const __nv_bfloat16 l0 = __float2bfloat16_rn(f0 - __bfloat162float(h0));
                const __nv_bfloat16 l1 = __float2bfloat16_rn(f1 - __bfloat162float(h1));
                const uint32_t off = r * 128 + ((((uint32_t)lane >> 2) ^ (r & 7)) << 4) + ((lane & 3) << 2);
                __nv_bfloat162 hh, ll;
                hh.x = h0; hh.y = h1;
                ll.x = l0; ll.y = l1;
                *reinterpret_cast<__nv_bfloat162 *>(st + off) = hh;
                *reinterpret_cast<__nv_bfloat162 *>(st + BG_A_BYTES + off) = ll;
            }
            }
            fence_proxy_async_smem();
            named_bar_sync(1, BG_BUILD_THREADS);
            if (tid == 0) {
                mbar_wait(&bar_tma[s], (li >> 1) & 1, status, ERR_TIMEOUT_BAND, false);
                tc_fence_after();
                const uint32_t sa = smem_u32(st);
                const uint32_t ahi = sa, alo = sa + BG_A_BYTES, bhi = sa + 2 * BG_A_BYTES, blo = bhi + b_bytes;
#pragma unroll
                for (int k = 0; k < BG_K / 16; ++k) {
                    const uint32_t o = k * 32;
                    mma_bf16(tmem, sw128_desc(ahi + o), sw128_desc(bhi + o), idesc, (li > 0 || k > 0) ? 1u : 0u);
                    mma_bf16(tmem, sw128_desc(ahi + o), sw128_desc(blo + o), idesc, 1u);
                    mma_bf16(tmem, sw128_desc(alo + o), sw128_desc(bhi + o), idesc, 1u);
                }
                mma_commit(&bar_mma[s]);
            }
        }
        if (tid == 0) mma_commit(bar_done);
        mbar_wait(bar_done, 0, status, ERR_TIMEOUT_BAND, false);
        tc_fence_after();

        // epilogue: warps w and w + 4 read lane quarter w % 4 (one model per thread), columns 32 (w / 4) + 64 i
        {
            const int q = warp & 3;
            const int r = q * 32 + lane, m = m0 + r;
            const uint32_t trow = tmem + ((uint32_t)(q * 32) << 16);
            for (int c0 = (warp >> 2) * 32; c0 < npad; c0 += 64) {
                float v[32];
                tmem_ld32(trow + c0, v);
                if (split) {
                    // the split's partial fluxes (band_finish_kernel sums them and forms the magnitudes)
                    if (m < a.n_models) {
                        float *dst = a.fpart + ((size_t)blockIdx.y * a.n_models + m) * npad + c0;
#pragma unroll
                        for (int i = 0; i < 32; i += 4)   // (npad is a multiple of 16)
                            if (c0 + i < npad)
                                *reinterpret_cast<float4 *>(dst + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
                    }
                    continue;
                }
                if (m < a.n_models) {
#pragma unroll
                    for (int i = 0; i < 32; ++i) {
                        const int b = c0 + i;
                        if (b < a.nbands) {
                            const double f = (double)v[i];
                            if (a.fband) a.fband[(size_t)m * a.nbands + b] = f;
                            if (a.mags) {
                                double mg = __longlong_as_double(0x7ff8000000000000LL);
                                if (a.do_band == nullptr || a.do_band[b] != 0)
                                    mg = band_mag(v[i], a.zp, a.dist[m]);
                                a.mags[(size_t)m * a.nbands + b] = mg;
                            }
                        }
                    }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, tcols);
    }
}

int band_gemm_npad(int nbands) { return (nbands + 15) / 16 * 16 < 32 ? 32 : (nbands + 15) / 16 * 16; }

// The split partial fluxes summed in split order, then the fluxes and magnitudes as the GEMM's epilogue forms them.
__global__ void band_finish_kernel(BandGemmArgs a) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)a.n_models * a.nbands) return;
    const int m = (int)(i / a.nbands), b = (int)(i % a.nbands);
    float v = 0.f;
    for (int s = 0; s < a.ksplit; ++s) v += a.fpart[((size_t)s * a.n_models + m) * a.npad + b];
    if (a.fband) a.fband[i] = (double)v;
    if (a.mags) {
        double mg = __longlong_as_double(0x7ff8000000000000LL);
        if (a.do_band == nullptr || a.do_band[b] != 0) mg = band_mag(v, a.zp, a.dist[m]);
        a.mags[i] = mg;
    }
}

// Splits of the pixel blocks when the batch's 128-model tiles give fewer than two CTAs per SM (two fit on an SM):
// up to two CTAs per SM, each split keeping at least 4 pixel blocks.
int band_gemm_ksplit(int n_models, int nkb, int num_sms) {
    const int tiles = (n_models + BG_M - 1) / BG_M;
    if (tiles >= 2 * num_sms || nkb < 8) return 1;
    return std::max(1, std::min((2 * num_sms + tiles - 1) / tiles, nkb / 4));
}

// Loads the band GEMM's module on the current device (CUDA loads modules lazily, on first use), so that a later
// launch loads nothing.
cudaError_t band_gemm_load() {
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, band_gemm_kernel);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, band_finish_kernel);
    return e;
}

cudaError_t run_band_gemm(const BandGemmArgs &a_in, const CUtensorMap &tm_hi, const CUtensorMap &tm_lo,
                          cudaStream_t st) {
    if (a_in.n_models <= 0 || a_in.nkb <= 0) return cudaSuccess;
    BandGemmArgs a = a_in;
    a.ksplit = a.fpart ? band_gemm_ksplit(a.n_models, a.nkb, a.num_sms) : 1;
    if (a.ksplit > 1 && (size_t)a.ksplit * a.n_models * a.npad > a.fpart_cap) a.ksplit = 1;
    const int smem = BandGemmSmem::total(a.npad);
    cudaError_t e = cudaFuncSetAttribute(band_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    const dim3 grid((a.n_models + BG_M - 1) / BG_M, a.ksplit);
    band_gemm_kernel<<<grid, BG_THREADS, smem, st>>>(tm_hi, tm_lo, a);
    if ((e = cudaGetLastError()) != cudaSuccess || a.ksplit == 1) return e;
    const size_t tot = (size_t)a.n_models * a.nbands;
    band_finish_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(a);
    return cudaGetLastError();
}

}  // namespace sps
