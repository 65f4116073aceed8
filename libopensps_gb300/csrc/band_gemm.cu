// Band fluxes and AB magnitudes as a tensor-core GEMM: fband(m, b) = sum_j Fobs(m, j) C(j, b); with, beside them,
// the FP64 mass and L_bol sums of the same models.
//
// compute_magnitudes_columns (OpenSPS src/spectra/opensps_batch_photometry.f90:53-180): each model's rest-frame
// spectrum resampled to the observed frame at its redshift, divided by lambda (observed_frame_z :819-903), then the
// trapezoid filter integrals regrouped by pixel, C(j, b) = band(j, b) (wtl(j - 1) + wtl(j)) (the split-K product
// :1002-1044, prepare_batch_grid :375-392), then magnitudes_from_fluxes :185-232 (AB, distance term, NaN for bands
// not computed). The division by lambda is folded into the band matrix (C(j, b) / lambda(j), formed in FP64 on the
// host), so the A operand is the resampled spectrum itself.
//
// Per CTA: 128 models (MMA M). K = the pixels that any band reaches, 64 per stage. The A operand (observed frame
// of 128 models x 64 pixels) is built by warps 0..7 in shared memory from the spectra, in the 128-byte swizzled
// K-major layout, split into bf16 hi and lo; the B operand (band matrix, hi and lo, bands x pixels) comes by TMA.
// fband = A_hi B_hi + A_hi B_lo + A_lo B_hi in f32 in tensor memory; the epilogue forms the magnitudes.
// Warp roles: warps 0..15 build the A operand (8 model rows each: two CTAs of 17 warps per SM at 56 registers, against
// 9 warps of 16 rows at 92), warp 16 issues the band matrix's TMA and the MMAs.
// Two stages with mbarriers: a builder warp signals its rows of stage s on full_a[s] and goes on to the next stage as
// soon as the MMAs that read that buffer have completed (empty[s], a tcgen05 commit), so that the warps do not wait
// for one another between stages.
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
constexpr int BG_BUILD_WARPS = 16;
constexpr int BG_BUILD_THREADS = BG_BUILD_WARPS * 32;
constexpr int BG_MMA_WARP = BG_BUILD_WARPS;             // TMA of the band matrix and the MMAs
constexpr int BG_THREADS = BG_BUILD_THREADS + 32;
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
    uint64_t *full_a = bars;         // [2] the builder warps' rows of a stage (8 arrivals)
    uint64_t *full_b = bars + 2;     // [2] the band matrix's TMA of a stage
    uint64_t *empty = bars + 4;      // [2] the MMAs that read a stage have completed
    uint64_t *bar_done = bars + 6;   // every MMA has completed
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 7);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * BG_M;
    // this CTA's pixel blocks: split blockIdx.y of gridDim.y
    const int kb0 = (int)((long long)blockIdx.y * a.nkb / gridDim.y), kb1 = (int)((long long)(blockIdx.y + 1) * a.nkb / gridDim.y);
    const int nst = kb1 - kb0;
    const bool split = gridDim.y > 1;
    int *status = a.status;
    const uint32_t tcols = npad <= 32 ? 32 : (npad <= 64 ? 64 : (npad <= 128 ? 128 : 256));
    __shared__ float4 zsm[BG_M];     // the observed-frame shift of the CTA's models (w = 2: no model in this row)
    __shared__ int2 rsh[BG_M];       // per row: the rest-frame offset d (observed pixel j reads j - d, j - d + 1) and
                                     // the last first-pixel j of a lane whose five rest pixels j - d .. j - d + 4 and
                                     // four observed ones lie inside the grid (the interior case: d <= j <= that;
                                     // a row without a model has none)

    if (tid == 0) {
        for (int s = 0; s < 2; ++s) { mbar_init(&full_a[s], BG_BUILD_WARPS); mbar_init(&full_b[s], 1); mbar_init(&empty[s], 1); }
        mbar_init(bar_done, 1);
        fence_mbar_init();
        tma_prefetch_desc(&tm_c_hi);
        tma_prefetch_desc(&tm_c_lo);
    }
    if (warp == 0) { tmem_alloc(tmem_slot, tcols); tmem_relinquish(); }
    for (int i = tid; i < BG_M; i += BG_THREADS) {
        const float4 zs = (m0 + i < a.n_models) ? a.zinfo[m0 + i] : make_float4(0.f, 0.f, 0.f, 2.f);
        zsm[i] = zs;
        // the interior interpolation's first rest pixel: n0 + 1 below the observed one unless the shift is whole
        const int kind = zs.w == 1.f ? 1 : (zs.w == 0.f ? 0 : 2);
        const int d = kind == 1 ? __float_as_int(zs.x) + (zs.y > 0.f ? 1 : 0) : 0;
        rsh[i] = make_int2(d, kind == 2 ? -1 : min(a.nspec - 5 + d, a.nspec - 4));
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == BG_MMA_WARP) {
        // ---------------------------------------------------------------- band matrix TMA and MMAs (one thread)
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16_f32(BG_M, npad);
            int last_fill[2] = {-1, -1};      // parity of the last TMA issued into each stage, -1: none
            bool ok = true;
            for (int li = 0; li < nst && ok; ++li) {
                const int s = li & 1, kb = kb0 + li;
                uint8_t *st = smem + s * stage_bytes;
                // the stage's B buffer is free once the MMAs of stage li - 2 have completed
                if (li >= 2 && !mbar_wait(&empty[s], ((li - 2) >> 1) & 1, status, ERR_TIMEOUT_BAND)) { ok = false; break; }
                mbar_arrive_expect_tx(&full_b[s], 2 * b_bytes);
                tma_load_2d(st + 2 * BG_A_BYTES, &tm_c_hi, kb * BG_K, 0, &full_b[s]);
                tma_load_2d(st + 2 * BG_A_BYTES + b_bytes, &tm_c_lo, kb * BG_K, 0, &full_b[s]);
                last_fill[s] = (li >> 1) & 1;
                if (!mbar_wait(&full_a[s], (li >> 1) & 1, status, ERR_TIMEOUT_BAND) ||
                    !mbar_wait(&full_b[s], (li >> 1) & 1, status, ERR_TIMEOUT_BAND)) { ok = false; break; }
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
                mma_commit(&empty[s]);
            }
            // every MMA issued completes on bar_done (the epilogue's wait, and the TMEM's release below); the copies
            // still in flight land before the CTA may exit
            mma_commit(bar_done);
            for (int s = 0; s < 2; ++s)
                if (last_fill[s] >= 0) mbar_wait(&full_b[s], (uint32_t)last_fill[s], status, ERR_TIMEOUT_BAND, false);
            if (!ok) mbar_wait(bar_done, 0, status, ERR_TIMEOUT_BAND, false);
        }
    } else {
        // ---------------------------------------------------------------- A operand builders (warps 0..15)
        const float dl2 = (float)(a.dlnl * 1.4426950408889634);   // grid step in log2 units
        const float inv_em1 = (float)(1.0 / expm1(a.dlnl));
        // each warp builds 8 model rows, two at a time: lane l takes row parity l / 16 and pixels 4 (l % 16) ..
        // 4 (l % 16) + 3 of the stage
        const int q = lane & 15, hr = lane >> 4;
        for (int li = 0; li < nst; ++li) {
            const int s = li & 1, kb = kb0 + li;
            uint8_t *st = smem + s * stage_bytes;
            // the stage's A buffer is free once the MMAs of stage li - 2 have completed
            if (li >= 2 && !mbar_wait(&empty[s], ((li - 2) >> 1) & 1, status, ERR_TIMEOUT_BAND)) break;
            const int j = a.j0 + kb * BG_K + 4 * q;          // first observed pixel of this lane
            // the loads of all 4 row pairs first (rows whose 5 rest pixels lie inside the grid: the interior case),
            // then the arithmetic
            float sv[4][5];
            bool inner[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int r = warp * 8 + 2 * i + hr;
                const int2 rs = rsh[r];
                inner[i] = j >= rs.x && j <= rs.y;
                const float *sp = a.spec + (size_t)(m0 + r) * a.ld_spec + (j - rs.x);
#pragma unroll
                for (int u = 0; u < 5; ++u) sv[i][u] = inner[i] ? __ldg(sp + u) : 0.f;
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int r = warp * 8 + 2 * i + hr;
                float f[4];
                if (inner[i]) {
                    // v = s(c) + t (s(c + 1) - s(c)), t = 0 for whole shifts and the rest frame (v = s(c) exactly
                    // for finite spectra); NaN -> 0 and negatives -> 0 in one fmaxf
                    const float t = zsm[r].y;
#pragma unroll
                    for (int u = 0; u < 4; ++u) f[u] = fmaxf(fmaf(t, sv[i][u + 1] - sv[i][u], sv[i][u]), 0.f);
                } else {
                    // the general case: no model, pixels past the grid's end, or intervals outside the grid (they
                    // extrapolate from the first / last one, the reference's clamped find_interval: position
                    // t = (e^(x dlnl) - 1) / (e^dlnl - 1), x pixels from the interval start)
                    const float4 zs = zsm[r];
                    const float *sp = a.spec + (size_t)(m0 + r) * a.ld_spec;
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int ju = j + u;
                        float v = 0.f;
                        if (zs.w == 1.f) {
                            const int n0 = __float_as_int(zs.x);
                            const int il = ju - n0 - ((zs.y > 0.f) ? 1 : 0);
                            const int cc = min(max(il, 0), a.nspec - 2);
                            const float tt = (cc == il) ? zs.y : (bg_ex2(((float)(ju - cc) - zs.z) * dl2) - 1.f) * inv_em1;
                            const float x0 = __ldg(sp + cc), x1 = __ldg(sp + cc + 1);
                            v = fmaf(tt, x1 - x0, x0);
                        } else if (zs.w == 0.f && ju < a.nspec) {
                            v = __ldg(sp + ju);
                        }
                        f[u] = fmaxf(v, 0.f);
                    }
                }
                // bf16 hi and lo parts, four pixels = 8 bytes of the row's 128-byte swizzled line
                const __nv_bfloat162 h01 = __floats2bfloat162_rn(f[0], f[1]), h23 = __floats2bfloat162_rn(f[2], f[3]);
                const float2 g01 = __bfloat1622float2(h01), g23 = __bfloat1622float2(h23);
                const __nv_bfloat162 l01 = __floats2bfloat162_rn(f[0] - g01.x, f[1] - g01.y);
                const __nv_bfloat162 l23 = __floats2bfloat162_rn(f[2] - g23.x, f[3] - g23.y);
                const uint32_t off = r * 128 + ((((uint32_t)q >> 1) ^ (r & 7)) << 4) + ((q & 1) << 3);
                uint2 hv, lv;
                hv.x = *reinterpret_cast<const uint32_t *>(&h01); hv.y = *reinterpret_cast<const uint32_t *>(&h23);
                lv.x = *reinterpret_cast<const uint32_t *>(&l01); lv.y = *reinterpret_cast<const uint32_t *>(&l23);
                *reinterpret_cast<uint2 *>(st + off) = hv;
                *reinterpret_cast<uint2 *>(st + BG_A_BYTES + off) = lv;
            }
            // this warp's rows of the stage, visible to the tensor core's (async) reads
            fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) mbar_arrive(&full_a[s]);
        }
        mbar_wait(bar_done, 0, status, ERR_TIMEOUT_BAND, false);
        tc_fence_after();

        // epilogue (warps 0..7): warps w and w + 4 read lane quarter w % 4 (one model per thread), columns
        // 32 (w / 4) + 64 i
        if (warp < 8 && *(volatile int *)status == 0) {
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
