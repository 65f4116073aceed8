// Band fluxes and AB magnitudes as a tensor-core GEMM: fband(m, b) = sum_j Fobs(m, j) C(j, b).
//
// compute_magnitudes_columns (OpenSPS src/spectra/opensps_batch_photometry.f90:53-180): each model's rest-frame
// spectrum resampled to the observed frame at its redshift, divided by lambda (observed_frame_z :819-903), then the
// trapezoid filter integrals regrouped by pixel, C(j, b) = band(j, b) (wtl(j - 1) + wtl(j)) (the split-K product
// :1002-1044, prepare_batch_grid :375-392), then magnitudes_from_fluxes :185-232 (AB, distance term, NaN for bands
// not computed).
//
// Per CTA: 128 models (MMA M). K = the pixels that any band reaches, 64 per stage. The A operand (observed frame
// of 128 models x 64 pixels) is built by the CTA's threads in shared memory from the spectra, in the 128-byte
// swizzled K-major layout, split into bf16 hi and lo; the B operand (band matrix, hi and lo, bands x pixels) comes
// by TMA. fband = A_hi B_hi + A_hi B_lo + A_lo B_hi in f32 in tensor memory; the epilogue forms the magnitudes.
// Two stages: the threads build stage s + 1 while the tensor core works on stage s.
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>
#include "sm103_ptx.cuh"
#include "csp_kernels.h"

namespace sps {

constexpr int BG_M = 128;
constexpr int BG_K = 64;
constexpr int BG_THREADS = 256;
constexpr int BG_A_BYTES = BG_M * BG_K * 2;   // 16 KB

struct BandGemmSmem {
    static int b_bytes(int npad) { return npad * BG_K * 2; }
    static int total(int npad) { return 2 * (2 * BG_A_BYTES + 2 * b_bytes(npad)) + 256 + 1024; }
};

// The rest-frame interval of observed pixel j when it falls outside the grid (extrapolation from the first or
// the last interval, as the reference's clamped find_interval): *il and the position t.
__device__ __noinline__ void clamped_interval(int j, float shift, float dlnl, float em1, int nspec, int *il, float *t) {
    const int c = (*il < 0) ? 0 : nspec - 2;
    *t = expm1f(((float)(j - c) - shift) * dlnl) / em1;
    *il = c;
}

__global__ void __launch_bounds__(BG_THREADS)
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
    int *status = a.status;
    const uint32_t tcols = npad <= 32 ? 32 : (npad <= 64 ? 64 : (npad <= 128 ? 128 : 256));

    if (tid == 0) {
        for (int s = 0; s < 2; ++s) { mbar_init(&bar_tma[s], 1); mbar_init(&bar_mma[s], 1); }
        mbar_init(bar_done, 1);
        fence_mbar_init();
        tma_prefetch_desc(&tm_c_hi);
        tma_prefetch_desc(&tm_c_lo);
    }
    if (warp == 0) { tmem_alloc(tmem_slot, tcols); tmem_relinquish(); }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t idesc = idesc_bf16_f32(BG_M, npad);
    const float dlnl_f = (float)a.dlnl;
    const float em1 = expm1f(dlnl_f);
    // the observed-frame shift of the CTA's models (w = 2: no model in this row)
    __shared__ float4 zsm[BG_M];
    for (int i = tid; i < BG_M; i += BG_THREADS)
        zsm[i] = (m0 + i < a.n_models) ? a.zinfo[m0 + i] : make_float4(0.f, 0.f, 0.f, 2.f);
    __syncthreads();

    // each warp builds 16 model rows; lane l takes pixels 2l, 2l + 1 of the stage
    for (int kb = 0; kb < a.nkb; ++kb) {
        const int s = kb & 1;
        uint8_t *st = smem + s * stage_bytes;
        if (kb >= 2) mbar_wait(&bar_mma[s], ((kb - 2) >> 1) & 1, status, ERR_TIMEOUT_BAND, false);
        if (tid == 0) {
            mbar_arrive_expect_tx(&bar_tma[s], 2 * b_bytes);
            tma_load_2d(st + 2 * BG_A_BYTES, &tm_c_hi, kb * BG_K, 0, &bar_tma[s]);
            tma_load_2d(st + 2 * BG_A_BYTES + b_bytes, &tm_c_lo, kb * BG_K, 0, &bar_tma[s]);
        }
        const int j = a.j0 + kb * BG_K + 2 * lane;       // observed pixel of this lane (and j + 1)
        float wl0 = 0.f, wl1 = 0.f;
        if (j < a.nspec) wl0 = __ldg(a.wl + j);
        if (j + 1 < a.nspec) wl1 = __ldg(a.wl + j + 1);
        // all 16 rows' loads are issued before any is used (the rows are independent)
        float s00[16], s01[16], s10[16], s11[16], t0v[16], t1v[16];
#pragma unroll
        for (int rr = 0; rr < 16; ++rr) {
            const int r = warp * 16 + rr;
            const float4 zs = zsm[r];                     // n0, t, s, (0: rest frame, 2: no model)
            const float *sp = a.spec + (size_t)(m0 + r) * a.ld_spec;
            s00[rr] = s01[rr] = s10[rr] = s11[rr] = 0.f;
            t0v[rr] = t1v[rr] = 0.f;
            if (zs.w == 1.f) {
                const int n0 = __float_as_int(zs.x);
                const int sub = (zs.y > 0.f) ? 1 : 0;
                int il0 = j - n0 - sub, il1 = il0 + 1;
                float t0 = zs.y, t1 = zs.y;
                if (il0 < 0 || il0 > a.nspec - 2) clamped_interval(j, zs.z, dlnl_f, em1, a.nspec, &il0, &t0);
                if (il1 < 0 || il1 > a.nspec - 2) clamped_interval(j + 1, zs.z, dlnl_f, em1, a.nspec, &il1, &t1);
                s00[rr] = __ldg(sp + il0); s01[rr] = __ldg(sp + il0 + 1);
                s10[rr] = __ldg(sp + il1); s11[rr] = __ldg(sp + il1 + 1);
                t0v[rr] = t0; t1v[rr] = t1;
            } else if (zs.w == 0.f) {
                // rest frame: v = s00 (t = 0)
                if (j < a.nspec) s00[rr] = __ldg(sp + j);
                if (j + 1 < a.nspec) s10[rr] = __ldg(sp + j + 1);
            }
        }
#pragma unroll
        for (int rr = 0; rr < 16; ++rr) {
            const int r = warp * 16 + rr;
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
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
            mbar_wait(&bar_tma[s], (kb >> 1) & 1, status, ERR_TIMEOUT_BAND, false);
            tc_fence_after();
            const uint32_t sa = smem_u32(st);
            const uint32_t ahi = sa, alo = sa + BG_A_BYTES, bhi = sa + 2 * BG_A_BYTES, blo = bhi + b_bytes;
#pragma unroll
            for (int k = 0; k < BG_K / 16; ++k) {
                const uint32_t o = k * 32;
                mma_bf16(tmem, sw128_desc(ahi + o), sw128_desc(bhi + o), idesc, (kb > 0 || k > 0) ? 1u : 0u);
                mma_bf16(tmem, sw128_desc(ahi + o), sw128_desc(blo + o), idesc, 1u);
                mma_bf16(tmem, sw128_desc(alo + o), sw128_desc(bhi + o), idesc, 1u);
            }
            mma_commit(&bar_mma[s]);
        }
    }
    if (tid == 0) mma_commit(bar_done);
    mbar_wait(bar_done, 0, status, ERR_TIMEOUT_BAND, false);
    tc_fence_after();

    // epilogue: warps 0..3 read their lane quarter (one model per thread)
    if (warp < 4) {
        const int r = warp * 32 + lane, m = m0 + r;
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
        for (int c0 = 0; c0 < npad; c0 += 32) {
            float v[32];
            tmem_ld32(trow + c0, v);
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
                                mg = (f > 0.0 ? -2.5 * log10(f) : __longlong_as_double(0x7ff8000000000000LL)) - a.zp +
                                     a.dist[m];
                            a.mags[(size_t)m * a.nbands + b] = mg;
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

cudaError_t run_band_gemm(const BandGemmArgs &a, const CUtensorMap &tm_hi, const CUtensorMap &tm_lo,
                          cudaStream_t st) {
    if (a.n_models <= 0 || a.nkb <= 0) return cudaSuccess;
    const int smem = BandGemmSmem::total(a.npad);
    cudaError_t e = cudaFuncSetAttribute(band_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    const int grid = (a.n_models + BG_M - 1) / BG_M;
    band_gemm_kernel<<<grid, BG_THREADS, smem, st>>>(tm_hi, tm_lo, a);
    return cudaGetLastError();
}

}  // namespace sps
