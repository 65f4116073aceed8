// A split-BF16 GEMM on the 5th-generation tensor cores: D(M x N) = A(M x K) B(N x K)^T with A = A_hi + A_lo and
// B = B_hi + B_lo (bf16, both K-major), D = A_hi B_hi + A_hi B_lo + A_lo B_hi accumulated in f32 in tensor memory,
// stored as f32 (row-major, ldd) for the rows < M and columns < N.
//
// The reverse pass's weight cotangent is this product: weights_z_bar(k, m) = sum_p basis(p, k) young_or_old_bar(p, m)
// (backward_age_sums, OpenSPS src/physics/opensps_csp_batch.f90:5226-5300), with A = the models' cotangents over the
// pixels and B = the transposed basis.
//
// Tile 128 x 256 x 64, two smem stages (96 KB each), persistent CTAs over tiles; warp 0 = TMA producer, warp 1 = MMA
// issuer and TMEM owner, warps 2..5 = epilogue (one accumulator row per thread); TMEM double-buffered. Every
// mbarrier wait is bounded (status word, no hang).
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>
#include "sm103_ptx.cuh"
#include "csp_kernels.h"

namespace sps {

constexpr int G_BM = 128, G_BN = 256, G_BK = 64, G_STAGES = 2;
constexpr int G_A_BYTES = G_BM * G_BK * 2, G_B_BYTES = G_BN * G_BK * 2;
constexpr int G_STAGE_BYTES = 2 * G_A_BYTES + 2 * G_B_BYTES;
constexpr int G_THREADS = 6 * 32;
constexpr int G_SMEM = G_STAGES * G_STAGE_BYTES + 256 + 1024;
constexpr uint32_t G_IDESC = idesc_bf16_f32(G_BM, G_BN);

__global__ void __launch_bounds__(G_THREADS, 1)
gemm_bf16x3_kernel(const __grid_constant__ CUtensorMap tm_a_hi, const __grid_constant__ CUtensorMap tm_a_lo,
                   const __grid_constant__ CUtensorMap tm_b_hi, const __grid_constant__ CUtensorMap tm_b_lo,
                   GemmArgs g) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + G_STAGES * G_STAGE_BYTES);
    uint64_t *full = bars, *empty = bars + G_STAGES, *tfull = bars + 2 * G_STAGES, *tempty = bars + 2 * G_STAGES + 2;
    uint64_t *mma_done = bars + 2 * G_STAGES + 4;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * G_STAGES + 5);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int mt_n = (g.M + G_BM - 1) / G_BM, nt_n = (g.N + G_BN - 1) / G_BN;
    const int n_tiles = mt_n * nt_n;
    const int nkb = (g.K + G_BK - 1) / G_BK;
    int *status = g.status;

    if (threadIdx.x == 0) {
        for (int s = 0; s < G_STAGES; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
        for (int b = 0; b < 2; ++b) { mbar_init(&tfull[b], 1); mbar_init(&tempty[b], 4); }
        mbar_init(mma_done, 1);
        fence_mbar_init();
    }
    if (warp == 1) { tmem_alloc(tmem_slot, 512); tmem_relinquish(); }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            int s = 0; uint32_t ph = 0;
            int last_fill[G_STAGES];
            for (int i = 0; i < G_STAGES; ++i) last_fill[i] = -1;
            bool ok = true;
            for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
                const int m0 = (tile % mt_n) * G_BM, n0 = (tile / mt_n) * G_BN;
                for (int kb = 0; kb < nkb; ++kb) {
                    if (!mbar_wait(&empty[s], ph ^ 1u, status, ERR_TIMEOUT_PRODUCER)) { ok = false; break; }
                    uint8_t *st = smem + s * G_STAGE_BYTES;
                    mbar_arrive_expect_tx(&full[s], G_STAGE_BYTES);
                    tma_load_2d(st, &tm_a_hi, kb * G_BK, m0, &full[s]);
                    tma_load_2d(st + G_A_BYTES, &tm_a_lo, kb * G_BK, m0, &full[s]);
                    tma_load_2d(st + 2 * G_A_BYTES, &tm_b_hi, kb * G_BK, g.b_row0 + n0, &full[s]);
                    tma_load_2d(st + 2 * G_A_BYTES + G_B_BYTES, &tm_b_lo, kb * G_BK, g.b_row0 + n0, &full[s]);
                    last_fill[s] = (int)ph;
                    if (++s == G_STAGES) { s = 0; ph ^= 1u; }
                }
            }
            for (int i = 0; i < G_STAGES; ++i)
                if (last_fill[i] >= 0) mbar_wait(&full[i], (uint32_t)last_fill[i], status, ERR_TIMEOUT_PRODUCER, false);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            int s = 0; uint32_t ph = 0;
            int acc = 0; uint32_t aph = 0;
            bool ok = true;
            for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
                if (!mbar_wait(&tempty[acc], aph ^ 1u, status, ERR_TIMEOUT_MMA)) { ok = false; break; }
                tc_fence_after();
                const uint32_t d = tmem_base + acc * G_BN;
                for (int kb = 0; kb < nkb; ++kb) {
                    if (!mbar_wait(&full[s], ph, status, ERR_TIMEOUT_MMA)) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t sa = smem_u32(smem + s * G_STAGE_BYTES);
                    const uint32_t a_hi = sa, a_lo = sa + G_A_BYTES, b_hi = sa + 2 * G_A_BYTES, b_lo = b_hi + G_B_BYTES;
#pragma unroll
                    for (int k = 0; k < G_BK / 16; ++k) {
                        const uint32_t off = k * 32;
                        mma_bf16(d, sw128_desc(a_hi + off), sw128_desc(b_hi + off), G_IDESC, (kb > 0 || k > 0) ? 1u : 0u);
                        mma_bf16(d, sw128_desc(a_hi + off), sw128_desc(b_lo + off), G_IDESC, 1u);
                        mma_bf16(d, sw128_desc(a_lo + off), sw128_desc(b_hi + off), G_IDESC, 1u);
                    }
                    mma_commit(&empty[s]);
                    if (++s == G_STAGES) { s = 0; ph ^= 1u; }
                }
                if (!ok) break;
                mma_commit(&tfull[acc]);
                if (++acc == 2) { acc = 0; aph ^= 1u; }
            }
            mma_commit(mma_done);
            mbar_wait(mma_done, 0, status, ERR_TIMEOUT_MMA, false);
        }
    } else {
        // epilogue: warp w reads TMEM lanes 32 (w % 4) .. : one row of D per thread
        const int q = warp & 3;
        int acc = 0; uint32_t aph = 0;
        for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
            const int m0 = (tile % mt_n) * G_BM, n0 = (tile / mt_n) * G_BN;
            mbar_wait(&tfull[acc], aph, status, ERR_TIMEOUT_EPILOGUE);
            named_bar_sync(1, 128);
            if (*(volatile int *)status != 0) break;
            tc_fence_after();
            const int row = m0 + q * 32 + lane;
            const uint32_t trow = tmem_base + ((uint32_t)(q * 32) << 16) + acc * G_BN;
            for (int c = 0; c < G_BN; c += 32) {
                float v[32];
                tmem_ld32(trow + c, v);
                if (row < g.M) {
                    float *dst = g.D + (size_t)row * g.ldd + n0 + c;
#pragma unroll
                    for (int i = 0; i < 32; ++i)
                        if (n0 + c + i < g.N) dst[i] = v[i];
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[acc]);
            if (++acc == 2) { acc = 0; aph ^= 1u; }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem_base, 512);
    }
}

int gemm_bk() { return G_BK; }
int gemm_bm() { return G_BM; }
int gemm_bn() { return G_BN; }

cudaError_t run_gemm_bf16x3(const GemmPlan &pl, const GemmArgs &g, cudaStream_t st) {
    if (g.M <= 0 || g.N <= 0 || g.K <= 0) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(gemm_bf16x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, G_SMEM);
    if (e != cudaSuccess) return e;
    const int tiles = ((g.M + G_BM - 1) / G_BM) * ((g.N + G_BN - 1) / G_BN);
    const int grid = tiles < pl.num_sms ? tiles : pl.num_sms;
    gemm_bf16x3_kernel<<<grid, G_THREADS, G_SMEM, st>>>(pl.tm_a_hi, pl.tm_a_lo, pl.tm_b_hi, pl.tm_b_lo, g);
    return cudaGetLastError();
}

}  // namespace sps
