// GEMMs on the 5th-generation tensor cores: D(M x N) = A(M x K) B(N x K)^T, both operands bf16 and K-major, f32
// accumulation in tensor memory, D stored as f32 (row-major, ldd) for the rows < M and columns < N.
//
// Two kinds:
//  * split-BF16 (three products): A = A_hi + A_lo, B = B_hi + B_lo, D = A_hi B_hi + A_hi B_lo + A_lo B_hi. The
//    reverse pass's weight cotangent (backward_age_sums, OpenSPS src/physics/opensps_csp_batch.f90:5226-5300) and
//    the SSP operator's template GEMM (template_columns, src/physics/opensps_ssp_batch.f90:3247-3385) use it.
//  * one product, bf16 or f16 operands: the emulator's training GEMMs (forward in f16; input cotangents and
//    weight gradients in bf16).
//
// Groups and split-K: the tile index runs over (group, K split, M tile, N tile). Group g reads the A rows from
// g * a_grp, the B rows from g * b_grp and writes D from g * d_grp (elements); K split s covers the K blocks
// [s * nkb / ksplit, (s + 1) * nkb / ksplit) and writes its partial sums from s * d_split. The emulator's five
// ensemble members are the groups; the weight gradients (K = the minibatch) are split over K.
//
// Tile 128 x 256 x 64, persistent CTAs over tiles; warp 0 = TMA producer, warp 1 = MMA issuer and TMEM owner,
// warps 2..5 = epilogue (one accumulator row per thread); TMEM double-buffered. Two smem stages of 96 KB (split) or
// four of 48 KB (plain). Every mbarrier wait is bounded (status word, no hang).
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>
#include "sm103_ptx.cuh"
#include "csp_kernels.h"

namespace sps {

constexpr int G_BM = 128, G_BN = 256, G_BK = 64;
constexpr int G_A_BYTES = G_BM * G_BK * 2, G_B_BYTES = G_BN * G_BK * 2;
constexpr int G_THREADS = 6 * 32;
constexpr uint32_t G_IDESC = idesc_bf16_f32(G_BM, G_BN);

template <int NPROD>
struct GemmCfg {
    static constexpr int STAGE_BYTES = NPROD == 3 ? 2 * G_A_BYTES + 2 * G_B_BYTES : G_A_BYTES + G_B_BYTES;
    static constexpr int STAGES = NPROD == 3 ? 2 : 4;
    static constexpr int SMEM = STAGES * STAGE_BYTES + 256 + 1024;
};

struct GemmTile {
    int g, s, m0, n0;
};
__device__ __forceinline__ GemmTile gemm_tile(const GemmArgs &g, int tile, int mt_n, int nt_n) {
    GemmTile t;
    t.m0 = (tile % mt_n) * G_BM;
    int r = tile / mt_n;
    t.n0 = (r % nt_n) * G_BN;
    r /= nt_n;
    t.s = r % g.ksplit;
    t.g = r / g.ksplit;
    return t;
}

template <int NPROD>
__global__ void __launch_bounds__(G_THREADS, 1)
gemm_bf16_kernel(const __grid_constant__ CUtensorMap tm_a_hi, const __grid_constant__ CUtensorMap tm_a_lo,
                 const __grid_constant__ CUtensorMap tm_b_hi, const __grid_constant__ CUtensorMap tm_b_lo,
                 GemmArgs g) {
    using C = GemmCfg<NPROD>;
    constexpr int NS = C::STAGES;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + NS * C::STAGE_BYTES);
    uint64_t *full = bars, *empty = bars + NS, *tfull = bars + 2 * NS, *tempty = bars + 2 * NS + 2;
    uint64_t *mma_done = bars + 2 * NS + 4;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * NS + 5);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int mt_n = (g.M + G_BM - 1) / G_BM, nt_n = (g.N + G_BN - 1) / G_BN;
    const int n_tiles = mt_n * nt_n * g.ksplit * g.groups;
    const int nkb = (g.K + G_BK - 1) / G_BK;
    int *status = g.status;

    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
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
            int last_fill[NS];
            for (int i = 0; i < NS; ++i) last_fill[i] = -1;
            bool ok = true;
            for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
                const GemmTile t = gemm_tile(g, tile, mt_n, nt_n);
                const int arow = (int)(t.g * g.a_grp) + t.m0;
                const int brow = (int)(t.g * g.b_grp) + g.b_row0 + t.n0;
                const int kb0 = t.s * nkb / g.ksplit, kb1 = (t.s + 1) * nkb / g.ksplit;
                for (int kb = kb0; kb < kb1; ++kb) {
                    if (!mbar_wait(&empty[s], ph ^ 1u, status, ERR_TIMEOUT_PRODUCER)) { ok = false; break; }
                    uint8_t *st = smem + s * C::STAGE_BYTES;
                    mbar_arrive_expect_tx(&full[s], C::STAGE_BYTES);
                    if (NPROD == 3) {
                        tma_load_2d(st, &tm_a_hi, kb * G_BK, arow, &full[s]);
                        tma_load_2d(st + G_A_BYTES, &tm_a_lo, kb * G_BK, arow, &full[s]);
                        tma_load_2d(st + 2 * G_A_BYTES, &tm_b_hi, kb * G_BK, brow, &full[s]);
                        tma_load_2d(st + 2 * G_A_BYTES + G_B_BYTES, &tm_b_lo, kb * G_BK, brow, &full[s]);
                    } else {
                        tma_load_2d(st, &tm_a_hi, kb * G_BK, arow, &full[s]);
                        tma_load_2d(st + G_A_BYTES, &tm_b_hi, kb * G_BK, brow, &full[s]);
                    }
                    last_fill[s] = (int)ph;
                    if (++s == NS) { s = 0; ph ^= 1u; }
                }
            }
            for (int i = 0; i < NS; ++i)
                if (last_fill[i] >= 0) mbar_wait(&full[i], (uint32_t)last_fill[i], status, ERR_TIMEOUT_PRODUCER, false);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            int s = 0; uint32_t ph = 0;
            int acc = 0; uint32_t aph = 0;
            bool ok = true;
            for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
                const GemmTile t = gemm_tile(g, tile, mt_n, nt_n);
                const int kb0 = t.s * nkb / g.ksplit, kb1 = (t.s + 1) * nkb / g.ksplit;
                if (!mbar_wait(&tempty[acc], aph ^ 1u, status, ERR_TIMEOUT_MMA)) { ok = false; break; }
                tc_fence_after();
                const uint32_t d = tmem_base + acc * G_BN;
                const uint32_t idesc = (NPROD == 1 && g.f16) ? idesc_f16_f32(G_BM, G_BN) : G_IDESC;
                for (int kb = kb0; kb < kb1; ++kb) {
                    if (!mbar_wait(&full[s], ph, status, ERR_TIMEOUT_MMA)) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t sa = smem_u32(smem + s * C::STAGE_BYTES);
#pragma unroll
                    for (int k = 0; k < G_BK / 16; ++k) {
                        const uint32_t off = k * 32;
                        const uint32_t first = (kb > kb0 || k > 0) ? 1u : 0u;
                        if (NPROD == 3) {
                            const uint32_t a_hi = sa, a_lo = sa + G_A_BYTES, b_hi = sa + 2 * G_A_BYTES, b_lo = b_hi + G_B_BYTES;
                            mma_bf16(d, sw128_desc(a_hi + off), sw128_desc(b_hi + off), G_IDESC, first);
                            mma_bf16(d, sw128_desc(a_hi + off), sw128_desc(b_lo + off), G_IDESC, 1u);
                            mma_bf16(d, sw128_desc(a_lo + off), sw128_desc(b_hi + off), G_IDESC, 1u);
                        } else {
                            mma_bf16(d, sw128_desc(sa + off), sw128_desc(sa + G_A_BYTES + off), idesc, first);
                        }
                    }
                    mma_commit(&empty[s]);
                    if (++s == NS) { s = 0; ph ^= 1u; }
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
            const GemmTile t = gemm_tile(g, tile, mt_n, nt_n);
            mbar_wait(&tfull[acc], aph, status, ERR_TIMEOUT_EPILOGUE);
            named_bar_sync(1, 128);
            if (*(volatile int *)status != 0) break;
            tc_fence_after();
            const int row = t.m0 + q * 32 + lane;
            const uint32_t trow = tmem_base + ((uint32_t)(q * 32) << 16) + acc * G_BN;
            float *dbase = g.D + t.g * g.d_grp + t.s * g.d_split;
            for (int c = 0; c < G_BN; c += 32) {
                if (t.n0 + c >= g.N) break;
                float v[32];
                tmem_ld32(trow + c, v);
                if (row < g.M) {
                    float *dst = dbase + (size_t)row * g.ldd + t.n0 + c;
                    if (t.n0 + c + 32 <= g.N && ((g.ldd | g.d_grp | g.d_split) & 3) == 0) {
#pragma unroll
                        for (int i = 0; i < 32; i += 4)
                            *reinterpret_cast<float4 *>(dst + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
                    } else {
#pragma unroll
                        for (int i = 0; i < 32; ++i)
                            if (t.n0 + c + i < g.N) dst[i] = v[i];
                    }
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

template <int NPROD>
static cudaError_t launch_gemm(const GemmPlan &pl, const GemmArgs &g, cudaStream_t st) {
    if (g.M <= 0 || g.N <= 0 || g.K <= 0 || g.groups <= 0 || g.ksplit <= 0) return cudaSuccess;
    const int nkb = (g.K + G_BK - 1) / G_BK;
    if (g.ksplit > nkb) return cudaErrorInvalidValue;          // every split needs a K block
    if ((reinterpret_cast<uintptr_t>(g.D) & 15) != 0) return cudaErrorInvalidValue;
    using C = GemmCfg<NPROD>;
    cudaError_t e = cudaFuncSetAttribute(gemm_bf16_kernel<NPROD>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
    if (e != cudaSuccess) return e;
    const long long tiles = (long long)((g.M + G_BM - 1) / G_BM) * ((g.N + G_BN - 1) / G_BN) * g.ksplit * g.groups;
    const int grid = tiles < pl.num_sms ? (int)tiles : pl.num_sms;
    gemm_bf16_kernel<NPROD><<<grid, G_THREADS, C::SMEM, st>>>(pl.tm_a_hi, pl.tm_a_lo, pl.tm_b_hi, pl.tm_b_lo, g);
    return cudaGetLastError();
}

cudaError_t run_gemm_bf16x3(const GemmPlan &pl, const GemmArgs &g, cudaStream_t st) { return launch_gemm<3>(pl, g, st); }
cudaError_t run_gemm_bf16(const GemmPlan &pl, const GemmArgs &g, cudaStream_t st) { return launch_gemm<1>(pl, g, st); }

}  // namespace sps
