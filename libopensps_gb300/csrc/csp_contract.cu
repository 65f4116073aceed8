// The CSP contraction with its fused per-pixel epilogue, on the 5th-generation tensor cores.
//
//   spec(p, m) = S( [ young(p, m) (T_birth (1 - frac_obrun) + frac_obrun) + old(p, m) T_dust3 ]
//                   (T_diffuse (1 - frac_nodust) + frac_nodust) T_igm(p, m) )
//   young / old(p, m) = sum_k basis(p, k) w(k, m) over the ages <= / > dust_tesc (k = age x metallicity)
//
// (OpenSPS compute_csp_batch stages 3-7: age_sums_w src/physics/opensps_csp_batch.f90:2269-2324, attenuate_batch
// :3576-3660, apply_igm_z :4205-4299, smoothing src/spectra/opensps_smoothing.f90:553-633.) The nebular lines are in
// the basis already (they are linear in the weights: the basis holds each young SSP with its lines).
//
// Matrix form: D(pixels x models) = basis(pixels x K) . W(models x K)^T, both operands K-major bf16 split into hi and
// lo parts (x = x_hi + x_lo); D = A_hi B_hi + A_hi B_lo + A_lo B_hi, accumulated in f32 in tensor memory. Tile: 128
// pixels x BN models x 64 K per stage; the 128 pixel rows of a tile are 120 output pixels with a halo of 4 on each
// side for the smoothing. One CTA per SM, persistent over tiles (model tile outer, pixel tile inner, so that the
// CTAs running together share the weights of a model tile in L2). Warp roles: warp 0 = TMA producer, warp 1 = MMA
// issuer (and TMEM owner), warps 2..5 = epilogue (TMEM lanes 32 (warp % 4) ..). Accumulators are double-buffered in
// TMEM so that the epilogue of a tile overlaps the MMAs of the next.
//
// NACC = 1: one accumulator (no birth-cloud or old-star screen in the batch: young and old are only ever summed).
// NACC = 2: young and old accumulators (the K range is ordered young block first, then old block).
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cstdint>
#include "sm103_ptx.cuh"
#include "csp_kernels.h"

namespace sps {

constexpr int BM = 128;          // pixel rows per tile (MMA M)
constexpr int BK = 64;           // K per stage (one 128-byte swizzled row of bf16)
constexpr int HALO = 4;          // smoothing halo (taps -4 .. 4)
constexpr int OUT_ROWS = BM - 2 * HALO;
constexpr int NSTAGE = 2;
constexpr int EPI_WARPS = 4;
constexpr int NTHREADS = (2 + EPI_WARPS) * 32;
constexpr int TROW = BM + 4;     // epilogue staging row (floats), padded

template <int NACC>
struct ContractCfg {
    static constexpr int BN = (NACC == 1) ? 256 : 128;           // models per tile (MMA N)
    static constexpr int A_BYTES = BM * BK * 2;                   // one of A_hi / A_lo
    static constexpr int B_BYTES = BN * BK * 2;
    static constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
    static constexpr int ACC_COLS = NACC * BN;                    // TMEM columns of one accumulator set
    static constexpr int TMEM_COLS = 2 * ACC_COLS;                // double-buffered (= 512)
    static constexpr int STAGE_T_BYTES = 32 * TROW * 4;           // epilogue staging, 32 models
    static constexpr int PAR_BYTES = 2 * 32 * MODEL_PAR_FLOATS * 4;
    static constexpr int SMEM_BYTES = NSTAGE * STAGE_BYTES + STAGE_T_BYTES + PAR_BYTES + 256 + 1024;
    static constexpr uint32_t IDESC = idesc_bf16_f32(BM, BN);
};

__device__ __forceinline__ float fast_exp(float x) { return exp2f(x * 1.4426950408889634f); }

template <int NACC>
__global__ void __launch_bounds__(NTHREADS, 1)
csp_contract_kernel(const __grid_constant__ CUtensorMap tm_a_hi, const __grid_constant__ CUtensorMap tm_a_lo,
                    const __grid_constant__ CUtensorMap tm_b_hi, const __grid_constant__ CUtensorMap tm_b_lo,
                    ContractArgs args) {
    using C = ContractCfg<NACC>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t *stage_base = smem;
    float *stageT = reinterpret_cast<float *>(smem + NSTAGE * C::STAGE_BYTES);
    float *parbuf = reinterpret_cast<float *>(smem + NSTAGE * C::STAGE_BYTES + C::STAGE_T_BYTES);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + NSTAGE * C::STAGE_BYTES + C::STAGE_T_BYTES + C::PAR_BYTES);
    uint64_t *full = bars;                 // [NSTAGE]
    uint64_t *empty = bars + NSTAGE;       // [NSTAGE]
    uint64_t *tfull = bars + 2 * NSTAGE;   // [2]
    uint64_t *tempty = bars + 2 * NSTAGE + 2;
    uint64_t *mma_done = bars + 2 * NSTAGE + 4;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 2 * NSTAGE + 5);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n_ptiles = args.n_ptiles;
    const int n_tiles = n_ptiles * args.n_mtiles;
    const int nkb = args.nkb_young + args.nkb_old;
    int *status = args.status;

    if (threadIdx.x == 0) {
        for (int s = 0; s < NSTAGE; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
        for (int b = 0; b < 2; ++b) { mbar_init(&tfull[b], 1); mbar_init(&tempty[b], EPI_WARPS); }
        mbar_init(mma_done, 1);
        fence_mbar_init();
    }
    if (warp == 1) { tmem_alloc(tmem_slot, C::TMEM_COLS); tmem_relinquish(); }
    if (warp == 0 && lane == 0) {
        tma_prefetch_desc(&tm_a_hi); tma_prefetch_desc(&tm_a_lo);
        tma_prefetch_desc(&tm_b_hi); tma_prefetch_desc(&tm_b_lo);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    if (warp == 0) {
        // ------------------------------------------------------------------ TMA producer
        if (lane == 0) {
            int s = 0; uint32_t ph = 0;
            int last_fill[NSTAGE];              // parity of the last fill issued into each stage, -1: none
            for (int i = 0; i < NSTAGE; ++i) last_fill[i] = -1;
            bool ok = true;
            for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
                const int mt = tile / n_ptiles, pt = tile % n_ptiles;
                const int p0 = pt * OUT_ROWS - HALO, m0 = mt * C::BN;
                for (int kb = 0; kb < nkb; ++kb) {
                    if (!mbar_wait(&empty[s], ph ^ 1u, status, ERR_TIMEOUT_PRODUCER)) { ok = false; break; }
                    uint8_t *st = stage_base + s * C::STAGE_BYTES;
                    mbar_arrive_expect_tx(&full[s], C::STAGE_BYTES);
                    tma_load_2d(st, &tm_a_hi, kb * BK, p0, &full[s]);
                    tma_load_2d(st + C::A_BYTES, &tm_a_lo, kb * BK, p0, &full[s]);
                    tma_load_2d(st + 2 * C::A_BYTES, &tm_b_hi, kb * BK, m0, &full[s]);
                    tma_load_2d(st + 2 * C::A_BYTES + C::B_BYTES, &tm_b_lo, kb * BK, m0, &full[s]);
                    last_fill[s] = (int)ph;
                    if (++s == NSTAGE) { s = 0; ph ^= 1u; }
                }
            }
            // Drain: every copy this thread issued must have landed before the CTA may exit.
            for (int i = 0; i < NSTAGE; ++i)
                if (last_fill[i] >= 0) mbar_wait(&full[i], (uint32_t)last_fill[i], status, ERR_TIMEOUT_PRODUCER, false);
        }
    } else if (warp == 1) {
        // ------------------------------------------------------------------ MMA issuer
        if (lane == 0) {
            int s = 0; uint32_t ph = 0;
            int acc = 0; uint32_t aph = 0;
            bool ok = true;
            for (int tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
                if (!mbar_wait(&tempty[acc], aph ^ 1u, status, ERR_TIMEOUT_MMA)) { ok = false; break; }
                tc_fence_after();
                const uint32_t d_base = tmem_base + acc * C::ACC_COLS;
                for (int kb = 0; kb < nkb; ++kb) {
                    if (!mbar_wait(&full[s], ph, status, ERR_TIMEOUT_MMA)) { ok = false; break; }
                    tc_fence_after();
                    const int which = (NACC == 2 && kb >= args.nkb_young) ? 1 : 0;
                    const uint32_t d = d_base + which * C::BN;
                    const int kfirst = (which == 0) ? 0 : args.nkb_young;
                    const uint32_t sa = smem_u32(stage_base + s * C::STAGE_BYTES);
                    const uint32_t a_hi = sa, a_lo = sa + C::A_BYTES;
                    const uint32_t b_hi = sa + 2 * C::A_BYTES, b_lo = b_hi + C::B_BYTES;
#pragma unroll
                    for (int k = 0; k < BK / 16; ++k) {
                        const uint32_t off = k * 32;
                        const uint32_t accum = (kb > kfirst || k > 0) ? 1u : 0u;
                        mma_bf16(d, sw128_desc(a_hi + off), sw128_desc(b_hi + off), C::IDESC, accum);
                        mma_bf16(d, sw128_desc(a_hi + off), sw128_desc(b_lo + off), C::IDESC, 1u);
                        mma_bf16(d, sw128_desc(a_lo + off), sw128_desc(b_hi + off), C::IDESC, 1u);
                    }
                    mma_commit(&empty[s]);          // frees the stage once these MMAs have read it
                    if (++s == NSTAGE) { s = 0; ph ^= 1u; }
                }
                if (!ok) break;
                mma_commit(&tfull[acc]);            // accumulator ready for the epilogue
                if (++acc == 2) { acc = 0; aph ^= 1u; }
            }
            // Every MMA issued by this thread must be complete before the TMEM is released.
            mma_commit(mma_done);
            mbar_wait(mma_done, 0, status, ERR_TIMEOUT_MMA, false);
        }
    } else {
        // ------------------------------------------------------------------ epilogue (warps 2..5)
        const int q = warp & 3;                 // TMEM lane quarter this warp may access
        const int r = q * 32 + lane;            // pixel row of the tile
        const int et = threadIdx.x - 64;        // 0..127
        int acc = 0; uint32_t aph = 0;
        int pb = 0;
        for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
            const int mt = tile / n_ptiles, pt = tile % n_ptiles;
            const int p0 = pt * OUT_ROWS - HALO, m0 = mt * C::BN;
            const int p = p0 + r;
            const bool inpix = (p >= 0 && p < args.nspec);
            // per-pixel data
            float ltab = 0.f, ia[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            bool sm_active = false;
            if (inpix) {
                const float *px = args.pix + (size_t)p * PIX_FLOATS;
                ltab = px[PIX_LTAB];
#pragma unroll
                for (int k = 0; k < 6; ++k) ia[k] = px[PIX_IGM_A + k];
                sm_active = px[PIX_SMOOTH] != 0.f;
            }
            const bool out_row = (r >= HALO && r < BM - HALO && inpix);
            const bool igm_pix = inpix && p < args.jtop;

            mbar_wait(&tfull[acc], aph, status, ERR_TIMEOUT_EPILOGUE);
            // all epilogue threads agree on whether to go on (a thread that gave up set the status first)
            named_bar_sync(1, 128);
            if (*(volatile int *)status != 0) break;
            tc_fence_after();
            const uint32_t t_row = tmem_base + ((uint32_t)(q * 32) << 16) + acc * C::ACC_COLS;

            for (int c = 0; c < C::BN / 32; ++c) {
                // model parameters of this chunk of 32 models (double-buffered)
                float *par = parbuf + pb * 32 * MODEL_PAR_FLOATS;
                for (int i = et; i < 32 * MODEL_PAR_FLOATS; i += 128) {
                    const int mm = m0 + c * 32 + i / MODEL_PAR_FLOATS;
                    par[i] = (mm < args.n_models) ? args.mpar[(size_t)mm * MODEL_PAR_FLOATS + (i % MODEL_PAR_FLOATS)] : 0.f;
                }
                float y[32];
                tmem_ld32(t_row + c * 32, y);
                float o[32];
                if constexpr (NACC == 2) {
                    tmem_ld32(t_row + C::BN + c * 32, o);
                    if (args.nkb_young == 0) {
#pragma unroll
                        for (int j = 0; j < 32; ++j) y[j] = 0.f;
                    }
                    if (args.nkb_old == 0) {
#pragma unroll
                        for (int j = 0; j < 32; ++j) o[j] = 0.f;
                    }
                }
                if (c == C::BN / 32 - 1) {
                    // all of this accumulator has been read: hand it back to the MMA warp
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&tempty[acc]);
                }
                named_bar_sync(1, 128);
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const float *mp = par + j * MODEL_PAR_FLOATS;
                    const float ed = mp[MP_DUST_INDEX];
                    const float curve = (ed != 0.f) ? fast_exp(ed * ltab) : 1.f;
                    const float td = fast_exp(-mp[MP_DUST2] * curve);
                    float ss;
                    if constexpr (NACC == 2) {
                        float tb = 1.f, to = 1.f;
                        if (mp[MP_DUST1] != 0.f) tb = fast_exp(-mp[MP_DUST1] * fast_exp(mp[MP_DUST1_INDEX] * ltab));
                        if (mp[MP_DUST3] != 0.f) to = fast_exp(-mp[MP_DUST3] * curve);
                        ss = (y[j] * tb * mp[MP_ONE_M_FO] + y[j] * mp[MP_FO]) + o[j] * to;
                    } else {
                        ss = y[j];
                    }
                    float tot = ss * (td * mp[MP_ONE_M_FND] + mp[MP_FND]);
                    if (igm_pix && mp[MP_IGM_ON] != 0.f) {
                        const int jmax = __float_as_int(mp[MP_IGM_JMAX]);
                        float tau;
                        if (p < jmax) tau = mp[MP_IGM_TMAX];
                        else tau = ia[0] * mp[MP_IGM_B + 0] + ia[1] * mp[MP_IGM_B + 1] + ia[2] * mp[MP_IGM_B + 2] +
                                   ia[3] * mp[MP_IGM_B + 3] + ia[4] * mp[MP_IGM_B + 4] + ia[5] * mp[MP_IGM_B + 5];
                        tot *= fast_exp(-tau * mp[MP_IGM_FACTOR]);
                    }
                    stageT[j * TROW + r] = tot;
                }
                named_bar_sync(1, 128);
                if (out_row) {
#pragma unroll 4
                    for (int j = 0; j < 32; ++j) {
                        const int mm = m0 + c * 32 + j;
                        if (mm >= args.n_models) break;
                        const float *mp = par + j * MODEL_PAR_FLOATS;
                        const float *row = stageT + j * TROW + r;
                        float v = row[0];
                        const int R = __float_as_int(mp[MP_SMOOTH_R]);
                        if (R >= 0 && sm_active) {
                            float s = 0.f;
#pragma unroll
                            for (int d = -HALO; d <= HALO; ++d) s = fmaf(mp[MP_TAPS + HALO + d], row[d], s);
                            v = s;
                        }
                        args.spec[(size_t)mm * args.ld_spec + p] = v;
                    }
                }
                pb ^= 1;
            }
            if (++acc == 2) { acc = 0; aph ^= 1u; }
        }
    }

    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem_base, C::TMEM_COLS);
    }
}

// ---------------------------------------------------------------------------------------------- host side
template <int NACC>
static cudaError_t launch_contract(const ContractPlan &pl, const ContractArgs &a, cudaStream_t st) {
    using C = ContractCfg<NACC>;
    auto kern = csp_contract_kernel<NACC>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    const int n_tiles = a.n_ptiles * a.n_mtiles;
    const int grid = n_tiles < pl.num_sms ? n_tiles : pl.num_sms;
    kern<<<grid, NTHREADS, C::SMEM_BYTES, st>>>(pl.tm_a_hi, pl.tm_a_lo, pl.tm_b_hi, pl.tm_b_lo, a);
    return cudaGetLastError();
}

int contract_models_per_tile(int nacc) { return nacc == 1 ? ContractCfg<1>::BN : ContractCfg<2>::BN; }
int contract_out_rows() { return OUT_ROWS; }
int contract_halo() { return HALO; }
int contract_bk() { return BK; }
int contract_bm() { return BM; }

cudaError_t run_contract(int nacc, const ContractPlan &pl, const ContractArgs &a, cudaStream_t st) {
    return nacc == 1 ? launch_contract<1>(pl, a, st) : launch_contract<2>(pl, a, st);
}

}  // namespace sps
