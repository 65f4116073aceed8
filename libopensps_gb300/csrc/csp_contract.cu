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
// issuer (and TMEM owner), warps 2..9 = epilogue in two groups of four (group g takes the models of column half g;
// in a group, warp w reads TMEM lanes 32 (w % 4) ..). Accumulators are double-buffered in TMEM so that the
// epilogue of a tile overlaps the MMAs of the next.
//
// Epilogue of a chunk of 16 models, per group: phase 1, thread = pixel row: the attenuated, IGM-absorbed spectrum
// of the 16 models into a staging tile; phase 2, thread = 4 consecutive output pixels of one model: the velocity
// smoothing (taps in registers) and the store.
//
// NACC = 1: one accumulator (no birth-cloud or old-star screen in the batch: young and old are only ever summed).
// NACC = 2: young and old accumulators (the K range is ordered young block first, then old block).
// Nebular emission's escaping ionizing light (frac_obrun above 0, nebular_kernels step 2 of OpenSPS,
// src/physics/opensps_csp_batch.f90:2726-2750): the basis holds the nebular ages' ionizing pixels absorbed (zero), and
// extra K blocks after the old block hold those ages' unabsorbed ionizing spectra against the weights times each
// model's escaping fraction; the ion young blocks accumulate into the young sums and the ion old blocks into the old
// ones. Only the pixel tiles that reach an ionizing pixel run them.
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
constexpr int EPI_GROUPS = 2;
constexpr int EPI_WARPS = 4 * EPI_GROUPS;
constexpr int NTHREADS = (2 + EPI_WARPS) * 32;
constexpr int CHUNK = 16;        // models per epilogue chunk
constexpr int TROW = BM + 4;     // staging row (floats): 16-byte aligned rows, and room for the phase-2 reads

template <int NACC>
struct ContractCfg {
    static constexpr int BN = (NACC == 1) ? 256 : 128;           // models per tile (MMA N)
    static constexpr int A_BYTES = BM * BK * 2;                   // one of A_hi / A_lo
    static constexpr int B_BYTES = BN * BK * 2;
    static constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
    static constexpr int ACC_COLS = NACC * BN;                    // TMEM columns of one accumulator set
    static constexpr int TMEM_COLS = 2 * ACC_COLS;                // double-buffered (= 512)
    static constexpr int GROUP_COLS = BN / EPI_GROUPS;            // models per epilogue group
    static constexpr int STAGE_T_FLOATS = CHUNK * TROW;           // per group
    static constexpr int PAR_FLOATS = 2 * CHUNK * MODEL_PAR_FLOATS;   // per group, double-buffered
    static constexpr int EPI_BYTES = EPI_GROUPS * (STAGE_T_FLOATS + PAR_FLOATS) * 4;
    static constexpr int SMEM_BYTES = NSTAGE * STAGE_BYTES + EPI_BYTES + 256 + 1024;
    static constexpr uint32_t IDESC = idesc_bf16_f32(BM, BN);
};

// 2^x by the SFU (relative error ~2^-22; flushes results below the smallest normal to zero).
__device__ __forceinline__ float ex2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

template <int NACC>
__global__ void __launch_bounds__(NTHREADS, 1)
csp_contract_kernel(const __grid_constant__ CUtensorMap tm_a_hi, const __grid_constant__ CUtensorMap tm_a_lo,
                    const __grid_constant__ CUtensorMap tm_b_hi, const __grid_constant__ CUtensorMap tm_b_lo,
                    ContractArgs args) {
    using C = ContractCfg<NACC>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t *stage_base = smem;
    float *epi_base = reinterpret_cast<float *>(smem + NSTAGE * C::STAGE_BYTES);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + NSTAGE * C::STAGE_BYTES + C::EPI_BYTES);
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
    const int nkb_ion = args.nkb_ion_young + args.nkb_ion_old;
    // K blocks of pixel tile pt: the escaping-light blocks only where the tile reaches an ionizing pixel
    auto tile_nkb = [&](int pt) { return (nkb_ion > 0 && pt * OUT_ROWS - HALO < args.ion_pix) ? nkb + nkb_ion : nkb; };
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
                const int kbn = tile_nkb(pt);
                for (int kb = 0; kb < kbn; ++kb) {
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
                const int kbn = tile_nkb(tile % n_ptiles);
                for (int kb = 0; kb < kbn; ++kb) {
                    if (!mbar_wait(&full[s], ph, status, ERR_TIMEOUT_MMA)) { ok = false; break; }
                    tc_fence_after();
                    // the accumulator of block kb: young / old blocks, then the escaping light's young / old blocks
                    // (which always add to sums their own range has begun: a young ion block exists only with young
                    // ages, an old one only with old ages)
                    const bool ion_old = kb >= nkb + args.nkb_ion_young;
                    const int which = (NACC == 2 && ((kb >= args.nkb_young && kb < nkb) || ion_old)) ? 1 : 0;
                    const uint32_t d = d_base + which * C::BN;
                    const int kfirst = kb >= nkb ? -1 : (which == 0) ? 0 : args.nkb_young;
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
        // ------------------------------------------------------------------ epilogue (warps 2..9)
        const int ew = warp - 2;                // 0..7
        const int g = ew >> 2;                  // group: column half
        const int wg = ew & 3;                  // warp within the group (phase 2: models 4 wg .. 4 wg + 3)
        const int q = warp & 3;                 // TMEM lane quarter this warp may access
        const int r = q * 32 + lane;            // pixel row of the tile (phase 1)
        const int et = wg * 32 + lane;          // 0..127 within the group
        const int bar_id = 1 + g;
        float *stageT = epi_base + g * (C::STAGE_T_FLOATS + C::PAR_FLOATS);
        float *parbuf = stageT + C::STAGE_T_FLOATS;
        const bool vec_store = (args.ld_spec & 1) == 0;
        int acc = 0; uint32_t aph = 0;
        int pb = 0;
        for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
            const int mt = tile / n_ptiles, pt = tile % n_ptiles;
            const int p0 = pt * OUT_ROWS - HALO, m0 = mt * C::BN;
            const int p = p0 + r;
            const bool inpix = (p >= 0 && p < args.nspec);
            // per-pixel data of this thread's row (phase 1)
            float ltab2 = 0.f, curve_u = 1.f, ia[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            float4 tcv = make_float4(0.f, 0.f, 0.f, 0.f);   // the curve tables T0..T3 (models' own tabulated curves)
            if (inpix) {
                const float4 *px = reinterpret_cast<const float4 *>(args.pix + (size_t)p * PIX_FLOATS);
                const float4 v0 = px[0], v1 = px[1];
                ltab2 = v0.x; curve_u = v0.y; ia[0] = v0.z; ia[1] = v0.w;
                ia[2] = v1.x; ia[3] = v1.y; ia[4] = v1.z; ia[5] = v1.w;
                if (args.tab_curve) tcv = px[PIX_T / 4];
            }
            const bool igm_pix = inpix && p < args.jtop;

            mbar_wait(&tfull[acc], aph, status, ERR_TIMEOUT_EPILOGUE);
            // the group agrees on whether to go on (a thread that gave up set the status first)
            named_bar_sync(bar_id, 128);
            if (*(volatile int *)status != 0) break;
            tc_fence_after();
            const uint32_t t_row = tmem_base + ((uint32_t)(q * 32) << 16) + acc * C::ACC_COLS;

            for (int c = 0; c < C::GROUP_COLS / CHUNK; ++c) {
                const int col0 = g * C::GROUP_COLS + c * CHUNK;      // first model of the chunk in the tile
                // model parameters of the chunk (double-buffered)
                float *par = parbuf + pb * CHUNK * MODEL_PAR_FLOATS;
                for (int i = et; i < CHUNK * MODEL_PAR_FLOATS / 4; i += 128) {
                    const int mm = m0 + col0 + (i * 4) / MODEL_PAR_FLOATS;
                    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (mm < args.n_models)
                        v = reinterpret_cast<const float4 *>(args.mpar + (size_t)mm * MODEL_PAR_FLOATS)[(i * 4) % MODEL_PAR_FLOATS / 4];
                    reinterpret_cast<float4 *>(par)[i] = v;
                }
                float y[16];
                tmem_ld16(t_row + col0, y);
                float o[16];
                if constexpr (NACC == 2) {
                    tmem_ld16(t_row + C::BN + col0, o);
                    if (args.nkb_young == 0) {
#pragma unroll
                        for (int j = 0; j < 16; ++j) y[j] = 0.f;
                    }
                    if (args.nkb_old == 0) {
#pragma unroll
                        for (int j = 0; j < 16; ++j) o[j] = 0.f;
                    }
                }
                if (c == C::GROUP_COLS / CHUNK - 1) {
                    // all of this group's accumulator columns have been read: hand them back to the MMA warp
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&tempty[acc]);
                }
                named_bar_sync(bar_id, 128);
                // ---- phase 1: thread = pixel row r, 16 models
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const float *mp = par + j * MODEL_PAR_FLOATS;
                    const float4 d0 = *reinterpret_cast<const float4 *>(mp);          // kd2, 1-fnd, fnd, index
                    const float curve = pix_curve(args.uniform_index, args.tab_curve, curve_u, ltab2, tcv,
                                                  make_float4(mp[MP_CS1], mp[MP_CS1 + 1], mp[MP_CS1 + 2], 0.f), d0.w);
                    float ss;
                    if constexpr (NACC == 2) {
                        if (args.young && inpix && r >= HALO && r < BM - HALO && m0 + col0 + j < args.n_models) {
                            // the parts: young and old age sums before dust (compute_csp_batch_parts)
                            args.young[(size_t)(m0 + col0 + j) * args.ld_spec + p] = y[j];
                            args.old[(size_t)(m0 + col0 + j) * args.ld_spec + p] = o[j];
                        }
                        const float4 d1 = *reinterpret_cast<const float4 *>(mp + 4);  // kd1, d1 index, 1-fo, fo
                        const float kd3 = mp[MP_KD3];
                        const float tb = (d1.x != 0.f) ? ex2(d1.x * ex2(d1.y * ltab2)) : 1.f;
                        const float to = (kd3 != 0.f) ? ex2(kd3 * curve) : 1.f;
                        ss = (y[j] * tb * d1.z + y[j] * d1.w) + o[j] * to;
                    } else {
                        ss = y[j];
                    }
                    float tot = ss * fmaf(ex2(d0.x * curve), d0.y, d0.z);
                    if (igm_pix) {
                        const float4 g0 = *reinterpret_cast<const float4 *>(mp + MP_IGM_ON);   // on, jmax, kcap, kd3
                        if (g0.x != 0.f) {
                            float arg;
                            if (p < __float_as_int(g0.y)) {
                                arg = g0.z;
                            } else {
                                const float4 g1 = *reinterpret_cast<const float4 *>(mp + MP_IGM_KB);   // kb0..kb3
                                const float2 g2 = *reinterpret_cast<const float2 *>(mp + MP_IGM_KB + 4);  // kb4, kb5
                                arg = ia[0] * g1.x + ia[1] * g1.y + ia[2] * g1.z + ia[3] * g1.w + ia[4] * g2.x +
                                      ia[5] * g2.y;
                            }
                            tot *= ex2(arg);
                        }
                    }
                    stageT[j * TROW + r] = tot;
                }
                named_bar_sync(bar_id, 128);
                // ---- phase 2: warp wg takes models 4 wg .. 4 wg + 3; lane l the output rows 4 + 4l .. 7 + 4l (no
                // spectra when a per-model epilogue forms them from the young and old sums)
                if (args.spec != nullptr && lane < OUT_ROWS / 4) {
                    const int row0 = HALO + 4 * lane;
                    const int pq = p0 + row0;                      // first output pixel of this lane
#pragma unroll 1
                    for (int jj = 0; jj < 4; ++jj) {
                        const int j = wg * 4 + jj;
                        const int mm = m0 + col0 + j;
                        if (mm >= args.n_models || pq >= args.nspec) continue;
                        const float *mp = par + j * MODEL_PAR_FLOATS;
                        const float *row = stageT + j * TROW + row0 - HALO;   // 16-byte aligned
                        const float4 w0 = *reinterpret_cast<const float4 *>(row);
                        const float4 w1 = *reinterpret_cast<const float4 *>(row + 4);
                        const float4 w2 = *reinterpret_cast<const float4 *>(row + 8);
                        const float win[12] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w, w2.x, w2.y, w2.z, w2.w};
                        float out[4] = {win[4], win[5], win[6], win[7]};
                        const int R = __float_as_int(mp[MP_SMOOTH_R]);
                        if (R >= 0 && pq + 3 >= args.sm_lo && pq <= args.sm_hi) {
                            const float4 ta = *reinterpret_cast<const float4 *>(mp + MP_TAPS);
                            const float4 tb = *reinterpret_cast<const float4 *>(mp + MP_TAPS + 4);
                            const float tc = mp[MP_TAPS + 8];
                            const float tap[9] = {ta.x, ta.y, ta.z, ta.w, tb.x, tb.y, tb.z, tb.w, tc};
#pragma unroll
                            for (int u = 0; u < 4; ++u) {
                                const int pu = pq + u;
                                if (pu < args.sm_lo || pu > args.sm_hi) continue;
                                float s = 0.f;
#pragma unroll
                                for (int d = 0; d < 9; ++d) s = fmaf(tap[d], win[u + d], s);
                                out[u] = s;
                            }
                        }
                        float *dst = args.spec + (size_t)mm * args.ld_spec + pq;
                        if (vec_store && pq + 3 < args.nspec) {
                            reinterpret_cast<float2 *>(dst)[0] = make_float2(out[0], out[1]);
                            reinterpret_cast<float2 *>(dst)[1] = make_float2(out[2], out[3]);
                        } else {
#pragma unroll
                            for (int u = 0; u < 4; ++u)
                                if (pq + u < args.nspec) dst[u] = out[u];
                        }
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
