// The emulator's inference: one fused persistent kernel per SM that runs the five members of the ensemble over a
// tile of 128 models, layer after layer, without leaving the SM.
//
// Per tile and member, five dense layers (12 features -> 512 -> 512 -> 512 -> 512 -> 128 outputs). Each hidden layer
// is two N chunks of 256 outputs (the output layer one chunk of 128): D(models x 256) = A(models x K) W(256 x K)^T
// on tcgen05 (M = 128 models, f16, f32 accumulator in TMEM). N = 256: on this GPU an N = 128 MMA takes as long as
// an N = 256 one. The activations never leave the SM and alternate between two homes:
//   input (S, K block 0) -> h1 (T) -> h2 (S) -> h3 (T) -> h4 (S) -> outputs (scratch)
// where S is shared memory (128 x 512 f16, eight 16 KB K blocks in the 128-byte swizzle: the MMA's A descriptor)
// and T is tensor memory (256 columns, two f16 per column: the MMA's A operand from TMEM). A layer reads one home
// and its epilogue writes the other. The accumulator (256 columns) is single-buffered: the epilogue first drains
// its 64 columns of the chunk into registers and releases the accumulator, so that the next chunk's MMAs run while
// it adds the biases, applies SiLU and stores the f16 activations; the next layer's first chunk starts on the
// 256 features already written (a ready barrier per 256 features).
// The weights stream through a three-stage TMA ring of 256 x 64 f16 tiles (32 KB), each CTA loading its own tiles
// (no clusters); the CTAs start on different members so that their reads spread over L2.
//
// Warp 0: TMA producer; warp 1: MMA issuer (one thread) and TMEM owner; warps 2..17: epilogue, four warps per
// TMEM lane quarter (one model row per thread, 64 of a chunk's 256 columns each). Each member's outputs go to the
// CTA's scratch (L2-resident); after the last member, each row's ensemble mean, spread (the population standard
// deviation over the members, the largest over the bands that are less than `faint` mag fainter than the
// brightest) and flag are formed from there.
//
// Every mbarrier wait is bounded (status word, no hang); drains wait for the copies and MMAs in flight.
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <algorithm>
#include <cmath>
#include <cstdint>
#include "sm103_ptx.cuh"
#include "csp_kernels.h"
#include "emulator.h"

namespace sps {

constexpr int EI_EPI_WARPS = 16;
constexpr int EI_THREADS = (2 + EI_EPI_WARPS) * 32;
constexpr int EI_NS = 3;                          // weight stages
constexpr int EI_KBLK = 128 * 64 * 2;             // one 128-row x 64 f16 K block of the activations (16 KB)
constexpr int EI_STAGE = 256 * 64 * 2;            // one 256 x 64 f16 weight tile (32 KB)
constexpr int EI_S_BYTES = 8 * EI_KBLK;           // activations: 8 K blocks
constexpr int EI_SMEM = EI_S_BYTES + EI_NS * EI_STAGE + 256 + 1024;
constexpr uint32_t EI_IDESC256 = idesc_f16_f32(128, 256), EI_IDESC128 = idesc_f16_f32(128, 128);
constexpr uint32_t EI_T_COL = 0, EI_ACC_COL = 256;
constexpr int EI_ROWS = 256;                      // rows of a hidden-layer weight tile (one TMA box)
constexpr int EI_ROWS4 = 128;                     // the same for the output layer's 128-row tiles

__device__ __forceinline__ float silu_fast(float z) {
    const float hz = 0.5f * z;
    return fmaf(hz, tanh_approx(hz), hz);          // z sigmoid(z) = hz (1 + tanh(hz))
}
__device__ __forceinline__ uint32_t pack_f16(float a, float b) {
    __half2 v = __floats2half2_rn(a, b);
    return *reinterpret_cast<uint32_t *>(&v);
}
// x = hi + lo, both f16 (the input's rounding error carried by the lo part)
__device__ __forceinline__ float f16_lo(float x) { return x - __half2float(__float2half_rn(x)); }
// byte offset of (row r, 16-byte chunk j) in a 128-row tile with the 128-byte swizzle
__device__ __forceinline__ uint32_t sw128_off(int r, int j) {
    return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((j ^ (r & 7)) << 4));
}
__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}

// The distance term of the magnitudes (as the batch's: 5 log10(d_L / 10 pc) - 2.5 log10(1 + z), zero at z = 0), on
// an FP32 copy of the cosmology table.
__device__ __forceinline__ float emu_distance(float z, const float *zt, const float *dl) {
    if (!(z > 0.f)) return 0.f;
    // the interval of find_interval0 (the table's redshifts fall with the index)
    const bool asc = zt[499] >= zt[0];
    int lower = 0, upper = 501;
    while (upper - lower > 1) {
        const int mid = (upper + lower) >> 1;
        if (asc == (z >= zt[mid - 1])) lower = mid; else upper = mid;
    }
    int lo = (z == zt[0]) ? 0 : (z == zt[499]) ? 498 : lower - 1;
    lo = min(max(lo, 0), 498);
    const float dm = dl[lo] + (dl[lo + 1] - dl[lo]) / (zt[lo + 1] - zt[lo]) * (z - zt[lo]);
    if (!(dm > 0.f)) return 0.f;
    return 5.f * log10f(dm * 0.1f) - 2.5f * log10f(1.f + z);
}

// The member a CTA runs at step mem of each tile: the order is rotated by the CTA index, so that the CTAs stream
// different members' weights at a time instead of all reading the same tiles from the same L2 lines.
__device__ __forceinline__ int emu_member(int mem) { return (mem + (int)blockIdx.x) % EMU_MEMBERS; }
// Tiles per CTA: the same count in every CTA, the ones past the last tile are run with no valid model.
__device__ __forceinline__ int emu_iters(int ntiles) { return (ntiles + (int)gridDim.x - 1) / (int)gridDim.x; }

// A warp-uniform bounded wait (every lane polls; the warp goes on only if all saw the phase complete).
__device__ __forceinline__ bool warp_wait(uint64_t *bar, uint32_t parity, int *status, int code) {
    const bool w = mbar_wait(bar, parity, status, code);
    return __all_sync(0xffffffffu, w);
}

// 32 consecutive 32-bit TMEM columns without the wait (the caller waits once for several loads).
__device__ __forceinline__ void tmem_ld32_nowait(uint32_t taddr, uint32_t *r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// The epilogue warps: lane quarter q (TMEM lanes 32q..32q+31, model rows), column slice cs (64 of a hidden chunk's
// 256 columns; 32 of the output chunk's 128).
__device__ __forceinline__ void emu_epilogue(const EmuInferArgs &a, uint8_t *S, uint64_t *bars, uint32_t tmem_base,
                                             int q, int cs, int lane) {
    uint64_t *afull = bars + 2 * EI_NS, *aempty = afull + 1, *hrdy = aempty + 1, *inrdy = hrdy + 2;
    const int r = q * 32 + lane;
    const uint32_t lane_base = (uint32_t)(q * 32) << 16;
    const uint32_t s_base = smem_u32(S);
    const float *par = a.par;
    const int ntiles = (a.n + 127) / 128;
    const int iters = emu_iters(ntiles);
    int *status = a.status;
    // this row's outputs of each member: scratch[cta][member][row][128]; then, per CTA, two slots x 128 rows x 16
    // words of tile inputs (the input row's 12 f16 words, zred, the flags)
    float *scr_row = a.scratch + ((size_t)blockIdx.x * EMU_SCRATCH_CTA + (size_t)r * EMU_NOUT);
    uint4 *in_row = reinterpret_cast<uint4 *>(a.scratch + (size_t)blockIdx.x * EMU_SCRATCH_CTA +
                                             (size_t)EMU_MEMBERS * 128 * EMU_NOUT) + (size_t)r * 4;
    constexpr size_t SCR_MEM = (size_t)128 * EMU_NOUT;
    uint32_t g = 0;
    bool ok = true;
    // the input words and flags of tile `tile` into slot `slot` (cs = 0 warps, one row each)
    auto prepare_input = [&](int tile, int slot) {
        if (cs != 0) return;
        const int m = tile * 128 + r;
        float xs[EMU_NFEAT];
        float zred = 0.f;
        uint32_t flags = 0;                      // bit 0: outside the box, bit 1: not finite
        bool use = m < a.n;
        if (use) {
            float x[EMU_NIN];
#pragma unroll
            for (int i = 0; i < EMU_NIN; ++i) x[i] = __ldg(a.x + (size_t)m * EMU_NIN + i);
            zred = x[5];
            if (!emu_features(x, par, xs)) flags |= 1u;
#pragma unroll
            for (int i = 0; i < EMU_NFEAT; ++i)
                if (!isfinite(xs[i])) use = false;
            if (!use) flags |= 2u;
        }
        if (!use) {
#pragma unroll
            for (int i = 0; i < EMU_NFEAT; ++i) xs[i] = 0.f;
        }
        uint32_t w[12];
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            w[i] = pack_f16(xs[2 * i], xs[2 * i + 1]);
            w[6 + i] = pack_f16(f16_lo(xs[2 * i]), f16_lo(xs[2 * i + 1]));
        }
        uint4 *dst = in_row + (size_t)slot * 128 * 4;
        dst[0] = make_uint4(w[0], w[1], w[2], w[3]);
        dst[1] = make_uint4(w[4], w[5], w[6], w[7]);
        dst[2] = make_uint4(w[8], w[9], w[10], w[11]);
        dst[3] = make_uint4(__float_as_uint(zred), flags, 0u, 0u);
    };
    // the input row into K block 0 of S (f16: the features' hi parts at K 0..11, lo parts at 16..27), from slot
    // `slot`; every epilogue warp arrives
    auto put_input = [&](int slot) {
        if (cs == 0) {
            const uint4 *src = in_row + (size_t)slot * 128 * 4;
            const uint4 w0 = src[0], w1 = src[1], w2 = src[2];
            st_shared_v4(s_base + sw128_off(r, 0), w0.x, w0.y, w0.z, w0.w);
            st_shared_v4(s_base + sw128_off(r, 1), w1.x, w1.y, 0u, 0u);
            st_shared_v4(s_base + sw128_off(r, 2), w1.z, w1.w, w2.x, w2.y);
            st_shared_v4(s_base + sw128_off(r, 3), w2.z, w2.w, 0u, 0u);
            fence_proxy_async_smem();
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(inrdy);
    };
    prepare_input(blockIdx.x, 0);
    put_input(0);
    for (int it = 0; it < iters && ok; ++it) {
        const int tile = blockIdx.x + it * gridDim.x;
        const int m = tile * 128 + r;
        for (int mem = 0; mem < EMU_MEMBERS && ok; ++mem) {
            const float *bm = a.bias + (size_t)emu_member(mem) * EMU_NBIAS;
            for (int L = 0; L < 5 && ok; ++L) {
                const int nch = L == 4 ? 1 : 2;
                for (int c = 0; c < nch; ++c) {
                    if (!warp_wait(afull, g & 1u, status, ERR_TIMEOUT_EPILOGUE)) { ok = false; break; }
                    ++g;
                    tc_fence_after();
                    if (L < 4) {
                        // drain this slice (64 columns) and release the accumulator
                        uint32_t v[64];
                        const uint32_t ta = tmem_base + lane_base + EI_ACC_COL + cs * 64;
                        tmem_ld32_nowait(ta, v);
                        tmem_ld32_nowait(ta + 32, v + 32);
                        tmem_wait_ld();
                        tc_fence_before();
                        __syncwarp();
                        if (lane == 0) mbar_arrive(aempty);
                        // bias, SiLU, f16 in groups of 16 features
                        const float4 *b4 = reinterpret_cast<const float4 *>(bm + L * EMU_H + c * 256 + cs * 64);
                        const uint32_t blk = s_base + (uint32_t)(c * 4 + cs) * EI_KBLK;   // h2, h4: K block 4c + cs
#pragma unroll
                        for (int grp = 0; grp < 4; ++grp) {
                            float b[16];
#pragma unroll
                            for (int i = 0; i < 4; ++i) {
                                const float4 t = __ldg(b4 + grp * 4 + i);
                                b[4 * i] = t.x; b[4 * i + 1] = t.y; b[4 * i + 2] = t.z; b[4 * i + 3] = t.w;
                            }
                            uint32_t pk[8];
#pragma unroll
                            for (int i = 0; i < 8; ++i)
                                pk[i] = pack_f16(silu_fast(__uint_as_float(v[grp * 16 + 2 * i]) + b[2 * i]),
                                                 silu_fast(__uint_as_float(v[grp * 16 + 2 * i + 1]) + b[2 * i + 1]));
                            if ((L & 1) == 0) {
                                // h1 (L = 0), h3 (L = 2) into tensor memory: features c*256 + cs*64 + grp*16 ...
                                tmem_st8(tmem_base + lane_base + EI_T_COL + c * 128 + cs * 32 + grp * 8, pk);
                            } else {
                                // h2 (L = 1), h4 (L = 3) into shared memory: 16-byte chunks 2 grp, 2 grp + 1
                                st_shared_v4(blk + sw128_off(r, 2 * grp), pk[0], pk[1], pk[2], pk[3]);
                                st_shared_v4(blk + sw128_off(r, 2 * grp + 1), pk[4], pk[5], pk[6], pk[7]);
                            }
                        }
                        if ((L & 1) == 0) {
                            tmem_wait_st();
                            tc_fence_before();
                        } else {
                            fence_proxy_async_smem();
                        }
                        __syncwarp();
                        if (lane == 0) mbar_arrive(&hrdy[c]);
                        // the next tile's inputs, where the epilogue has time to spare
                        if (mem == 0 && L == 1 && c == 0 && it + 1 < iters) prepare_input(tile + gridDim.x, (it + 1) & 1);
                    } else {
                        // the output chunk (128 columns): this slice's 32
                        uint32_t v[32];
                        tmem_ld32_nowait(tmem_base + lane_base + EI_ACC_COL + cs * 32, v);
                        tmem_wait_ld();
                        tc_fence_before();
                        __syncwarp();
                        if (lane == 0) mbar_arrive(aempty);
                        // S is free (the output layer's MMAs are done): the next member's input row, or the next
                        // tile's after the last member
                        if (mem + 1 < EMU_MEMBERS) put_input(it & 1);
                        else if (it + 1 < iters) put_input((it + 1) & 1);
                        const float4 *b4 = reinterpret_cast<const float4 *>(bm + 4 * EMU_H + cs * 32);
                        float4 *dst = reinterpret_cast<float4 *>(scr_row + mem * SCR_MEM + cs * 32);
#pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            const float4 t = __ldg(b4 + i);
                            dst[i] = make_float4(__uint_as_float(v[4 * i]) + t.x, __uint_as_float(v[4 * i + 1]) + t.y,
                                                 __uint_as_float(v[4 * i + 2]) + t.z, __uint_as_float(v[4 * i + 3]) + t.w);
                        }
                    }
                }
            }
        }
        // ---- the ensemble's outputs of the quarter's rows: the four slices' scratch writes are in. The barrier is
        // passed by all four warps whatever happened, and they stop together if any of them, or the status word,
        // says so (a wait that gave up)
        if (named_bar_or(1 + q, 128, !ok || *(volatile int *)status != 0)) break;
        if (m >= a.n) continue;
        const float invm = 1.f / (float)EMU_MEMBERS;
        if (cs < 2) {
            if (a.coef) {
                float *dst = a.coef + (size_t)m * EMU_NPC + cs * 32;
#pragma unroll 2
                for (int j = 0; j < 32; j += 4) {
                    const int col = cs * 32 + j;
                    float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                    for (int k = 0; k < EMU_MEMBERS; ++k) {
                        const float4 t = *reinterpret_cast<const float4 *>(scr_row + k * SCR_MEM + col);
                        sum.x += t.x; sum.y += t.y; sum.z += t.z; sum.w += t.w;
                    }
                    float4 o;
                    o.x = par[EMU_P_OMU + col] + par[EMU_P_OSIG + col] * sum.x * invm;
                    o.y = par[EMU_P_OMU + col + 1] + par[EMU_P_OSIG + col + 1] * sum.y * invm;
                    o.z = par[EMU_P_OMU + col + 2] + par[EMU_P_OSIG + col + 2] * sum.z * invm;
                    o.w = par[EMU_P_OMU + col + 3] + par[EMU_P_OSIG + col + 3] * sum.w * invm;
                    *reinterpret_cast<float4 *>(dst + j) = o;
                }
            }
        } else if (cs == 2) {
            // the row's zred and flags from the tile's input slot (written by this quarter's cs = 0 warp)
            const uint4 info = in_row[(size_t)(it & 1) * 128 * 4 + 3];
            const bool outside = (info.y & 1u) != 0, bad = (info.y & 2u) != 0;
            const float dd = emu_distance(__uint_as_float(info.x), par + EMU_P_ZT, par + EMU_P_DL);
            const float *scr = scr_row + EMU_NPC;
            // pass 1: the ensemble mean of each band (its magnitude) and the brightest band
            float mmin = INFINITY;
            bool finite = true;
            float *mdst = a.mags + (size_t)m * a.nb;
            for (int j = 0; j < a.nb; ++j) {
                float sum = 0.f;
#pragma unroll
                for (int k = 0; k < EMU_MEMBERS; ++k) sum += scr[k * SCR_MEM + j];
                const int o = EMU_NPC + j;
                const float mag = par[EMU_P_OMU + o] + par[EMU_P_OSIG + o] * sum * invm + dd;
                if (!isfinite(mag)) finite = false;
                mmin = fminf(mmin, mag);
                mdst[j] = mag;
            }
            // pass 2: the spread of the bands that count
            float spread = 0.f;
            for (int j = 0; j < a.nb; ++j) {
                float z[EMU_MEMBERS], mean = 0.f;
#pragma unroll
                for (int k = 0; k < EMU_MEMBERS; ++k) { z[k] = scr[k * SCR_MEM + j]; mean += z[k]; }
                mean *= invm;
                float var = 0.f;
#pragma unroll
                for (int k = 0; k < EMU_MEMBERS; ++k) var += (z[k] - mean) * (z[k] - mean);
                const int o = EMU_NPC + j;
                const float sd = par[EMU_P_OSIG + o] * sqrtf(var * invm);
                const float mag = par[EMU_P_OMU + o] + par[EMU_P_OSIG + o] * mean + dd;
                if (!isfinite(sd)) finite = false;
                if (mag < mmin + a.faint) spread = fmaxf(spread, sd);
            }
            const int f = outside ? 1 : (bad || !finite) ? 3 : (spread > a.spread_max) ? 2 : 0;
            if (a.spread) a.spread[m] = spread;
            a.flag[m] = f;
            if (f) {
                const int k = atomicAdd(a.nflag, 1);
                a.flagged[k] = m;
            }
        }
    }
}

__global__ void __launch_bounds__(EI_THREADS, 1)
emu_infer_kernel(const __grid_constant__ CUtensorMap tm_w0, const __grid_constant__ CUtensorMap tm_wh,
                 const __grid_constant__ CUtensorMap tm_w4, EmuInferArgs a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t *S = smem;
    uint8_t *W = smem + EI_S_BYTES;
    uint64_t *bars = reinterpret_cast<uint64_t *>(W + EI_NS * EI_STAGE);
    uint64_t *full = bars, *empty = bars + EI_NS;
    uint64_t *afull = bars + 2 * EI_NS, *aempty = afull + 1, *hrdy = aempty + 1, *inrdy = hrdy + 2;
    uint64_t *mma_done = inrdy + 1;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mma_done + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ntiles = (a.n + 127) / 128;
    int *status = a.status;

    if (threadIdx.x == 0) {
        for (int s = 0; s < EI_NS; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
        mbar_init(afull, 1);
        mbar_init(aempty, EI_EPI_WARPS);
        for (int c = 0; c < 2; ++c) mbar_init(&hrdy[c], EI_EPI_WARPS);
        mbar_init(inrdy, EI_EPI_WARPS);
        mbar_init(mma_done, 1);
        fence_mbar_init();
    }
    if (warp == 1) { tmem_alloc(tmem_slot, 512); tmem_relinquish(); }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;
    const int iters = emu_iters(ntiles);

    if (warp == 0) {
        if (lane == 0) {
            int s = 0; uint32_t ph = 0;
            int last_fill[EI_NS];
            for (int i = 0; i < EI_NS; ++i) last_fill[i] = -1;
            bool ok = true;
            for (int it = 0; it < iters && ok; ++it)
                for (int mem = 0; mem < EMU_MEMBERS && ok; ++mem)
                    for (int L = 0; L < 5 && ok; ++L) {
                        const int nch = L == 4 ? 1 : 2, nkb = L == 0 ? 1 : 8;
                        for (int c = 0; c < nch && ok; ++c)
                            for (int kb = 0; kb < nkb; ++kb) {
                                // the stage is free once the MMAs that read it have completed
                                if (!mbar_wait(&empty[s], ph ^ 1u, status, ERR_TIMEOUT_PRODUCER)) { ok = false; break; }
                                const int mw = emu_member(mem);
                                uint8_t *st = W + s * EI_STAGE;
                                if (L < 4) {
                                    mbar_arrive_expect_tx(&full[s], EI_STAGE);
                                    if (L == 0)
                                        tma_load_2d(st, &tm_w0, 0, mw * EMU_H + c * 256, &full[s]);
                                    else
                                        tma_load_2d(st, &tm_wh, kb * 64, ((L - 1) * EMU_MEMBERS + mw) * EMU_H + c * 256,
                                                    &full[s]);
                                } else {
                                    mbar_arrive_expect_tx(&full[s], EI_STAGE / 2);
                                    tma_load_2d(st, &tm_w4, kb * 64, mw * EMU_NOUT, &full[s]);
                                }
                                last_fill[s] = (int)ph;
                                if (++s == EI_NS) { s = 0; ph ^= 1u; }
                            }
                    }
            for (int i = 0; i < EI_NS; ++i)
                if (last_fill[i] >= 0) mbar_wait(&full[i], (uint32_t)last_fill[i], status, ERR_TIMEOUT_PRODUCER, false);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            int s = 0; uint32_t ph = 0;
            uint32_t g = 0, icnt = 0, hcnt = 0;
            bool ok = true;
            const uint32_t s_base = smem_u32(S);
            const uint32_t d = tmem_base + EI_ACC_COL;
            for (int it = 0; it < iters && ok; ++it)
                for (int mem = 0; mem < EMU_MEMBERS && ok; ++mem) {
                    if (!mbar_wait(inrdy, icnt & 1u, status, ERR_TIMEOUT_MMA)) { ok = false; break; }
                    ++icnt;
                    tc_fence_after();
                    for (int L = 0; L < 5 && ok; ++L) {
                        const int nch = L == 4 ? 1 : 2, nkb = L == 0 ? 1 : 8;
                        const uint32_t idesc = L == 4 ? EI_IDESC128 : EI_IDESC256;
                        for (int c = 0; c < nch && ok; ++c) {
                            // the accumulator is free once the epilogue has drained the previous chunk
                            if (!mbar_wait(aempty, (g & 1u) ^ 1u, status, ERR_TIMEOUT_MMA)) { ok = false; break; }
                            tc_fence_after();
                            for (int kb = 0; kb < nkb; ++kb) {
                                if (L >= 1 && c == 0 && (kb & 3) == 0) {
                                    if (!mbar_wait(&hrdy[kb >> 2], hcnt & 1u, status, ERR_TIMEOUT_MMA)) { ok = false; break; }
                                    tc_fence_after();
                                }
                                if (!mbar_wait(&full[s], ph, status, ERR_TIMEOUT_MMA)) { ok = false; break; }
                                tc_fence_after();
                                const uint32_t b0 = smem_u32(W + s * EI_STAGE);
                                if (L == 0) {
                                    // the input layer: two K steps (the features' hi parts, then their lo parts
                                    // against the same weights repeated in W0's columns 16..27)
                                    mma_bf16(d, sw128_desc(s_base), sw128_desc(b0), idesc, 0u);
                                    mma_bf16(d, sw128_desc(s_base + 32), sw128_desc(b0 + 32), idesc, 1u);
                                } else {
#pragma unroll
                                    for (int k = 0; k < 4; ++k) {
                                        const uint32_t acc = (kb > 0 || k > 0) ? 1u : 0u;
                                        if (L & 1)   // h1, h3 in tensor memory
                                            mma_bf16_ts(d, tmem_base + EI_T_COL + kb * 32 + k * 8, sw128_desc(b0 + k * 32), idesc, acc);
                                        else         // h2, h4 in shared memory
                                            mma_bf16(d, sw128_desc(s_base + kb * EI_KBLK + k * 32), sw128_desc(b0 + k * 32), idesc, acc);
                                    }
                                }
                                mma_commit(&empty[s]);   // frees the stage once these MMAs complete
                                if (++s == EI_NS) { s = 0; ph ^= 1u; }
                            }
                            if (!ok) break;
                            mma_commit(afull);
                            ++g;
                        }
                        if (L >= 1) ++hcnt;
                    }
                }
            mma_commit(mma_done);
            mbar_wait(mma_done, 0, status, ERR_TIMEOUT_MMA, false);
        }
    } else {
        emu_epilogue(a, S, bars, tmem_base, warp & 3, (warp - 2) >> 2, lane);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem_base, 512);
    }
}

int emu_infer_smem() { return EI_SMEM; }
// rows of the inference kernel's weight boxes: hidden layers (one CTA's share of a 256-row tile), output layer
int emu_weight_box_rows() { return EI_ROWS; }
int emu_weight_box_rows4() { return EI_ROWS4; }

cudaError_t run_emu_infer(const Emulator &e, const EmuInferArgs &a, int num_sms, cudaStream_t st) {
    if (a.n <= 0) return cudaSuccess;
    if (a.nb < 1 || a.nb > EMU_MAX_BANDS) return cudaErrorInvalidValue;
    cudaError_t err = cudaFuncSetAttribute(emu_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, EI_SMEM);
    if (err != cudaSuccess) return err;
    cudaLaunchConfig_t cfg = {};
    cfg.blockDim = dim3(EI_THREADS);
    cfg.dynamicSmemBytes = EI_SMEM;
    cfg.stream = st;
    cfg.attrs = nullptr;
    cfg.numAttrs = 0;
    // persistent: one CTA per SM (its shared memory allows no more), no more CTAs than tiles
    const int ntiles = (a.n + 127) / 128;
    cfg.gridDim = dim3(std::min(num_sms, ntiles));
    err = cudaLaunchKernelEx(&cfg, emu_infer_kernel, e.tm_w0, e.tm_wh, e.tm_w4, a);
    if (err != cudaSuccess) return err;
    return cudaGetLastError();
}

}  // namespace sps
