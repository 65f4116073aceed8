// The emulator's inference: one fused persistent kernel per SM that runs the five members of the ensemble over a
// tile of 128 models, layer after layer, without leaving the SM.
//
// Per tile and member, five dense layers (64 -> 512 -> 512 -> 512 -> 512 -> 128). Each layer is four (the output
// layer: one) N chunks of 128 outputs, D(models x 128) = A(models x K) W_chunk(128 x K)^T on tcgen05 (M = 128 models,
// N = 128, f16, f32 accumulator in TMEM). The activations never leave the SM and alternate between two homes:
//   input (S, K block 0) -> h1 (T) -> h2 (S) -> h3 (T) -> h4 (S) -> outputs (registers)
// where S is shared memory (128 x 512 f16, eight 16 KB K blocks in the 128-byte swizzle: the MMA's A descriptor)
// and T is tensor memory (256 columns, two f16 per column: the MMA's A operand from TMEM). A layer reads one home
// and its epilogue writes the other, so the epilogue of chunk c (TMEM accumulator -> bias, SiLU -> f16) runs
// while the MMAs of chunk c + 1 read the unchanged input. The accumulators are double-buffered (2 x 128 columns),
// and the next layer's first chunk starts on the K blocks already written (a ready barrier per 128 features).
// The weights stream through a six-stage TMA ring (128 x 64 f16 tiles, 16 KB).
//
// Warp 0: TMA producer; warp 1: MMA issuer (one thread) and TMEM owner; warps 2..9: epilogue, two warps per TMEM
// lane quarter (one model row per thread, 64 of the 128 columns each). The output epilogue keeps, per model, the
// members' sum of the PCA coefficients and a running mean and M2 (Welford) of the magnitudes, then writes the
// ensemble mean, the spread (the population standard deviation over the members, the largest over the bands that
// are less than `faint` mag fainter than the brightest) and the flag.
//
// Every mbarrier wait is bounded (status word, no hang); drains wait for the copies and MMAs in flight.
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cmath>
#include <cstdint>
#include "sm103_ptx.cuh"
#include "csp_kernels.h"
#include "emulator.h"

namespace sps {

constexpr int EI_THREADS = 320;
constexpr int EI_NS = 6;                          // weight stages
constexpr int EI_TILE = 128 * 64 * 2;             // one 128 x 64 f16 tile (16 KB)
constexpr int EI_S_BYTES = 8 * EI_TILE;           // activations: 8 K blocks
constexpr int EI_SMEM = EI_S_BYTES + EI_NS * EI_TILE + 256 + 1024;
constexpr uint32_t EI_IDESC = idesc_f16_f32(128, 128);
constexpr uint32_t EI_T_COL = 0, EI_ACC_COL = 256;

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

// A warp-uniform bounded wait (every lane polls; the warp goes on only if all saw the phase complete).
__device__ __forceinline__ bool warp_wait(uint64_t *bar, uint32_t parity, int *status, int code) {
    const bool w = mbar_wait(bar, parity, status, code);
    return __all_sync(0xffffffffu, w);
}

// The epilogue warps of one column half H (H = 0: columns 0..63 of each chunk, the PCA outputs of the last layer;
// H = 1: columns 64..127, the magnitudes), one model row per thread.
template <int H>
__device__ __forceinline__ void emu_epilogue(const EmuInferArgs &a, uint8_t *S, uint64_t *bars, uint32_t tmem_base,
                                             int q, int lane) {
    uint64_t *afull = bars + 2 * EI_NS, *aempty = afull + 2, *hrdy = aempty + 2, *inrdy = hrdy + 4;
    const int r = q * 32 + lane;
    const uint32_t lane_base = (uint32_t)(q * 32) << 16;
    const uint32_t s_base = smem_u32(S);
    const float *par = a.par;
    const int ntiles = (a.n + 127) / 128;
    int *status = a.status;
    uint32_t g = 0;
    bool ok = true;
    constexpr int NACC = H == 0 ? EMU_NPC : EMU_MAX_BANDS;
    float acc1[NACC];            // H = 0: the members' sum (standardised); H = 1: Welford mean
    float acc2[H == 0 ? 1 : EMU_MAX_BANDS];   // H = 1: Welford M2
    for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int m = tile * 128 + r;
        const bool valid = m < a.n;
        float xs[EMU_NFEAT];
        bool outside = false, bad = false;
        float zred = 0.f;
        if (valid) {
            float x[EMU_NIN];
#pragma unroll
            for (int i = 0; i < EMU_NIN; ++i) x[i] = __ldg(a.x + (size_t)m * EMU_NIN + i);
            zred = x[5];
            outside = !emu_features(x, par, xs);
#pragma unroll
            for (int i = 0; i < EMU_NFEAT; ++i)
                if (!isfinite(xs[i])) bad = true;
        }
        if (!valid || bad) {
#pragma unroll
            for (int i = 0; i < EMU_NFEAT; ++i) xs[i] = 0.f;
        }
        // the input row as f16 words: the features' hi parts (K 0..11), then their lo parts (K 16..27)
        uint32_t xin[12];
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            xin[i] = pack_f16(xs[2 * i], xs[2 * i + 1]);
            xin[6 + i] = pack_f16(f16_lo(xs[2 * i]), f16_lo(xs[2 * i + 1]));
        }
#pragma unroll
        for (int j = 0; j < NACC; ++j) acc1[j] = 0.f;
        if (H == 1) {
#pragma unroll
            for (int j = 0; j < EMU_MAX_BANDS; ++j) acc2[j] = 0.f;
        }
        for (int mem = 0; mem < EMU_MEMBERS && ok; ++mem) {
            // the input row (K block 0 of S, f16): K 0..11 the features' hi parts, K 16..27 their lo parts, zeros
            if (H == 0) {
                st_shared_v4(s_base + sw128_off(r, 0), xin[0], xin[1], xin[2], xin[3]);
                st_shared_v4(s_base + sw128_off(r, 1), xin[4], xin[5], 0u, 0u);
                st_shared_v4(s_base + sw128_off(r, 2), xin[6], xin[7], xin[8], xin[9]);
                st_shared_v4(s_base + sw128_off(r, 3), xin[10], xin[11], 0u, 0u);
                fence_proxy_async_smem();
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(inrdy);
            const float *bm = a.bias + (size_t)mem * EMU_NBIAS;
            for (int L = 0; L < 5 && ok; ++L) {
                const int nch = L == 4 ? 1 : 4;
                for (int c = 0; c < nch; ++c) {
                    const uint32_t buf = g & 1u;
                    if (!warp_wait(&afull[buf], (g >> 1) & 1u, status, ERR_TIMEOUT_EPILOGUE)) { ok = false; break; }
                    ++g;
                    tc_fence_after();
                    const uint32_t ta = tmem_base + lane_base + EI_ACC_COL + buf * 128 + H * 64;
                    float v[32];
                    if (L < 4) {
                        const float *b = bm + L * EMU_H + c * 128 + H * 64;
                        uint32_t p[32];
#pragma unroll
                        for (int half = 0; half < 2; ++half) {
                            tmem_ld32(ta + half * 32, v);
#pragma unroll
                            for (int i = 0; i < 16; ++i)
                                p[half * 16 + i] = pack_f16(silu_fast(v[2 * i] + __ldg(b + half * 32 + 2 * i)),
                                                            silu_fast(v[2 * i + 1] + __ldg(b + half * 32 + 2 * i + 1)));
                        }
                        tc_fence_before();
                        __syncwarp();
                        if (lane == 0) mbar_arrive(&aempty[buf]);
                        if ((L & 1) == 0) {
                            // h1 (L = 0) and h3 (L = 2) into tensor memory
                            tmem_st32(tmem_base + lane_base + EI_T_COL + c * 64 + H * 32, p);
                            tmem_wait_st();
                            tc_fence_before();
                        } else {
                            // h2 (L = 1) and h4 (L = 3) into shared memory, K block 2c + H
                            const uint32_t blk = s_base + (uint32_t)(2 * c + H) * EI_TILE;
#pragma unroll
                            for (int j = 0; j < 8; ++j)
                                st_shared_v4(blk + sw128_off(r, j), p[4 * j], p[4 * j + 1], p[4 * j + 2], p[4 * j + 3]);
                            fence_proxy_async_smem();
                        }
                        __syncwarp();
                        if (lane == 0) mbar_arrive(&hrdy[c]);
                    } else {
                        const float *b = bm + 4 * EMU_H + H * 64;
                        const float inv = 1.f / (float)(mem + 1);
#pragma unroll
                        for (int half = 0; half < 2; ++half) {
                            tmem_ld32(ta + half * 32, v);
#pragma unroll
                            for (int i = 0; i < 32; ++i) {
                                const int j = half * 32 + i;
                                if (H == 0) {
                                    acc1[j < NACC ? j : 0] += v[i] + __ldg(b + j);
                                } else if (j < EMU_MAX_BANDS) {
                                    const float z = v[i] + __ldg(b + j);
                                    const float d = z - acc1[j];
                                    acc1[j] += d * inv;
                                    acc2[j] = fmaf(d, z - acc1[j], acc2[j]);
                                }
                            }
                        }
                        tc_fence_before();
                        __syncwarp();
                        if (lane == 0) mbar_arrive(&aempty[buf]);
                    }
                }
            }
        }
        if (!ok || !valid) continue;
        // ---- the ensemble's outputs of model m
        const float invm = 1.f / (float)EMU_MEMBERS;
        if (H == 0) {
            if (a.coef) {
                float *dst = a.coef + (size_t)m * EMU_NPC;
#pragma unroll
                for (int j = 0; j < EMU_NPC; j += 4) {
                    float4 o;
                    o.x = par[EMU_P_OMU + j] + par[EMU_P_OSIG + j] * acc1[j] * invm;
                    o.y = par[EMU_P_OMU + j + 1] + par[EMU_P_OSIG + j + 1] * acc1[j + 1] * invm;
                    o.z = par[EMU_P_OMU + j + 2] + par[EMU_P_OSIG + j + 2] * acc1[j + 2] * invm;
                    o.w = par[EMU_P_OMU + j + 3] + par[EMU_P_OSIG + j + 3] * acc1[j + 3] * invm;
                    *reinterpret_cast<float4 *>(dst + j) = o;
                }
            }
        } else {
            const float dd = emu_distance(zred, par + EMU_P_ZT, par + EMU_P_DL);
            float mmin = INFINITY;
            bool finite = true;
#pragma unroll
            for (int j = 0; j < EMU_MAX_BANDS; ++j)
                if (j < a.nb) {
                    const int o = EMU_NPC + j;
                    acc1[j] = par[EMU_P_OMU + o] + par[EMU_P_OSIG + o] * acc1[j] + dd;     // the magnitude
                    acc2[j] = par[EMU_P_OSIG + o] * sqrtf(fmaxf(acc2[j] * invm, 0.f));     // its spread
                    if (!isfinite(acc1[j]) || !isfinite(acc2[j])) finite = false;
                    mmin = fminf(mmin, acc1[j]);
                }
            float spread = 0.f;
            float *dst = a.mags + (size_t)m * a.nb;
#pragma unroll
            for (int j = 0; j < EMU_MAX_BANDS; ++j)
                if (j < a.nb) {
                    if (acc1[j] < mmin + a.faint) spread = fmaxf(spread, acc2[j]);
                    dst[j] = acc1[j];
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
    uint64_t *bars = reinterpret_cast<uint64_t *>(W + EI_NS * EI_TILE);
    uint64_t *full = bars, *empty = bars + EI_NS;
    uint64_t *afull = bars + 2 * EI_NS, *aempty = afull + 2, *hrdy = aempty + 2, *inrdy = hrdy + 4;
    uint64_t *mma_done = inrdy + 1;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mma_done + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ntiles = (a.n + 127) / 128;
    int *status = a.status;

    if (threadIdx.x == 0) {
        for (int s = 0; s < EI_NS; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
        for (int b = 0; b < 2; ++b) { mbar_init(&afull[b], 1); mbar_init(&aempty[b], 8); }
        for (int c = 0; c < 4; ++c) mbar_init(&hrdy[c], 8);
        mbar_init(inrdy, 8);
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
            int last_fill[EI_NS];
            for (int i = 0; i < EI_NS; ++i) last_fill[i] = -1;
            bool ok = true;
            for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x)
                for (int mem = 0; mem < EMU_MEMBERS && ok; ++mem)
                    for (int L = 0; L < 5 && ok; ++L) {
                        const int nch = L == 4 ? 1 : 4, nkb = L == 0 ? 1 : 8;
                        for (int c = 0; c < nch && ok; ++c)
                            for (int kb = 0; kb < nkb; ++kb) {
                                if (!mbar_wait(&empty[s], ph ^ 1u, status, ERR_TIMEOUT_PRODUCER)) { ok = false; break; }
                                uint8_t *dst = W + s * EI_TILE;
                                mbar_arrive_expect_tx(&full[s], EI_TILE);
                                if (L == 0)
                                    tma_load_2d(dst, &tm_w0, 0, mem * EMU_H + c * 128, &full[s]);
                                else if (L < 4)
                                    tma_load_2d(dst, &tm_wh, kb * 64, ((L - 1) * EMU_MEMBERS + mem) * EMU_H + c * 128, &full[s]);
                                else
                                    tma_load_2d(dst, &tm_w4, kb * 64, mem * EMU_NOUT, &full[s]);
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
            for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x)
                for (int mem = 0; mem < EMU_MEMBERS && ok; ++mem) {
                    if (!mbar_wait(inrdy, icnt & 1u, status, ERR_TIMEOUT_MMA)) { ok = false; break; }
                    ++icnt;
                    tc_fence_after();
                    for (int L = 0; L < 5 && ok; ++L) {
                        const int nch = L == 4 ? 1 : 4, nkb = L == 0 ? 1 : 8;
                        for (int c = 0; c < nch && ok; ++c) {
                            const uint32_t buf = g & 1u;
                            if (!mbar_wait(&aempty[buf], ((g >> 1) & 1u) ^ 1u, status, ERR_TIMEOUT_MMA)) { ok = false; break; }
                            tc_fence_after();
                            const uint32_t d = tmem_base + EI_ACC_COL + buf * 128;
                            for (int kb = 0; kb < nkb; ++kb) {
                                if (L >= 1 && c == 0 && (kb & 1) == 0) {
                                    if (!mbar_wait(&hrdy[kb >> 1], hcnt & 1u, status, ERR_TIMEOUT_MMA)) { ok = false; break; }
                                    tc_fence_after();
                                }
                                if (!mbar_wait(&full[s], ph, status, ERR_TIMEOUT_MMA)) { ok = false; break; }
                                tc_fence_after();
                                const uint32_t b0 = smem_u32(W + s * EI_TILE);
                                if (L == 0) {
                                    // the input layer: two K steps (the features' hi parts, then their lo parts
                                    // against the same weights repeated in W0's columns 16..27)
                                    mma_bf16(d, sw128_desc(s_base), sw128_desc(b0), EI_IDESC, 0u);
                                    mma_bf16(d, sw128_desc(s_base + 32), sw128_desc(b0 + 32), EI_IDESC, 1u);
                                } else {
#pragma unroll
                                    for (int k = 0; k < 4; ++k) {
                                        const uint32_t acc = (kb > 0 || k > 0) ? 1u : 0u;
                                        if (L & 1)   // h1, h3 in tensor memory
                                            mma_bf16_ts(d, tmem_base + EI_T_COL + kb * 32 + k * 8, sw128_desc(b0 + k * 32), EI_IDESC, acc);
                                        else         // h2, h4 in shared memory
                                            mma_bf16(d, sw128_desc(s_base + kb * EI_TILE + k * 32), sw128_desc(b0 + k * 32), EI_IDESC, acc);
                                    }
                                }
                                mma_commit(&empty[s]);
                                if (++s == EI_NS) { s = 0; ph ^= 1u; }
                            }
                            if (!ok) break;
                            mma_commit(&afull[buf]);
                            ++g;
                        }
                        if (L >= 1) ++hcnt;
                    }
                }
            mma_commit(mma_done);
            mbar_wait(mma_done, 0, status, ERR_TIMEOUT_MMA, false);
        }
    } else {
        const int q = warp & 3;
        if (warp < 6) emu_epilogue<0>(a, S, bars, tmem_base, q, lane);
        else emu_epilogue<1>(a, S, bars, tmem_base, q, lane);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem_base, 512);
    }
}

int emu_infer_smem() { return EI_SMEM; }

cudaError_t run_emu_infer(const Emulator &e, const EmuInferArgs &a, int num_sms, cudaStream_t st) {
    if (a.n <= 0) return cudaSuccess;
    if (a.nb < 1 || a.nb > EMU_MAX_BANDS) return cudaErrorInvalidValue;
    cudaError_t err = cudaFuncSetAttribute(emu_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, EI_SMEM);
    if (err != cudaSuccess) return err;
    const int ntiles = (a.n + 127) / 128;
    const int grid = ntiles < num_sms ? ntiles : num_sms;
    emu_infer_kernel<<<grid, EI_THREADS, EI_SMEM, st>>>(e.tm_w0, e.tm_wh, e.tm_w4, a);
    return cudaGetLastError();
}

}  // namespace sps
