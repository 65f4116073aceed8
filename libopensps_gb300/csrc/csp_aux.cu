// The prologue kernels of the batched CSP path.
//
// weights_convert_sums: model_sums_zw (OpenSPS src/physics/opensps_csp_batch.f90:2090-2120) per model: the weights
//   floored at SAFE_FLOOR, the FP64 mass and L_bol sums (young and old parts apart when asked), and the weights cast
//   once to the contraction's operand (bf16 hi + lo, in its K order, through the operand's column map), in one pass.
// weights_prep: the FP64 sums alone (the plain FP64 path).
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cfloat>
#include <cstdint>
#include "csp_kernels.h"

namespace sps {

// ---------------------------------------------------------------------------------------------- weights
// The operand and, from the same FP64 weights, the FP64 sums of model_sums_zw (one warp per model, the sums in the
// operand's column order; young ages by the column map's KMAP_YOUNG bit): the sums ride the FP64 pipe while the
// conversion waits on memory, instead of a second pass over the weights bound by that pipe. Escaping-light columns
// (KMAP_ION) carry the weight times the model's escaping fraction clamp(frac_obrun, 0, 1) (nebular_kernels step 2,
// OpenSPS src/physics/opensps_csp_batch.f90:2726-2750, with fesc of batch_nebular_indices :1696) and join no sum.
template <bool PARTS>
__global__ void __launch_bounds__(256) weights_convert_sums_kernel(WeightsArgs a) {
    const int m = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (m >= a.n_models) return;
    const double *w = a.wz + (size_t)m * a.nt * a.nz;
    __nv_bfloat16 *hi = a.w_hi + (size_t)m * a.kpad, *lo = a.w_lo + (size_t)m * a.kpad;
    double ms = 0.0, ls = 0.0, msy = 0.0, lsy = 0.0, mso = 0.0, lso = 0.0;
    const float fesc = a.mpar ? fminf(fmaxf(__ldg(a.mpar + (size_t)m * MODEL_PAR_FLOATS + MP_FO), 0.f), 1.f) : 0.f;
#pragma unroll 4
    for (int k = lane; k < a.kpad; k += 32) {
        const int code = __ldg(a.kmap + k);
        float wf = 0.f;
        if (code >= 0) {
            const int idx = code & KMAP_SRC;
            const double wv = __ldg(w + idx);
            wf = weight_to_f32(wv);
            if (code & KMAP_ION) {
                wf *= fesc;
            } else if (__double_as_longlong(wv) > 0x0010000000000000LL) {   // wv > DBL_MIN (and not negative)
                const double mk = __ldg(a.mass + idx), lk = __ldg(a.llin + idx);
                ms = fma(wv, mk, ms);
                ls = fma(wv, lk, ls);
                if (PARTS) {
                    if (code & KMAP_YOUNG) { msy = fma(wv, mk, msy); lsy = fma(wv, lk, lsy); }
                    else { mso = fma(wv, mk, mso); lso = fma(wv, lk, lso); }
                }
            }
        }
        const __nv_bfloat16 h = __float2bfloat16_rn(wf);
        hi[k] = h;
        lo[k] = __float2bfloat16_rn(wf - __bfloat162float(h));
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        ms += __shfl_xor_sync(0xffffffffu, ms, off);
        ls += __shfl_xor_sync(0xffffffffu, ls, off);
        if (PARTS) {
            msy += __shfl_xor_sync(0xffffffffu, msy, off);
            lsy += __shfl_xor_sync(0xffffffffu, lsy, off);
            mso += __shfl_xor_sync(0xffffffffu, mso, off);
            lso += __shfl_xor_sync(0xffffffffu, lso, off);
        }
    }
    if (lane == 0 && a.sums) {
        double *o = a.sums + (size_t)m * 6;
        o[0] = ms; o[1] = ls;
        if (PARTS) { o[2] = msy; o[3] = mso; o[4] = lsy; o[5] = lso; }
    }
}

cudaError_t run_weights_convert_sums(const WeightsArgs &a, cudaStream_t st) {
    if (a.n_models <= 0) return cudaSuccess;
    const int threads = 256, per_block = threads / 32, blocks = (a.n_models + per_block - 1) / per_block;
    if (a.parts) weights_convert_sums_kernel<true><<<blocks, threads, 0, st>>>(a);
    else weights_convert_sums_kernel<false><<<blocks, threads, 0, st>>>(a);
    return cudaGetLastError();
}

// The FP64 sums of model_sums_zw: one warp per model over the source weights (age fastest).
template <bool PARTS>
__global__ void __launch_bounds__(256) weights_prep_kernel(WeightsArgs a) {
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int m = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; m < a.n_models; m += nwarps) {
    const double *w = a.wz + (size_t)m * a.nt * a.nz;
    double ms = 0.0, ls = 0.0, msy = 0.0, lsy = 0.0, mso = 0.0, lso = 0.0;
    const int ntz = a.nt * a.nz;
    int t = lane % a.nt;
#pragma unroll 4
    for (int k = lane; k < ntz; k += 32) {
        const double wv = __ldg(w + k);
        if (__double_as_longlong(wv) > 0x0010000000000000LL) {   // wv > DBL_MIN (and not negative)
            // (fused multiply-adds: the kernel is bound by GB300's FP64 pipe, and one FMA is half a multiply and an add)
            const double mk = __ldg(a.mass + k), lk = __ldg(a.llin + k);
            ms = fma(wv, mk, ms);
            ls = fma(wv, lk, ls);
            if (PARTS) {
                if (t < a.itesc) { msy = fma(wv, mk, msy); lsy = fma(wv, lk, lsy); }
                else { mso = fma(wv, mk, mso); lso = fma(wv, lk, lso); }
            }
        }
        if (PARTS) { t += 32; while (t >= a.nt) t -= a.nt; }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        ms += __shfl_xor_sync(0xffffffffu, ms, off);
        ls += __shfl_xor_sync(0xffffffffu, ls, off);
        if (PARTS) {
            msy += __shfl_xor_sync(0xffffffffu, msy, off);
            lsy += __shfl_xor_sync(0xffffffffu, lsy, off);
            mso += __shfl_xor_sync(0xffffffffu, mso, off);
            lso += __shfl_xor_sync(0xffffffffu, lso, off);
        }
    }
    if (lane == 0 && a.sums) {
        double *o = a.sums + (size_t)m * 6;
        o[0] = ms; o[1] = ls;
        if (PARTS) { o[2] = msy; o[3] = mso; o[4] = lsy; o[5] = lso; }
    }
    }
}

cudaError_t run_weights_prep(const WeightsArgs &a, cudaStream_t st) {
    if (a.n_models <= 0) return cudaSuccess;
    const int threads = a.grid > 0 ? 64 : 256, per_block = threads / 32;
    const int blocks = a.grid > 0 ? a.grid : (a.n_models + per_block - 1) / per_block;
    if (a.parts) weights_prep_kernel<true><<<blocks, threads, 0, st>>>(a);
    else weights_prep_kernel<false><<<blocks, threads, 0, st>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------- emission lines
// line_profiles' luminosities (src/physics/opensps_csp_batch.f90:3133-3166 with the line table of the ages that have
// lines): one block per model, one thread per line, over the (age, metallicity) entries with lines.
__global__ void emlines_kernel(EmlineArgs a) {
    const int m = blockIdx.x;
    const double *w = a.wz + (size_t)m * a.ntz;
    for (int l = threadIdx.x; l < a.nline; l += blockDim.x) {
        float s = 0.f;
        for (int i = 0; i < a.nnz; ++i) {
            const float wv = weight_to_f32(__ldg(w + __ldg(a.kidx + i)));
            s = fmaf(wv, __ldg(a.lum + (size_t)i * a.nline + l), s);
        }
        a.eml[(size_t)m * a.nline + l] = s;
    }
}

cudaError_t run_emlines(const EmlineArgs &a, cudaStream_t st) {
    if (a.n_models <= 0 || a.nline <= 0) return cudaSuccess;
    emlines_kernel<<<a.n_models, 128, 0, st>>>(a);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------------- casts
__global__ void spec_to_f64_kernel(const float *src, int ld, int nspec, int n_models, double *dst) {
    const size_t total = (size_t)nspec * n_models;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const size_t m = i / nspec, j = i % nspec;
        dst[i] = (double)src[m * ld + j];
    }
}

cudaError_t run_spec_to_f64(const float *src, int ld, int nspec, int n_models, double *dst, cudaStream_t st) {
    if (n_models <= 0) return cudaSuccess;
    spec_to_f64_kernel<<<1216, 256, 0, st>>>(src, ld, nspec, n_models, dst);
    return cudaGetLastError();
}

}  // namespace sps
