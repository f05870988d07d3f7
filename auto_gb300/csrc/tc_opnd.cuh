// Operand building and GEMM issue shared by the tensor-core passes (step_tc.cu, step_tc_row.cu).
//
// Operands live in shared memory in the K-major layout of tc_ptx.cuh (kmajor_offset), as bf16 hi
// and lo copies (BF16x3: hi*hi + hi*lo + lo*hi) or one tf32 copy.  A hand-over between two GEMMs
// reads the accumulator from TMEM, does its pointwise work and stores the next GEMM's A operand.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "fft_core.cuh"
#include "tc_ptx.cuh"

namespace lenia {
namespace tc {

// BF16x3 split of two values at once: hi = bf16(v) and lo = bf16(v - hi) for a and b, packed as
// bf16x2 (a in the low half).  One paired conversion for both his, one f32x2 subtract for both
// (exact) residuals, one paired conversion for both los: the same bits as the per-value split.
__device__ __forceinline__ void split_bf16x2(float a, float b, uint32_t& hi, uint32_t& lo) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    const float2 hf = __bfloat1622float2(h);
    const float2 r = lfft::f2sub(make_float2(a, b), hf);
    const __nv_bfloat162 l = __floats2bfloat162_rn(r.x, r.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
}

// One value at (row r, k) of an operand with K elements per row (hi at op, lo opnd_bytes later).
template <bool X3, int LBO>
__device__ __forceinline__ void store_elem(uint8_t* op, int opnd_bytes, int r, int k, int K, float v) {
    if (X3) {
        const uint32_t off = kmajor_offset(r, k, K, 2, LBO);
        const __nv_bfloat16 hi = __float2bfloat16_rn(v);
        const __nv_bfloat16 lo = __float2bfloat16_rn(v - __bfloat162float(hi));
        *reinterpret_cast<__nv_bfloat16*>(op + off) = hi;
        *reinterpret_cast<__nv_bfloat16*>(op + opnd_bytes + off) = lo;
    } else {
        *reinterpret_cast<uint32_t*>(op + kmajor_offset(r, k, K, 4, LBO)) = to_tf32(v);
    }
}

// 16 bytes of consecutive K: 8 values (bf16 hi and lo) or 4 (tf32), starting at k0.
template <bool X3, int LBO>
__device__ __forceinline__ void store_chunk(uint8_t* op, int opnd_bytes, int r, int k0, int K, const float* v) {
    if (X3) {
        uint32_t hi[4], lo[4];
#pragma unroll
        for (int i = 0; i < 4; i++) split_bf16x2(v[2 * i], v[2 * i + 1], hi[i], lo[i]);
        const uint32_t off = kmajor_offset(r, k0, K, 2, LBO);
        *reinterpret_cast<uint4*>(op + off) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
        *reinterpret_cast<uint4*>(op + opnd_bytes + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
    } else {
        *reinterpret_cast<uint4*>(op + kmajor_offset(r, k0, K, 4, LBO)) =
            make_uint4(to_tf32(v[0]), to_tf32(v[1]), to_tf32(v[2]), to_tf32(v[3]));
    }
}

// 8 values of consecutive m (m0 a multiple of 8) at one k of an MN-major bf16 operand with M rows,
// as hi and lo (BF16x3): one 16-byte store each.
__device__ __forceinline__ void store_mn_chunk(uint8_t* op, int opnd_bytes, int m0, int k, int M, const float* v) {
    uint32_t hi[4], lo[4];
#pragma unroll
    for (int i = 0; i < 4; i++) split_bf16x2(v[2 * i], v[2 * i + 1], hi[i], lo[i]);
    const uint32_t off = mnmajor_offset(m0, k, M);
    *reinterpret_cast<uint4*>(op + off) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
    *reinterpret_cast<uint4*>(op + opnd_bytes + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
}

// One BF16x3 GEMM with A MN-major (mnmajor_offset, M rows) and F K-major (f_K elements a row, LBO
// apart): D[rows of M in blocks of 128] (+)= A (M x K) * F^T.  A row block starts 16 core matrices
// (2048 bytes) further along MN; an MMA consumes 16 K, two K-groups of A.
template <int LBO>
__device__ __forceinline__ void issue_gemm_amn(uint32_t d_tmem, uint32_t a_saddr, uint32_t a_lo_off, int M, int K,
                                               uint32_t f_saddr, uint32_t f_lo_off, int f_K, int N, uint32_t idesc) {
    const uint32_t a_lbo = (uint32_t)(M / 8) * 128u, a_sbo = 128u, f_sbo = (uint32_t)(f_K * 2 / 16 * LBO);
    const int ksteps = K / 16;
    for (int b = 0; b < M / 128; b++) {
        const uint32_t d = d_tmem + (uint32_t)(b * N);
        const uint32_t a0 = a_saddr + (uint32_t)b * 2048u;
        for (int s = 0; s < ksteps; s++) {
            const uint64_t ad = smem_desc(a0 + 2u * a_lbo * s, a_lbo, a_sbo);
            const uint32_t fo = f_saddr + 2u * LBO * s;
            const uint64_t bd = smem_desc(fo, LBO, f_sbo);
            mma<false>(d, ad, bd, idesc, s > 0 ? 1u : 0u);
            mma<false>(d, ad, smem_desc(fo + f_lo_off, LBO, f_sbo), idesc, 1u);
            mma<false>(d, smem_desc(a0 + a_lo_off + 2u * a_lbo * s, a_lbo, a_sbo), bd, idesc, 1u);
        }
    }
}

// One GEMM: D[rows of M in blocks of 128] (+)= A (M x K) * F^T (F: N x K), both K-major with
// K-adjacent core matrices LBO bytes apart.  A is laid out with a_K elements per row and F with f_K
// (f_K > K multiplies by the first K columns of F only), so each has its own 8-row-group stride
// (SBO).  An MMA consumes 32 bytes of K (two core matrices), so consecutive MMAs start 2 LBO apart.
template <bool X3, int LBO = 128>
__device__ __forceinline__ void issue_gemm_k(uint32_t d_tmem, uint32_t a_saddr, uint32_t a_lo_off, int M, int K, int a_K,
                                             uint32_t f_saddr, uint32_t f_lo_off, int f_K, int N, uint32_t idesc) {
    constexpr int E = X3 ? 2 : 4;
    const uint32_t a_sbo = (uint32_t)(a_K * E / 16 * LBO), f_sbo = (uint32_t)(f_K * E / 16 * LBO);
    const int ksteps = K * E / 32;
    for (int b = 0; b < M / 128; b++) {
        const uint32_t d = d_tmem + (uint32_t)(b * N);
        const uint32_t a0 = a_saddr + (uint32_t)b * 16u * a_sbo;
        for (int s = 0; s < ksteps; s++) {
            const uint32_t ko = 2u * LBO * s;
            const uint64_t ad = smem_desc(a0 + ko, LBO, a_sbo);
            const uint64_t bd = smem_desc(f_saddr + ko, LBO, f_sbo);
            mma<!X3>(d, ad, bd, idesc, s > 0 ? 1u : 0u);
            if (X3) {
                mma<false>(d, ad, smem_desc(f_saddr + f_lo_off + ko, LBO, f_sbo), idesc, 1u);
                mma<false>(d, smem_desc(a0 + a_lo_off + ko, LBO, a_sbo), bd, idesc, 1u);
            }
        }
    }
}
// Both operands with K elements per row.
template <bool X3, int LBO = 128>
__device__ __forceinline__ void issue_gemm(uint32_t d_tmem, uint32_t a_saddr, uint32_t a_lo_off, int M, int K,
                                           uint32_t f_saddr, uint32_t f_lo_off, int N, uint32_t idesc) {
    issue_gemm_k<X3, LBO>(d_tmem, a_saddr, a_lo_off, M, K, K, f_saddr, f_lo_off, K, N, idesc);
}

// Twiddle exp(-2 pi i a b / H) from the global table (TWN entries).
template <int H>
__device__ __forceinline__ float2 twid(const float2* __restrict__ tw, int a, int b) {
    return tw[((a * b) % H) * (lfft::TWN / H)];
}

}  // namespace tc
}  // namespace lenia
