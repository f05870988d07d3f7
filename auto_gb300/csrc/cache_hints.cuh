// Global loads and stores with an L2 eviction priority (createpolicy + .L2::cache_hint).
//
// Between the two launches of a step the half-spectrum is written by one pass and read by the
// next; for a 4096 x 4096 world it is 64 MiB, and with the 17 MiB kernel spectrum it fits in the
// 129 MB L2.  The state is read and written once per step.  Spectrum traffic is tagged
// evict_last and state traffic evict_first, so the streaming state does not push the spectrum
// out.  The hints are per instruction: nothing about the device's cache configuration changes.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace lenia {
namespace hint {

__device__ __forceinline__ uint64_t policy_keep() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ uint64_t policy_stream() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ float2 ld2(const float2* p, uint64_t pol) {
    float2 v;
    asm volatile("ld.global.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(v.x), "=f"(v.y) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ float4 ld4(const float4* p, uint64_t pol) {
    float4 v;
    asm volatile("ld.global.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ float ld1(const float* p, uint64_t pol) {
    float v;
    asm volatile("ld.global.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ void st2(float2* p, float2 v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(p), "f"(v.x), "f"(v.y), "l"(pol) : "memory");
}
__device__ __forceinline__ void st4(float4* p, float4 v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "f"(v.x), "f"(v.y), "f"(v.z),
                 "f"(v.w), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ void st1(float* p, float v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(p), "f"(v), "l"(pol) : "memory");
}

// The same loads with .cg (cached in L2 only, not in the SM's L1), for data that another CTA of the
// same launch may have written since this SM last read it: L1 is not coherent across SMs.
__device__ __forceinline__ float2 ld2_cg(const float2* p, uint64_t pol) {
    float2 v;
    asm volatile("ld.global.cg.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(v.x), "=f"(v.y) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ float4 ld4_cg(const float4* p, uint64_t pol) {
    float4 v;
    asm volatile("ld.global.cg.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "l"(p), "l"(pol));
    return v;
}
template <bool CG>
__device__ __forceinline__ float2 ld2c(const float2* p, uint64_t pol) { return CG ? ld2_cg(p, pol) : ld2(p, pol); }
template <bool CG>
__device__ __forceinline__ float4 ld4c(const float4* p, uint64_t pol) { return CG ? ld4_cg(p, pol) : ld4(p, pol); }

// The same with a compile-time byte offset folded into the address ([p + OFF]), so that a run of
// accesses off one base pointer does not need a 64-bit register pair per address.
template <int OFF>
__device__ __forceinline__ float ld1_at(const float* p, uint64_t pol) {
    float v;
    asm volatile("ld.global.L2::cache_hint.f32 %0, [%1+%3], %2;" : "=f"(v) : "l"(p), "l"(pol), "n"(OFF));
    return v;
}
template <int OFF>
__device__ __forceinline__ float ld1_at_cg(const float* p, uint64_t pol) {
    float v;
    asm volatile("ld.global.cg.L2::cache_hint.f32 %0, [%1+%3], %2;" : "=f"(v) : "l"(p), "l"(pol), "n"(OFF));
    return v;
}
template <int OFF, bool CG>
__device__ __forceinline__ float ld1_atc(const float* p, uint64_t pol) {
    return CG ? ld1_at_cg<OFF>(p, pol) : ld1_at<OFF>(p, pol);
}
template <int OFF>
__device__ __forceinline__ void st1_at(float* p, float v, uint64_t pol) {
    asm volatile("st.global.L2::cache_hint.f32 [%0+%3], %1, %2;" ::"l"(p), "f"(v), "l"(pol), "n"(OFF) : "memory");
}

}  // namespace hint
}  // namespace lenia
