// Device helpers shared by the kernel files: packed FP32x2 arithmetic on
// 64-bit register pairs (one instruction computes two lanes) and cp.async
// copies into shared memory.
#pragma once

namespace lp {

__device__ __forceinline__ unsigned long long pk2(float lo, float hi) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ float2 up2(unsigned long long v) {
    float lo, hi;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
    return make_float2(lo, hi);
}
__device__ __forceinline__ unsigned long long mul2(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b, unsigned long long c) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// FP64 <-> FP32 conversions by bit manipulation, so that the stage copies of
// the mixed path do not occupy the narrow FP64 unit: FP64 -> FP32 truncates
// toward zero (within one FP32 ulp) and flushes magnitudes below the FP32
// normal range to signed zero; FP32 -> FP64 is exact for normal numbers and
// zero (FP32 subnormals become signed zero).
__device__ __forceinline__ float f64_to_f32_bits(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;
    if (e <= 0) return __uint_as_float(sign);
    if (e >= 255) return __uint_as_float(sign | 0x7f800000u);
    return __uint_as_float(sign | ((unsigned)e << 23) | (unsigned)((b >> 29) & 0x7fffffu));
}
__device__ __forceinline__ double f32_to_f64_bits(float f) {
    const unsigned u = __float_as_uint(f), sign = u & 0x80000000u, e = (u >> 23) & 0xffu;
    if (e == 0) return __longlong_as_double((long long)((unsigned long long)sign << 32));
    const unsigned long long ee = e == 255 ? 0x7ffull : (unsigned long long)(e - 127 + 1023);
    return __longlong_as_double(
        (long long)(((unsigned long long)sign << 32) | (ee << 52) | ((unsigned long long)(u & 0x7fffffu) << 29)));
}

// A sum of FP32 terms as an unevaluated pair hi + lo: each term enters by
// an error-free two-sum (Knuth), a weighted term w x as the exact pair
// (w x rounded, its FMA residual).
struct DFSum {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float s = __fadd_rn(hi, x), bp = __fsub_rn(s, hi);
        lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(x, bp)));
        hi = s;
    }
    __device__ __forceinline__ void addw(float w, float x) {
        const float p = __fmul_rn(w, x);
        add(p);
        lo = __fadd_rn(lo, fmaf(w, x, -p));
    }
    __device__ __forceinline__ double get() const { return f32_to_f64_bits(hi) + f32_to_f64_bits(lo); }
};

}  // namespace lp
