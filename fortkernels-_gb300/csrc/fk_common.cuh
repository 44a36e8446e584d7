// fk_common.cuh -- device helpers shared by the GPP and FF kernels.
//
// Complex values live in HBM as interleaved (re, im) doubles (double2), the
// layout of std::complex<double> / GPUComplex in the reference.  The device
// arithmetic below replaces the reference's complex classes (FFKer_cori/
// Complex.h, BGW-Kernels/GPUComplex.h): products are (ac-bd, ad+bc).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define FK_DEV __device__ __forceinline__

// ---------------------------------------------------------------- complex
FK_DEV double2 cmul(double2 a, double2 b) {
    return make_double2(__dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)),
                        __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
}
FK_DEV double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
FK_DEV double2 cadd(double2 a, double2 b) { return make_double2(__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y)); }
FK_DEV double2 csub(double2 a, double2 b) { return make_double2(__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y)); }
FK_DEV double2 cscale(double2 a, double s) { return make_double2(__dmul_rn(a.x, s), __dmul_rn(a.y, s)); }
FK_DEV double cnorm2(double2 a) { return __dadd_rn(__dmul_rn(a.x, a.x), __dmul_rn(a.y, a.y)); }
// fused accumulate: acc += a*b (contracted; for sums whose rounding order is free)
FK_DEV void cfma(double2& acc, double2 a, double2 b) {
    acc.x = fma(a.x, b.x, fma(-a.y, b.y, acc.x));
    acc.y = fma(a.x, b.y, fma(a.y, b.x, acc.y));
}

FK_DEV float2 cmulf(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
FK_DEV void cfmaf(float2& acc, float2 a, float2 b) {
    acc.x = fmaf(a.x, b.x, fmaf(-a.y, b.y, acc.x));
    acc.y = fmaf(a.x, b.y, fmaf(a.y, b.x, acc.y));
}

// ------------------------------------------------ FP64 -> FP32 without the FP64 pipe
// On GB300 cvt.f32.f64 issues on the (narrow) FP64 pipe.  This conversion
// works on the IEEE-754 bit fields with integer instructions: it adds half
// an FP32 ulp to the 64-bit pattern (round half away from zero; a carry out
// of the mantissa correctly bumps the exponent), then rebiases the exponent
// (1023 -> 127) and keeps the top 23 mantissa bits.  Magnitudes below 2^-126
// flush to signed zero.  Inputs must satisfy |x| < 2^127 (the kernels' data
// are O(1); larger values are rejected by the host-side checks where the
// mixed path is used on user data).
FK_DEV float f64_to_f32_bits(double d) {
    unsigned long long u = (unsigned long long)__double_as_longlong(d) + 0x10000000ull;
    unsigned hi = (unsigned)(u >> 32), lo = (unsigned)u;
    unsigned sign = hi & 0x80000000u;
    unsigned mag = hi & 0x7FFFFFFFu;
    unsigned f = mag < (897u << 20) ? 0u : __funnelshift_l(lo, mag - (896u << 20), 3);
    return __uint_as_float(f | sign);
}
FK_DEV float2 c64_to_f32(double2 v) { return make_float2(f64_to_f32_bits(v.x), f64_to_f32_bits(v.y)); }
// FP32 -> FP64 with integer instructions (exact); zeros and subnormals give a
// signed zero, infinities and NaNs are not expected by the callers
FK_DEV double f32_to_f64_bits(float f) {
    const unsigned u = __float_as_uint(f), e = (u >> 23) & 0xFFu;
    const unsigned long long s = (unsigned long long)(u & 0x80000000u) << 32;
    if (e == 0) return __longlong_as_double((long long)s);
    return __longlong_as_double(
        (long long)(s | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)(u & 0x7FFFFFu) << 29)));
}

// x[0] + x[stride] + ... + x[(n-1)*stride], added left to right.  The loads
// of a group are issued together ahead of the adds, so a long sum waits for
// memory once per group.  Every load reads a valid address (the index is
// clamped) and every add is unconditional (+0.0 for the indices past n, which
// leaves a sum that starts at +0.0 unchanged): an add guarded by a branch lets
// the compiler move each load next to its add, and the group's loads then wait
// for memory one after another (measured: 3.5x slower on GB300).
template <int G>
FK_DEV double2 ordered_sum_g(const double2* x, long stride, int n) {
    double2 s = make_double2(0.0, 0.0);
    for (int i0 = 0; i0 < n; i0 += G) {
        double2 v[G];
#pragma unroll
        for (int j = 0; j < G; ++j) v[j] = x[(long)min(i0 + j, n - 1) * stride];
#pragma unroll
        for (int j = 0; j < G; ++j) s = cadd(s, i0 + j < n ? v[j] : make_double2(0.0, 0.0));
    }
    return s;
}
FK_DEV double2 ordered_sum(const double2* x, long stride, int n) { return ordered_sum_g<8>(x, stride, n); }
// The same with the loads of up to 16 terms in flight.
FK_DEV double2 ordered_sum16(const double2* x, long stride, int n) { return ordered_sum_g<16>(x, stride, n); }

// --------------------------------------------- compensated FP32 accumulation
// float-float (hi, lo) accumulator updated with Knuth's TwoSum: exact sum of
// the running value and the incoming FP32 block sum, error kept in lo.
struct ff32 { float hi, lo; };
FK_DEV void ff_add(ff32& a, float b) {
    float s = a.hi + b;
    float bb = s - a.hi;
    float err = (a.hi - (s - bb)) + (b - bb);
    a.hi = s;
    a.lo += err;
}

// ------------------------------------------------------- index map (GPP)
// igp for column my_igp, BGW-Kernels/gppKer.cpp:322-328: inv_igp_index equal
// to ncouls maps to ncouls-1 without reading indinv; anything mapping outside
// [0, ncouls) returns -1 and the column is skipped.
FK_DEV int gpp_igp_of(int my_igp, int ncouls, const int* inv_igp_index, const int* indinv) {
    int indigp = inv_igp_index[my_igp];
    int igp;
    if (indigp == ncouls) igp = ncouls - 1;
    else if (indigp < 0 || indigp > ncouls) return -1;
    else igp = indinv[indigp];
    return (igp >= ncouls || igp < 0) ? -1 : igp;
}

#define FK_CUDA_OK(call) ((call) == cudaSuccess)
