// fp.cuh - separately rounded float operations shared by the kernels and by
// the host-side test of the radius routine.
//
// Every operation of the pass is written with an explicit rounding so that
// nvcc cannot contract a multiply and an add into an FMA: the kernels must
// reproduce, bit for bit, the reference's GLM / BoundingSphere arithmetic
// (one rounding per operation, left to right).
#pragma once

#include <stdint.h>
#include <string.h>
#include <math.h>

#if defined(__CUDACC__)
#define CADR_HD __host__ __device__ __forceinline__
#else
#define CADR_HD static inline
#endif

namespace cadr {

CADR_HD float fmul(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    volatile float r = a * b;
    return r;
#endif
}

CADR_HD float fadd(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    volatile float r = a + b;
    return r;
#endif
}

CADR_HD float fsub(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    volatile float r = a - b;
    return r;
#endif
}

CADR_HD float ffma(float a, float b, float c)
{
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}

CADR_HD float fsqrt(float a)
{
#if defined(__CUDA_ARCH__)
    return __fsqrt_rn(a);
#else
    return sqrtf(a);
#endif
}

CADR_HD float fdiv(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fdiv_rn(a, b);
#else
    volatile float r = a / b;
    return r;
#endif
}

CADR_HD uint32_t fbits(float x)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    uint32_t u;
    memcpy(&u, &x, 4);
    return u;
#endif
}

CADR_HD float bitsf(uint32_t u)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float x;
    memcpy(&x, &u, 4);
    return x;
#endif
}

// The reference radius, float(sqrt(double(x)) * double(r)), evaluated in
// double: the exact (slow) path.
CADR_HD float radius_double(float x, float r)
{
#if defined(__CUDA_ARCH__)
    return __double2float_rn(__dmul_rn(__dsqrt_rn((double)x), (double)r));
#else
    volatile double s = sqrt((double)x);
    volatile double p = s * (double)r;
    return (float)p;
#endif
}

// Bounding-sphere radius of src/CadR/BoundingSphere.h:85 in the reference's
// precision: RN_float(RN_double(RN_double(sqrt(x)) * r)), where x is the
// largest squared column length and r the local radius.
//
// The device has little FP64 throughput, so the common case is computed in
// float-float arithmetic: sqrt(x) = s + t (s = RN(sqrt x), t = (x - s*s)/2s
// with the residual exact by FMA), then (s + t) * r = p + lo with p = RN(s*r)
// and the product error recovered exactly by FMA.  The total error of p + lo
// against the double-rounded reference value is below 2^-44.5 |p|.  The
// result is f = RN(p + lo) unless p + lo lies within 2^-43 |f| of a rounding
// midpoint of f (or f is a power of two, whose lower midpoint is closer);
// only then, about once per million spheres, the double path runs.
// Inputs outside x in [2^-100, 2^100], r in [2^-60, 2^60] (or negative,
// zero, subnormal, infinite, NaN) take the double path as well.
CADR_HD float sphere_radius(float x, float r)
{
    const uint32_t xb = fbits(x), rb = fbits(r);
    const uint32_t xe = xb >> 23, re = rb >> 23;  // sign bit included: negative -> out of range
    if (xe >= 27u && xe <= 227u && re >= 67u && re <= 187u) {
        const float s = fsqrt(x);
        const float e = ffma(-s, s, x);      // exact residual x - s*s
        const float t = fdiv(e, fadd(s, s));
        const float p = fmul(s, r);
        const float q = ffma(s, r, -p);      // exact: s*r - p
        const float lo = fadd(q, fmul(t, r));
        const float f = fadd(p, lo);
        const float d = fadd(fsub(p, f), lo);  // offset of p + lo from f
        const uint32_t fb = fbits(f);
        const uint32_t fe = fb >> 23;          // biased exponent (f > 0, normal)
        const float half_ulp = bitsf((fe - 24u) << 23);
        const float margin = bitsf((fe - 43u) << 23);
        const float gap = fsub(fabsf(d), half_ulp);
        const bool hard = (fabsf(gap) <= margin) || ((fb & 0x7fffffu) == 0u);
        if (!hard) return f;
    }
    return radius_double(x, r);
}

}  // namespace cadr
