/*
 * cf_pinned_math.h — the floating-point operations of the clustered-forward
 * path, pinned so that the CUDA kernels and any host restatement produce the
 * same bits.
 *
 * GLSL leaves three things of the reference shaders to the implementation:
 *
 *  1. pow(): the GLSL 4.60 specification only says that pow's precision is
 *     inherited from exp2(y * log2(x)).  AABBGenerator.comp:72-75 calls it for
 *     the exponential slice depths.  This header defines one deterministic
 *     cf_pow_pinned(x, y) = cf_exp2_pinned(y * cf_log2_pinned(x)), written from
 *     two published series using only correctly rounded IEEE-754 binary32
 *     + - * / and exact bit manipulation:
 *       - log2: x = m * 2^e with m in [sqrt(1/2), sqrt(2)), then
 *         ln(m) = 2 atanh(s), s = (m - 1) / (m + 1), with the odd power series
 *         atanh(s) = s + s^3/3 + s^5/5 + s^7/7 + s^9/9 (|s| <= 0.1716, the
 *         truncation error is below 2e-9 relative);
 *       - exp2: t = n + f with n = nearest integer, |f| <= 1/2, and
 *         2^f = sum_{k=0..7} (f ln 2)^k / k! (Taylor series of exp; the
 *         truncation error is below 8e-9 relative), then scaled by 2^n
 *         through the exponent field.
 *     Its error is a few ulp of binary32 over the slice-depth domain, inside
 *     the GLSL bound.
 *  2. The summation order of mat4 * vec4.  GLSL defines M * v as
 *     v.x*M[0] + v.y*M[1] + v.z*M[2] + v.w*M[3] but not how it is rounded.
 *     The pinned order is left to right, one rounding per operation:
 *        r[i] = ((M[0][i]*v.x + M[1][i]*v.y) + M[2][i]*v.z) + M[3][i]*v.w
 *  3. Contraction into fused multiply-add.  None is allowed: every product
 *     is rounded before it is added.  Device code calls the __fmul_rn /
 *     __fadd_rn / __fdiv_rn intrinsics, which the compiler never contracts;
 *     host code must be built with -ffp-contract=off (GCC contracts by
 *     default on AArch64) and without -ffast-math.
 *
 * min/max follow the GLSL definitions exactly (min(x, y) = y < x ? y : x,
 * max(x, y) = x < y ? y : x), which differ from fminf/fmaxf on signed zeros
 * and NaN.
 *
 * No libm function is used anywhere in this header.
 */
#ifndef CF_PINNED_MATH_H
#define CF_PINNED_MATH_H

#include <stdint.h>
#if !defined(__CUDA_ARCH__)
#include <string.h>
#endif

#if defined(__CUDACC__)
#define CF_HD __host__ __device__ __forceinline__
#else
#define CF_HD static inline
#endif

CF_HD uint32_t cf_float_bits(float f)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, sizeof(u));
    return u;
#endif
}

CF_HD float cf_bits_float(uint32_t u)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, sizeof(f));
    return f;
#endif
}

CF_HD float cf_fmul(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}

CF_HD float cf_fadd(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}

CF_HD float cf_fsub(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}

CF_HD float cf_fdiv(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}

/* Correctly rounded square root (IEEE 754 requires it of sqrt). */
CF_HD float cf_fsqrt(float a)
{
#if defined(__CUDA_ARCH__)
    return __fsqrt_rn(a);
#else
    return __builtin_sqrtf(a);
#endif
}

/* GLSL min / max (GLSL 4.60 §8.3). */
CF_HD float cf_glsl_min(float x, float y) { return (y < x) ? y : x; }
CF_HD float cf_glsl_max(float x, float y) { return (x < y) ? y : x; }

/* Row i of M * v in the pinned order; m is column-major (m[col*4 + row]). */
CF_HD float cf_mat4_row(const float* m, int i, float x, float y, float z, float w)
{
    float r = cf_fadd(cf_fmul(m[0 + i], x), cf_fmul(m[4 + i], y));
    r = cf_fadd(r, cf_fmul(m[8 + i], z));
    return cf_fadd(r, cf_fmul(m[12 + i], w));
}

/* log2 for binary32.  x <= 0 -> -inf (x == 0) or NaN; +inf -> +inf; NaN -> NaN. */
CF_HD float cf_log2_pinned(float x)
{
    if (!(x > 0.0f)) {
        if (x == 0.0f) return cf_bits_float(0xff800000u); /* -inf */
        return cf_bits_float(0x7fc00000u);                /* NaN  */
    }
    uint32_t b = cf_float_bits(x);
    if (b >= 0x7f800000u) return x; /* +inf */
    int e = 0;
    if (b < 0x00800000u) {          /* subnormal: scale by 2^24, exact */
        x = cf_fmul(x, 16777216.0f);
        b = cf_float_bits(x);
        e = -24;
    }
    e += (int)((b >> 23) & 0xffu) - 127;
    float m = cf_bits_float((b & 0x007fffffu) | 0x3f800000u); /* [1, 2) */
    if (m > 0x1.6a09e6p+0f) {                                  /* sqrt(2) */
        m = cf_fmul(m, 0.5f);
        e += 1;
    }
    const float s = cf_fdiv(cf_fsub(m, 1.0f), cf_fadd(m, 1.0f));
    const float s2 = cf_fmul(s, s);
    float p = 0x1.c71c72p-4f;                       /* 1/9 */
    p = cf_fadd(cf_fmul(p, s2), 0x1.24924ap-3f);    /* 1/7 */
    p = cf_fadd(cf_fmul(p, s2), 0x1.99999ap-3f);    /* 1/5 */
    p = cf_fadd(cf_fmul(p, s2), 0x1.555556p-2f);    /* 1/3 */
    p = cf_fadd(cf_fmul(p, s2), 1.0f);
    const float ln_m = cf_fmul(cf_fmul(2.0f, s), p);
    return cf_fadd((float)e, cf_fmul(ln_m, 0x1.715476p+0f)); /* 1/ln 2 */
}

/* 2^t for binary32. */
CF_HD float cf_exp2_pinned(float t)
{
    if (t != t) return t;
    if (t >= 128.0f) return cf_bits_float(0x7f800000u);
    if (t < -151.0f) return 0.0f;
    /* nearest integer (ties to even) by the 1.5 * 2^23 shift; exact here */
    const float n = cf_fsub(cf_fadd(t, 12582912.0f), 12582912.0f);
    const float f = cf_fsub(t, n); /* exact, |f| <= 1/2 */
    float p = 0x1.ffcbfcp-17f;                    /* (ln2)^7/7! */
    p = cf_fadd(cf_fmul(p, f), 0x1.430912p-13f);  /* (ln2)^6/6! */
    p = cf_fadd(cf_fmul(p, f), 0x1.5d87fep-10f);  /* (ln2)^5/5! */
    p = cf_fadd(cf_fmul(p, f), 0x1.3b2ab6p-7f);   /* (ln2)^4/4! */
    p = cf_fadd(cf_fmul(p, f), 0x1.c6b08ep-5f);   /* (ln2)^3/3! */
    p = cf_fadd(cf_fmul(p, f), 0x1.ebfbe0p-3f);   /* (ln2)^2/2! */
    p = cf_fadd(cf_fmul(p, f), 0x1.62e430p-1f);   /*  ln2       */
    p = cf_fadd(cf_fmul(p, f), 1.0f);
    int ni = (int)n;
    /* scale by 2^ni in at most two exact power-of-two steps */
    if (ni > 127) {
        p = cf_fmul(p, cf_bits_float((uint32_t)(127 + 127) << 23));
        ni -= 127;
    } else if (ni < -126) {
        p = cf_fmul(p, cf_bits_float((uint32_t)(-126 + 127) << 23));
        ni += 126;
    }
    if (ni < -126) return cf_fmul(p, 0.0f);
    return cf_fmul(p, cf_bits_float((uint32_t)(ni + 127) << 23));
}

/* pow(x, y) := exp2(y * log2(x)), the form GLSL specifies pow's precision by. */
CF_HD float cf_pow_pinned(float x, float y)
{
    return cf_exp2_pinned(cf_fmul(y, cf_log2_pinned(x)));
}

#endif /* CF_PINNED_MATH_H */
