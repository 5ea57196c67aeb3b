/*
 * slg_half.h - IEEE binary16 conversions shared by the device kernels, the
 * CPU checker and the LightSky compatibility layer the reference sources are
 * compiled against, so that all three store a half depth the same way.
 *
 * float -> half rounds to nearest, ties to even; values past the largest half
 * become infinities, values below half the smallest subnormal become signed
 * zeros, and a NaN becomes sign | 0x7E00 (quiet, payload dropped).
 * half -> float is exact. Integer arithmetic only, so host and device agree
 * bit for bit.
 */
#ifndef SLG_HALF_H
#define SLG_HALF_H

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
    #define SLG_HALF_HD __host__ __device__ __forceinline__
#else
    #define SLG_HALF_HD static inline
#endif

SLG_HALF_HD uint32_t slg_f32_bits(float f)
{
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t x;
    memcpy(&x, &f, 4);
    return x;
#endif
}

SLG_HALF_HD float slg_f32_from_bits(uint32_t x)
{
#if defined(__CUDA_ARCH__)
    return __uint_as_float(x);
#else
    float f;
    memcpy(&f, &x, 4);
    return f;
#endif
}

SLG_HALF_HD uint16_t slg_float_to_half(float f)
{
    const uint32_t x = slg_f32_bits(f);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const uint32_t e8 = (x >> 23) & 0xFFu;
    const int32_t exp = (int32_t)e8 - 127 + 15;
    uint32_t mant = x & 0x7FFFFFu;
    if (e8 == 0xFFu) return (uint16_t)(sign | 0x7C00u | (mant ? 0x200u : 0u));
    if (exp >= 31) return (uint16_t)(sign | 0x7C00u);
    if (exp <= 0)
    {
        if (exp < -10) return (uint16_t)sign;
        mant |= 0x800000u;
        const uint32_t shift = (uint32_t)(14 - exp);
        uint32_t h = mant >> shift;
        const uint32_t rem = mant & ((1u << shift) - 1u), halfway = 1u << (shift - 1u);
        if (rem > halfway || (rem == halfway && (h & 1u))) ++h;
        return (uint16_t)(sign | h);
    }
    uint32_t h = ((uint32_t)exp << 10) | (mant >> 13);
    const uint32_t rem = mant & 0x1FFFu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
    return (uint16_t)(sign | h);
}

SLG_HALF_HD float slg_half_to_float(uint16_t h)
{
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    const uint32_t exp = (uint32_t)(h >> 10) & 0x1Fu;
    const uint32_t mant = (uint32_t)h & 0x3FFu;
    if (exp == 0)
    {
        if (!mant) return slg_f32_from_bits(sign);
        /* subnormal: mant * 2^-24, exact in binary32 */
        return slg_f32_from_bits(slg_f32_bits((float)mant * (1.f / 16777216.f)) | sign);
    }
    if (exp == 31) return slg_f32_from_bits(sign | 0x7F800000u | (mant << 13));
    return slg_f32_from_bits(sign | ((exp - 15u + 127u) << 23) | (mant << 13));
}

#endif /* SLG_HALF_H */
