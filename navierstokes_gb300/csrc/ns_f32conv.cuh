// ns_f32conv.cuh -- FP32 <-> FP64 conversions on the integer pipe for the
// split-precision and batched FP32 paths.
//
// On GB300 the F2F conversions run on the FP64 pipe, about 60x slower than
// FP32 arithmetic, so these build the IEEE-754 bit patterns with integer
// operations (round to nearest even where a rounding happens).  Magnitudes
// below the FP32 normal range (2^-126) convert to a signed zero instead of
// a subnormal: a value that small is 1e-26 of the smallest perturbation the
// paths resolve, and taking the plain conversion there (an FP64-pipe
// instruction in a divergent branch) slowed the stage kernel by a tenth
// once the far field of a long run filled with such values.  Overflow,
// infinities and NaNs take the plain conversions.
#pragma once

namespace ns {

// x exactly (FP32 subnormals as a signed zero)
__device__ __forceinline__ double f2d_exact(float x)
{
    const unsigned b = __float_as_uint(x);
    const unsigned e = (b >> 23) & 0xffu;
    if (e == 0xffu) return (double)x;  // inf, nan
    const unsigned m = b & 0x7fffffu;
    const unsigned hi = (b & 0x80000000u) | (e ? (((e + (1023u - 127u)) << 20) | (m >> 3)) : 0u);
    const unsigned lo = e ? (m << 29) : 0u;
    return __hiloint2double((int)hi, (int)lo);
}

// x rounded to FP32, nearest even (|x| < 2^-126 as a signed zero)
__device__ __forceinline__ float d2f_rn(double x)
{
    const unsigned hi = (unsigned)__double2hiint(x);
    const unsigned lo = (unsigned)__double2loint(x);
    const unsigned e = (hi >> 20) & 0x7ffu;
    if (e > 1023u + 127u) return (float)x;                            // overflow, inf, nan
    if (e < 1023u - 126u) return __uint_as_float(hi & 0x80000000u);  // zero, tiny
    const unsigned top = ((hi & 0xfffffu) << 3) | (lo >> 29);  // 23 mantissa bits
    const unsigned rest = lo & 0x1fffffffu;                    // 29 discarded bits
    unsigned f = (hi & 0x80000000u) | ((e - (1023u - 127u)) << 23) | top;
    const unsigned half = 1u << 28;
    if (rest > half || (rest == half && (top & 1u))) f += 1u;  // carry may bump the exponent
    return __uint_as_float(f);
}

// hi = x rounded to FP32 (nearest even) and lo = x - hi rounded to FP32, with
// integer operations and one integer-to-float conversion: the remainder is
// the 29 discarded mantissa bits, minus 2^29 when hi rounded up, times
// 2^(e - 1075).  Below 2^-74 lo would fall under the FP32 normal range and
// is zero (hi as d2f_rn); from 2^128 on the plain conversion.
__device__ __forceinline__ void d2f_split(double x, float &hi, float &lo)
{
    const unsigned xh = (unsigned)__double2hiint(x), xl = (unsigned)__double2loint(x);
    const unsigned e = (xh >> 20) & 0x7ffu;
    if (e < 949u || e > 1150u) {
        hi = d2f_rn(x);
        lo = 0.f;
        return;
    }
    const unsigned top = ((xh & 0xfffffu) << 3) | (xl >> 29);  // 23 mantissa bits
    const unsigned rest = xl & 0x1fffffffu;                    // 29 discarded bits
    unsigned f = (xh & 0x80000000u) | ((e - 896u) << 23) | top;
    int r = (int)rest;
    const unsigned half = 1u << 28;
    if (rest > half || (rest == half && (top & 1u))) {  // carry may bump the exponent
        f += 1u;
        r -= (1 << 29);
    }
    hi = __uint_as_float(f);
    const float mag = __int2float_rn(r) * __uint_as_float((e - 948u) << 23);
    lo = (xh & 0x80000000u) ? -mag : mag;
}

}  // namespace ns
