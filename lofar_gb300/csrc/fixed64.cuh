// Integer-pipe arithmetic for the FP64 form's fixed-point kernels (the
// integer FFT, the FP64 gridder's and degridder's taps).  On this part an
// FP64 instruction issues at 1/64 of the integer rate, so conversions and
// products that keep about 60 significant bits are done with integer
// instructions only.
#pragma once

#include <cuda_runtime.h>

namespace wsg {

// round(x * 2^s) for the FP64 bit pattern `bits`, |x| * 2^s < 2^62; ties
// round away from zero.  Zero and values below 2^-s/2 give 0.
__device__ __forceinline__ long long to_fixed(long long bits, int s)
{
    const int e = (int)((bits >> 52) & 0x7FF);
    const long long m = (bits & 0xFFFFFFFFFFFFFll) | (e ? 0x10000000000000ll : 0ll);
    const int sh = max(e, 1) - 1075 + s;      // |x| 2^s = m 2^sh
    long long r;
    if (sh >= 0)
        r = m << sh;
    else if (sh > -64)
        r = (m + (1ll << (-sh - 1))) >> (-sh);
    else
        r = 0;
    return bits < 0 ? -r : r;
}

// v * 2^k as an FP64 bit pattern, rounded to nearest even; the result is
// assumed to be zero or a normal number.
__device__ __forceinline__ long long from_fixed(long long v, int k)
{
    if (v == 0) return 0;
    const unsigned long long neg = v < 0 ? 0x8000000000000000ull : 0ull;
    const unsigned long long a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
    const int lz = __clzll((long long)a);
    const unsigned long long n = a << lz;                  // top bit set
    unsigned long long mant = n >> 11;                     // 53 bits, hidden bit included
    const unsigned long long rest = n & 0x7FFull;
    mant += (rest > 0x400ull || (rest == 0x400ull && (mant & 1ull))) ? 1ull : 0ull;
    // |v| = n 2^-lz = mant 2^(11 - lz): biased exponent 1086 - lz + k; a carry
    // of the rounding into bit 53 moves into the exponent by the addition
    const long long e = 1086 - lz + k;
    return (long long)(neg | (((unsigned long long)(e - 1) << 52) + mant));
}

// Biased FP64 exponent of x (2047: NaN or infinity; |x| < 2^(e - 1022)).
__device__ __forceinline__ unsigned exp_field(double x)
{
    return (unsigned)(__double_as_longlong(x) >> 52) & 0x7FFu;
}

// v = h 2^32 + l with l in [-2^31, 2^31).
struct Half64 {
    int h, l;
};

__device__ __forceinline__ Half64 split64(long long v)
{
    const int l = (int)(unsigned)v;
    return {(int)(v >> 32) + (int)((unsigned)v >> 31), l};
}

// a b / 2^64 with the low product a_l b_l (below 2^62) dropped and the middle
// sum rounded: the error is below one unit and unbiased.  Requires
// |a_h b_l + a_l b_h| < 2^63 - 2^31.
__device__ __forceinline__ long long mulhi_bal(Half64 a, Half64 b)
{
    const long long mid = (1ll << 31) + (long long)a.h * b.l + (long long)a.l * b.h;
    return (long long)a.h * b.h + (mid >> 32);
}

}  // namespace wsg
