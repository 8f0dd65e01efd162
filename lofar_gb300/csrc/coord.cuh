// Bit-exact coordinate step of the reference gridder.
//
// The reference converts a normalised coordinate to a cell with
//     pos = uu / dx;  cell = (int)pos              (w-stacking.cu:66-71)
// and uses pos again for the tap distances j + 0.5 - pos (w-stacking.cu:85,89).
//
// When dx is an exact power of two (dx = 2^-k, the case whenever the grid
// size is a power of two, init.c:16), uu/dx equals uu*2^k exactly, so the
// truncation and the fraction pos - cell are read straight off the IEEE-754
// bit pattern with integer instructions: no FP64 arithmetic, which runs at
// 1/64 of the FP32 rate on GB300.  Otherwise the IEEE FP64 division is used,
// as in the reference.  Either way cell is identical to the reference's and
// frac = pos - cell is exact before its final rounding to the stored type.
#pragma once

#include <stdint.h>

namespace wsg {

struct Split {
    long long g;       // trunc(x * 2^k), toward zero
    uint64_t fb;       // |frac| = fb * 2^s
    int s;
    unsigned neg;      // sign bit of x (and of frac)
    bool ok;           // finite and |x * 2^k| < 2^30
};

__device__ __forceinline__ Split split_pow2(double x, int k)
{
    Split r;
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    r.neg = (unsigned)(b >> 63);
    const int e = (int)((b >> 52) & 0x7FF);
    uint64_t m = b & 0xFFFFFFFFFFFFFull;
    r.g = 0;
    r.fb = 0;
    r.s = 0;
    if (e == 0x7FF) {  // NaN or infinity
        r.ok = false;
        return r;
    }
    int E = e;
    if (e) m |= (1ull << 52);
    else E = 1;
    const int s = E - 1075 + k;  // x * 2^k = m * 2^s
    if (s >= 0) {                // |x * 2^k| >= 2^52: far outside any grid
        r.ok = false;
        return r;
    }
    const int sh = -s;
    uint64_t ip, fb;
    if (sh >= 64) {
        ip = 0;
        fb = m;
    } else {
        ip = m >> sh;
        fb = m & ((1ull << sh) - 1ull);
    }
    r.ok = ip < (1ull << 30);
    r.g = r.neg ? -(long long)ip : (long long)ip;
    r.fb = fb;
    r.s = s;
    return r;
}

// (-1)^neg * fb * 2^s rounded to nearest-even float, integer instructions only.
__device__ __forceinline__ float split_frac_f32(const Split &r)
{
    if (r.fb == 0) return r.neg ? -0.0f : 0.0f;
    const int lz = __clzll((long long)r.fb);
    const uint64_t top = r.fb << lz;
    uint32_t m = (uint32_t)(top >> 40);
    const uint64_t rem = top & 0xFFFFFFFFFFull;
    int ex = 63 - lz + r.s;
    if (rem > 0x8000000000ull || (rem == 0x8000000000ull && (m & 1u))) {
        m += 1u;
        if (m == (1u << 24)) {
            m >>= 1;
            ex += 1;
        }
    }
    const int be = ex + 127;
    if (be <= 0) return r.neg ? -0.0f : 0.0f;
    return __uint_as_float((r.neg << 31) | ((uint32_t)be << 23) | (m & 0x7FFFFFu));
}

// (-1)^neg * fb * 2^s exactly as a double (fb < 2^53).
__device__ __forceinline__ double split_frac_f64(const Split &r)
{
    if (r.fb == 0) return r.neg ? -0.0 : 0.0;
    const int lz = __clzll((long long)r.fb);
    const uint64_t mant = r.fb << (lz - 11);
    const int be = 63 - lz + r.s + 1023;
    if (be <= 0) return r.neg ? -0.0 : 0.0;
    return __longlong_as_double((long long)(((uint64_t)r.neg << 63) | ((uint64_t)be << 52) |
                                            (mant & 0xFFFFFFFFFFFFFull)));
}

template <typename F> __device__ __forceinline__ F split_frac(const Split &r);
template <> __device__ __forceinline__ float split_frac<float>(const Split &r)
{
    return split_frac_f32(r);
}
template <> __device__ __forceinline__ double split_frac<double>(const Split &r)
{
    return split_frac_f64(r);
}

template <typename F> struct Cell {
    int g;
    F frac;
    bool ok;
};

// cell = (int)(x/d) and frac = x/d - cell, exactly as the reference.
template <bool POW2, typename F>
__device__ __forceinline__ Cell<F> coord_step(double x, int k, double d)
{
    Cell<F> c;
    if (POW2) {
        const Split r = split_pow2(x, k);
        c.ok = r.ok;
        c.g = (int)r.g;
        c.frac = split_frac<F>(r);
    } else {
        const double pos = x / d;
        c.ok = fabs(pos) < 1073741824.0;  // false for NaN
        const int g = c.ok ? (int)pos : 0;
        c.g = g;
        c.frac = (F)(pos - (double)g);
    }
    return c;
}

// The cell alone, cell = (int)(x/d).  With a power-of-two d = 2^-k and a
// non-negative normal x whose x * 2^k has its integer part in the high word of
// the mantissa (1075 - e - k in [33, 52], e the biased exponent: every x in
// [2^-(k+20), 1) for k <= 20), the integer part is one shift of the high word;
// other inputs take the general path.  Same result as coord_step's cell.
template <bool POW2>
__device__ __forceinline__ int coord_cell(double x, int k, double d, bool &ok)
{
    if (POW2) {
        const unsigned hi = (unsigned)__double2hiint(x);
        const int e = (int)((hi >> 20) & 0x7FFu);
        const int sh = 1075 - e - k;
        if ((hi >> 31) == 0u && e != 0 && sh >= 33 && sh <= 52) {
            ok = true;
            return (int)(((hi & 0xFFFFFu) | 0x100000u) >> (sh - 32));
        }
        const Split r = split_pow2(x, k);
        ok = r.ok;
        return (int)r.g;
    }
    const double pos = x / d;
    ok = fabs(pos) < 1073741824.0;  // false for NaN
    return ok ? (int)pos : 0;
}

// The cell and the fraction as the FP32C record stores it: q24 =
// (frac + 1) * 2^23 rounded to an integer, at most 2^24 - 1.  On coord_cell's
// fast path the fraction's bits are rounded once, to nearest even, straight
// from the mantissa; otherwise the fraction is first rounded to a float.
template <bool POW2>
__device__ __forceinline__ int coord_cell_q24(double x, int k, double d, unsigned &q24, bool &ok)
{
    if (POW2) {
        const unsigned hi = (unsigned)__double2hiint(x);
        const int e = (int)((hi >> 20) & 0x7FFu);
        const int sh = 1075 - e - k;
        if ((hi >> 31) == 0u && e != 0 && sh >= 33 && sh <= 52) {
            const unsigned lo = (unsigned)__double2loint(x);
            const unsigned mh = (hi & 0xFFFFFu) | 0x100000u;
            const unsigned fh = mh & ((1u << (sh - 32)) - 1u);   // fraction = fh:lo * 2^-sh
            const int r = sh - 23;                               // in [10, 29]
            const unsigned t = __funnelshift_r(lo, fh, r);       // floor(frac * 2^23) < 2^23
            const unsigned rem = lo & ((1u << r) - 1u), half = 1u << (r - 1);
            const unsigned up = (rem > half || (rem == half && (t & 1u))) ? 1u : 0u;
            q24 = min((1u << 23) + t + up, 0xFFFFFFu);
            ok = true;
            return (int)(mh >> (sh - 32));
        }
    }
    const Cell<float> c = coord_step<POW2, float>(x, k, d);
    q24 = min((unsigned)__float2int_rn((c.frac + 1.0f) * 8388608.0f), 0xFFFFFFu);
    ok = c.ok;
    return c.g;
}

}  // namespace wsg
