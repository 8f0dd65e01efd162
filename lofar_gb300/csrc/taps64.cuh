// Gaussian tap weights of the FP64 gridder and degridder.
//
// On this part an FP64 instruction issues at 1/64 of the FP32 and integer
// rates, so the weights of the reference's kernel (w-stacking.cu:80-92:
// norm * exp(-(du^2 + dv^2) / 2), du = i + 0.5 - pos) are evaluated per axis
// as
//     exp(-(m + c)^2 / 2) = exp(-m^2 / 2) * exp(-c^2 / 2) * exp(-c)^m,
// with c = 0.5 - frac (frac the record's offset inside its cell) and
// m = -K..K the tap's offset from the cell; for m < 0, exp(-c)^m is taken as
// (1 / exp(-c))^|m|.  A record needs four exponentials (two per axis)
// instead of 2(2K+1), so one warp-wide FP64 exponential serves eight
// records: lane q of the pass computes value q % 4 of record q / 4, and a
// warp-wide reciprocal follows.  That pass is the only FP64 arithmetic of
// the fixed-point kernels: the factors exp(-m^2/2) are per-lane constants
// and the K-step power ladders run in Q62 integers (taps64_factors_q).  The
// FP64 ladders (taps64_factors) serve the FP64-atomic fallback.  The
// rounding differs from the direct form by a few units in the last place.
//
// Tap layout: a group of G lanes (G = 4, 8 or 16, at least 2K+1) takes one
// record, lane i of the group holding the u-factor of column i and the
// v-factor of row i, so R = 32/G records share every tap instruction.
#pragma once

#include <cuda_runtime.h>

#include "fixed64.cuh"

namespace wsg {

template <int K> struct Taps64 {
    static constexpr int NT = 2 * K + 1;
    static constexpr int G = NT <= 4 ? 4 : (NT <= 8 ? 8 : 16);
    static constexpr int R = 32 / G;                   // records per tap pass
    static constexpr int RE = 8;                       // records per exponential pass
    static constexpr int SUB = RE / R;                 // tap passes per exponential pass
    static_assert(NT <= 16, "support above 31 points");
};

// Per-lane constants: exp(-m^2/2) (times norm for the u-factor) for the lane's
// index i = lane % G; zero for lanes past the window.
template <int K>
__device__ __forceinline__ void taps64_consts(int lane, double norm, double &nt_u, double &t_v)
{
    using P = Taps64<K>;
    const int i = lane % P::G;
    const double m = (double)(i - K);
    const double t = i < P::NT ? exp(-(m * m) * 0.5) : 0.0;
    nt_u = norm * t;
    t_v = t;
}

// The exponential pass for records first .. first + count - 1 of `fr`
// (count <= RE = 8): lane l holds value l % 4 of record l / 4, in the order
// exp(-cu^2/2), exp(-cu), exp(-cv^2/2), exp(-cv), and its reciprocal.
struct Exps64 {
    double e, inv;
};

__device__ __forceinline__ Exps64 taps64_exps(const double2 *__restrict__ fr, unsigned count,
                                              int lane)
{
    const int r = lane >> 2, t = lane & 3;
    double f = 0.0;
    if ((unsigned)r < count) {
        const double2 v = __ldg(fr + r);
        f = t < 2 ? v.x : v.y;
    }
    const double c = 0.5 - f;
    const double e = exp((t & 1) ? -c : -(c * c) * 0.5);
    return {e, 1.0 / e};
}

// The factors of lane i = lane % G for record r of the exponential pass:
// gu = norm * exp(-(m + cu)^2 / 2), gv = exp(-(m + cv)^2 / 2), m = i - K
// (zero past the window).  Every lane of the warp must call it.
template <int K>
__device__ __forceinline__ void taps64_factors(const Exps64 &E, int r, int lane, double nt_u,
                                               double t_v, double &gu, double &gv)
{
    using P = Taps64<K>;
    const int m = lane % P::G - K;
    const int am = m < 0 ? -m : m;
    const int q = 4 * r;
    const double au = __shfl_sync(0xFFFFFFFFu, E.e, q);
    const double bu_p = __shfl_sync(0xFFFFFFFFu, E.e, q + 1);
    const double bu_n = __shfl_sync(0xFFFFFFFFu, E.inv, q + 1);
    const double av = __shfl_sync(0xFFFFFFFFu, E.e, q + 2);
    const double bv_p = __shfl_sync(0xFFFFFFFFu, E.e, q + 3);
    const double bv_n = __shfl_sync(0xFFFFFFFFu, E.inv, q + 3);
    const double bu = m > 0 ? bu_p : bu_n;
    const double bv = m > 0 ? bv_p : bv_n;
    double pu = 1.0, pv = 1.0;
#pragma unroll
    for (int t = 1; t <= K; t++) {
        if (t <= am) {
            pu *= bu;
            pv *= bv;
        }
    }
    gu = nt_u * au * pu;
    gv = t_v * av * pv;
}

// Integer form of the factors: Q62 values of gu and gv (zero past the
// window).  The reference's cell is pos truncated toward zero, so frac lies
// in (-1, 1), c in (-1/2, 3/2), and the exponential pass's values reach
// e^{3/2}; they are converted to Q60 (below 8) on their own lanes.  Each
// ladder starts from exp(-m^2/2) exp(-c^2/2) and multiplies by exp(-+c) |m|
// times; every partial product exp(-(m^2 + c^2 - 2|i c|)/2), i <= |m|, is at
// most 1, so gu and gv stay in Q62.  A product is rounded to within 16 units
// of 2^-62.
struct Exps64Q {
    long long e, inv;   // Q60
};

__device__ __forceinline__ Exps64Q taps64_exps_q60(const Exps64 &E)
{
    return {to_fixed(__double_as_longlong(E.e), 60), to_fixed(__double_as_longlong(E.inv), 60)};
}

// (a b) >> 60 for a in Q62 and b in Q60 (b below 2^62.6).
__device__ __forceinline__ long long q60mul_bal(long long a, long long b)
{
    return mulhi_bal(split64(a), split64(b)) << 4;
}

template <int K>
__device__ __forceinline__ void taps64_factors_q(const Exps64Q &E, int r, int lane,
                                                   long long nt_u, long long t_v, long long &gu,
                                                   long long &gv)
{
    using P = Taps64<K>;
    const int m = lane % P::G - K;
    const int am = m < 0 ? -m : m;
    const int q = 4 * r;
    const long long au = __shfl_sync(0xFFFFFFFFu, E.e, q);
    const long long bu_p = __shfl_sync(0xFFFFFFFFu, E.e, q + 1);
    const long long bu_n = __shfl_sync(0xFFFFFFFFu, E.inv, q + 1);
    const long long av = __shfl_sync(0xFFFFFFFFu, E.e, q + 2);
    const long long bv_p = __shfl_sync(0xFFFFFFFFu, E.e, q + 3);
    const long long bv_n = __shfl_sync(0xFFFFFFFFu, E.inv, q + 3);
    const long long bu = m > 0 ? bu_p : bu_n;
    const long long bv = m > 0 ? bv_p : bv_n;
    gu = q60mul_bal(nt_u, au);
    gv = q60mul_bal(t_v, av);
#pragma unroll
    for (int t = 1; t <= K; t++) {
        if (t <= am) {
            gu = q60mul_bal(gu, bu);
            gv = q60mul_bal(gv, bv);
        }
    }
}

}  // namespace wsg
