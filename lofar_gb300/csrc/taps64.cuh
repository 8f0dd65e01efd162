// FP64 Gaussian tap weights for the FP64 gridder and degridder.
//
// On this part an FP64 instruction issues at a small fraction of the FP32
// rate, so the FP64 kernels are bound by the number of FP64 warp instructions
// per record, not by memory.  The weights of the reference's kernel
// (w-stacking.cu:80-92: norm * exp(-(du^2 + dv^2) / 2), du = i + 0.5 - pos)
// are evaluated per axis as
//     exp(-(m + c)^2 / 2) = exp(-m^2 / 2) * exp(-c^2 / 2) * exp(-c)^m,
// with c = 0.5 - frac (frac the record's offset inside its cell) and
// m = -K..K the tap's offset from the cell; for m < 0, exp(-c)^m is taken as
// exp(c)^|m|.  A record needs six exponentials (three per axis) instead of
// 2(2K+1), so one warp-wide exponential serves several records: lane q of
// the exponential pass computes value q % 6 of record q / 6.  The factors
// exp(-m^2/2) are per-lane constants, and the powers take K multiplies.  The
// rounding differs from the direct form by a few units in the last place
// (at most K + 4 roundings per factor).
//
// Tap layout: a group of G lanes (G = 4, 8 or 16, at least 2K+1) takes one
// record, lane i of the group holding the u-factor of column i and the
// v-factor of row i, so R = 32/G records share every tap instruction.
#pragma once

#include <cuda_runtime.h>

namespace wsg {

template <int K> struct Taps64 {
    static constexpr int NT = 2 * K + 1;
    static constexpr int G = NT <= 4 ? 4 : (NT <= 8 ? 8 : 16);
    static constexpr int R = 32 / G;                   // records per tap pass
    static constexpr int SUB = R >= 4 ? 1 : 2;         // tap passes per exponential pass
    static constexpr int RE = R * SUB;                 // records per exponential pass
    static constexpr int EP = (6 * RE + 31) / 32;      // exponential passes (warp-wide)
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
// (count <= RE): E[p] on lane l holds value (32 p + l) % 6 of record
// (32 p + l) / 6, in the order exp(-cu^2/2), exp(-cu), exp(cu), exp(-cv^2/2),
// exp(-cv), exp(cv).
template <int K>
__device__ __forceinline__ void taps64_exps(double (&E)[Taps64<K>::EP],
                                            const double2 *__restrict__ fr, unsigned count,
                                            int lane)
{
    using P = Taps64<K>;
#pragma unroll
    for (int p = 0; p < P::EP; p++) {
        const int q = 32 * p + lane;
        const int r = q / 6, t = q - 6 * (q / 6);
        double f = 0.0;
        if ((unsigned)r < count) {
            const double2 v = __ldg(fr + r);
            f = t < 3 ? v.x : v.y;
        }
        const double c = 0.5 - f;
        const int kind = t < 3 ? t : t - 3;
        const double arg = kind == 0 ? -(c * c) * 0.5 : (kind == 1 ? -c : c);
        E[p] = exp(arg);
    }
}

template <int EP>
__device__ __forceinline__ double taps64_fetch(const double (&E)[EP], int q)
{
    double v = __shfl_sync(0xFFFFFFFFu, E[0], q & 31);
#pragma unroll
    for (int p = 1; p < EP; p++) {
        const double w = __shfl_sync(0xFFFFFFFFu, E[p], q & 31);
        if ((q >> 5) == p) v = w;
    }
    return v;
}

// The factors of lane i = lane % G for record r of the exponential pass:
// gu = norm * exp(-(m + cu)^2 / 2), gv = exp(-(m + cv)^2 / 2), m = i - K
// (zero past the window).  Every lane of the warp must call it.
template <int K>
__device__ __forceinline__ void taps64_factors(const double (&E)[Taps64<K>::EP], int r, int lane,
                                               double nt_u, double t_v, double &gu, double &gv)
{
    using P = Taps64<K>;
    const int m = lane % P::G - K;
    const int am = m < 0 ? -m : m;
    const int q = 6 * r;
    const double au = taps64_fetch(E, q);
    const double bu = taps64_fetch(E, q + (m > 0 ? 1 : 2));
    const double av = taps64_fetch(E, q + 3);
    const double bv = taps64_fetch(E, q + (m > 0 ? 4 : 5));
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

}  // namespace wsg
