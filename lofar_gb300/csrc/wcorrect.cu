// W-term phase correction and plane sum (phase_correction.cu:11-85 / :147-207)
// and its adjoint.
//
// The reference runs one thread per (plane, pixel) and adds into the image
// with P-way contended FP64 atomics.  Here one thread owns a pixel and walks
// the planes: every plane is read once, coalesced, and the image is written
// once, with no atomics.  The FFT's 1/(Nx*Ny) is folded into `scale`.
//
// Pixel geometry (phase_correction.cu:48-58): x = sin(wrap(iu)*resolution),
// y likewise, r2 = x*x + y*y (evaluated without FMA contraction so the NaN
// mask r2 > 1 matches the reference bit for bit), and for plane w
//     phi_w = 2*PI*(wmin + w*dw)*(sqrt(1-r2) - 1),   amp = dwnorm*sqrt(1-r2).
//
// FP64 form: the plane phasor is advanced by a complex rotation,
// e_{w+1} = e_w * e^{i*2*PI*dw*t}, so each pixel needs two FP64 sincos and
// P complex multiplies instead of 2P FP64 sin/cos (FP64 runs at 1/64 rate).
//
// Adjoint: pixels where the forward image is NaN (r2 > 1) carry no data and
// are excluded (written as zero), so the adjoint is that of the forward
// restricted to its finite pixels.
//
// FP32C form: per pixel, the phase in cycles a + w*b (mod 1) is tabulated once
// per plan (computed in FP64) as Q32 fractions of a cycle; per plane the cycle
// fraction is one integer multiply-add, reduced modulo 1 by the 32-bit
// wrap-around, then one hardware sincos of an argument in [-pi, pi).
#include <cuda_runtime.h>
#include <math.h>

#include "fixed64.cuh"
#include "wsg_internal.cuh"

namespace wsg {

namespace {

__device__ __forceinline__ double pixel_sin(int i, int ntot, double res)
{
    double c = (double)(i - ntot / 2);
    if (c < 0.0) c = (double)(i + ntot / 2);
    return sin(c * res);
}

__global__ void k_wscreen_tables(WcParams p, double *sinx, double *siny)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < p.xaxis) sinx[i] = pixel_sin(i, p.xaxistot, p.resolution);
    if (i < p.yaxis) siny[i] = pixel_sin(i, p.yaxistot, p.resolution);
}

// sqrt(1 - r2) with r2 formed as the reference's CPU path does (no FMA).
__device__ __forceinline__ double pixel_cosine(double xs, double ys)
{
    const double r2 = __dadd_rn(__dmul_rn(xs, xs), __dmul_rn(ys, ys));
    return sqrt(__dadd_rn(1.0, -r2));
}

__global__ void k_wscreen_build(WcParams p, WScreen ws)
{
    const long long npix = (long long)p.xaxis * p.yaxis;
    const double dw = (p.wmax - p.wmin) / (double)p.planes;
    const double dwnorm = dw / (p.wmax - p.wmin);
    // cycles = phi / (2 pi) = (PI / pi) * wterm * t
    const double kappa = kRefPi / 3.141592653589793238462643383279502884;
    for (long long pix = (long long)blockIdx.x * blockDim.x + threadIdx.x; pix < npix;
         pix += (long long)gridDim.x * blockDim.x) {
        const int iu = (int)(pix % p.xaxis);
        const int iv = (int)(pix / p.xaxis);
        const double s = pixel_cosine(ws.sinx[iu], ws.siny[iv]);
        const double t = s - 1.0;
        double a = (p.wmin * t) * kappa;
        double b = (dw * t) * kappa;
        a -= rint(a);
        b -= rint(b);
        // |a|, |b| <= 1/2: a * 2^32 rounded to an integer, taken modulo 2^32
        ws.aq[pix] = (unsigned)llrint(a * 4294967296.0);
        ws.bq[pix] = (unsigned)llrint(b * 4294967296.0);
        ws.amp[pix] = (float)(dwnorm * s);
    }
}

__device__ __forceinline__ void two_sum_acc(float &hi, float &lo, float x)
{
    const float s = hi + x;
    const float z = s - hi;
    lo += (hi - (s - z)) + (x - z);
    hi = s;
}

// ---- FP64 form on the integer pipe --------------------------------------
//
// The phase of plane w at a pixel is the cycle count (wmin + w dw) t kappa
// (kappa = PI / pi, the reference's PI), taken modulo 1 as a Q64 fraction.
// Its cosine and sine come from a 256-entry table of e^{2 pi i k / 256} (Q62,
// built per CTA with FP64 sincospi) and Taylor series of the remaining angle
// (below 2 pi / 256, terms to the 7th power, truncation below 1e-17);
// the planes' phasors then follow by the recurrence e_{w+1} = e_w e_step in
// Q62.  The plane values enter as 53-bit mantissas with a shared exponent
// per complex value, the products are balanced 32-bit-half products, and
// the sum over planes is block floating point (a 64-bit pair with one
// exponent, realigned when a larger term arrives), so about 51 bits of the
// largest term are kept.  No FP64 instruction runs per (pixel, plane).

// (a * b) >> 62, exact floor, for signed a and b.
__device__ __forceinline__ long long q62mul(long long a, long long b)
{
    const long long hi = __mul64hi(a, b);
    const unsigned long long lo = (unsigned long long)a * (unsigned long long)b;
    return (hi << 2) | (long long)(lo >> 62);
}

// frac(c) * 2^64 for the FP64 value c (bits below 2^-64 truncated).
__device__ __forceinline__ unsigned long long cycles_q64(double c)
{
    const long long bits = __double_as_longlong(c);
    const int e = (int)((bits >> 52) & 0x7FF);
    const unsigned long long m =
        (unsigned long long)(bits & 0xFFFFFFFFFFFFFll) | (e ? 0x10000000000000ull : 0ull);
    const int k = max(e, 1) - 1075 + 64;        // c 2^64 = m 2^k
    unsigned long long q;
    if (k >= 64 || k <= -64) q = 0ull;
    else if (k >= 0) q = m << k;
    else q = m >> (-k);
    return bits < 0 ? 0ull - q : q;
}

// e^{2 pi i q / 2^64} in Q62; tab[k] = e^{2 pi i k / 256} in Q62.
__device__ __forceinline__ longlong2 cis_q62(unsigned long long q, const longlong2 *tab)
{
    constexpr long long ONE = 1ll << 62;
    constexpr long long PI_2 = 0x6487ED5110B4611All;   // pi/2 in Q62
    const longlong2 t = tab[q >> 56];
    const unsigned long long r = q & 0x00FFFFFFFFFFFFFFull;   // < 2^56
    // d = 2 pi r / 2^64 in Q62 = r pi / 2
    const long long d = (long long)__umul64hi(r << 2, (unsigned long long)PI_2);
    const long long d2 = q62mul(d, d);
    const long long d4 = q62mul(d2, d2);
    const long long d6 = q62mul(d4, d2);
    const long long c = ONE - (d2 >> 1) + d4 / 24 - d6 / 720;
    const long long sp = ONE - d2 / 6 + d4 / 120 - d6 / 5040;
    const long long sn = q62mul(d, sp);
    return make_longlong2(q62mul(t.x, c) - q62mul(t.y, sn), q62mul(t.y, c) + q62mul(t.x, sn));
}

// The table, built by the CTA's first 256 threads (needs a barrier after).
__device__ __forceinline__ void cis_table(longlong2 *tab)
{
    if (threadIdx.x < 256) {
        double sn, cs;
        sincospi((double)threadIdx.x / 128.0, &sn, &cs);
        const double q = 4611686018427387904.0;   // 2^62
        tab[threadIdx.x] = make_longlong2(__double2ll_rn(cs * q), __double2ll_rn(sn * q));
    }
}

// a * b / 2^62 for Q62 phasors (|a|, |b| <= 1).
__device__ __forceinline__ longlong2 cmul_q62(longlong2 a, longlong2 b)
{
    const Half64 ar = split64(a.x), ai = split64(a.y), br = split64(b.x), bi = split64(b.y);
    return make_longlong2((mulhi_bal(ar, br) - mulhi_bal(ai, bi)) << 2,
                          (mulhi_bal(ar, bi) + mulhi_bal(ai, br)) << 2);
}

// A complex FP64 value as signed 53-bit mantissas with one exponent:
// value = m * 2^(e - 1075).  e = 2047 marks NaN or infinity.
struct Mant2 {
    long long r, i;
    int e;
};

__device__ __forceinline__ Mant2 to_mant2(double2 v)
{
    const long long br = __double_as_longlong(v.x), bi = __double_as_longlong(v.y);
    const int er = (int)((br >> 52) & 0x7FF), ei = (int)((bi >> 52) & 0x7FF);
    long long mr = (br & 0xFFFFFFFFFFFFFll) | (er ? 0x10000000000000ll : 0ll);
    long long mi = (bi & 0xFFFFFFFFFFFFFll) | (ei ? 0x10000000000000ll : 0ll);
    const int xr = max(er, 1), xi = max(ei, 1), e = max(xr, xi);
    const int sr = e - xr, si = e - xi;
    mr = sr >= 63 ? 0 : (sr ? ((mr >> (sr - 1)) + 1) >> 1 : mr);
    mi = si >= 63 ? 0 : (si ? ((mi >> (si - 1)) + 1) >> 1 : mi);
    return {br < 0 ? -mr : mr, bi < 0 ? -mi : mi, max(er, ei) == 2047 ? 2047 : e};
}

// x >> k rounded, k >= 0 (0 for k >= 63).
__device__ __forceinline__ long long shr_rn(long long x, int k)
{
    return k >= 63 ? 0 : (k ? ((x >> (k - 1)) + 1) >> 1 : x);
}

// v 2^k as FP64, flushing results below the normal range to zero.
__device__ __forceinline__ double fixed_to_f64(long long v, int k)
{
    if (v == 0) return 0.0;
    const unsigned long long a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
    if (1086 - __clzll((long long)a) + k < 1) return 0.0;
    return __longlong_as_double(from_fixed(v, k));
}

__global__ void __launch_bounds__(256)
k_wcorrect_f32c(WcParams p, WScreen ws, const float2 *__restrict__ planes,
                float2 *__restrict__ image, float scale)
{
    const long long npix = (long long)p.xaxis * p.yaxis;
    const bool phase = p.phase_on && p.planes > 1;
    for (long long pix = (long long)blockIdx.x * blockDim.x + threadIdx.x; pix < npix;
         pix += (long long)gridDim.x * blockDim.x) {
        float hr = 0.f, lr = 0.f, hi = 0.f, li = 0.f;
        if (phase) {
            const unsigned aq = ws.aq[pix], bq = ws.bq[pix];
#pragma unroll 8
            for (int w = 0; w < p.planes; w++) {
                const float2 g = __ldcs(planes + (size_t)w * npix + pix);
                float sn, cs;
                __sincosf(wscreen_angle(aq, bq, (unsigned)w), &sn, &cs);
                two_sum_acc(hr, lr, g.x * cs - g.y * sn);
                two_sum_acc(hi, li, g.x * sn + g.y * cs);
            }
            const float amp = ws.amp[pix] * scale;
            image[pix] = make_float2((hr + lr) * amp, (hi + li) * amp);
        } else {
#pragma unroll 8
            for (int w = 0; w < p.planes; w++) {
                const float2 g = __ldcs(planes + (size_t)w * npix + pix);
                two_sum_acc(hr, lr, g.x);
                two_sum_acc(hi, li, g.y);
            }
            image[pix] = make_float2((hr + lr) * scale, (hi + li) * scale);
        }
    }
}

__global__ void __launch_bounds__(256)
k_wcorrect_adj_f32c(WcParams p, WScreen ws, const float2 *__restrict__ image,
                    float2 *__restrict__ planes, float scale)
{
    const long long npix = (long long)p.xaxis * p.yaxis;
    const bool phase = p.phase_on && p.planes > 1;
    for (long long pix = (long long)blockIdx.x * blockDim.x + threadIdx.x; pix < npix;
         pix += (long long)gridDim.x * blockDim.x) {
        const float2 im = image[pix];
        if (phase) {
            const unsigned aq = ws.aq[pix], bq = ws.bq[pix];
            const float amp = ws.amp[pix] * scale;
            if (!(amp == amp)) {  // pixel where the forward is NaN: excluded
                for (int w = 0; w < p.planes; w++)
                    __stcs(planes + (size_t)w * npix + pix, make_float2(0.f, 0.f));
                continue;
            }
            const float xr = im.x * amp, xi = im.y * amp;
#pragma unroll 8
            for (int w = 0; w < p.planes; w++) {
                float sn, cs;
                __sincosf(wscreen_angle(aq, bq, (unsigned)w), &sn, &cs);
                __stcs(planes + (size_t)w * npix + pix,
                       make_float2(cs * xr + sn * xi, cs * xi - sn * xr));
            }
        } else {
            const float2 v = make_float2(im.x * scale, im.y * scale);
            for (int w = 0; w < p.planes; w++) __stcs(planes + (size_t)w * npix + pix, v);
        }
    }
}

__global__ void __launch_bounds__(256)
k_wcorrect_f64(WcParams p, const double *__restrict__ sinx, const double *__restrict__ siny,
               const double2 *__restrict__ planes, double2 *__restrict__ image,
               double *__restrict__ image_re, double *__restrict__ image_im, double scale)
{
    __shared__ longlong2 tab[256];
    cis_table(tab);
    __syncthreads();
    const long long npix = (long long)p.xaxis * p.yaxis;
    const bool phase = p.phase_on && p.planes > 1;
    const double dw = (p.wmax - p.wmin) / (double)p.planes;
    const double dwnorm = dw / (p.wmax - p.wmin);
    const double kappa = kRefPi / 3.141592653589793238462643383279502884;
    for (long long pix = (long long)blockIdx.x * blockDim.x + threadIdx.x; pix < npix;
         pix += (long long)gridDim.x * blockDim.x) {
        double s = 1.0;
        longlong2 ph = make_longlong2(1ll << 62, 0), step = ph;
        if (phase) {
            const int iu = (int)(pix % p.xaxis);
            const int iv = (int)(pix / p.xaxis);
            s = pixel_cosine(sinx[iu], siny[iv]);
            const double t = s - 1.0;
            ph = cis_q62(cycles_q64((p.wmin * t) * kappa), tab);
            step = cis_q62(cycles_q64((dw * t) * kappa), tab);
        }
        // sum_w plane_w e_w, block floating point: (ar, ai) 2^(ea - 1075 + 2)
        long long ar = 0, ai = 0;
        int ea = 0;
        bool bad = false;
        for (int w = 0; w < p.planes; w++) {
            const Mant2 g = to_mant2(__ldcs(planes + (size_t)w * npix + pix));
            bad |= g.e == 2047;
            const Half64 gr = split64(g.r), gi = split64(g.i);
            const Half64 pr = split64(ph.x), pi = split64(ph.y);
            const long long tr = mulhi_bal(gr, pr) - mulhi_bal(gi, pi);
            const long long ti = mulhi_bal(gr, pi) + mulhi_bal(gi, pr);
            if (g.e > ea) {
                ar = shr_rn(ar, g.e - ea);
                ai = shr_rn(ai, g.e - ea);
                ea = g.e;
            }
            ar += shr_rn(tr, ea - g.e);
            ai += shr_rn(ti, ea - g.e);
            if (phase) ph = cmul_q62(ph, step);
        }
        double sr, si;
        if (bad || !(s == s)) {
            sr = si = __longlong_as_double(0x7FF8000000000000ll);
        } else {
            const double amp = phase ? dwnorm * s * scale : scale;
            sr = fixed_to_f64(ar, ea - 1075 + 2) * amp;
            si = fixed_to_f64(ai, ea - 1075 + 2) * amp;
        }
        if (image) image[pix] = make_double2(sr, si);
        if (image_re) image_re[pix] = sr;
        if (image_im) image_im[pix] = si;
    }
}

__global__ void __launch_bounds__(256)
k_wcorrect_adj_f64(WcParams p, const double *__restrict__ sinx, const double *__restrict__ siny,
                   const double2 *__restrict__ image, double2 *__restrict__ planes, double scale)
{
    __shared__ longlong2 tab[256];
    cis_table(tab);
    __syncthreads();
    const long long npix = (long long)p.xaxis * p.yaxis;
    const bool phase = p.phase_on && p.planes > 1;
    const double dw = (p.wmax - p.wmin) / (double)p.planes;
    const double dwnorm = dw / (p.wmax - p.wmin);
    const double kappa = kRefPi / 3.141592653589793238462643383279502884;
    for (long long pix = (long long)blockIdx.x * blockDim.x + threadIdx.x; pix < npix;
         pix += (long long)gridDim.x * blockDim.x) {
        const double2 im = image[pix];
        if (!phase) {
            const double2 v = make_double2(im.x * scale, im.y * scale);
            for (int w = 0; w < p.planes; w++) __stcs(planes + (size_t)w * npix + pix, v);
            continue;
        }
        const int iu = (int)(pix % p.xaxis);
        const int iv = (int)(pix / p.xaxis);
        const double s = pixel_cosine(sinx[iu], siny[iv]);
        const double t = s - 1.0;
        const double amp = dwnorm * s * scale;
        if (!(amp == amp)) {  // pixel where the forward is NaN: excluded
            for (int w = 0; w < p.planes; w++)
                __stcs(planes + (size_t)w * npix + pix, make_double2(0.0, 0.0));
            continue;
        }
        longlong2 ph = cis_q62(cycles_q64((p.wmin * t) * kappa), tab);
        const longlong2 step = cis_q62(cycles_q64((dw * t) * kappa), tab);
        const Mant2 x = to_mant2(make_double2(im.x * amp, im.y * amp));
        const Half64 xr = split64(x.r), xi = split64(x.i);
        const int k = x.e - 1075 + 2;
        for (int w = 0; w < p.planes; w++) {
            // conj(e_w) x
            const Half64 pr = split64(ph.x), pi = split64(ph.y);
            const long long orr = mulhi_bal(xr, pr) + mulhi_bal(xi, pi);
            const long long oi = mulhi_bal(xi, pr) - mulhi_bal(xr, pi);
            double2 o;
            if (x.e == 2047)
                o.x = o.y = __longlong_as_double(0x7FF8000000000000ll);
            else
                o = make_double2(fixed_to_f64(orr, k), fixed_to_f64(oi, k));
            __stcs(planes + (size_t)w * npix + pix, o);
            ph = cmul_q62(ph, step);
        }
    }
}

__global__ void k_scale_f64(double2 *x, long long n, double scale)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        double2 v = x[i];
        v.x *= scale;
        v.y *= scale;
        x[i] = v;
    }
}

__global__ void k_f64_to_f32(const double2 *in, float2 *out, long long n)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double2 v = in[i];
        out[i] = make_float2((float)v.x, (float)v.y);
    }
}

__global__ void k_f32_to_f64(const float2 *in, double2 *out, long long n)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float2 v = in[i];
        out[i] = make_double2((double)v.x, (double)v.y);
    }
}

int elem_grid(long long n)
{
    const long long want = (n + 255) / 256;
    const long long cap = (long long)num_sms() * 16;
    return (int)max(1ll, min(want, cap));
}

}  // namespace

cudaError_t launch_wscreen_tables(const WcParams &p, double *sinx, double *siny, cudaStream_t s)
{
    const int n = max(p.xaxis, p.yaxis);
    k_wscreen_tables<<<(n + 255) / 256, 256, 0, s>>>(p, sinx, siny);
    return cudaGetLastError();
}

cudaError_t launch_wscreen_build(const WcParams &p, const WScreen &ws, cudaStream_t s)
{
    k_wscreen_build<<<elem_grid((long long)p.xaxis * p.yaxis), 256, 0, s>>>(p, ws);
    return cudaGetLastError();
}

cudaError_t launch_wcorrect_f32c(const WcParams &p, const WScreen &ws, const float2 *planes,
                                 float2 *image, double scale, cudaStream_t s)
{
    k_wcorrect_f32c<<<elem_grid((long long)p.xaxis * p.yaxis), 256, 0, s>>>(p, ws, planes, image,
                                                                           (float)scale);
    return cudaGetLastError();
}

cudaError_t launch_wcorrect_adj_f32c(const WcParams &p, const WScreen &ws, const float2 *image,
                                     float2 *planes, double scale, cudaStream_t s)
{
    k_wcorrect_adj_f32c<<<elem_grid((long long)p.xaxis * p.yaxis), 256, 0, s>>>(p, ws, image,
                                                                               planes, (float)scale);
    return cudaGetLastError();
}

cudaError_t launch_wcorrect_f64(const WcParams &p, const double *sinx, const double *siny,
                                const double2 *planes, double2 *image, double *image_re,
                                double *image_im, double scale, cudaStream_t s)
{
    k_wcorrect_f64<<<elem_grid((long long)p.xaxis * p.yaxis), 256, 0, s>>>(
        p, sinx, siny, planes, image, image_re, image_im, scale);
    return cudaGetLastError();
}

cudaError_t launch_wcorrect_adj_f64(const WcParams &p, const double *sinx, const double *siny,
                                    const double2 *image, double2 *planes, double scale,
                                    cudaStream_t s)
{
    k_wcorrect_adj_f64<<<elem_grid((long long)p.xaxis * p.yaxis), 256, 0, s>>>(p, sinx, siny,
                                                                              image, planes, scale);
    return cudaGetLastError();
}

cudaError_t launch_scale_f64(double2 *x, long long n, double scale, cudaStream_t s)
{
    k_scale_f64<<<elem_grid(n), 256, 0, s>>>(x, n, scale);
    return cudaGetLastError();
}

cudaError_t launch_f64_to_f32(const double2 *in, float2 *out, long long n, cudaStream_t s)
{
    k_f64_to_f32<<<elem_grid(n), 256, 0, s>>>(in, out, n);
    return cudaGetLastError();
}

cudaError_t launch_f32_to_f64(const float2 *in, double2 *out, long long n, cudaStream_t s)
{
    k_f32_to_f64<<<elem_grid(n), 256, 0, s>>>(in, out, n);
    return cudaGetLastError();
}

}  // namespace wsg
