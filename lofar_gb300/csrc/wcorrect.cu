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
// per plan as reduced float-float pairs (computed in FP64); per plane the
// fractional cycle is recovered exactly in FP32 with an error-free product
// and TwoSum, then one hardware sincos of an argument in [-pi, pi].
#include <cuda_runtime.h>
#include <math.h>

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
        const float ah = (float)a, bh = (float)b;
        ws.ah[pix] = ah;
        ws.al[pix] = (float)(a - (double)ah);
        ws.bh[pix] = bh;
        ws.bl[pix] = (float)(b - (double)bh);
        ws.amp[pix] = (float)(dwnorm * s);
    }
}

// Fractional cycle of a + w*b, |a|,|b| <= 1/2 given as float-float pairs.
__device__ __forceinline__ float cycle_frac(float ah, float al, float bh, float bl, float wf)
{
    const float p = wf * bh;
    const float pe = fmaf(wf, bh, -p);          // exact product error
    const float s = ah + p;
    const float z = s - ah;
    const float se = (ah - (s - z)) + (p - z);  // TwoSum error
    const float lo = fmaf(wf, bl, al) + (pe + se);
    return (s - rintf(s)) + lo;                 // s - rint(s) is exact
}

__device__ __forceinline__ void two_sum_acc(float &hi, float &lo, float x)
{
    const float s = hi + x;
    const float z = s - hi;
    lo += (hi - (s - z)) + (x - z);
    hi = s;
}

constexpr float kTwoPiF = 6.28318530717958647692f;

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
            const float ah = ws.ah[pix], al = ws.al[pix], bh = ws.bh[pix], bl = ws.bl[pix];
#pragma unroll 8
            for (int w = 0; w < p.planes; w++) {
                const float2 g = __ldcs(planes + (size_t)w * npix + pix);
                const float c = cycle_frac(ah, al, bh, bl, (float)w);
                float sn, cs;
                __sincosf(kTwoPiF * c, &sn, &cs);
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
            const float ah = ws.ah[pix], al = ws.al[pix], bh = ws.bh[pix], bl = ws.bl[pix];
            const float amp = ws.amp[pix] * scale;
            if (!(amp == amp)) {  // pixel where the forward is NaN: excluded
                for (int w = 0; w < p.planes; w++)
                    __stcs(planes + (size_t)w * npix + pix, make_float2(0.f, 0.f));
                continue;
            }
            const float xr = im.x * amp, xi = im.y * amp;
#pragma unroll 8
            for (int w = 0; w < p.planes; w++) {
                const float c = cycle_frac(ah, al, bh, bl, (float)w);
                float sn, cs;
                __sincosf(kTwoPiF * c, &sn, &cs);
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
    const long long npix = (long long)p.xaxis * p.yaxis;
    const bool phase = p.phase_on && p.planes > 1;
    const double dw = (p.wmax - p.wmin) / (double)p.planes;
    const double dwnorm = dw / (p.wmax - p.wmin);
    for (long long pix = (long long)blockIdx.x * blockDim.x + threadIdx.x; pix < npix;
         pix += (long long)gridDim.x * blockDim.x) {
        double sr = 0.0, si = 0.0;
        if (phase) {
            const int iu = (int)(pix % p.xaxis);
            const int iv = (int)(pix / p.xaxis);
            const double s = pixel_cosine(sinx[iu], siny[iv]);
            const double t = s - 1.0;
            double er, ei, rr, ri;
            sincos(2.0 * kRefPi * p.wmin * t, &ei, &er);
            sincos(2.0 * kRefPi * dw * t, &ri, &rr);
            for (int w = 0; w < p.planes; w++) {
                const double2 g = __ldcs(planes + (size_t)w * npix + pix);
                sr += g.x * er - g.y * ei;
                si += g.x * ei + g.y * er;
                const double nr = er * rr - ei * ri;
                ei = er * ri + ei * rr;
                er = nr;
            }
            const double amp = dwnorm * s * scale;
            sr *= amp;
            si *= amp;
        } else {
            for (int w = 0; w < p.planes; w++) {
                const double2 g = __ldcs(planes + (size_t)w * npix + pix);
                sr += g.x;
                si += g.y;
            }
            sr *= scale;
            si *= scale;
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
    const long long npix = (long long)p.xaxis * p.yaxis;
    const bool phase = p.phase_on && p.planes > 1;
    const double dw = (p.wmax - p.wmin) / (double)p.planes;
    const double dwnorm = dw / (p.wmax - p.wmin);
    for (long long pix = (long long)blockIdx.x * blockDim.x + threadIdx.x; pix < npix;
         pix += (long long)gridDim.x * blockDim.x) {
        const double2 im = image[pix];
        if (phase) {
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
            const double xr = im.x * amp, xi = im.y * amp;
            double er, ei, rr, ri;
            sincos(2.0 * kRefPi * p.wmin * t, &ei, &er);
            sincos(2.0 * kRefPi * dw * t, &ri, &rr);
            for (int w = 0; w < p.planes; w++) {
                __stcs(planes + (size_t)w * npix + pix,
                       make_double2(er * xr + ei * xi, er * xi - ei * xr));
                const double nr = er * rr - ei * ri;
                ei = er * ri + ei * rr;
                er = nr;
            }
        } else {
            const double2 v = make_double2(im.x * scale, im.y * scale);
            for (int w = 0; w < p.planes; w++) __stcs(planes + (size_t)w * npix + pix, v);
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
