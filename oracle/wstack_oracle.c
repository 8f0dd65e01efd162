/*
 * CPU restatement of the w-stacking hot path (TEST INFRASTRUCTURE ONLY).
 *
 * This file is the oracle that the CUDA library is checked against.  It is
 * never linked into, loaded by, or called from the product library
 * (lofar_gb300/libwstack_gb300.so); only the tests, the smoke check and the
 * CPU-baseline leg of bench.py load it.
 *
 * Each function restates, in plain C with OpenMP, the arithmetic of one
 * reference routine (nandhanas/LOFAR, the HPC_Imaging w-stacking imager),
 * keeping the reference's evaluation order so that a single-threaded run
 * reproduces the reference's CPU path bit for bit:
 *
 *   oracle_wstack             w-stacking.cu:222-311 (OpenMP CPU body of wstack)
 *   oracle_phase_correction   phase_correction.cu:147-207 (OpenMP CPU body,
 *                             PHASE_ON defined)
 *   oracle_degrid             the exact transpose of oracle_wstack's map from
 *                             the folded measurement value to the grid (the
 *                             reference has no adjoint)
 *   oracle_phase_adjoint      the exact adjoint of oracle_phase_correction
 *   oracle_grid_plane,        oracle_wstack / oracle_degrid restricted to
 *   oracle_degrid_plane       the measurements of one w-plane, on a single
 *                             [Ny][Nx] plane buffer
 *   oracle_phase_window       oracle_phase_correction (and its adjoint) for
 *                             one plane on a window of pixels
 * The last three let oracle.py evaluate a window of the image of grids whose
 * FP64 cube does not fit in host memory, one plane at a time.
 *
 * Parity is pinned against the reference itself: oracle/Makefile compiles the
 * reference's w-stacking.cu and phase_correction.cu as C into oracle/_ref/,
 * and tests/golden/ holds fixtures produced by that build.
 *
 * Differences from the reference, all outside its defined behaviour:
 *   - grid offsets are computed in 64-bit arithmetic (the reference computes
 *     j + k*Nx + w*Nx*Ny in int, which overflows once P*Nx*Ny >= 2^31);
 *   - a measurement whose w-plane index falls outside [0, P) is skipped (the
 *     reference writes outside the grid for it, w-stacking.cu:69,90).
 */
#include <math.h>
#include <stddef.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* The reference's pi (w-stacking.h:6); deliberately not M_PI. */
#define ORACLE_PI 3.14159265359

/* Gaussian convolution weight, w-stacking.cu:17-22. */
static double oracle_gauss(double norm, double std22, double du, double dv)
{
    return norm * exp(-((du * du) + (dv * dv)) * std22);
}

/*
 * Gridding, w-stacking.cu:222-311.  Accumulates (+=) into grid, laid out as
 * [plane][v][u][re,im] doubles (w-stacking.cu:274).
 */
void oracle_wstack(int num_w_planes, long num_points, long freq_per_chan,
                   long polarizations, const double *uu, const double *vv,
                   const double *ww, const float *vis_real,
                   const float *vis_img, const float *weight, double dx,
                   double dw, int w_support, int grid_size_x,
                   int grid_size_y, double *grid, int num_threads)
{
    /* kernel constants, w-stacking.cu:148-151 */
    const int half = (w_support - 1) / 2;
    const double sigma = 1.0;
    const double std22 = 1.0 / (2.0 * sigma * sigma);
    const double norm = std22 / ORACLE_PI;
    const long plane_cells = (long)grid_size_x * (long)grid_size_y;

#ifdef _OPENMP
    if (num_threads > 0) omp_set_num_threads(num_threads);
#else
    (void)num_threads;
#endif

#pragma omp parallel for schedule(static)
    for (long m = 0; m < num_points; m++) {
        const long vbase = m * freq_per_chan * polarizations;
        /* coordinate step, w-stacking.cu:250-255 */
        const double pu = uu[m] / dx;
        const double pv = vv[m] / dx;
        const double pw = ww[m] / dw;
        const int cw = (int)pw;
        const int cu = (int)pu;
        const int cv = (int)pv;
        if (cw < 0 || cw >= num_w_planes) continue;

        /* clipped support window, w-stacking.cu:258-261 */
        const long j0 = (cu > half - 1) ? cu - half : 0;
        const long j1 = (cu < grid_size_x - half) ? cu + half : grid_size_x - 1;
        const long k0 = (cv > half - 1) ? cv - half : 0;
        const long k1 = (cv < grid_size_y - half) ? cv + half : grid_size_y - 1;

        for (long k = k0; k <= k1; k++) {
            const double dist_v = (double)k + 0.5 - pv;
            for (long j = j0; j <= j1; j++) {
                const double dist_u = (double)j + 0.5 - pu;
                const long cell = 2 * (j + k * (long)grid_size_x + (long)cw * plane_cells);
                const double cwt = oracle_gauss(norm, std22, dist_u, dist_v);
                /* frequency/polarisation fold, w-stacking.cu:279-298:
                 * weight*vis is a float product, then promoted to double. */
                double acc_re = 0.0, acc_im = 0.0;
                long fine = vbase;
                for (long f = 0; f < freq_per_chan; f++) {
                    long iw = vbase / freq_per_chan;
                    for (long p = 0; p < polarizations; p++) {
                        if (!isnan(vis_real[fine])) {
                            acc_re += weight[iw] * vis_real[fine] * cwt;
                            acc_im += weight[iw] * vis_img[fine] * cwt;
                        }
                        fine++;
                        iw++;
                    }
                }
#pragma omp atomic
                grid[cell] += acc_re;
#pragma omp atomic
                grid[cell + 1] += acc_im;
            }
        }
    }
}

/* Pixel direction cosine, phase_correction.cu:164-169 (half-grid wrap). */
static double oracle_pixel_sin(int i, int ntot, double resolution)
{
    double c = (double)(i - ntot / 2);
    if (c < 0.0) c = (double)(i + ntot / 2);
    return sin(c * resolution);
}

/*
 * W-term phase correction and plane sum, phase_correction.cu:147-207 with
 * PHASE_ON.  Accumulates (+=) into image_real/image_imag ([v][u] doubles).
 * phase_on = 0 reproduces the build without PHASE_ON (plain plane sum).
 */
void oracle_phase_correction(const double *gridss, double *image_real,
                             double *image_imag, int xaxis, int yaxis,
                             int num_w_planes, int xaxistot, int yaxistot,
                             double resolution, double wmin, double wmax,
                             int num_threads, int phase_on)
{
    /* phase_correction.cu:92-94 */
    const double dw = (wmax - wmin) / (double)num_w_planes;
    const double dwnorm = dw / (wmax - wmin);
    const long plane_cells = (long)xaxis * (long)yaxis;

#ifdef _OPENMP
    if (num_threads > 0) omp_set_num_threads(num_threads);
#else
    (void)num_threads;
#endif

#pragma omp parallel for collapse(3) schedule(static)
    for (int iw = 0; iw < num_w_planes; iw++) {
        for (int iv = 0; iv < yaxis; iv++) {
            for (int iu = 0; iu < xaxis; iu++) {
                const long src = 2 * (iu + (long)iv * xaxis + plane_cells * iw);
                const long pix = iu + (long)iv * xaxis;
                const double wterm = wmin + iw * dw;
                if (phase_on && num_w_planes > 1) {
                    const double xs = oracle_pixel_sin(iu, xaxistot, resolution);
                    const double ys = oracle_pixel_sin(iv, yaxistot, resolution);
                    const double r2 = (xs * xs + ys * ys);
                    const double pre = cos(2.0 * ORACLE_PI * wterm * (sqrt(1 - r2) - 1.0));
                    const double pim = sin(2.0 * ORACLE_PI * wterm * (sqrt(1 - r2) - 1.0));
                    const double a = gridss[src];
                    const double b = gridss[src + 1];
#pragma omp atomic
                    image_real[pix] += (a * pre - b * pim) * dwnorm * sqrt(1 - r2);
#pragma omp atomic
                    image_imag[pix] += (a * pim + b * pre) * dwnorm * sqrt(1 - r2);
                } else {
#pragma omp atomic
                    image_real[pix] += gridss[src];
#pragma omp atomic
                    image_imag[pix] += gridss[src + 1];
                }
            }
        }
    }
}

/*
 * Adjoint of the gridding map.  The forward map sends the folded measurement
 * value V_m = sum_{f,p} weight*vis (complex) to grid cells with real weights
 * c_m(cell) = norm*exp(-(du^2+dv^2)/2); its transpose is
 *     out[m] = sum_{cell in window(m)} c_m(cell) * grid[plane(m)][cell]
 * with the same window, clipping and plane rule as oracle_wstack.
 * out is [num_points][re,im] doubles, overwritten.
 */
void oracle_degrid(int num_w_planes, long num_points, const double *uu,
                   const double *vv, const double *ww, double dx, double dw,
                   int w_support, int grid_size_x, int grid_size_y,
                   const double *grid, double *out, int num_threads)
{
    const int half = (w_support - 1) / 2;
    const double std22 = 0.5;
    const double norm = std22 / ORACLE_PI;
    const long plane_cells = (long)grid_size_x * (long)grid_size_y;

#ifdef _OPENMP
    if (num_threads > 0) omp_set_num_threads(num_threads);
#else
    (void)num_threads;
#endif

#pragma omp parallel for schedule(static)
    for (long m = 0; m < num_points; m++) {
        const double pu = uu[m] / dx;
        const double pv = vv[m] / dx;
        const int cw = (int)(ww[m] / dw);
        const int cu = (int)pu;
        const int cv = (int)pv;
        double sre = 0.0, sim = 0.0;
        if (cw >= 0 && cw < num_w_planes) {
            const long j0 = (cu > half - 1) ? cu - half : 0;
            const long j1 = (cu < grid_size_x - half) ? cu + half : grid_size_x - 1;
            const long k0 = (cv > half - 1) ? cv - half : 0;
            const long k1 = (cv < grid_size_y - half) ? cv + half : grid_size_y - 1;
            for (long k = k0; k <= k1; k++) {
                const double dist_v = (double)k + 0.5 - pv;
                for (long j = j0; j <= j1; j++) {
                    const double dist_u = (double)j + 0.5 - pu;
                    const long cell = 2 * (j + k * (long)grid_size_x + (long)cw * plane_cells);
                    const double cwt = oracle_gauss(norm, std22, dist_u, dist_v);
                    sre += cwt * grid[cell];
                    sim += cwt * grid[cell + 1];
                }
            }
        }
        out[2 * m] = sre;
        out[2 * m + 1] = sim;
    }
}

/*
 * Adjoint of oracle_phase_correction (PHASE_ON): broadcasts the complex image
 * back to every plane with the conjugate phase,
 *     planes[w][pix] = conj(e^{i phi_w(pix)}) * dwnorm * sqrt(1-r2) * image[pix]
 * and, for a single plane, planes[0] = image.  planes is overwritten.
 */
void oracle_phase_adjoint(const double *image_real, const double *image_imag,
                          double *planes, int xaxis, int yaxis,
                          int num_w_planes, int xaxistot, int yaxistot,
                          double resolution, double wmin, double wmax,
                          int num_threads, int phase_on)
{
    const double dw = (wmax - wmin) / (double)num_w_planes;
    const double dwnorm = dw / (wmax - wmin);
    const long plane_cells = (long)xaxis * (long)yaxis;

#ifdef _OPENMP
    if (num_threads > 0) omp_set_num_threads(num_threads);
#else
    (void)num_threads;
#endif

#pragma omp parallel for collapse(3) schedule(static)
    for (int iw = 0; iw < num_w_planes; iw++) {
        for (int iv = 0; iv < yaxis; iv++) {
            for (int iu = 0; iu < xaxis; iu++) {
                const long dst = 2 * (iu + (long)iv * xaxis + plane_cells * iw);
                const long pix = iu + (long)iv * xaxis;
                const double xr = image_real[pix];
                const double xi = image_imag[pix];
                if (phase_on && num_w_planes > 1) {
                    const double wterm = wmin + iw * dw;
                    const double xs = oracle_pixel_sin(iu, xaxistot, resolution);
                    const double ys = oracle_pixel_sin(iv, yaxistot, resolution);
                    const double r2 = (xs * xs + ys * ys);
                    const double pre = cos(2.0 * ORACLE_PI * wterm * (sqrt(1 - r2) - 1.0));
                    const double pim = sin(2.0 * ORACLE_PI * wterm * (sqrt(1 - r2) - 1.0));
                    const double amp = dwnorm * sqrt(1 - r2);
                    planes[dst] = (pre * xr + pim * xi) * amp;
                    planes[dst + 1] = (pre * xi - pim * xr) * amp;
                } else {
                    planes[dst] = xr;
                    planes[dst + 1] = xi;
                }
            }
        }
    }
}

/*
 * The reference's image resolution, gridding.c:160:
 *     resolution = 1.0/MAX(abs(uvmin), abs(uvmax))
 * compiled as C, so abs() is the int abs and the metadata values are
 * truncated to int first.
 */
double oracle_resolution(double uvmin, double uvmax)
{
    int a = (int)uvmin;
    int b = (int)uvmax;
    if (a < 0) a = -a;
    if (b < 0) b = -b;
    return 1.0 / (double)(a > b ? a : b);
}


/* ------------------------------------------------------------------------
 * Per-plane and windowed forms, for grids whose FP64 cube does not fit in
 * host memory (oracle.py composes them with the per-plane FFT).
 * ---------------------------------------------------------------------- */

/*
 * oracle_wstack for the measurements of plane w only, into buf ([ny][nx][2],
 * accumulated); rows[k] is set for every grid row that receives a tap.
 */
void oracle_grid_plane(int w, int num_w_planes, long num_points, long freq_per_chan,
                       long polarizations, const double *uu, const double *vv,
                       const double *ww, const float *vis_real, const float *vis_img,
                       const float *weight, double dx, double dw, int w_support,
                       int grid_size_x, int grid_size_y, double *buf, unsigned char *rows,
                       int num_threads)
{
    const int half = (w_support - 1) / 2;
    const double std22 = 0.5;
    const double norm = std22 / ORACLE_PI;
#ifdef _OPENMP
    if (num_threads > 0) omp_set_num_threads(num_threads);
#else
    (void)num_threads;
#endif
#pragma omp parallel for schedule(static)
    for (long m = 0; m < num_points; m++) {
        const int cw = (int)(ww[m] / dw);
        if (cw != w || cw < 0 || cw >= num_w_planes) continue;
        const long vbase = m * freq_per_chan * polarizations;
        const double pu = uu[m] / dx;
        const double pv = vv[m] / dx;
        const int cu = (int)pu;
        const int cv = (int)pv;
        const long j0 = (cu > half - 1) ? cu - half : 0;
        const long j1 = (cu < grid_size_x - half) ? cu + half : grid_size_x - 1;
        const long k0 = (cv > half - 1) ? cv - half : 0;
        const long k1 = (cv < grid_size_y - half) ? cv + half : grid_size_y - 1;
        for (long k = k0; k <= k1; k++) {
            const double dist_v = (double)k + 0.5 - pv;
#pragma omp atomic write
            rows[k] = 1;
            for (long j = j0; j <= j1; j++) {
                const double dist_u = (double)j + 0.5 - pu;
                const long cell = 2 * (j + k * (long)grid_size_x);
                const double cwt = oracle_gauss(norm, std22, dist_u, dist_v);
                double acc_re = 0.0, acc_im = 0.0;
                long fine = vbase;
                for (long f = 0; f < freq_per_chan; f++) {
                    long iw = vbase / freq_per_chan;
                    for (long p = 0; p < polarizations; p++) {
                        if (!isnan(vis_real[fine])) {
                            acc_re += weight[iw] * vis_real[fine] * cwt;
                            acc_im += weight[iw] * vis_img[fine] * cwt;
                        }
                        fine++;
                        iw++;
                    }
                }
#pragma omp atomic
                buf[cell] += acc_re;
#pragma omp atomic
                buf[cell + 1] += acc_im;
            }
        }
    }
}

/*
 * oracle_degrid for the measurements of plane w only, reading the single
 * plane buf ([ny][nx][2]); out[m] ([num_points][2]) is written for those
 * measurements and left alone for the others.  rows[k] is set for every row
 * they read (so a caller can evaluate the plane on those rows only).
 * With buf == NULL only rows is set.
 */
void oracle_degrid_plane(int w, int num_w_planes, long num_points, const double *uu,
                         const double *vv, const double *ww, double dx, double dw,
                         int w_support, int grid_size_x, int grid_size_y, const double *buf,
                         double *out, unsigned char *rows, int num_threads)
{
    const int half = (w_support - 1) / 2;
    const double std22 = 0.5;
    const double norm = std22 / ORACLE_PI;
#ifdef _OPENMP
    if (num_threads > 0) omp_set_num_threads(num_threads);
#else
    (void)num_threads;
#endif
#pragma omp parallel for schedule(static)
    for (long m = 0; m < num_points; m++) {
        const int cw = (int)(ww[m] / dw);
        if (cw != w || cw < 0 || cw >= num_w_planes) continue;
        const double pu = uu[m] / dx;
        const double pv = vv[m] / dx;
        const int cu = (int)pu;
        const int cv = (int)pv;
        const long j0 = (cu > half - 1) ? cu - half : 0;
        const long j1 = (cu < grid_size_x - half) ? cu + half : grid_size_x - 1;
        const long k0 = (cv > half - 1) ? cv - half : 0;
        const long k1 = (cv < grid_size_y - half) ? cv + half : grid_size_y - 1;
        double sre = 0.0, sim = 0.0;
        for (long k = k0; k <= k1; k++) {
#pragma omp atomic write
            rows[k] = 1;
            if (!buf) continue;
            const double dist_v = (double)k + 0.5 - pv;
            for (long j = j0; j <= j1; j++) {
                const double dist_u = (double)j + 0.5 - pu;
                const double cwt = oracle_gauss(norm, std22, dist_u, dist_v);
                sre += cwt * buf[2 * (j + k * (long)grid_size_x)];
                sim += cwt * buf[2 * (j + k * (long)grid_size_x) + 1];
            }
        }
        if (buf) {
            out[2 * m] = sre;
            out[2 * m + 1] = sim;
        }
    }
}

/*
 * One plane of oracle_phase_correction (adjoint = 0: image += phase * plane,
 * accumulated) or of oracle_phase_adjoint (adjoint = 1: plane = conj(phase) *
 * image, overwritten) on the window [x0, x0+wx) x [y0, y0+wy) of an
 * xaxistot x yaxistot image; plane and image are [wy][wx] (plane interleaved
 * re,im; image as two arrays).
 */
void oracle_phase_window(double *plane, double *image_real, double *image_imag, int w,
                         int num_w_planes, int x0, int y0, int wx, int wy, int xaxistot,
                         int yaxistot, double resolution, double wmin, double wmax, int adjoint,
                         int num_threads)
{
    const double dw = (wmax - wmin) / (double)num_w_planes;
    const double dwnorm = dw / (wmax - wmin);
    const double wterm = wmin + w * dw;
#ifdef _OPENMP
    if (num_threads > 0) omp_set_num_threads(num_threads);
#else
    (void)num_threads;
#endif
#pragma omp parallel for collapse(2) schedule(static)
    for (int jy = 0; jy < wy; jy++) {
        for (int i = 0; i < wx; i++) {
            const size_t pix = (size_t)jy * wx + i;
            if (num_w_planes <= 1) {
                if (adjoint) {
                    plane[2 * pix] = image_real[pix];
                    plane[2 * pix + 1] = image_imag[pix];
                } else {
                    image_real[pix] += plane[2 * pix];
                    image_imag[pix] += plane[2 * pix + 1];
                }
                continue;
            }
            const double xs = oracle_pixel_sin(x0 + i, xaxistot, resolution);
            const double ys = oracle_pixel_sin(y0 + jy, yaxistot, resolution);
            const double r2 = (xs * xs + ys * ys);
            const double pre = cos(2.0 * ORACLE_PI * wterm * (sqrt(1 - r2) - 1.0));
            const double pim = sin(2.0 * ORACLE_PI * wterm * (sqrt(1 - r2) - 1.0));
            if (adjoint) {
                const double amp = dwnorm * sqrt(1 - r2);
                const double xr = image_real[pix], xi = image_imag[pix];
                plane[2 * pix] = (pre * xr + pim * xi) * amp;
                plane[2 * pix + 1] = (pre * xi - pim * xr) * amp;
            } else {
                const double a = plane[2 * pix], b = plane[2 * pix + 1];
                image_real[pix] += (a * pre - b * pim) * dwnorm * sqrt(1 - r2);
                image_imag[pix] += (a * pim + b * pre) * dwnorm * sqrt(1 - r2);
            }
        }
    }
}
