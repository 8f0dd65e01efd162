// wsg_run_paramfile: the reference's main() (main.c:8-94) for one process on
// one GPU, over the plan API.  Per dataset:
//
//   init      meta file, drop-last-1000 partition, binary files    init.c:10-65
//   gridding  rows of v-slab 0 gridded into a resident cube         gridding.c:159-263
//   dump      grid as float64 planes                    (WRITE_DATA) gridding.c:366-447
//   fft       per-plane FFTW_BACKWARD * 1/(Nx*Ny)                    fourier_transform.c:7-72
//   dump      transformed planes                        (WRITE_DATA) fourier_transform.c:74-159
//   phase     w-correction and plane sum -> image                    fourier_transform.c:165-173
//   dump      image                                    (WRITE_IMAGE) fourier_transform.c:177-219
//   timings   one line per dataset                                   result.c:49-62
//
// The reference's MPI decomposition becomes one resident grid: with one rank
// it has one v-slab, whose rows are those with (int)vv == 0
// (gridding.c:42-56), so rows with |vv| >= 1 (or NaN) are not gridded here
// either.  The reference hands the slab's rows to wstack in reverse order
// (gridding.c:193); the order changes only the rounding of the sums.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>

#include "plan.cuh"
#include "wstack_gb300_io.h"

using namespace wsg;

namespace {

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct HostDeleter {
    void operator()(void *p) const
    {
        if (p) cudaFreeHost(p);
    }
};
struct DevDeleter {
    void operator()(void *p) const
    {
        if (p) cudaFree(p);
    }
};
struct PlanDeleter {
    void operator()(wsg_plan *p) const
    {
        if (p) wsg_plan_destroy(p);
    }
};
struct StreamDeleter {
    void operator()(CUstream_st *s) const
    {
        if (s) cudaStreamDestroy(s);
    }
};
using HostPtr = std::unique_ptr<void, HostDeleter>;
using DevPtr = std::unique_ptr<void, DevDeleter>;

int host_alloc(HostPtr &out, size_t bytes)
{
    void *p = nullptr;
    WSG_CUDA(cudaHostAlloc(&p, bytes ? bytes : 16, cudaHostAllocDefault));
    out.reset(p);
    return WSG_OK;
}

int dev_alloc(DevPtr &out, size_t bytes)
{
    void *p = nullptr;
    WSG_CUDA(cudaMalloc(&p, bytes ? bytes : 16));
    out.reset(p);
    return WSG_OK;
}

std::string out_path(const wsg_run_options &o, int dataset, const char *name)
{
    std::string s(o.outdir);
    if (!s.empty() && s.back() != '/') s += '/';
    return s + std::to_string(dataset) + name;
}

// Keeps the rows the reference's single slab grids: (int)(vv * 1) == 0.
// Returns the number kept; compacts in place only when some row is dropped.
long keep_slab_rows(long n, long nf, long np, double *uu, double *vv, double *ww, float *wt,
                    float *vr, float *vi)
{
    long bad = 0;
    for (long i = 0; i < n; ++i) bad += !(vv[i] > -1.0 && vv[i] < 1.0);
    if (!bad) return n;
    long k = 0;
    const long nv = nf * np;
    for (long i = 0; i < n; ++i) {
        if (!(vv[i] > -1.0 && vv[i] < 1.0)) continue;
        if (k != i) {
            uu[k] = uu[i];
            vv[k] = vv[i];
            ww[k] = ww[i];
            memmove(wt + k * np, wt + i * np, sizeof(float) * np);
            memmove(vr + k * nv, vr + i * nv, sizeof(float) * nv);
            memmove(vi + k * nv, vi + i * nv, sizeof(float) * nv);
        }
        ++k;
    }
    return k;
}

int run_dataset(const wsg_params &prm, int index, const wsg_run_options &o, cudaStream_t stream,
                wsg_run_report &rep)
{
    const double t_start = now_s();
    if (o.verbose) printf("\nDataset %d\n", index);

    // ---- init: meta file, partition, binary files ----------------------------
    wsg_metadata meta;
    const std::string metapath = std::string(prm.datapath[index]) + prm.metafile;
    WSG_TRY(wsg_read_metadata(metapath.c_str(), &meta));
    if (o.verbose) printf("Subtracting last %d measurements\n", WSG_DROPPED_ROWS);
    long startrow = 0;
    WSG_TRY(wsg_partition_measurements(&meta, 0, 1, &startrow));
    if (o.verbose) {
        printf("N. measurements %ld\n", meta.Nmeasures);
        printf("N. visibilities %ld\n", meta.Nvis);
        printf("READING DATA\n");
    }
    const long n = meta.Nmeasures, nf = meta.freq_per_chan, np = meta.polarisations;
    HostPtr h_uu, h_vv, h_ww, h_wt, h_vr, h_vi;
    WSG_TRY(host_alloc(h_uu, sizeof(double) * n));
    WSG_TRY(host_alloc(h_vv, sizeof(double) * n));
    WSG_TRY(host_alloc(h_ww, sizeof(double) * n));
    WSG_TRY(host_alloc(h_wt, sizeof(float) * meta.Nweights));
    WSG_TRY(host_alloc(h_vr, sizeof(float) * meta.Nvis));
    WSG_TRY(host_alloc(h_vi, sizeof(float) * meta.Nvis));
    int st = wsg_read_measurements(&prm, index, &meta, startrow, (double *)h_uu.get(),
                                   (double *)h_vv.get(), (double *)h_ww.get(), (float *)h_wt.get(),
                                   (float *)h_vr.get(), (float *)h_vi.get());
    if (st != WSG_OK) {
        // a short file: the reference prints and carries on with zeros
        if (st != WSG_ERR_IO || strncmp(wstack_gb300_last_error_string(), "an error occurred", 17))
            return st;
        fprintf(stderr, "%s\n", wstack_gb300_last_error_string());
        clear_error();
    }
    const long rows = keep_slab_rows(n, nf, np, (double *)h_uu.get(), (double *)h_vv.get(),
                                     (double *)h_ww.get(), (float *)h_wt.get(), (float *)h_vr.get(),
                                     (float *)h_vi.get());
    double resolution = 0.0;
    WSG_TRY(wsg_reference_resolution(meta.uvmin, meta.uvmax, &resolution));
    const double t_setup = now_s();

    // ---- gridding ------------------------------------------------------------
    const int nx = prm.grid_size_x, ny = prm.grid_size_y, planes = prm.num_w_planes;
    if (o.verbose)
        printf("RESOLUTION = %f rad, %f arcsec\n", resolution,
               resolution * (3600.0 * 180.0) / 3.14159265359);
    wsg_plan *raw = nullptr;
    WSG_TRY(wsg_plan_create(&raw, nx, ny, planes, prm.w_support, 1.0 / (double)nx,
                            1.0 / (double)planes, o.precision, stream));
    std::unique_ptr<wsg_plan, PlanDeleter> plan(raw);
    WSG_TRY(wsg_plan_set_wcorrection(plan.get(), resolution, meta.wmin, meta.wmax));
    DevPtr d_uu, d_vv, d_ww, d_wt, d_vr, d_vi;
    const size_t b_uvw = sizeof(double) * rows, b_wt = sizeof(float) * rows * np,
                 b_vis = sizeof(float) * rows * nf * np;
    WSG_TRY(dev_alloc(d_uu, b_uvw));
    WSG_TRY(dev_alloc(d_vv, b_uvw));
    WSG_TRY(dev_alloc(d_ww, b_uvw));
    WSG_TRY(dev_alloc(d_wt, b_wt));
    WSG_TRY(dev_alloc(d_vr, b_vis));
    WSG_TRY(dev_alloc(d_vi, b_vis));
    if (rows > 0) {
        WSG_CUDA(cudaMemcpyAsync(d_uu.get(), h_uu.get(), b_uvw, cudaMemcpyHostToDevice, stream));
        WSG_CUDA(cudaMemcpyAsync(d_vv.get(), h_vv.get(), b_uvw, cudaMemcpyHostToDevice, stream));
        WSG_CUDA(cudaMemcpyAsync(d_ww.get(), h_ww.get(), b_uvw, cudaMemcpyHostToDevice, stream));
        WSG_CUDA(cudaMemcpyAsync(d_wt.get(), h_wt.get(), b_wt, cudaMemcpyHostToDevice, stream));
        WSG_CUDA(cudaMemcpyAsync(d_vr.get(), h_vr.get(), b_vis, cudaMemcpyHostToDevice, stream));
        WSG_CUDA(cudaMemcpyAsync(d_vi.get(), h_vi.get(), b_vis, cudaMemcpyHostToDevice, stream));
    }
    WSG_TRY(wsg_bin(plan.get(), rows, nf, np, (const double *)d_uu.get(), (const double *)d_vv.get(),
                    (const double *)d_ww.get(), (const float *)d_vr.get(),
                    (const float *)d_vi.get(), (const float *)d_wt.get()));
    WSG_CUDA(cudaStreamSynchronize(stream));
    const double t_compose = now_s();
    // the measurements are binned into the plan's records: free the raw inputs
    d_uu.reset();
    d_vv.reset();
    d_ww.reset();
    d_wt.reset();
    d_vr.reset();
    d_vi.reset();

    const size_t elem = o.precision == WSG_FP64 ? 2 * sizeof(double) : 2 * sizeof(float);
    const long long npix = (long long)nx * ny;
    DevPtr d_cube, d_image;
    WSG_TRY(dev_alloc(d_cube, elem * (size_t)planes * npix));
    WSG_TRY(dev_alloc(d_image, elem * (size_t)npix));
    WSG_TRY(wsg_grid(plan.get(), d_cube.get()));
    WSG_CUDA(cudaStreamSynchronize(stream));
    const double t_kernel = now_s();
    double t_write = 0.0;

    if (o.write_data) {
        if (o.verbose) printf("WRITING GRIDDED DATA\n");
        const double t0 = now_s();
        WSG_TRY(wsg_plan_dump_cube(plan.get(), d_cube.get(), 1.0,
                                   out_path(o, index, prm.outfile2).c_str(),
                                   out_path(o, index, prm.outfile3).c_str()));
        t_write += now_s() - t0;
    }

    // ---- fft + phase correction -----------------------------------------------
    if (o.verbose) printf("PERFORMING FFT\n");
    const double scale = 1.0 / (double)npix;
    double t_fft0 = now_s(), t_fft = 0.0, t_phase0 = 0.0;
    if (o.write_data) {
        WSG_TRY(wsg_fft(plan.get(), d_cube.get(), +1));
        WSG_CUDA(cudaStreamSynchronize(stream));
        t_fft = now_s() - t_fft0;
        if (o.verbose) printf("WRITING FFT TRANSFORMED DATA\n");
        const double t0 = now_s();
        WSG_TRY(wsg_plan_dump_cube(plan.get(), d_cube.get(), scale,
                                   out_path(o, index, prm.fftfile2).c_str(),
                                   out_path(o, index, prm.fftfile3).c_str()));
        t_write += now_s() - t0;
        if (o.verbose) printf("PHASE CORRECTION\n");
        t_phase0 = now_s();
        WSG_TRY(wsg_wcorrect(plan.get(), d_cube.get(), d_image.get(), scale));
    } else if (o.precision == WSG_FP64) {
        WSG_TRY(wsg_fft(plan.get(), d_cube.get(), +1));
        WSG_CUDA(cudaStreamSynchronize(stream));
        t_fft = now_s() - t_fft0;
        if (o.verbose) printf("PHASE CORRECTION\n");
        t_phase0 = now_s();
        WSG_TRY(wsg_wcorrect(plan.get(), d_cube.get(), d_image.get(), scale));
    } else {
        // one fused launch transforms each plane and applies the w-correction
        WSG_TRY(wsg_fft_wcorrect(plan.get(), d_cube.get(), d_image.get(), 1));
        WSG_CUDA(cudaStreamSynchronize(stream));
        t_fft = now_s() - t_fft0;
        if (o.verbose) printf("PHASE CORRECTION\n");
        t_phase0 = now_s();
    }
    HostPtr h_img, h_re, h_im;
    WSG_TRY(host_alloc(h_img, elem * (size_t)npix));
    WSG_CUDA(cudaMemcpyAsync(h_img.get(), d_image.get(), elem * (size_t)npix, cudaMemcpyDeviceToHost,
                             stream));
    WSG_CUDA(cudaStreamSynchronize(stream));
    const double t_phase = now_s() - t_phase0;

    if (o.write_image) {
        if (o.verbose) printf("WRITING IMAGE\n");
        const double t0 = now_s();
        WSG_TRY(host_alloc(h_re, sizeof(double) * (size_t)npix));
        WSG_TRY(host_alloc(h_im, sizeof(double) * (size_t)npix));
        double *re = (double *)h_re.get(), *im = (double *)h_im.get();
        if (o.precision == WSG_FP64) {
            const double *z = (const double *)h_img.get();
            for (long long i = 0; i < npix; ++i) {
                re[i] = z[2 * i];
                im[i] = z[2 * i + 1];
            }
        } else {
            const float *z = (const float *)h_img.get();
            for (long long i = 0; i < npix; ++i) {
                re[i] = (double)z[2 * i];
                im[i] = (double)z[2 * i + 1];
            }
        }
        WSG_TRY(wsg_write_image_dump(re, im, (long)npix, out_path(o, index, prm.fftfile2).c_str(),
                                     out_path(o, index, prm.fftfile3).c_str()));
        t_write += now_s() - t0;
    }

    wsg_stats stats;
    WSG_TRY(wsg_plan_get_stats(plan.get(), &stats));
    const double total = now_s() - t_start;
    const double setup = t_setup - t_start, compose = t_compose - t_setup,
                 kernel = t_kernel - t_compose;
    if (o.write_timings) {
        const double s[7] = {setup, kernel, compose, 0.0, t_fft, t_phase, total};
        WSG_TRY(wsg_write_timings(out_path(o, index, prm.timingfile).c_str(), s));
    }
    if (o.verbose) {
        printf("%14s time : %f sec\n", "Setup", setup);
        printf("%10s Kernel time = %f, Array Composition time %f, Reduce time: %f sec\n", "", kernel,
               compose, 0.0);
        printf("%14s time : %f sec\n", "FFTW", t_fft);
        printf("%14s time : %f sec\n", "Phase", t_phase);
        printf("%14s time : %f sec\n\n", "TOTAL", total);
    }
    rep.datasets += 1;
    rep.Nmeasures = rows;
    rep.Nvis = rows * nf * np;
    rep.resolution = resolution;
    rep.dropped += (n - rows) + stats.dropped_plane;   // off the slab, or w outside the cube
    rep.setup += setup;
    rep.compose += compose;
    rep.kernel += kernel;
    rep.fft += t_fft;
    rep.phase += t_phase;
    rep.write += t_write;
    rep.total += total;
    return WSG_OK;
}

}  // namespace

extern "C" {

void wsg_run_options_default(wsg_run_options *opt)
{
    if (!opt) return;
    memset(opt, 0, sizeof(*opt));
    opt->precision = WSG_FP64;
    opt->write_timings = 1;
}

int wsg_run_paramfile(const char *paramfile, const wsg_run_options *opt, wsg_run_report *report)
{
    clear_error();
    if (!paramfile) return set_error(WSG_ERR_ARG, "NULL argument");
    wsg_run_options o;
    if (opt)
        o = *opt;
    else
        wsg_run_options_default(&o);
    if (o.precision != WSG_FP64 && o.precision != WSG_FP32C)
        return set_error(WSG_ERR_ARG, "invalid precision %d", o.precision);
    if (memchr(o.outdir, 0, sizeof(o.outdir)) == nullptr)
        return set_error(WSG_ERR_ARG, "outdir is not NUL-terminated");
    wsg_run_report rep;
    memset(&rep, 0, sizeof(rep));
    if (report) *report = rep;

    // the parameter set is ~125 KB: keep it off the stack
    std::unique_ptr<wsg_params> prm(new wsg_params);
    WSG_TRY(wsg_read_parameter_file(paramfile, prm.get()));
    if (prm->num_threads == 0)
        return set_error(WSG_ERR_ARG, "Usage: %d number_of_OMP_Threads", prm->num_threads);
    if (prm->ndatasets > WSG_MAX_DATASETS)
        return set_error(WSG_ERR_ARG, "ndatasets %d above %d", prm->ndatasets, WSG_MAX_DATASETS);
    if (prm->grid_size_x <= 0 || prm->grid_size_y <= 0 || prm->num_w_planes <= 0)
        return set_error(WSG_ERR_ARG, "grid_size_x, grid_size_y and num_w_planes must be positive");

    cudaStream_t s = nullptr;
    WSG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    std::unique_ptr<CUstream_st, StreamDeleter> stream(s);
    for (int i = 0; i < prm->ndatasets; ++i) {
        const int st = run_dataset(*prm, i, o, s, rep);
        if (report) *report = rep;
        if (st != WSG_OK) return st;
    }
    return WSG_OK;
}

}  // extern "C"
