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
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "plan.cuh"
#include "wstack_gb300_io.h"

using namespace wsg;

namespace {

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

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
using DevPtr = std::unique_ptr<void, DevDeleter>;

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

// The device side of one dataset, prepared on a second host thread while the
// files are read: the plan with its records, resident grid and FFT plan, the
// input buffers and the image buffers.
struct DeviceSide {
    std::unique_ptr<wsg_plan, PlanDeleter> plan;
    DevPtr in[6];          // uu, vv, ww, weights, vis_real, vis_img
    DevPtr image, split;   // complex image; its real and imaginary float64 planes
    int status = WSG_OK;
    std::string message;
};

int prepare_device(DeviceSide &d, const wsg_params &prm, const wsg_metadata &meta,
                   double resolution, const wsg_run_options &o, cudaStream_t stream)
{
    const int nx = prm.grid_size_x, ny = prm.grid_size_y, planes = prm.num_w_planes;
    wsg_plan *raw = nullptr;
    WSG_TRY(wsg_plan_create(&raw, nx, ny, planes, prm.w_support, 1.0 / (double)nx,
                            1.0 / (double)planes, o.precision, stream));
    d.plan.reset(raw);
    WSG_TRY(wsg_plan_set_wcorrection(raw, resolution, meta.wmin, meta.wmax));
    // the reference's measurement sets are written dump by dump, `baselines`
    // rows each; one rank reads them from row 0
    if (meta.baselines > 1) WSG_TRY(wsg_plan_set_layout(raw, meta.baselines));
    WSG_TRY(wsg_plan_reserve(raw, meta.Nmeasures));
    const size_t b_uvw = sizeof(double) * meta.Nmeasures, b_wt = sizeof(float) * meta.Nweights,
                 b_vis = sizeof(float) * meta.Nvis;
    const size_t bytes[6] = {b_uvw, b_uvw, b_uvw, b_wt, b_vis, b_vis};
    for (int k = 0; k < 6; ++k) WSG_TRY(dev_alloc(d.in[k], bytes[k]));
    const size_t npix = (size_t)nx * ny;
    WSG_TRY(dev_alloc(d.image, (o.precision == WSG_FP64 ? 16 : 8) * npix));
    WSG_TRY(dev_alloc(d.split, 2 * sizeof(double) * npix));
    return WSG_OK;
}

int run_dataset(const wsg_params &prm, int index, const wsg_run_options &o, int device,
                cudaStream_t stream, wsg_run_report &rep)
{
    const double t_start = now_s();
    if (o.verbose) printf("\nDataset %d\n", index);

    // ---- init: meta file, partition ------------------------------------------
    wsg_metadata meta;
    const std::string metapath = std::string(prm.datapath[index]) + prm.metafile;
    WSG_TRY(wsg_read_metadata(metapath.c_str(), &meta));
    if (o.verbose) printf("Subtracting last %d measurements\n", WSG_DROPPED_ROWS);
    long startrow = 0;
    WSG_TRY(wsg_partition_measurements(&meta, 0, 1, &startrow));
    if (o.verbose) {
        printf("N. measurements %ld\n", meta.Nmeasures);
        printf("N. visibilities %ld\n", meta.Nvis);
    }
    double resolution = 0.0;
    WSG_TRY(wsg_reference_resolution(meta.uvmin, meta.uvmax, &resolution));
    const long n = meta.Nmeasures, nf = meta.freq_per_chan, np = meta.polarisations;

    // ---- the device side on a second thread, the binary files on this one -----
    DeviceSide dev;
    std::thread prep([&]() {
        cudaSetDevice(device);
        dev.status = prepare_device(dev, prm, meta, resolution, o, stream);
        if (dev.status != WSG_OK) dev.message = wstack_gb300_last_error_string();
    });
    if (o.verbose) printf("READING DATA\n");
    // pageable buffers: no pinning cost, and first-touched by the reader threads
    const size_t bytes[6] = {sizeof(double) * n, sizeof(double) * n, sizeof(double) * n,
                             sizeof(float) * meta.Nweights, sizeof(float) * meta.Nvis,
                             sizeof(float) * meta.Nvis};
    std::unique_ptr<unsigned char[]> host[6];
    for (int k = 0; k < 6; ++k) host[k].reset(new (std::nothrow) unsigned char[bytes[k] ? bytes[k] : 1]);
    int st = WSG_OK;
    for (int k = 0; k < 6; ++k)
        if (!host[k]) st = set_error(WSG_ERR_NOMEM, "host buffer of %zu bytes", bytes[k]);
    if (st == WSG_OK) {
        st = wsg_read_measurements(&prm, index, &meta, startrow, (double *)host[0].get(),
                                   (double *)host[1].get(), (double *)host[2].get(),
                                   (float *)host[3].get(), (float *)host[4].get(),
                                   (float *)host[5].get());
        if (st == WSG_ERR_IO && !strncmp(wstack_gb300_last_error_string(), "an error occurred", 17)) {
            // a short file: the reference prints and carries on with zeros
            fprintf(stderr, "%s\n", wstack_gb300_last_error_string());
            clear_error();
            st = WSG_OK;
        }
    }
    prep.join();
    if (st != WSG_OK) return st;
    if (dev.status != WSG_OK) return set_error(dev.status, "%s", dev.message.c_str());
    double *h_uu = (double *)host[0].get(), *h_vv = (double *)host[1].get(),
           *h_ww = (double *)host[2].get();
    float *h_wt = (float *)host[3].get(), *h_vr = (float *)host[4].get(),
          *h_vi = (float *)host[5].get();
    const long rows = keep_slab_rows(n, nf, np, h_uu, h_vv, h_ww, h_wt, h_vr, h_vi);
    const double t_setup = now_s();

    // ---- gridding ------------------------------------------------------------
    const int nx = prm.grid_size_x, ny = prm.grid_size_y;
    if (o.verbose)
        printf("RESOLUTION = %f rad, %f arcsec\n", resolution,
               resolution * (3600.0 * 180.0) / 3.14159265359);
    wsg_plan *plan = dev.plan.get();
    const size_t rbytes[6] = {sizeof(double) * rows, sizeof(double) * rows, sizeof(double) * rows,
                              sizeof(float) * rows * np, sizeof(float) * rows * nf * np,
                              sizeof(float) * rows * nf * np};
    for (int k = 0; k < 6 && rows > 0; ++k)
        WSG_CUDA(cudaMemcpyAsync(dev.in[k].get(), host[k].get(), rbytes[k], cudaMemcpyHostToDevice,
                                 stream));
    WSG_TRY(wsg_bin(plan, rows, nf, np, (const double *)dev.in[0].get(),
                    (const double *)dev.in[1].get(), (const double *)dev.in[2].get(),
                    (const float *)dev.in[4].get(), (const float *)dev.in[5].get(),
                    (const float *)dev.in[3].get()));
    WSG_CUDA(cudaStreamSynchronize(stream));
    const double t_compose = now_s();
    // the inputs are now binned into the plan's records; their buffers are
    // released with the dataset (a cudaFree here would wait for the device)
    void *cube = wsg_plan_grid(plan);
    WSG_TRY(wsg_grid(plan, cube));
    WSG_CUDA(cudaStreamSynchronize(stream));
    const double t_kernel = now_s();
    double t_write = 0.0;

    if (o.write_data) {
        if (o.verbose) printf("WRITING GRIDDED DATA\n");
        const double t0 = now_s();
        WSG_TRY(wsg_plan_dump_cube(plan, cube, 1.0, out_path(o, index, prm.outfile2).c_str(),
                                   out_path(o, index, prm.outfile3).c_str()));
        t_write += now_s() - t0;
    }

    // ---- fft + phase correction -----------------------------------------------
    if (o.verbose) printf("PERFORMING FFT\n");
    const long long npix = (long long)nx * ny;
    const double scale = 1.0 / (double)npix;
    const double t_fft0 = now_s();
    double t_fft = 0.0, t_phase0 = 0.0;
    if (o.write_data || o.precision == WSG_FP64) {
        WSG_TRY(wsg_fft(plan, cube, +1));
        WSG_CUDA(cudaStreamSynchronize(stream));
        t_fft = now_s() - t_fft0;
        if (o.write_data) {
            if (o.verbose) printf("WRITING FFT TRANSFORMED DATA\n");
            const double t0 = now_s();
            WSG_TRY(wsg_plan_dump_cube(plan, cube, scale, out_path(o, index, prm.fftfile2).c_str(),
                                       out_path(o, index, prm.fftfile3).c_str()));
            t_write += now_s() - t0;
        }
        if (o.verbose) printf("PHASE CORRECTION\n");
        t_phase0 = now_s();
        WSG_TRY(wsg_wcorrect(plan, cube, dev.image.get(), scale));
    } else {
        // one fused launch transforms each plane and applies the w-correction
        WSG_TRY(wsg_fft_wcorrect(plan, cube, dev.image.get(), 1));
        WSG_CUDA(cudaStreamSynchronize(stream));
        t_fft = now_s() - t_fft0;
        if (o.verbose) printf("PHASE CORRECTION\n");
        t_phase0 = now_s();
    }
    // image_real / image_imag in host memory, as the reference's phase_correction
    // leaves them (fourier_transform.c:170-173)
    std::unique_ptr<double[]> image_re(new (std::nothrow) double[npix]),
        image_im(new (std::nothrow) double[npix]);   // not zero-filled: the download writes all
    if (!image_re || !image_im) return set_error(WSG_ERR_NOMEM, "host image of %lld pixels", npix);
    double *d_re = (double *)dev.split.get(), *d_im = d_re + npix;
    WSG_CUDA(launch_split_complex(dev.image.get(), o.precision, d_re, d_im, npix, 1.0, stream));
    WSG_CUDA(cudaMemcpyAsync(image_re.get(), d_re, sizeof(double) * npix, cudaMemcpyDeviceToHost,
                             stream));
    WSG_CUDA(cudaMemcpyAsync(image_im.get(), d_im, sizeof(double) * npix, cudaMemcpyDeviceToHost,
                             stream));
    WSG_CUDA(cudaStreamSynchronize(stream));
    const double t_phase = now_s() - t_phase0;

    if (o.write_image) {
        if (o.verbose) printf("WRITING IMAGE\n");
        const double t0 = now_s();
        WSG_TRY(wsg_write_image_dump(image_re.get(), image_im.get(), (long)npix,
                                     out_path(o, index, prm.fftfile2).c_str(),
                                     out_path(o, index, prm.fftfile3).c_str()));
        t_write += now_s() - t0;
    }

    wsg_stats stats;
    WSG_TRY(wsg_plan_get_stats(plan, &stats));
    const double total = now_s() - t_start;
    const double setup = t_setup - t_start, compose = t_compose - t_setup,
                 kernel = t_kernel - t_compose;
    if (o.write_timings) {
        const double sec[7] = {setup, kernel, compose, 0.0, t_fft, t_phase, total};
        WSG_TRY(wsg_write_timings(out_path(o, index, prm.timingfile).c_str(), sec));
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

    int device = 0;
    WSG_CUDA(cudaGetDevice(&device));
    cudaStream_t s = nullptr;
    WSG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    std::unique_ptr<CUstream_st, StreamDeleter> stream(s);
    for (int i = 0; i < prm->ndatasets; ++i) {
        const int st = run_dataset(*prm, i, o, device, s, rep);
        if (report) *report = rep;
        if (st != WSG_OK) return st;
    }
    return WSG_OK;
}

}  // extern "C"
