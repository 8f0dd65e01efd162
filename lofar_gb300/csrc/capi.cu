// C ABI of libwstack_gb300.so: the reference's drop-in entry points and the
// device-resident plan API.  See include/wstack_gb300.h for the contract.
#include <cuda_runtime.h>

#include <atomic>
#include <cufft.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <new>

#include "plan.cuh"

using namespace wsg;

// ---------------------------------------------------------------------------
// error state and shared helpers
// ---------------------------------------------------------------------------

namespace {
thread_local int tl_status = WSG_OK;
thread_local char tl_msg[512] = "";
}  // namespace

int wsg::set_error(int status, const char *fmt, ...)
{
    tl_status = status;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(tl_msg, sizeof(tl_msg), fmt, ap);
    va_end(ap);
    return status;
}

int wsg::clear_error()
{
    tl_status = WSG_OK;
    tl_msg[0] = 0;
    return WSG_OK;
}

bool wsg::is_pow2_recip(double d, int &k)
{
    if (!(d > 0.0) || !isfinite(d)) return false;
    int e;
    const double m = frexp(d, &e);
    if (m != 0.5) return false;
    k = 1 - e;
    return k >= 0 && k <= 1000;
}

bool wsg::device_accessible(const void *ptr)
{
    if (!ptr) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Records a status and message as this thread's last error (for entry points
// defined in other translation units).
int wsg::report_status(int status, const char *msg)
{
    return set_error(status, "%s", msg ? msg : "");
}

// SM count of the current device, cached per device ordinal (a process may
// drive GPUs with different SM counts from several threads).
int wsg::num_sms()
{
    constexpr int kDevs = 64;
    static std::atomic<int> cache[kDevs];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        dev = 0;
    }
    const bool cached = dev >= 0 && dev < kDevs;
    if (cached) {
        const int n = cache[dev].load(std::memory_order_relaxed);
        if (n > 0) return n;
    }
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) {
        cudaGetLastError();
        v = 148;
    }
    if (cached) cache[dev].store(v, std::memory_order_relaxed);
    return v;
}

// ---------------------------------------------------------------------------
// plan
// ---------------------------------------------------------------------------

WScreen wsg::plan_wscreen(const wsg_plan *p)
{
    WScreen ws;
    unsigned *base = p->wscreen.as<unsigned>();
    const long long n = p->npix();
    ws.aq = base;
    ws.bq = base ? base + n : nullptr;
    ws.amp = base ? reinterpret_cast<float *>(base + 2 * n) : nullptr;
    ws.sinx = p->sinx.as<double>();
    ws.siny = p->siny.as<double>();
    return ws;
}

int wsg::plan_configure(wsg_plan *p)
{
    GeomParams &g = p->geom;
    g.nx = p->nx;
    g.ny = p->ny;
    g.half = p->half;
    g.tile = p->tile;
    g.tile_shift = 0;
    while ((1 << g.tile_shift) < p->tile) g.tile_shift++;
    g.ntu = (p->nx + p->tile - 1) / p->tile;
    g.ntv = (p->ny + p->tile - 1) / p->tile;
    g.wplanes = p->planes;
    g.planes = (int)p->cube_planes();
    g.nbins = p->cube_planes() * g.ntv * g.ntu;
    g.dx = p->dx;
    g.dw = p->dw;
    // the [dump][baseline] walk serves FP32C plans; the FP64 gridder's
    // record groups would collide on the shared cells of one track's records
    g.rows = p->prec == WSG_FP32C ? p->rows : 0;
    int k = 0;
    g.u_pow2 = is_pow2_recip(p->dx, k) ? 1 : 0;
    g.ku = g.u_pow2 ? k : 0;
    g.w_pow2 = is_pow2_recip(p->dw, k) ? 1 : 0;
    g.kw = g.w_pow2 ? k : 0;
    if (g.nbins * 2 * kSub >= (1ll << 32) - 1)
        return set_error(WSG_ERR_UNSUPPORTED, "too many (plane, tile) bins: %lld", g.nbins);
    const int sms = num_sms();
    const int og = grid_max_ctas_per_sm(p->prec, p->tile, p->half);
    const int od = degrid_max_ctas_per_sm(p->prec, p->tile, p->half);
    if (og <= 0 || od <= 0)
        return set_error(WSG_ERR_UNSUPPORTED, "no tile kernel for tile=%d support=%d", p->tile,
                         p->support);
    const char *fft_env = getenv("WSTACK_GB300_FFT");
    p->fused = p->prec == WSG_FP32C && fft_fused_supported(p->nx, p->ny, p->tile) &&
               !(fft_env && strcmp(fft_env, "cufft") == 0);
    p->fft64 = p->prec == WSG_FP64 && fft64_supported(p->nx, p->ny, p->cube_planes()) &&
               !(fft_env && strcmp(fft_env, "cufft") == 0);
    p->masks_valid = false;
    p->ctas_grid = p->ctas_user > 0 ? p->ctas_user : og * sms;
    p->ctas_degrid = p->ctas_user > 0 ? p->ctas_user : od * sms;
    p->rec_cap = 0;  // bin table and partial-tile sizes depend on tile and split
    p->n_binned = -1;
    return WSG_OK;
}

int wsg::ensure_records(wsg_plan *p, long long n)
{
    // a support window of <= tile cells touches at most 2x2 tiles
    const unsigned long long need = (unsigned long long)(n > 0 ? n : 1) * 4ull;
    if (need <= p->rec_cap) return WSG_OK;
    WSG_CUDA(p->bins.ensure(bin_buffer_bytes(p->geom.nbins, max_split_items(need, p->split), kSub)));
    WSG_CUDA(p->partials.ensure(max_slots(need, p->split) * (size_t)p->tile * p->tile *
                                (p->prec == WSG_FP64 ? sizeof(double2) : sizeof(float2))));
    WSG_CUDA(p->ridx.ensure(need * sizeof(unsigned)));
    if (p->prec == WSG_FP64) {
        WSG_CUDA(p->rcell.ensure(need * sizeof(unsigned)));
        WSG_CUDA(p->rfrac.ensure(need * sizeof(double2)));
        WSG_CUDA(p->rval.ensure(need * sizeof(double2)));
    } else {
        WSG_CUDA(p->rec16.ensure(need * sizeof(uint4)));
    }
    p->rec_cap = need;
    return WSG_OK;
}

namespace {

int ensure_fft(wsg_plan *p)
{
    if (p->fft_ready) return WSG_OK;
    const cufftType type = p->prec == WSG_FP64 ? CUFFT_Z2Z : CUFFT_C2C;
    int n[2] = {p->ny, p->nx};
    const long long dist = p->npix();
    // largest divisor of P whose work area stays within 4 GiB
    const size_t limit = (size_t)4 << 30;
    int batch = p->planes;
    for (;;) {
        size_t ws = 0;
        WSG_CUFFT(cufftEstimateMany(2, n, nullptr, 1, (int)dist, nullptr, 1, (int)dist, type,
                                    batch, &ws));
        if (ws <= limit || batch == 1) break;
        int b = batch - 1;
        while (b > 1 && p->planes % b) b--;
        batch = b;
    }
    WSG_CUFFT(cufftCreate(&p->fft));
    WSG_CUFFT(cufftSetAutoAllocation(p->fft, 0));
    size_t ws = 0;
    long long nn[2] = {p->ny, p->nx};
    WSG_CUFFT(cufftMakePlanMany64(p->fft, 2, nn, nullptr, 1, dist, nullptr, 1, dist, type, batch,
                                  &ws));
    WSG_CUDA(p->fft_work.ensure(ws));
    WSG_CUFFT(cufftSetWorkArea(p->fft, p->fft_work.p));
    p->fft_batch = batch;
    p->fft_ready = true;
    return WSG_OK;
}

}  // namespace

FftMasks wsg::mask_view(const wsg_plan *p)
{
    FftMasks m;
    const size_t nt = (size_t)p->cube_planes() * p->geom.ntv * p->geom.ntu;
    const size_t nc = (size_t)p->cube_planes() * p->geom.ntu;
    unsigned char *b = p->masks.as<unsigned char>();
    m.occ_tile = b;
    m.need_tile = b + nt;
    m.occ_col = b + 2 * nt;
    m.need_col = b + 2 * nt + nc;
    m.plane_occ = b + 2 * nt + 2 * nc;
    m.plane_need = b + 2 * nt + 2 * nc + p->cube_planes();
    return m;
}

int wsg::ensure_fused(wsg_plan *p)
{
    if (!p->tw_ready) {
        WSG_CUDA(p->twx.ensure(sizeof(float2) * p->nx));
        WSG_CUDA(p->twy.ensure(sizeof(float2) * p->ny));
        WSG_CUDA(launch_twiddles(p->twx.as<float2>(), p->nx, p->stream));
        WSG_CUDA(launch_twiddles(p->twy.as<float2>(), p->ny, p->stream));
        p->tw_ready = true;
    }
    return ensure_masks(p);
}

int wsg::ensure_masks(wsg_plan *p)
{
    const size_t nt = (size_t)p->cube_planes() * p->geom.ntv * p->geom.ntu;
    const size_t nc = (size_t)p->cube_planes() * p->geom.ntu;
    WSG_CUDA(p->masks.ensure(2 * nt + 2 * nc + 2 * (size_t)p->cube_planes()));
    return WSG_OK;
}

int wsg::ensure_wscreen(wsg_plan *p)
{
    if (!p->wc_set) return set_error(WSG_ERR_STATE, "w-correction geometry not set");
    if (p->ws_ready) return WSG_OK;
    WSG_CUDA(p->sinx.ensure(sizeof(double) * p->nx));
    WSG_CUDA(p->siny.ensure(sizeof(double) * p->ny));
    WSG_CUDA(launch_wscreen_tables(p->wc, p->sinx.as<double>(), p->siny.as<double>(), p->stream));
    if (p->prec == WSG_FP32C && p->wc.phase_on && p->planes > 1) {
        WSG_CUDA(p->wscreen.ensure(sizeof(unsigned) * 3 * (size_t)p->npix()));
        WSG_CUDA(launch_wscreen_build(p->wc, plan_wscreen(p), p->stream));
    }
    p->ws_ready = true;
    return WSG_OK;
}

int wsg::finish_binning(wsg_plan *p)
{
    p->masks_valid = false;
    if (p->fused || p->fft64) {
        // the transforms of the imaging calls read (FP32C forward) and write
        // (adjoint) only the tiles these masks mark
        WSG_TRY(p->fused ? ensure_fused(p) : ensure_masks(p));
        WSG_CUDA(launch_fft_masks(p->geom, p->binbufs(), mask_view(p), p->stream));
        p->masks_valid = true;
    }
    return WSG_OK;
}


extern "C" {

int wsg_plan_create(wsg_plan **out, int grid_size_x, int grid_size_y, int num_w_planes,
                    int w_support, double dx, double dw, int precision, void *stream)
{
    clear_error();
    if (!out) return set_error(WSG_ERR_ARG, "plan pointer is NULL");
    *out = nullptr;
    if (grid_size_x <= 0 || grid_size_y <= 0 || num_w_planes <= 0)
        return set_error(WSG_ERR_ARG, "grid sizes and plane count must be positive");
    if (grid_size_x > 65536 || grid_size_y > 65536)
        return set_error(WSG_ERR_UNSUPPORTED, "grid edge above 65536");
    if (w_support < 1 || w_support > 2 * kMaxHalf + 1)
        return set_error(WSG_ERR_UNSUPPORTED, "w_support %d outside [1, %d]", w_support,
                         2 * kMaxHalf + 1);
    if (precision != WSG_FP64 && precision != WSG_FP32C)
        return set_error(WSG_ERR_ARG, "unknown precision %d", precision);
    if (!(dx > 0.0) || !(dw > 0.0) || !isfinite(dx) || !isfinite(dw))
        return set_error(WSG_ERR_ARG, "dx and dw must be positive and finite");
    wsg_plan *p = new (std::nothrow) wsg_plan();
    if (!p) return set_error(WSG_ERR_NOMEM, "host allocation failed");
    p->nx = grid_size_x;
    p->ny = grid_size_y;
    p->planes = num_w_planes;
    p->support = w_support;
    p->half = (w_support - 1) / 2;
    p->prec = precision;
    p->dx = dx;
    p->dw = dw;
    p->stream = (cudaStream_t)stream;
    p->tile = 64;
    // FP32C work items sort and sum up to 16384 records in stages; the FP64
    // gridder sums items of up to 4096 records in fixed point
    p->split = precision == WSG_FP32C ? kDefaultSplitF32 : kDefaultSplit;
    int st = WSG_OK;
    cudaError_t e = p->ctr.ensure(sizeof(DevCounters));
    if (e != cudaSuccess) st = set_error(WSG_ERR_NOMEM, "%s", cudaGetErrorString(e));
    if (st == WSG_OK) st = plan_configure(p);
    if (st != WSG_OK) {
        wsg_plan_destroy(p);
        return st;
    }
    *out = p;
    return WSG_OK;
}

int wsg_plan_destroy(wsg_plan *p)
{
    if (!p) return WSG_OK;
    if (p->a_ready) {
        cudaStreamSynchronize(p->s_in);
        cudaStreamSynchronize(p->s_out);
        if (p->stream) cudaStreamSynchronize(p->stream);
        cudaEvent_t ev[] = {p->e_in[0], p->e_in[1], p->e_free[0], p->e_free[1], p->e_adj,
                            p->e_vis_down};
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
        cudaStreamDestroy(p->s_in);
        cudaStreamDestroy(p->s_out);
        for (auto &slot : p->a_in)
            for (DevBuf &b : slot) b.release();
        p->a_img_fwd.release();
        p->a_img_adj.release();
        p->a_vis.release();
    }
    if (p->fft) cufftDestroy(p->fft);
    DevBuf *bufs[] = {&p->grid, &p->bins, &p->ctr, &p->rec16, &p->partials, &p->rcell, &p->rfrac, &p->rval, &p->ridx, &p->rpos, &p->rvrec,
                      &p->h_uu, &p->h_vv, &p->h_ww, &p->h_vr, &p->h_vi, &p->h_wt, &p->h_image,
                      &p->h_out, &p->sinx, &p->siny, &p->wscreen, &p->fft_work};
    for (DevBuf *b : bufs) b->release();
    p->twx.release();
    p->twy.release();
    p->masks.release();
    delete p;
    return WSG_OK;
}

int wsg_plan_set_stream(wsg_plan *p, void *stream)
{
    clear_error();
    if (!p) return set_error(WSG_ERR_ARG, "plan is NULL");
    p->stream = (cudaStream_t)stream;
    return WSG_OK;
}

int wsg_plan_set_tuning(wsg_plan *p, int tile, int ctas, int chunk)
{
    clear_error();
    if (!p) return set_error(WSG_ERR_ARG, "plan is NULL");
    if (tile != 0 && tile != 32 && tile != 64)
        return set_error(WSG_ERR_UNSUPPORTED, "tile must be 32 or 64");
    if (tile && 2 * p->half + 1 > tile)
        return set_error(WSG_ERR_UNSUPPORTED, "tile smaller than the support");
    if (chunk < 0 || ctas < 0) return set_error(WSG_ERR_ARG, "negative tuning value");
    if (chunk > 0 && chunk < kStage)
        return set_error(WSG_ERR_UNSUPPORTED, "split size below %d records", kStage);
    if (chunk > 0) p->split = chunk;
    p->ctas_user = ctas;
    if (tile) p->tile = tile;
    return plan_configure(p);
}

int wsg_plan_set_layout(wsg_plan *p, long rows_per_dump)
{
    clear_error();
    if (!p) return set_error(WSG_ERR_ARG, "plan is NULL");
    if (rows_per_dump < 0) return set_error(WSG_ERR_ARG, "negative rows per dump");
    p->rows = rows_per_dump;
    p->geom.rows = p->prec == WSG_FP32C ? rows_per_dump : 0;
    return WSG_OK;
}

int wsg_plan_reserve(wsg_plan *p, long max_points)
{
    clear_error();
    if (!p) return set_error(WSG_ERR_ARG, "plan is NULL");
    if (max_points < 0 || max_points > 1000000000L)
        return set_error(WSG_ERR_UNSUPPORTED, "max_points outside [0, 1e9]");
    WSG_TRY(ensure_records(p, max_points));
    WSG_CUDA(p->grid.ensure(p->elem() * (size_t)p->cube_planes() * p->npix()));
    // the FP32C power-of-two grids transform with the library's own kernels
    WSG_TRY(p->fused ? ensure_fused(p) : ensure_fft(p));
    if (p->wc_set) WSG_TRY(ensure_wscreen(p));
    return WSG_OK;
}

int wsg_plan_set_wcorrection(wsg_plan *p, double resolution, double wmin, double wmax)
{
    clear_error();
    if (!p) return set_error(WSG_ERR_ARG, "plan is NULL");
    if (!isfinite(resolution) || !isfinite(wmin) || !isfinite(wmax))
        return set_error(WSG_ERR_ARG, "non-finite w-correction geometry");
    p->wc.xaxis = p->nx;
    p->wc.yaxis = p->ny;
    p->wc.xaxistot = p->nx;
    p->wc.yaxistot = p->ny;
    p->wc.planes = p->planes;
    p->wc.resolution = resolution;
    p->wc.wmin = wmin;
    p->wc.wmax = wmax;
    p->wc.phase_on = 1;
    p->wc_set = true;
    p->ws_ready = false;
    return WSG_OK;
}

int wsg_plan_get_stats(wsg_plan *p, wsg_stats *s)
{
    clear_error();
    if (!p || !s) return set_error(WSG_ERR_ARG, "NULL argument");
    DevCounters c;
    WSG_CUDA(cudaMemcpyAsync(&c, p->ctr.p, sizeof(c), cudaMemcpyDeviceToHost, p->stream));
    WSG_CUDA(cudaStreamSynchronize(p->stream));
    if (fft_tma_timed_out())
        return set_error(WSG_ERR_CUDA, "a column FFT gave up waiting for its staged strip");
    if (degrid_tma_timed_out())
        return set_error(WSG_ERR_CUDA, "a degridding CTA gave up waiting for its staged tile");
    s->points_in = p->n_binned;
    s->records = (long long)c.records;
    s->dropped_plane = (long long)c.dropped_plane;
    s->dropped_window = (long long)c.dropped_window;
    s->bins = (int)p->geom.nbins;
    s->tile = p->tile;
    s->max_bin_records = (int)c.max_bin;
    s->ctas = p->ctas_grid;
    return WSG_OK;
}

long long wsg_plan_device_bytes(wsg_plan *p)
{
    if (!p) return 0;
    const DevBuf *bufs[] = {&p->grid, &p->bins, &p->ctr, &p->rec16, &p->partials, &p->rcell, &p->rfrac, &p->rval,
                            &p->ridx, &p->rpos, &p->rvrec, &p->h_uu, &p->h_vv, &p->h_ww, &p->h_vr, &p->h_vi,
                            &p->h_wt, &p->h_image, &p->h_out, &p->sinx, &p->siny,
                            &p->wscreen, &p->fft_work};
    long long t = 0;
    for (const DevBuf *b : bufs) t += (long long)b->bytes;
    return t;
}

void *wsg_plan_grid(wsg_plan *p) { return p ? p->grid.p : nullptr; }

int wsg_bin(wsg_plan *p, long n, long nf, long np, const double *uu, const double *vv,
            const double *ww, const float *vr, const float *vi, const float *wt)
{
    clear_error();
    if (!p) return set_error(WSG_ERR_ARG, "plan is NULL");
    if (p->jobs != 1) return set_error(WSG_ERR_STATE, "a batch plan is binned by wsg_batch_bind");
    if (n < 0 || nf <= 0 || np <= 0) return set_error(WSG_ERR_ARG, "bad measurement counts");
    if (n > 1000000000L) return set_error(WSG_ERR_UNSUPPORTED, "more than 1e9 measurements");
    if (n > 0 && (!uu || !vv || !ww || !vr || !vi || !wt))
        return set_error(WSG_ERR_ARG, "NULL input pointer");
    WSG_TRY(ensure_records(p, n));
    if (rows_walk(p->geom, n)) {
        WSG_CUDA(p->rpos.ensure(sizeof(unsigned) * (size_t)n));
        WSG_CUDA(p->rvrec.ensure(sizeof(float2) * (size_t)p->rec_cap));
    }
    const BinBuffers b = p->binbufs();
    WSG_CUDA(cudaMemsetAsync(b.sub_prim, 0, bin_counter_bytes(p->geom.nbins, b.nsub), p->stream));
    WSG_CUDA(cudaMemsetAsync(b.ctr, 0, sizeof(DevCounters), p->stream));
    WSG_CUDA(launch_bin_count(p->geom, uu, vv, ww, n, b, p->stream));
    WSG_CUDA(launch_bin_scan(p->geom, b, p->stream));
    WSG_CUDA(launch_bin_scatter(p->geom, p->prec, uu, vv, ww, vr, vi, wt, n, nf, np, b,
                                p->recbufs(), p->stream));
    p->n_binned = n;
    p->walked = rows_walk(p->geom, n);
    return finish_binning(p);
}

int wsg_grid(wsg_plan *p, void *grid)
{
    clear_error();
    if (!p || !grid) return set_error(WSG_ERR_ARG, "NULL argument");
    if (p->n_binned < 0) return set_error(WSG_ERR_STATE, "wsg_grid before wsg_bin");
    const BinBuffers b = p->binbufs();
    WSG_CUDA(cudaMemsetAsync(&b.ctr->work_grid, 0, sizeof(unsigned), p->stream));
    WSG_CUDA(launch_grid(p->geom, p->prec, b, p->recbufs(), grid, p->partials.p, p->ctas_grid,
                         p->stream, false, p->walked));
    return WSG_OK;
}

int wsg_grid_occupied(wsg_plan *p, void *grid)
{
    clear_error();
    if (!p || !grid) return set_error(WSG_ERR_ARG, "NULL argument");
    if (p->n_binned < 0) return set_error(WSG_ERR_STATE, "wsg_grid_occupied before wsg_bin");
    const BinBuffers b = p->binbufs();
    WSG_CUDA(cudaMemsetAsync(&b.ctr->work_grid, 0, sizeof(unsigned), p->stream));
    WSG_CUDA(launch_grid(p->geom, p->prec, b, p->recbufs(), grid, p->partials.p, p->ctas_grid,
                         p->stream, p->fused, p->walked));
    return WSG_OK;
}

// Tile masks serve the FP64 column pass when a CTA's columns (at most 16)
// share one tile column, and the column's tile mask fits its shared copy.
static bool fft64_masks_ok(const wsg_plan *p)
{
    return p->geom.tile >= 16 && p->ny / p->geom.tile <= p->ny / 16 && p->nx % p->geom.tile == 0 &&
           p->ny % p->geom.tile == 0;
}

// The FP64 plan's integer-pipe transform of its cube; `pruned` (adjoint):
// with the tile masks of the last binning, only the tiles the degridder reads
// are written.
static int fft64_planes(wsg_plan *p, void *grid, int sign, bool pruned)
{
    if (!p->tw64_ready) {
        WSG_CUDA(p->tw64x.ensure((size_t)2 * p->nx * sizeof(int4)));
        WSG_CUDA(p->tw64y.ensure((size_t)2 * p->ny * sizeof(int4)));
        WSG_CUDA(build_twiddles64(p->tw64x.as<int4>(), p->nx, p->stream));
        WSG_CUDA(build_twiddles64(p->tw64y.as<int4>(), p->ny, p->stream));
        p->tw64_ready = true;
    }
    const FftMasks m = mask_view(p);
    WSG_CUDA(launch_fft64(reinterpret_cast<double2 *>(grid), p->nx, p->ny, (int)p->cube_planes(),
                          sign, p->tw64x.as<int4>(), p->tw64y.as<int4>(), 0, p->stream,
                          pruned ? &m : nullptr, p->geom.tile_shift));
    return WSG_OK;
}

int wsg_fft(wsg_plan *p, void *grid, int sign)
{
    clear_error();
    if (!p || !grid) return set_error(WSG_ERR_ARG, "NULL argument");
    if (sign != 1 && sign != -1) return set_error(WSG_ERR_ARG, "sign must be +1 or -1");
    if (p->fused) {
        WSG_TRY(ensure_fused(p));
        WSG_CUDA(launch_fft2d_plain(p->geom, reinterpret_cast<float2 *>(grid), p->twx.as<float2>(),
                                    p->twy.as<float2>(), sign, p->stream));
        return WSG_OK;
    }
    if (p->fft64) return fft64_planes(p, grid, sign, false);
    WSG_TRY(ensure_fft(p));
    WSG_CUFFT(cufftSetStream(p->fft, p->stream));
    const int dir = sign > 0 ? CUFFT_INVERSE : CUFFT_FORWARD;
    const long long step = (long long)p->fft_batch * p->npix();
    for (int b0 = 0; b0 < p->planes; b0 += p->fft_batch) {
        if (p->prec == WSG_FP64) {
            cufftDoubleComplex *x = reinterpret_cast<cufftDoubleComplex *>(grid) + (b0 / p->fft_batch) * step;
            WSG_CUFFT(cufftExecZ2Z(p->fft, x, x, dir));
        } else {
            cufftComplex *x = reinterpret_cast<cufftComplex *>(grid) + (b0 / p->fft_batch) * step;
            WSG_CUFFT(cufftExecC2C(p->fft, x, x, dir));
        }
    }
    return WSG_OK;
}

int wsg_wcorrect(wsg_plan *p, const void *planes, void *image, double scale)
{
    clear_error();
    if (!p || !planes || !image) return set_error(WSG_ERR_ARG, "NULL argument");
    WSG_TRY(ensure_wscreen(p));
    if (p->prec == WSG_FP64) {
        WSG_CUDA(launch_wcorrect_f64(p->wc, p->sinx.as<double>(), p->siny.as<double>(),
                                     reinterpret_cast<const double2 *>(planes),
                                     reinterpret_cast<double2 *>(image), nullptr, nullptr, scale,
                                     p->stream));
    } else {
        WSG_CUDA(launch_wcorrect_f32c(p->wc, plan_wscreen(p),
                                      reinterpret_cast<const float2 *>(planes),
                                      reinterpret_cast<float2 *>(image), scale, p->stream));
    }
    return WSG_OK;
}

int wsg_wcorrect_adjoint(wsg_plan *p, const void *image, void *planes, double scale)
{
    clear_error();
    if (!p || !planes || !image) return set_error(WSG_ERR_ARG, "NULL argument");
    WSG_TRY(ensure_wscreen(p));
    if (p->prec == WSG_FP64) {
        WSG_CUDA(launch_wcorrect_adj_f64(p->wc, p->sinx.as<double>(), p->siny.as<double>(),
                                         reinterpret_cast<const double2 *>(image),
                                         reinterpret_cast<double2 *>(planes), scale, p->stream));
    } else {
        WSG_CUDA(launch_wcorrect_adj_f32c(p->wc, plan_wscreen(p),
                                          reinterpret_cast<const float2 *>(image),
                                          reinterpret_cast<float2 *>(planes), scale, p->stream));
    }
    return WSG_OK;
}

int wsg_degrid(wsg_plan *p, const void *grid, void *out)
{
    clear_error();
    if (!p || !grid || (!out && p->n_binned > 0)) return set_error(WSG_ERR_ARG, "NULL argument");
    if (p->n_binned < 0) return set_error(WSG_ERR_STATE, "wsg_degrid before wsg_bin");
    if (p->n_binned == 0) return WSG_OK;
    const BinBuffers b = p->binbufs();
    WSG_CUDA(cudaMemsetAsync(&b.ctr->work_degrid, 0, sizeof(unsigned), p->stream));
    WSG_CUDA(launch_degrid(p->geom, p->prec, b, p->recbufs(), grid, out, p->n_binned,
                           p->ctas_degrid, p->stream, p->walked));
    return WSG_OK;
}

int wsg_fft_wcorrect(wsg_plan *p, void *grid, void *image, int prune)
{
    clear_error();
    if (!p || !grid || !image) return set_error(WSG_ERR_ARG, "NULL argument");
    WSG_TRY(ensure_wscreen(p));
    const double scale = 1.0 / (double)p->npix();
    if (!p->fused) {
        WSG_TRY(wsg_fft(p, grid, +1));
        WSG_TRY(wsg_wcorrect(p, grid, image, scale));
        return WSG_OK;
    }
    WSG_TRY(ensure_fused(p));
    if (prune && !p->masks_valid) return set_error(WSG_ERR_STATE, "pruned transform before wsg_bin");
    if (!prune) {
        // dense transform: plain 2D FFT then the w-correction kernel
        WSG_CUDA(launch_fft2d_plain(p->geom, reinterpret_cast<float2 *>(grid),
                                    p->twx.as<float2>(), p->twy.as<float2>(), +1, p->stream));
        WSG_TRY(wsg_wcorrect(p, grid, image, scale));
        return WSG_OK;
    }
    WSG_CUDA(launch_image_fwd_fused(p->geom, reinterpret_cast<float2 *>(grid),
                                    reinterpret_cast<float2 *>(image), p->twx.as<float2>(),
                                    p->twy.as<float2>(), plan_wscreen(p), mask_view(p),
                                    p->wc.phase_on && p->planes > 1, scale, p->stream));
    return WSG_OK;
}

int wsg_wcorrect_adjoint_fft(wsg_plan *p, const void *image, void *grid, int prune)
{
    clear_error();
    if (!p || !grid || !image) return set_error(WSG_ERR_ARG, "NULL argument");
    WSG_TRY(ensure_wscreen(p));
    const double scale = 1.0 / (double)p->npix();
    if (!p->fused || !prune) {
        WSG_TRY(wsg_wcorrect_adjoint(p, image, grid, scale));
        if (prune && p->fft64 && p->masks_valid && fft64_masks_ok(p))
            WSG_TRY(fft64_planes(p, grid, -1, true));
        else
            WSG_TRY(wsg_fft(p, grid, -1));
        return WSG_OK;
    }
    WSG_TRY(ensure_fused(p));
    if (!p->masks_valid) return set_error(WSG_ERR_STATE, "pruned transform before wsg_bin");
    WSG_CUDA(launch_image_adj_fused(p->geom, reinterpret_cast<const float2 *>(image),
                                    reinterpret_cast<float2 *>(grid), p->twx.as<float2>(),
                                    p->twy.as<float2>(), plan_wscreen(p), mask_view(p),
                                    p->wc.phase_on && p->planes > 1, scale, p->stream));
    return WSG_OK;
}

int wsg_image_forward(wsg_plan *p, long n, long nf, long np, const double *uu, const double *vv,
                      const double *ww, const float *vr, const float *vi, const float *wt,
                      void *image)
{
    clear_error();
    if (!p || !image) return set_error(WSG_ERR_ARG, "NULL argument");
    WSG_CUDA(p->grid.ensure(p->elem() * (size_t)p->cube_planes() * p->npix()));
    WSG_TRY(ensure_wscreen(p));
    WSG_TRY(wsg_bin(p, n, nf, np, uu, vv, ww, vr, vi, wt));
    // the fused transforms read occupied tiles only: the gridder skips the
    // tiles of empty bins, which would only be written with zeros
    WSG_TRY(wsg_grid_occupied(p, p->grid.p));
    WSG_TRY(wsg_fft_wcorrect(p, p->grid.p, image, 1));
    return WSG_OK;
}

int wsg_image_adjoint(wsg_plan *p, const void *image, void *out)
{
    clear_error();
    if (!p || !image) return set_error(WSG_ERR_ARG, "NULL argument");
    if (p->n_binned < 0) return set_error(WSG_ERR_STATE, "adjoint before a forward/bin call");
    WSG_CUDA(p->grid.ensure(p->elem() * (size_t)p->cube_planes() * p->npix()));
    WSG_TRY(wsg_wcorrect_adjoint_fft(p, image, p->grid.p, 1));
    WSG_TRY(wsg_degrid(p, p->grid.p, out));
    return WSG_OK;
}

int wsg_image_forward_host(wsg_plan *p, long n, long nf, long np, const double *uu,
                           const double *vv, const double *ww, const float *vr, const float *vi,
                           const float *wt, void *image)
{
    clear_error();
    if (!p || !image) return set_error(WSG_ERR_ARG, "NULL argument");
    if (n < 0 || nf <= 0 || np <= 0) return set_error(WSG_ERR_ARG, "bad measurement counts");
    if (n > 0 && (!uu || !vv || !ww || !vr || !vi || !wt))
        return set_error(WSG_ERR_ARG, "NULL input pointer");
    const size_t nb = sizeof(double) * (size_t)n;
    const size_t nvis = sizeof(float) * (size_t)n * nf * np;
    const size_t nwt = sizeof(float) * (size_t)n * np;
    WSG_CUDA(p->h_uu.ensure(nb));
    WSG_CUDA(p->h_vv.ensure(nb));
    WSG_CUDA(p->h_ww.ensure(nb));
    WSG_CUDA(p->h_vr.ensure(nvis));
    WSG_CUDA(p->h_vi.ensure(nvis));
    WSG_CUDA(p->h_wt.ensure(nwt));
    WSG_CUDA(p->h_image.ensure(p->elem() * (size_t)p->npix()));
    if (n > 0) {
        WSG_CUDA(cudaMemcpyAsync(p->h_uu.p, uu, nb, cudaMemcpyHostToDevice, p->stream));
        WSG_CUDA(cudaMemcpyAsync(p->h_vv.p, vv, nb, cudaMemcpyHostToDevice, p->stream));
        WSG_CUDA(cudaMemcpyAsync(p->h_ww.p, ww, nb, cudaMemcpyHostToDevice, p->stream));
        WSG_CUDA(cudaMemcpyAsync(p->h_vr.p, vr, nvis, cudaMemcpyHostToDevice, p->stream));
        WSG_CUDA(cudaMemcpyAsync(p->h_vi.p, vi, nvis, cudaMemcpyHostToDevice, p->stream));
        WSG_CUDA(cudaMemcpyAsync(p->h_wt.p, wt, nwt, cudaMemcpyHostToDevice, p->stream));
    }
    WSG_TRY(wsg_image_forward(p, n, nf, np, p->h_uu.as<double>(), p->h_vv.as<double>(),
                              p->h_ww.as<double>(), p->h_vr.as<float>(), p->h_vi.as<float>(),
                              p->h_wt.as<float>(), p->h_image.p));
    WSG_CUDA(cudaMemcpyAsync(image, p->h_image.p, p->elem() * (size_t)p->npix(),
                             cudaMemcpyDeviceToHost, p->stream));
    WSG_CUDA(cudaStreamSynchronize(p->stream));
    return WSG_OK;
}

int wsg_image_adjoint_host(wsg_plan *p, const void *image, void *out)
{
    clear_error();
    if (!p || !image) return set_error(WSG_ERR_ARG, "NULL argument");
    if (p->n_binned < 0) return set_error(WSG_ERR_STATE, "adjoint before a forward/bin call");
    const size_t ibytes = p->elem() * (size_t)p->npix();
    const size_t obytes = p->elem() * (size_t)p->n_binned;
    WSG_CUDA(p->h_image.ensure(ibytes));
    WSG_CUDA(p->h_out.ensure(obytes));
    WSG_CUDA(cudaMemcpyAsync(p->h_image.p, image, ibytes, cudaMemcpyHostToDevice, p->stream));
    WSG_TRY(wsg_image_adjoint(p, p->h_image.p, p->h_out.p));
    if (obytes)
        WSG_CUDA(cudaMemcpyAsync(out, p->h_out.p, obytes, cudaMemcpyDeviceToHost, p->stream));
    WSG_CUDA(cudaStreamSynchronize(p->stream));
    return WSG_OK;
}

// ---- asynchronous host pipeline ---------------------------------------------

namespace {

// A large copy is issued as 32 MiB pieces: copies of one direction from
// different streams share the copy engines in order, and a latency-critical
// small copy (the adjoint's image) must not queue behind a whole prefetch.
cudaError_t copy_pieces(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind,
                        cudaStream_t s)
{
    const size_t piece = (size_t)32 << 20;
    for (size_t o = 0; o < bytes; o += piece) {
        const cudaError_t e = cudaMemcpyAsync(static_cast<char *>(dst) + o,
                                              static_cast<const char *>(src) + o,
                                              bytes - o < piece ? bytes - o : piece, kind, s);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// Copies between pinned host memory and the device done by a kernel on the
// compute stream: they bypass the copy engines, where an image copy would
// queue behind the next step's input upload (copies of one direction run in
// order), and they sit on the compute stream's critical path, which is where
// the image's round trip belongs.
__global__ void k_copy16(const uint4 *__restrict__ src, uint4 *__restrict__ dst, size_t n)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        dst[i] = src[i];
}

// dst <- src (bytes); `host` is whichever of the two is host memory.  Falls
// back to cudaMemcpyAsync unless the host side is pinned and everything is
// 16-byte aligned.
cudaError_t copy_by_kernel(void *dst, const void *src, size_t bytes, const void *host,
                           cudaMemcpyKind kind, cudaStream_t s)
{
    if (bytes == 0) return cudaSuccess;
    cudaPointerAttributes a;
    const bool pinned = cudaPointerGetAttributes(&a, host) == cudaSuccess &&
                        a.type == cudaMemoryTypeHost && a.devicePointer != nullptr;
    if (!pinned) cudaGetLastError();
    const bool aligned = (((uintptr_t)dst | (uintptr_t)src | bytes) & 15) == 0;
    if (!pinned || !aligned) return cudaMemcpyAsync(dst, src, bytes, kind, s);
    // a.devicePointer is the device view of `host` itself
    const void *dsrc = host == src ? a.devicePointer : src;
    void *ddst = host == dst ? a.devicePointer : dst;
    const size_t n = bytes / 16;
    const int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)num_sms() * 4);
    k_copy16<<<blocks, 256, 0, s>>>(static_cast<const uint4 *>(dsrc), static_cast<uint4 *>(ddst), n);
    return cudaGetLastError();
}

// The device's view of a pinned host buffer (8-byte aligned), or nullptr.
void *pinned_view(const void *host)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer || ((uintptr_t)a.devicePointer & 7))
        return nullptr;
    return a.devicePointer;
}

int ensure_async(wsg_plan *p)
{
    if (p->a_ready) return WSG_OK;
    WSG_CUDA(cudaStreamCreateWithFlags(&p->s_in, cudaStreamNonBlocking));
    WSG_CUDA(cudaStreamCreateWithFlags(&p->s_out, cudaStreamNonBlocking));
    cudaEvent_t *ev[] = {&p->e_in[0], &p->e_in[1], &p->e_free[0], &p->e_free[1], &p->e_adj,
                         &p->e_vis_down};
    for (cudaEvent_t *e : ev) WSG_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    p->a_ready = true;
    return WSG_OK;
}

}  // namespace

int wsg_image_forward_host_async(wsg_plan *p, long n, long nf, long np, const double *uu,
                                 const double *vv, const double *ww, const float *vr,
                                 const float *vi, const float *wt, void *image)
{
    clear_error();
    if (!p || !image) return set_error(WSG_ERR_ARG, "NULL argument");
    if (n < 0 || nf <= 0 || np <= 0) return set_error(WSG_ERR_ARG, "bad measurement counts");
    if (n > 0 && (!uu || !vv || !ww || !vr || !vi || !wt))
        return set_error(WSG_ERR_ARG, "NULL input pointer");
    WSG_TRY(ensure_async(p));
    const int s = p->a_slot;
    const size_t nb = sizeof(double) * (size_t)n;
    const size_t nvis = sizeof(float) * (size_t)n * nf * np;
    const size_t nwt = sizeof(float) * (size_t)n * np;
    const size_t bytes[6] = {nb, nb, nb, nvis, nvis, nwt};
    const void *src[6] = {uu, vv, ww, vr, vi, wt};
    for (int k = 0; k < 6; ++k) WSG_CUDA(p->a_in[s][k].ensure(bytes[k]));
    WSG_CUDA(p->a_img_fwd.ensure(p->elem() * (size_t)p->npix()));
    // the slot's previous inputs must have been binned before they are replaced
    WSG_CUDA(cudaStreamWaitEvent(p->s_in, p->e_free[s], 0));
    if (n > 0)
        for (int k = 0; k < 6; ++k)
            WSG_CUDA(copy_pieces(p->a_in[s][k].p, src[k], bytes[k], cudaMemcpyHostToDevice,
                                 p->s_in));
    WSG_CUDA(cudaEventRecord(p->e_in[s], p->s_in));
    WSG_CUDA(cudaStreamWaitEvent(p->stream, p->e_in[s], 0));
    // A fused plan's row kernel writes each image row once: with a pinned host
    // image it writes the rows straight into host memory, and the image's
    // download leaves the critical path.
    void *direct = p->fused ? pinned_view(image) : nullptr;
    WSG_TRY(wsg_image_forward(p, n, nf, np, p->a_in[s][0].as<double>(), p->a_in[s][1].as<double>(),
                              p->a_in[s][2].as<double>(), p->a_in[s][3].as<float>(),
                              p->a_in[s][4].as<float>(), p->a_in[s][5].as<float>(),
                              direct ? direct : p->a_img_fwd.p));
    WSG_CUDA(cudaEventRecord(p->e_free[s], p->stream));
    // otherwise the download stays on the compute stream (see copy_by_kernel)
    if (!direct)
        WSG_CUDA(copy_by_kernel(image, p->a_img_fwd.p, p->elem() * (size_t)p->npix(), image,
                                cudaMemcpyDeviceToHost, p->stream));
    p->a_slot = s ^ 1;
    return WSG_OK;
}

int wsg_image_adjoint_host_async(wsg_plan *p, const void *image, void *out)
{
    clear_error();
    if (!p || !image) return set_error(WSG_ERR_ARG, "NULL argument");
    if (p->n_binned < 0) return set_error(WSG_ERR_STATE, "adjoint before a forward/bin call");
    WSG_TRY(ensure_async(p));
    const size_t ibytes = p->elem() * (size_t)p->npix();
    const size_t obytes = p->elem() * (size_t)p->n_binned;
    if (obytes && !out) return set_error(WSG_ERR_ARG, "NULL output");
    WSG_CUDA(p->a_vis.ensure(obytes));
    // A fused plan's adjoint row kernel reads each image row once: a pinned
    // host image is read in place.  Otherwise it is uploaded on the compute
    // stream, after the forward's download of the same host image.
    const void *direct = p->fused ? pinned_view(image) : nullptr;
    if (!direct) {
        WSG_CUDA(p->a_img_adj.ensure(ibytes));
        WSG_CUDA(copy_by_kernel(p->a_img_adj.p, image, ibytes, image, cudaMemcpyHostToDevice,
                                p->stream));
    }
    // the previous adjoint output must have left the device buffer
    WSG_CUDA(cudaStreamWaitEvent(p->stream, p->e_vis_down, 0));
    WSG_TRY(wsg_image_adjoint(p, direct ? direct : p->a_img_adj.p, p->a_vis.p));
    WSG_CUDA(cudaEventRecord(p->e_adj, p->stream));
    WSG_CUDA(cudaStreamWaitEvent(p->s_out, p->e_adj, 0));
    if (obytes) WSG_CUDA(copy_pieces(out, p->a_vis.p, obytes, cudaMemcpyDeviceToHost, p->s_out));
    WSG_CUDA(cudaEventRecord(p->e_vis_down, p->s_out));
    return WSG_OK;
}

int wsg_plan_synchronize(wsg_plan *p)
{
    clear_error();
    if (!p) return set_error(WSG_ERR_ARG, "plan is NULL");
    if (p->a_ready) {
        WSG_CUDA(cudaStreamSynchronize(p->s_in));
        WSG_CUDA(cudaStreamSynchronize(p->s_out));
    }
    WSG_CUDA(cudaStreamSynchronize(p->stream));
    return WSG_OK;
}

}  // extern "C"


// ---------------------------------------------------------------------------
// drop-in entry points (reference signatures)
// ---------------------------------------------------------------------------

namespace {

struct Legacy {
    std::mutex mu;
    int precision = WSG_FP64;
    wsg_plan *plan = nullptr;
    cudaStream_t stream = nullptr;
    DevBuf uu, vv, ww, vr, vi, wt, grid64, image_re, image_im, planes, sinx, siny;
    // FFT entry
    cufftHandle fft = 0;
    int fft_nx = 0, fft_ny = 0, fft_batch = 0;
    DevBuf fft_work, fft_buf;
    int tw64_nx = 0, tw64_ny = 0;   // twiddles of the integer-pipe FFT
    DevBuf tw64x, tw64y;
};

Legacy &legacy()
{
    static Legacy L;
    return L;
}

int legacy_stream(Legacy &L)
{
    if (!L.stream) WSG_CUDA(cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking));
    return WSG_OK;
}

template <typename T>
int stage_in(Legacy &L, DevBuf &buf, const T *src, size_t count, const T **dst)
{
    if (count == 0) {
        *dst = src;
        return WSG_OK;
    }
    if (device_accessible(src)) {
        *dst = src;
        return WSG_OK;
    }
    WSG_CUDA(buf.ensure(sizeof(T) * count));
    WSG_CUDA(cudaMemcpyAsync(buf.p, src, sizeof(T) * count, cudaMemcpyHostToDevice, L.stream));
    *dst = buf.as<T>();
    return WSG_OK;
}

int legacy_wstack(int P, long n, long nf, long np, double *uu, double *vv, double *ww,
                  float *vr, float *vi, float *wt, double dx, double dw, int support, int nx,
                  int ny, double *grid)
{
    if (!grid) return set_error(WSG_ERR_ARG, "grid is NULL");
    Legacy &L = legacy();
    std::lock_guard<std::mutex> lock(L.mu);
    WSG_TRY(legacy_stream(L));
    wsg_plan *p = L.plan;
    if (!p || p->nx != nx || p->ny != ny || p->planes != P || p->support != support ||
        p->dx != dx || p->dw != dw || p->prec != L.precision) {
        if (p) wsg_plan_destroy(p);
        L.plan = nullptr;
        WSG_TRY(wsg_plan_create(&L.plan, nx, ny, P, support, dx, dw, L.precision, L.stream));
        p = L.plan;
    }
    p->stream = L.stream;
    const double *duu, *dvv, *dww;
    const float *dvr, *dvi, *dwt;
    const size_t nvis = (size_t)n * nf * np;
    WSG_TRY(stage_in(L, L.uu, uu, (size_t)n, &duu));
    WSG_TRY(stage_in(L, L.vv, vv, (size_t)n, &dvv));
    WSG_TRY(stage_in(L, L.ww, ww, (size_t)n, &dww));
    WSG_TRY(stage_in(L, L.vr, vr, nvis, &dvr));
    WSG_TRY(stage_in(L, L.vi, vi, nvis, &dvi));
    WSG_TRY(stage_in(L, L.wt, wt, (size_t)n * np, &dwt));
    WSG_TRY(wsg_bin(p, n, nf, np, duu, dvv, dww, dvr, dvi, dwt));
    const size_t cells = (size_t)P * nx * ny;
    const bool grid_dev = device_accessible(grid);
    if (p->prec == WSG_FP64) {
        void *target = grid;
        if (!grid_dev) {
            WSG_CUDA(L.grid64.ensure(cells * sizeof(double2)));
            target = L.grid64.p;
        }
        WSG_TRY(wsg_grid(p, target));
        if (!grid_dev)
            WSG_CUDA(cudaMemcpyAsync(grid, target, cells * sizeof(double2), cudaMemcpyDeviceToHost,
                                     L.stream));
    } else {
        WSG_CUDA(p->grid.ensure(cells * sizeof(float2)));
        WSG_TRY(wsg_grid(p, p->grid.p));
        void *target = grid;
        if (!grid_dev) {
            WSG_CUDA(L.grid64.ensure(cells * sizeof(double2)));
            target = L.grid64.p;
        }
        WSG_CUDA(launch_f32_to_f64(p->grid.as<float2>(), reinterpret_cast<double2 *>(target),
                                   (long long)cells, L.stream));
        if (!grid_dev)
            WSG_CUDA(cudaMemcpyAsync(grid, target, cells * sizeof(double2), cudaMemcpyDeviceToHost,
                                     L.stream));
    }
    WSG_CUDA(cudaStreamSynchronize(L.stream));
    DevCounters c;
    WSG_CUDA(cudaMemcpy(&c, p->ctr.p, sizeof(c), cudaMemcpyDeviceToHost));
    if (c.dropped_plane)
        return set_error(WSG_OK, "%llu measurements had a w-plane index outside [0, %d) and were skipped",
                         (unsigned long long)c.dropped_plane, P);
    return WSG_OK;
}

int legacy_phase(double *gridss, double *image_re, double *image_im, int xaxis, int yaxis,
                 int P, int xaxistot, int yaxistot, double resolution, double wmin, double wmax)
{
    if (!gridss || !image_re || !image_im) return set_error(WSG_ERR_ARG, "NULL argument");
    if (xaxis <= 0 || yaxis <= 0 || P <= 0) return set_error(WSG_ERR_ARG, "bad sizes");
    Legacy &L = legacy();
    std::lock_guard<std::mutex> lock(L.mu);
    WSG_TRY(legacy_stream(L));
    WcParams wc;
    wc.xaxis = xaxis;
    wc.yaxis = yaxis;
    wc.planes = P;
    wc.xaxistot = xaxistot;
    wc.yaxistot = yaxistot;
    wc.resolution = resolution;
    wc.wmin = wmin;
    wc.wmax = wmax;
    wc.phase_on = 1;
    const size_t npix = (size_t)xaxis * yaxis;
    const double2 *planes;
    WSG_TRY(stage_in(L, L.planes, reinterpret_cast<const double2 *>(gridss), npix * P, &planes));
    WSG_CUDA(L.sinx.ensure(sizeof(double) * xaxis));
    WSG_CUDA(L.siny.ensure(sizeof(double) * yaxis));
    WSG_CUDA(launch_wscreen_tables(wc, L.sinx.as<double>(), L.siny.as<double>(), L.stream));
    double *ore = image_re, *oim = image_im;
    const bool re_dev = device_accessible(image_re), im_dev = device_accessible(image_im);
    if (!re_dev) {
        WSG_CUDA(L.image_re.ensure(sizeof(double) * npix));
        ore = L.image_re.as<double>();
    }
    if (!im_dev) {
        WSG_CUDA(L.image_im.ensure(sizeof(double) * npix));
        oim = L.image_im.as<double>();
    }
    WSG_CUDA(launch_wcorrect_f64(wc, L.sinx.as<double>(), L.siny.as<double>(), planes, nullptr,
                                 ore, oim, 1.0, L.stream));
    if (!re_dev)
        WSG_CUDA(cudaMemcpyAsync(image_re, ore, sizeof(double) * npix, cudaMemcpyDeviceToHost, L.stream));
    if (!im_dev)
        WSG_CUDA(cudaMemcpyAsync(image_im, oim, sizeof(double) * npix, cudaMemcpyDeviceToHost, L.stream));
    WSG_CUDA(cudaStreamSynchronize(L.stream));
    return WSG_OK;
}

int legacy_fft(const double *in, double *out, int nx, int ny, int nplanes)
{
    if (!in || !out) return set_error(WSG_ERR_ARG, "NULL argument");
    if (nx <= 0 || ny <= 0 || nplanes <= 0) return set_error(WSG_ERR_ARG, "bad sizes");
    Legacy &L = legacy();
    std::lock_guard<std::mutex> lock(L.mu);
    WSG_TRY(legacy_stream(L));
    const long long npix = (long long)nx * ny;
    const size_t bytes = sizeof(double2) * (size_t)npix * nplanes;
    const char *fft_env = getenv("WSTACK_GB300_FFT");
    const bool int_fft =
        fft64_supported(nx, ny, nplanes) && !(fft_env && strcmp(fft_env, "cufft") == 0);
    if (int_fft && (L.tw64_nx != nx || L.tw64_ny != ny)) {
        WSG_CUDA(L.tw64x.ensure((size_t)2 * nx * sizeof(int4)));
        WSG_CUDA(L.tw64y.ensure((size_t)2 * ny * sizeof(int4)));
        WSG_CUDA(build_twiddles64(L.tw64x.as<int4>(), nx, L.stream));
        WSG_CUDA(build_twiddles64(L.tw64y.as<int4>(), ny, L.stream));
        L.tw64_nx = nx;
        L.tw64_ny = ny;
    }
    if (!int_fft && (!L.fft || L.fft_nx != nx || L.fft_ny != ny)) {
        if (L.fft) cufftDestroy(L.fft);
        L.fft = 0;
        WSG_CUFFT(cufftCreate(&L.fft));
        WSG_CUFFT(cufftSetAutoAllocation(L.fft, 0));
        long long n2[2] = {ny, nx};
        size_t ws = 0;
        WSG_CUFFT(cufftMakePlanMany64(L.fft, 2, n2, nullptr, 1, npix, nullptr, 1, npix, CUFFT_Z2Z,
                                      1, &ws));
        WSG_CUDA(L.fft_work.ensure(ws));
        WSG_CUFFT(cufftSetWorkArea(L.fft, L.fft_work.p));
        L.fft_nx = nx;
        L.fft_ny = ny;
    }
    if (!int_fft) WSG_CUFFT(cufftSetStream(L.fft, L.stream));
    const bool in_dev = device_accessible(in), out_dev = device_accessible(out);
    double2 *work;
    if (out_dev) {
        work = reinterpret_cast<double2 *>(out);
        if (in != out)
            WSG_CUDA(cudaMemcpyAsync(work, in, bytes, in_dev ? cudaMemcpyDeviceToDevice
                                                             : cudaMemcpyHostToDevice, L.stream));
    } else {
        WSG_CUDA(L.fft_buf.ensure(bytes));
        work = L.fft_buf.as<double2>();
        WSG_CUDA(cudaMemcpyAsync(work, in, bytes, in_dev ? cudaMemcpyDeviceToDevice
                                                         : cudaMemcpyHostToDevice, L.stream));
    }
    if (int_fft) {
        // 1/(nx ny) is an exact power of two, applied as the FFT's output exponent
        int lg = 0;
        while ((1ll << lg) < npix) lg++;
        WSG_CUDA(launch_fft64(work, nx, ny, nplanes, +1, L.tw64x.as<int4>(), L.tw64y.as<int4>(),
                              -lg, L.stream));
    } else {
        for (int w = 0; w < nplanes; w++) {
            cufftDoubleComplex *x = reinterpret_cast<cufftDoubleComplex *>(work) + (size_t)w * npix;
            WSG_CUFFT(cufftExecZ2Z(L.fft, x, x, CUFFT_INVERSE));
        }
        WSG_CUDA(launch_scale_f64(work, npix * nplanes, 1.0 / (double)npix, L.stream));
    }
    if (!out_dev) WSG_CUDA(cudaMemcpyAsync(out, work, bytes, cudaMemcpyDeviceToHost, L.stream));
    WSG_CUDA(cudaStreamSynchronize(L.stream));
    return WSG_OK;
}

}  // namespace

extern "C" {

void wstack(int num_w_planes, long num_points, long freq_per_chan, long polarizations, double *uu,
            double *vv, double *ww, float *vis_real, float *vis_img, float *weight, double dx,
            double dw, int w_support, int grid_size_x, int grid_size_y, double *grid,
            int num_threads)
{
    (void)num_threads;
    clear_error();
    legacy_wstack(num_w_planes, num_points, freq_per_chan, polarizations, uu, vv, ww, vis_real,
                  vis_img, weight, dx, dw, w_support, grid_size_x, grid_size_y, grid);
}

void phase_correction(double *gridss, double *image_real, double *image_imag, int xaxis,
                      int yaxis, int num_w_planes, int xaxistot, int yaxistot, double resolution,
                      double wmin, double wmax, int num_threads)
{
    (void)num_threads;
    clear_error();
    legacy_phase(gridss, image_real, image_imag, xaxis, yaxis, num_w_planes, xaxistot, yaxistot,
                 resolution, wmin, wmax);
}

int test(int nnn) { return nnn + 1; }

int wstack_fft_planes(const double *in, double *out, int nx, int ny, int nplanes)
{
    clear_error();
    return legacy_fft(in, out, nx, ny, nplanes);
}

int wstack_gb300_last_error(void) { return tl_status; }

const char *wstack_gb300_last_error_string(void) { return tl_msg; }

int wstack_gb300_set_precision(int precision)
{
    if (precision != WSG_FP64 && precision != WSG_FP32C) return -1;
    Legacy &L = legacy();
    std::lock_guard<std::mutex> lock(L.mu);
    const int old = L.precision;
    L.precision = precision;
    return old;
}

void wstack_gb300_release(void)
{
    Legacy &L = legacy();
    std::lock_guard<std::mutex> lock(L.mu);
    if (L.plan) wsg_plan_destroy(L.plan);
    L.plan = nullptr;
    if (L.fft) cufftDestroy(L.fft);
    L.fft = 0;
    L.tw64_nx = L.tw64_ny = 0;
    DevBuf *bufs[] = {&L.uu, &L.vv, &L.ww, &L.vr, &L.vi, &L.wt, &L.grid64, &L.image_re,
                      &L.image_im, &L.planes, &L.sinx, &L.siny, &L.fft_work, &L.fft_buf,
                      &L.tw64x, &L.tw64y};
    for (DevBuf *b : bufs) b->release();
    if (L.stream) cudaStreamDestroy(L.stream);
    L.stream = nullptr;
}

}  // extern "C"
