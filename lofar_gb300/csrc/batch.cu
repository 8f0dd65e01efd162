// (channel, polarisation) batches, CUDA-graph replay of the batched forward,
// and the autotuner of the tile edge, split size and persistent CTA count.
//
// A batch is a plan whose cube holds one job of P planes per (channel,
// polarisation) pair, stacked along the plane axis: bins, records, the tile
// kernels, the column FFTs and the degridder see J*P planes and need nothing
// batch-specific; only the binning pass (which maps a measurement to its
// channel and emits one record set per polarisation) and the row FFT +
// w-correction (one image per job) know about jobs.
#include <cuda_runtime.h>
#include <math.h>

#include <functional>
#include <new>
#include <vector>

#include "plan.cuh"

using namespace wsg;

struct wsg_batch {
    wsg_plan *p = nullptr;
    int channels = 0, pols = 0;
    std::vector<ChanDesc> table;
    std::vector<long long> m0;
    DevBuf dtable, dm0;
    ChanTable tab{};
    long long ntot = 0;              // bound measurements
    unsigned long long nvis = 0;     // bound visibilities (ntot * pols)
    bool bound = false;
    // graph of the forward
    cudaStream_t gstream = nullptr;  // capture stream when the plan's stream is the legacy one
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    const void *graph_images = nullptr;
    unsigned long long gen = 1, graph_gen = 0;
    bool forwarded = false;
};

namespace {

void drop_graph(wsg_batch *B)
{
    if (B->exec) cudaGraphExecDestroy(B->exec);
    if (B->graph) cudaGraphDestroy(B->graph);
    B->exec = nullptr;
    B->graph = nullptr;
    B->graph_images = nullptr;
    B->graph_gen = 0;
}

// Device storage for the bound inputs (no allocation afterwards, so the
// forward can be captured).
int batch_prepare(wsg_batch *B)
{
    wsg_plan *p = B->p;
    if (!B->bound) return set_error(WSG_ERR_STATE, "no channels bound (wsg_batch_bind)");
    if (!p->wc_set) return set_error(WSG_ERR_STATE, "w-correction geometry not set");
    WSG_TRY(ensure_records(p, (long long)B->nvis));
    WSG_CUDA(p->grid.ensure(p->elem() * (size_t)p->cube_planes() * p->npix()));
    WSG_TRY(ensure_wscreen(p));
    WSG_TRY(ensure_fused(p));
    return WSG_OK;
}

// The forward's stream work: allocation-free, so it can be captured.
int batch_enqueue_forward(wsg_batch *B, void *images)
{
    wsg_plan *p = B->p;
    const BinBuffers b = p->binbufs();
    const RecBuffers r = p->recbufs();
    WSG_CUDA(cudaMemsetAsync(b.sub_prim, 0, bin_counter_bytes(p->geom.nbins, b.nsub), p->stream));
    WSG_CUDA(cudaMemsetAsync(b.ctr, 0, sizeof(DevCounters), p->stream));
    WSG_CUDA(launch_bin_count_batch(p->geom, B->tab, b, p->stream));
    WSG_CUDA(launch_bin_scan(p->geom, b, p->stream));
    WSG_CUDA(launch_bin_scatter_batch(p->geom, p->prec, B->tab, b, r, p->stream));
    WSG_CUDA(launch_fft_masks(p->geom, b, mask_view(p), p->stream));
    WSG_CUDA(launch_grid(p->geom, p->prec, b, r, p->grid.p, p->partials.p, p->ctas_grid,
                         p->stream, true));   // occupied tiles only: the fused transforms skip the rest
    WSG_CUDA(launch_image_fwd_fused(p->geom, p->grid.as<float2>(), reinterpret_cast<float2 *>(images),
                                    p->twx.as<float2>(), p->twy.as<float2>(), plan_wscreen(p),
                                    mask_view(p), p->wc.phase_on && p->planes > 1,
                                    1.0 / (double)p->npix(), p->stream));
    return WSG_OK;
}

int batch_capture(wsg_batch *B, void *images, cudaStream_t cs)
{
    drop_graph(B);
    wsg_plan *p = B->p;
    cudaStream_t keep = p->stream;
    p->stream = cs;
    WSG_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed));
    const int st = batch_enqueue_forward(B, images);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(cs, &g);
    p->stream = keep;
    if (st != WSG_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    WSG_CUDA(e);
    B->graph = g;
    WSG_CUDA(cudaGraphInstantiate(&B->exec, g, 0));
    B->graph_images = images;
    B->graph_gen = B->gen;
    return WSG_OK;
}

int batch_forward(wsg_batch *B, void *images, int use_graph)
{
    wsg_plan *p = B->p;
    WSG_TRY(batch_prepare(B));
    if (!use_graph) {
        WSG_TRY(batch_enqueue_forward(B, images));
    } else {
        // the legacy default stream cannot be captured: run the graph on a
        // private stream ordered after and before it with events
        const bool own = p->stream == nullptr;
        cudaStream_t cs = p->stream;
        if (own) {
            if (!B->gstream) WSG_CUDA(cudaStreamCreateWithFlags(&B->gstream, cudaStreamNonBlocking));
            if (!B->ev_in) WSG_CUDA(cudaEventCreateWithFlags(&B->ev_in, cudaEventDisableTiming));
            if (!B->ev_out) WSG_CUDA(cudaEventCreateWithFlags(&B->ev_out, cudaEventDisableTiming));
            cs = B->gstream;
        }
        if (!B->exec || B->graph_gen != B->gen || B->graph_images != images)
            WSG_TRY(batch_capture(B, images, cs));
        if (own) {
            WSG_CUDA(cudaEventRecord(B->ev_in, p->stream));
            WSG_CUDA(cudaStreamWaitEvent(cs, B->ev_in, 0));
        }
        WSG_CUDA(cudaGraphLaunch(B->exec, cs));
        if (own) {
            WSG_CUDA(cudaEventRecord(B->ev_out, cs));
            WSG_CUDA(cudaStreamWaitEvent(p->stream, B->ev_out, 0));
        }
    }
    p->n_binned = (long long)B->nvis;
    p->walked = false;
    p->masks_valid = true;
    B->forwarded = true;
    return WSG_OK;
}

// Autotuner: one parameter at a time (tile edge, then split size, then CTAs
// per SM), each candidate timed over `iters` runs after one warm-up run.
struct Tuner {
    wsg_plan *p;
    std::function<int()> prepare, run;
    int iters;
    std::vector<wsg_tuning> tried;

    int time_one(int tile, int ctas, int chunk, float &ms)
    {
        p->tile = tile;
        p->ctas_user = ctas;
        p->split = chunk;
        WSG_TRY(plan_configure(p));
        WSG_TRY(prepare());
        WSG_TRY(run());
        cudaEvent_t e0, e1;
        WSG_CUDA(cudaEventCreate(&e0));
        WSG_CUDA(cudaEventCreate(&e1));
        int st = WSG_OK;
        cudaError_t ce = cudaEventRecord(e0, p->stream);
        for (int i = 0; i < iters && st == WSG_OK && ce == cudaSuccess; i++) st = run();
        if (ce == cudaSuccess) ce = cudaEventRecord(e1, p->stream);
        if (ce == cudaSuccess) ce = cudaEventSynchronize(e1);
        float t = 0.f;
        if (ce == cudaSuccess) ce = cudaEventElapsedTime(&t, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (st != WSG_OK) return st;
        WSG_CUDA(ce);
        ms = t / (float)iters;
        tried.push_back(wsg_tuning{tile, ctas, chunk, ms});
        return WSG_OK;
    }

    int tune(wsg_tuning &best)
    {
        const int half = p->half;
        std::vector<int> tiles;
        for (int t : {64, 32}) {
            if (2 * half + 1 > t) continue;
            if (p->fused && !fft_fused_supported(p->nx, p->ny, t)) continue;
            if (grid_max_ctas_per_sm(p->prec, t, half) <= 0) continue;
            tiles.push_back(t);
        }
        if (tiles.empty()) return set_error(WSG_ERR_UNSUPPORTED, "no tile edge to tune");
        best = wsg_tuning{p->tile, 0, p->split, INFINITY};
        for (int t : tiles) {
            float ms = 0.f;
            WSG_TRY(time_one(t, 0, best.chunk, ms));
            if (ms < best.ms) best = wsg_tuning{t, 0, best.chunk, ms};
        }
        for (int c : {2048, 4096, 8192, 16384}) {
            if (c == best.chunk) continue;
            float ms = 0.f;
            WSG_TRY(time_one(best.tile, 0, c, ms));
            if (ms < best.ms) best = wsg_tuning{best.tile, 0, c, ms};
        }
        const int kmax = grid_max_ctas_per_sm(p->prec, best.tile, half);
        const int auto_k = kmax;   // ctas 0 = kmax per SM, already timed
        for (int k = 1; k < kmax; k++) {
            if (k == auto_k) continue;
            float ms = 0.f;
            WSG_TRY(time_one(best.tile, k * num_sms(), best.chunk, ms));
            if (ms < best.ms) best = wsg_tuning{best.tile, k * num_sms(), best.chunk, ms};
        }
        p->tile = best.tile;
        p->ctas_user = best.ctas;
        p->split = best.chunk;
        WSG_TRY(plan_configure(p));
        return prepare();
    }
};

void copy_tried(const std::vector<wsg_tuning> &v, wsg_tuning *tried, int max_tried, int *n_tried)
{
    int n = 0;
    for (const wsg_tuning &t : v) {
        if (tried && n < max_tried) tried[n] = t;
        n++;
    }
    if (n_tried) *n_tried = n;
}

}  // namespace

extern "C" {

int wsg_plan_autotune(wsg_plan *p, long n, long nf, long np, const double *uu, const double *vv,
                      const double *ww, const float *vr, const float *vi, const float *wt,
                      void *image, int iters, wsg_tuning *best, wsg_tuning *tried, int max_tried,
                      int *n_tried)
{
    clear_error();
    if (!p || !image) return set_error(WSG_ERR_ARG, "NULL argument");
    if (p->jobs != 1) return set_error(WSG_ERR_STATE, "batch plans are tuned by wsg_batch_autotune");
    if (iters <= 0) return set_error(WSG_ERR_ARG, "iters must be positive");
    if (!p->wc_set) return set_error(WSG_ERR_STATE, "w-correction geometry not set");
    Tuner T{p, [] { return (int)WSG_OK; },
            [=] { return wsg_image_forward(p, n, nf, np, uu, vv, ww, vr, vi, wt, image); }, iters,
            {}};
    wsg_tuning b{};
    const int st = T.tune(b);
    copy_tried(T.tried, tried, max_tried, n_tried);
    if (st != WSG_OK) return st;
    if (best) *best = b;
    return WSG_OK;
}

int wsg_batch_create(wsg_batch **out, int nx, int ny, int planes, int support, double dx,
                     double dw, int channels, int pols, void *stream)
{
    clear_error();
    if (!out) return set_error(WSG_ERR_ARG, "batch pointer is NULL");
    *out = nullptr;
    if (channels <= 0 || pols <= 0) return set_error(WSG_ERR_ARG, "channels and pols must be positive");
    if (channels > kMaxChannels)
        return set_error(WSG_ERR_UNSUPPORTED, "more than %d channels in one batch", kMaxChannels);
    if ((long long)channels * pols * (planes > 0 ? planes : 1) > 65535)
        return set_error(WSG_ERR_UNSUPPORTED, "channels*pols*planes above 65535");
    if (!fft_fused_supported(nx, ny, 64))
        return set_error(WSG_ERR_UNSUPPORTED, "batches need power-of-two grid edges in [256, 8192]");
    wsg_batch *B = new (std::nothrow) wsg_batch();
    if (!B) return set_error(WSG_ERR_NOMEM, "host allocation failed");
    int st = wsg_plan_create(&B->p, nx, ny, planes, support, dx, dw, WSG_FP32C, stream);
    if (st == WSG_OK) {
        B->channels = channels;
        B->pols = pols;
        B->p->jobs = channels * pols;
        st = plan_configure(B->p);
    }
    if (st == WSG_OK && !B->p->fused)
        st = set_error(WSG_ERR_UNSUPPORTED, "the fused FFT is disabled (WSTACK_GB300_FFT)");
    if (st != WSG_OK) {
        const int keep = st;
        wsg_batch_destroy(B);
        return keep;
    }
    *out = B;
    return WSG_OK;
}

int wsg_batch_destroy(wsg_batch *B)
{
    if (!B) return WSG_OK;
    drop_graph(B);
    if (B->gstream) cudaStreamDestroy(B->gstream);
    if (B->ev_in) cudaEventDestroy(B->ev_in);
    if (B->ev_out) cudaEventDestroy(B->ev_out);
    B->dtable.release();
    B->dm0.release();
    if (B->p) wsg_plan_destroy(B->p);
    delete B;
    return WSG_OK;
}

int wsg_batch_set_stream(wsg_batch *B, void *stream)
{
    clear_error();
    if (!B) return set_error(WSG_ERR_ARG, "batch is NULL");
    if (B->p->stream != (cudaStream_t)stream) B->gen++;
    B->p->stream = (cudaStream_t)stream;
    return WSG_OK;
}

int wsg_batch_set_wcorrection(wsg_batch *B, double resolution, double wmin, double wmax)
{
    clear_error();
    if (!B) return set_error(WSG_ERR_ARG, "batch is NULL");
    WSG_TRY(wsg_plan_set_wcorrection(B->p, resolution, wmin, wmax));
    B->gen++;
    return WSG_OK;
}

int wsg_batch_set_tuning(wsg_batch *B, int tile, int ctas, int chunk)
{
    clear_error();
    if (!B) return set_error(WSG_ERR_ARG, "batch is NULL");
    const int st = wsg_plan_set_tuning(B->p, tile, ctas, chunk);
    B->gen++;
    B->forwarded = false;
    return st;
}

int wsg_batch_bind(wsg_batch *B, const wsg_channel *ch)
{
    clear_error();
    if (!B || !ch) return set_error(WSG_ERR_ARG, "NULL argument");
    std::vector<ChanDesc> t(B->channels);
    std::vector<long long> m0(B->channels);
    long long tot = 0;
    for (int c = 0; c < B->channels; c++) {
        const wsg_channel &x = ch[c];
        if (x.num_points < 0) return set_error(WSG_ERR_ARG, "channel %d: negative num_points", c);
        if (x.num_points > 0 && (!x.uu || !x.vv || !x.ww || !x.vis_real || !x.vis_img || !x.weight))
            return set_error(WSG_ERR_ARG, "channel %d: NULL input pointer", c);
        t[c] = ChanDesc{x.uu, x.vv, x.ww, x.vis_real, x.vis_img, x.weight, tot, x.num_points,
                        (unsigned long long)tot * B->pols};
        m0[c] = tot;
        tot += x.num_points;
    }
    const unsigned long long nvis = (unsigned long long)tot * B->pols;
    // record positions and indices are 32-bit; each visibility gives <= 4 records
    if (nvis * 4ull >= (1ull << 32))
        return set_error(WSG_ERR_UNSUPPORTED, "%llu visibilities in one batch (limit %llu)", nvis,
                         ((1ull << 32) - 1) / 4);
    WSG_CUDA(B->dtable.ensure(sizeof(ChanDesc) * B->channels));
    WSG_CUDA(B->dm0.ensure(sizeof(long long) * B->channels));
    WSG_CUDA(cudaMemcpyAsync(B->dtable.p, t.data(), sizeof(ChanDesc) * B->channels,
                             cudaMemcpyHostToDevice, B->p->stream));
    WSG_CUDA(cudaMemcpyAsync(B->dm0.p, m0.data(), sizeof(long long) * B->channels,
                             cudaMemcpyHostToDevice, B->p->stream));
    WSG_CUDA(cudaStreamSynchronize(B->p->stream));
    B->table.swap(t);
    B->m0.swap(m0);
    B->tab = ChanTable{B->dtable.as<ChanDesc>(), B->dm0.as<long long>(), B->channels, B->pols, tot};
    B->ntot = tot;
    B->nvis = nvis;
    B->bound = true;
    B->forwarded = false;
    B->gen++;
    return batch_prepare(B);
}

int wsg_batch_forward(wsg_batch *B, void *images, int use_graph)
{
    clear_error();
    if (!B || !images) return set_error(WSG_ERR_ARG, "NULL argument");
    return batch_forward(B, images, use_graph);
}

int wsg_batch_adjoint(wsg_batch *B, const void *images, void *vis_out)
{
    clear_error();
    if (!B || !images || (!vis_out && B->nvis)) return set_error(WSG_ERR_ARG, "NULL argument");
    if (!B->forwarded) return set_error(WSG_ERR_STATE, "adjoint before a forward");
    wsg_plan *p = B->p;
    WSG_TRY(batch_prepare(B));
    WSG_CUDA(launch_image_adj_fused(p->geom, reinterpret_cast<const float2 *>(images),
                                    p->grid.as<float2>(), p->twx.as<float2>(), p->twy.as<float2>(),
                                    plan_wscreen(p), mask_view(p), p->wc.phase_on && p->planes > 1,
                                    1.0 / (double)p->npix(), p->stream));
    if (B->nvis == 0) return WSG_OK;
    const BinBuffers b = p->binbufs();
    WSG_CUDA(cudaMemsetAsync(&b.ctr->work_degrid, 0, sizeof(unsigned), p->stream));
    WSG_CUDA(launch_degrid(p->geom, p->prec, b, p->recbufs(), p->grid.p, vis_out,
                           (long long)B->nvis, p->ctas_degrid, p->stream));
    return WSG_OK;
}

int wsg_batch_autotune(wsg_batch *B, void *images, int iters, wsg_tuning *best, wsg_tuning *tried,
                       int max_tried, int *n_tried)
{
    clear_error();
    if (!B || !images) return set_error(WSG_ERR_ARG, "NULL argument");
    if (iters <= 0) return set_error(WSG_ERR_ARG, "iters must be positive");
    WSG_TRY(batch_prepare(B));
    Tuner T{B->p, [B] { return batch_prepare(B); },
            [B, images] { return batch_forward(B, images, 0); }, iters, {}};
    wsg_tuning b{};
    const int st = T.tune(b);
    B->gen++;
    copy_tried(T.tried, tried, max_tried, n_tried);
    if (st != WSG_OK) return st;
    if (best) *best = b;
    B->forwarded = false;
    return WSG_OK;
}

long long wsg_batch_vis_offset(wsg_batch *B, int channel)
{
    if (!B || !B->bound || channel < 0 || channel > B->channels) return -1;
    if (channel == B->channels) return (long long)B->nvis;
    return (long long)B->table[channel].vis0;
}

void *wsg_batch_grids(wsg_batch *B) { return B ? B->p->grid.p : nullptr; }

int wsg_batch_get_stats(wsg_batch *B, wsg_stats *s)
{
    clear_error();
    if (!B) return set_error(WSG_ERR_ARG, "batch is NULL");
    return wsg_plan_get_stats(B->p, s);
}

long long wsg_batch_device_bytes(wsg_batch *B)
{
    if (!B) return 0;
    return wsg_plan_device_bytes(B->p) + (long long)B->dtable.bytes + (long long)B->dm0.bytes;
}

}  // extern "C"
