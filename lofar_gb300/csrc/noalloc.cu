// wsg_grid_noalloc: FP64 gridding that allocates no device memory.
//
// Some callers cannot call cudaMalloc at the point where they grid: a
// real-time pipeline that reserves all of its device memory up front and
// forbids allocation while observing, a host application that owns the
// device's memory and hands plug-ins only its own buffers, or code running in
// a context where an allocation would synchronise the device.  For them this
// entry point grids measurements that are already on the device into a grid
// that is already on the device, and keeps every intermediate (the bin table
// and the sorted measurement records) in the static array below instead of
// allocating it.
//
// The array is a fixed 64 MiB of device memory per GPU that loads the library,
// held until the process exits.  A call needs at most
//     2560 + 36*nbins + 16*ceil(nbins/256) + 161*num_points   bytes
//     (alignment padding included),
//     nbins = num_w_planes * ceil(grid_size_y/64) * ceil(grid_size_x/64),
// and is rejected with WSG_ERR_CAPACITY when that exceeds the array: for a
// 4096x4096x32 grid that is about 387,000 measurements per call.  Every call
// overwrites the whole grid (as wstack() does), so a caller splitting a larger
// set grids each part into its own grid and sums the grids.  Its bin table
// keeps one counter per bin and kind (no sub-counters).
//
// All calls share the array and it keeps what the last call left in it; each
// call clears the counters it needs before using them.  Calls whose GPU work
// may overlap (different streams without ordering, or several host threads)
// race on the array and must be serialised by the caller.
//
// The device address of the array is looked up once per device (with that
// device current) by the first call made on it; that first call may also load
// the library's device code, so make it before any stream capture.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>

#include <mutex>

#include "wsg_internal.cuh"

namespace wsg {
int report_status(int status, const char *msg);  // capi.cu: per-thread last error
}

using namespace wsg;

namespace {

constexpr size_t kNoAllocBytes = (size_t)64 << 20;
constexpr int kNoAllocTile = 64;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_addr_mu;
void *g_addr[kMaxDevices] = {};

size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

int fail(int status, const char *fmt, ...)
{
    char msg[384];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof(msg), fmt, ap);
    va_end(ap);
    return report_status(status, msg);
}

int scratch_address(void **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(WSG_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices)
        return fail(WSG_ERR_UNSUPPORTED, "device ordinal %d above %d", dev, kMaxDevices - 1);
    std::lock_guard<std::mutex> lock(g_addr_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(WSG_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return WSG_OK;
}

bool pow2_recip(double d, int &k)
{
    if (!(d > 0.0) || !isfinite(d)) return false;
    int e;
    if (frexp(d, &e) != 0.5) return false;
    k = 1 - e;
    return k >= 0 && k <= 1000;
}

bool on_device(const void *ptr)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace

extern "C" int wsg_grid_noalloc(int num_w_planes, long num_points, long freq_per_chan,
                                long polarizations, const double *uu, const double *vv,
                                const double *ww, const float *vis_real, const float *vis_img,
                                const float *weight, double dx, double dw, int w_support,
                                int grid_size_x, int grid_size_y, double *grid, void *stream)
{
    report_status(WSG_OK, "");
    if (num_w_planes <= 0 || grid_size_x <= 0 || grid_size_y <= 0 || num_points < 0 ||
        freq_per_chan <= 0 || polarizations <= 0)
        return fail(WSG_ERR_ARG, "wsg_grid_noalloc: sizes must be positive");
    if (grid_size_x > 65536 || grid_size_y > 65536)
        return fail(WSG_ERR_UNSUPPORTED, "wsg_grid_noalloc: grid edge above 65536");
    if (w_support < 1 || w_support > 2 * kMaxHalf + 1)
        return fail(WSG_ERR_UNSUPPORTED, "wsg_grid_noalloc: w_support %d outside [1, %d]",
                    w_support, 2 * kMaxHalf + 1);
    if (!(dx > 0.0) || !(dw > 0.0) || !isfinite(dx) || !isfinite(dw))
        return fail(WSG_ERR_ARG, "wsg_grid_noalloc: dx and dw must be positive and finite");
    if (!grid || (num_points > 0 && (!uu || !vv || !ww || !vis_real || !vis_img || !weight)))
        return fail(WSG_ERR_ARG, "wsg_grid_noalloc: NULL pointer");
    const void *ptrs[] = {uu, vv, ww, vis_real, vis_img, weight};
    if (!on_device(grid)) return fail(WSG_ERR_ARG, "wsg_grid_noalloc: grid must be device memory");
    if (num_points > 0)
        for (const void *q : ptrs)
            if (!on_device(q))
                return fail(WSG_ERR_ARG, "wsg_grid_noalloc: inputs must be device memory");

    GeomParams g{};
    g.nx = grid_size_x;
    g.ny = grid_size_y;
    g.planes = num_w_planes;
    g.wplanes = num_w_planes;
    g.half = (w_support - 1) / 2;
    g.tile = kNoAllocTile;
    g.tile_shift = 6;   // log2(kNoAllocTile)
    g.ntu = (grid_size_x + kNoAllocTile - 1) / kNoAllocTile;
    g.ntv = (grid_size_y + kNoAllocTile - 1) / kNoAllocTile;
    g.nbins = (long long)num_w_planes * g.ntv * g.ntu;
    g.dx = dx;
    g.dw = dw;
    int k = 0;
    g.u_pow2 = pow2_recip(dx, k) ? 1 : 0;
    g.ku = g.u_pow2 ? k : 0;
    g.w_pow2 = pow2_recip(dw, k) ? 1 : 0;
    g.kw = g.w_pow2 ? k : 0;

    // Bound the sizes before any layout arithmetic: a measurement needs at
    // least 160 bytes of the array (four records of 40 bytes), so larger
    // counts cannot fit and would overflow the products below; the value
    // index m*freq_per_chan*polarizations must stay well inside 63 bits.
    if ((unsigned long long)num_points > kNoAllocBytes / 160)
        return fail(WSG_ERR_CAPACITY,
                    "wsg_grid_noalloc: %ld measurements cannot fit its fixed %zu-byte scratch "
                    "array (at most %zu); grid the parts into separate grids and sum them, or "
                    "use the plan API",
                    num_points, kNoAllocBytes, kNoAllocBytes / 160);
    if (freq_per_chan > (1l << 20) || polarizations > (1l << 20) ||
        (double)num_points * (double)freq_per_chan * (double)polarizations > 4.0e18)
        return fail(WSG_ERR_ARG,
                    "wsg_grid_noalloc: freq_per_chan %ld x polarizations %ld too large",
                    freq_per_chan, polarizations);

    // scratch layout: counters | bin table | record cells | indices | fracs | values
    const unsigned long long cap = 4ull * (unsigned long long)(num_points > 0 ? num_points : 1);
    const size_t o_bins = up256(sizeof(DevCounters));
    const size_t o_cell = o_bins + up256(bin_buffer_bytes(g.nbins, max_split_items(cap, kDefaultSplit), 1));
    const size_t o_idx = o_cell + up256(cap * sizeof(unsigned));
    const size_t o_frac = o_idx + up256(cap * sizeof(unsigned));
    const size_t o_val = o_frac + up256(cap * sizeof(double2));
    const size_t need = o_val + up256(cap * sizeof(double2));
    if (g.nbins >= (1ll << 31) || need > kNoAllocBytes)
        return fail(WSG_ERR_CAPACITY,
                    "wsg_grid_noalloc: needs %zu bytes of scratch (about 36*%lld bins + 161*%ld "
                    "measurements), above its fixed %zu-byte array; every call overwrites the "
                    "whole grid, so grid the parts into separate grids and sum them, or use "
                    "the plan API",
                    need, g.nbins, num_points, kNoAllocBytes);

    void *base = nullptr;
    int st = scratch_address(&base);
    if (st != WSG_OK) return st;
    unsigned char *s = reinterpret_cast<unsigned char *>(base);
    cudaStream_t cs = reinterpret_cast<cudaStream_t>(stream);

    BinBuffers b;
    b.ctr = reinterpret_cast<DevCounters *>(s);
    unsigned *bins = reinterpret_cast<unsigned *>(s + o_bins);
    bin_buffer_carve(bins, g.nbins, 1, b);
    b.split_size = kDefaultSplit;
    RecBuffers r{};
    r.rec16 = nullptr;
    r.cell = reinterpret_cast<unsigned *>(s + o_cell);
    r.idx = reinterpret_cast<unsigned *>(s + o_idx);
    r.frac = s + o_frac;
    r.val = s + o_val;
    r.capacity = cap;

    const int per_sm = grid_max_ctas_per_sm(WSG_FP64, kNoAllocTile, g.half);
    if (per_sm <= 0)
        return fail(WSG_ERR_UNSUPPORTED, "wsg_grid_noalloc: no FP64 tile kernel for support %d",
                    w_support);

    // the array keeps the previous call's contents: clear counters and bin counts
    cudaError_t e = cudaMemsetAsync(b.ctr, 0, sizeof(DevCounters), cs);
    if (e == cudaSuccess) e = cudaMemsetAsync(b.sub_prim, 0, bin_counter_bytes(g.nbins, b.nsub), cs);
    if (e == cudaSuccess) e = launch_bin_count(g, uu, vv, ww, num_points, b, cs);
    if (e == cudaSuccess) e = launch_bin_scan(g, b, cs);
    if (e == cudaSuccess)
        e = launch_bin_scatter(g, WSG_FP64, uu, vv, ww, vis_real, vis_img, weight, num_points,
                               freq_per_chan, polarizations, b, r, cs);
    if (e == cudaSuccess)
        e = launch_grid(g, WSG_FP64, b, r, grid, nullptr, per_sm * num_sms(), cs);
    if (e != cudaSuccess)
        return fail(WSG_ERR_CUDA, "wsg_grid_noalloc: %s", cudaGetErrorString(e));
    return WSG_OK;
}
