// Host-side state of a plan, shared by the translation units that implement
// the C ABI (capi.cu: single-image plan and drop-in entry points; batch.cu:
// (channel, polarisation) batches, CUDA-graph capture and the autotuner).
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>

#include "wsg_internal.cuh"

namespace wsg {

// Thread-local last error (wstack_gb300_last_error*); set_error returns its
// status so call sites can `return set_error(...)`.
int set_error(int status, const char *fmt, ...);
int clear_error();

#define WSG_CUDA(call)                                                                  \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            return ::wsg::set_error(e_ == cudaErrorMemoryAllocation ? WSG_ERR_NOMEM       \
                                                                    : WSG_ERR_CUDA,       \
                                    "%s: %s (%s:%d)", #call, cudaGetErrorString(e_),       \
                                    __FILE__, __LINE__);                                \
        }                                                                               \
    } while (0)

#define WSG_CUFFT(call)                                                                 \
    do {                                                                                \
        cufftResult r_ = (call);                                                        \
        if (r_ != CUFFT_SUCCESS)                                                        \
            return ::wsg::set_error(WSG_ERR_CUFFT, "%s: cufft status %d (%s:%d)", #call,  \
                                    (int)r_, __FILE__, __LINE__);                       \
    } while (0)

#define WSG_TRY(call)                 \
    do {                              \
        int s_ = (call);              \
        if (s_ != WSG_OK) return s_;  \
    } while (0)

// A device allocation that only grows.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t n)
    {
        if (n <= bytes && p) return cudaSuccess;
        release();
        cudaError_t e = cudaMalloc(&p, n ? n : 16);
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        bytes = n ? n : 16;
        return cudaSuccess;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <typename T> T *as() const { return reinterpret_cast<T *>(p); }
};

// src: n complex values (complex128 when prec == WSG_FP64, else complex64) ->
// re[i] = scale * real, im[i] = scale * imag as float64 (binms.cu).
cudaError_t launch_split_complex(const void *src, int prec, double *re, double *im, long long n,
                                 double scale, cudaStream_t stream);

// d == 2^-k exactly (0 <= k <= 1000).
bool is_pow2_recip(double d, int &k);
// ptr is device (or managed) memory of the current context.
bool device_accessible(const void *ptr);

}  // namespace wsg

struct wsg_plan {
    int nx, ny, planes, support, half, prec;   // planes: w-planes of one job
    int jobs = 1;                              // images in the cube (batch: channels * pols)
    double dx, dw;
    cudaStream_t stream = nullptr;
    int tile = 64, ctas_grid = 0, ctas_degrid = 0, split = wsg::kDefaultSplit, ctas_user = 0;
    long long rows = 0;   // measurements per dump of the inputs' layout (0 = unknown)
    bool walked = false;  // the binned records came from the [dump][baseline] walk
    wsg::GeomParams geom{};

    wsg::DevBuf grid;                          // resident [jobs*P][Ny][Nx] complex
    wsg::DevBuf bins;                          // bin_buffer_bytes(nbins)
    wsg::DevBuf ctr;                           // DevCounters
    wsg::DevBuf rec16, rcell, rfrac, rval, ridx;   // records (FP32C: rec16+idx; FP64: SoA)
    wsg::DevBuf rpos, rvrec;                       // the walk's record map and degridded values
    wsg::DevBuf partials;                      // FP32C partial tiles of split bins
    unsigned long long rec_cap = 0;
    long long n_binned = -1;                   // measurements (batch: visibilities) binned

    // staging for *_host calls
    wsg::DevBuf h_uu, h_vv, h_ww, h_vr, h_vi, h_wt, h_image, h_out;

    bool wc_set = false, ws_ready = false;
    wsg::WcParams wc{};
    wsg::DevBuf sinx, siny, wscreen;

    cufftHandle fft = 0;
    bool fft_ready = false;
    int fft_batch = 0;
    wsg::DevBuf fft_work;

    // asynchronous host pipeline (wsg_image_*_host_async): input uploads on
    // s_in into two slots, the adjoint output's download on s_out, compute
    // and the image's round trip on `stream`
    cudaStream_t s_in = nullptr, s_out = nullptr;
    cudaEvent_t e_in[2] = {nullptr, nullptr};     // slot's inputs on the device
    cudaEvent_t e_free[2] = {nullptr, nullptr};   // slot's inputs consumed
    cudaEvent_t e_adj = nullptr;                  // adjoint output ready
    cudaEvent_t e_vis_down = nullptr;             // adjoint output downloaded
    wsg::DevBuf a_in[2][6], a_img_fwd, a_img_adj, a_vis;
    int a_slot = 0;
    bool a_ready = false;

    // FP64 integer-pipe FFT (power-of-two grids)
    bool fft64 = false;
    bool tw64_ready = false;
    wsg::DevBuf tw64x, tw64y;

    // FP32C fused FFT + w-correction (power-of-two grids)
    bool fused = false;
    bool tw_ready = false;
    bool masks_valid = false;
    wsg::DevBuf twx, twy, masks;

    size_t elem() const { return prec == WSG_FP64 ? sizeof(double2) : sizeof(float2); }
    long long npix() const { return (long long)nx * ny; }
    long long cube_planes() const { return (long long)jobs * planes; }
    wsg::BinBuffers binbufs() const
    {
        wsg::BinBuffers b;
        wsg::bin_buffer_carve(bins.p, geom.nbins, wsg::kSub, b);
        b.ctr = ctr.as<wsg::DevCounters>();
        b.split_size = (unsigned)split;
        return b;
    }
    wsg::RecBuffers recbufs() const
    {
        wsg::RecBuffers r;
        r.rec16 = rec16.as<uint4>();
        r.cell = rcell.as<unsigned>();
        r.frac = rfrac.p;
        r.val = rval.p;
        r.idx = ridx.as<unsigned>();
        r.capacity = rec_cap;
        r.pos = rpos.as<unsigned>();
        r.vrec = rvrec.as<float2>();
        return r;
    }
};

namespace wsg {

WScreen plan_wscreen(const wsg_plan *p);
FftMasks mask_view(const wsg_plan *p);
int ensure_masks(wsg_plan *p);
// Derived geometry, CTA counts and the fused-FFT switch from the plan's
// sizes and tuning; drops the record capacity (bin tables depend on them).
int plan_configure(wsg_plan *p);
// Record, bin-table and partial-tile storage for up to n source points
// (each gives at most 4 records).
int ensure_records(wsg_plan *p, long long n);
int ensure_fused(wsg_plan *p);
int ensure_wscreen(wsg_plan *p);
// Shared bin-table epilogue of every binning: the FFT tile masks.
int finish_binning(wsg_plan *p);

}  // namespace wsg
