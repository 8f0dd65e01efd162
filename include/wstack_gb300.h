/*
 * wstack_gb300.h -- C ABI of the GB300 (sm_103a) w-stacking library
 * (lofar_gb300/libwstack_gb300.so).
 *
 * Two layers:
 *
 * 1. Drop-in symbols with the reference's exact signatures and argument
 *    meaning (nandhanas/LOFAR, w-stacking.h).  A reference build links this
 *    library instead of compiling w-stacking.cu / phase_correction.cu.  All
 *    pointers may be ordinary host memory (the reference's contract) or device
 *    memory; the library detects which.  They return void like the reference;
 *    failures are recorded for wstack_gb300_last_error().
 *
 * 2. A device-resident plan API (wsg_*).  The grid stays in HBM between
 *    gridding, the per-plane FFT and the w-correction (the reference's
 *    MPI/NUMA reduction collapses to this resident grid).  All data pointers
 *    are device pointers unless the name ends in _host.  Every call returns a
 *    wsg_status.  Calls are ordered on the plan's CUDA stream.
 *
 * Layouts (as in the reference):
 *   uu, vv, ww    double[num_points], normalised so that cell = (int)(uu/dx),
 *                 plane = (int)(ww/dw)            (w-stacking.cu:66-71)
 *   vis_real/img  float[num_points*freq_per_chan*polarizations], [m][f][p]
 *   weight        float[num_points*polarizations], [m][p]
 *   grid          [plane][v][u] complex (re, im interleaved); complex128 for
 *                 WSG_FP64, complex64 for WSG_FP32C    (w-stacking.cu:90)
 *   image         [v][u] complex, same precision as the plan's grid
 */
#ifndef WSTACK_GB300_H_
#define WSTACK_GB300_H_

#if defined(__GNUC__)
#define WSG_API __attribute__((visibility("default")))
#else
#define WSG_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* 1. Drop-in entry points (reference signatures)                      */
/* ------------------------------------------------------------------ */

/*
 * Replaces wstack() (declared w-stacking.h:12-29; CUDA body
 * w-stacking.cu:123-220; OpenMP body w-stacking.cu:222-311).
 * Grids num_points measurements into grid[num_w_planes][grid_size_y]
 * [grid_size_x][2] (FP64).  Like the reference's CUDA build the grid is
 * overwritten (the OpenMP build accumulates; the two agree on a zeroed grid,
 * which is what the reference's caller passes, init.c:369).  num_threads is
 * accepted and ignored.  Measurements whose w-plane index is outside
 * [0, num_w_planes) are skipped and counted (the reference writes outside the
 * grid for them).  The precision is FP64 unless wstack_gb300_set_precision()
 * selected WSG_FP32C.
 */
WSG_API void wstack(int num_w_planes, long num_points, long freq_per_chan, long polarizations,
            double *uu, double *vv, double *ww, float *vis_real, float *vis_img,
            float *weight, double dx, double dw, int w_support, int grid_size_x,
            int grid_size_y, double *grid, int num_threads);

/*
 * Replaces phase_correction() (declared w-stacking.h:39-51; definition
 * phase_correction.cu:89-212, PHASE_ON).  gridss is the per-plane FFT output
 * already scaled by 1/(Nx*Ny) (fourier_transform.c:56-57); image_real and
 * image_imag ([yaxis][xaxis] doubles) are overwritten, like the reference's
 * CUDA build.  Pixels with sin^2+sin^2 > 1 come out NaN exactly as in the
 * reference.  num_threads is ignored.
 */
WSG_API void phase_correction(double *gridss, double *image_real, double *image_imag, int xaxis,
                      int yaxis, int num_w_planes, int xaxistot, int yaxistot,
                      double resolution, double wmin, double wmax, int num_threads);

/* Replaces test() (w-stacking.h:34, w-stacking.cu:316-322): returns nnn+1. */
WSG_API int test(int nnn);

/*
 * The per-plane inverse FFT of fftw_data() (fourier_transform.c:25-59), which
 * the reference runs inline with FFTW over globals: for each of nplanes
 * planes, out = (1/(nx*ny)) * sum_k in_k e^{+2 pi i k.x/n} (FFTW_BACKWARD).
 * in and out are [nplanes][ny][nx] complex128 and may alias.  Returns a
 * wsg_status.  A patched fftw_data() calls this instead of fftw_execute().
 */
WSG_API int wstack_fft_planes(const double *in, double *out, int nx, int ny, int nplanes);

/* Status of the last drop-in call made by this thread (wsg_status). */
WSG_API int wstack_gb300_last_error(void);
/* Human-readable message for the last drop-in failure of this thread. */
WSG_API const char *wstack_gb300_last_error_string(void);
/* Precision used by the drop-in wstack()/phase_correction(): WSG_FP64
 * (default) or WSG_FP32C.  Returns the previous value, or -1 if invalid. */
WSG_API int wstack_gb300_set_precision(int precision);
/* Frees the device state that the drop-in calls keep between calls. */
WSG_API void wstack_gb300_release(void);

/* ------------------------------------------------------------------ */
/* 2. Device-resident plan API                                         */
/* ------------------------------------------------------------------ */

typedef enum {
    WSG_OK = 0,
    WSG_ERR_ARG = 1,        /* invalid argument (size, pointer, support)   */
    WSG_ERR_CUDA = 2,       /* a CUDA runtime call failed                  */
    WSG_ERR_CUFFT = 3,      /* a cuFFT call failed                         */
    WSG_ERR_NOMEM = 4,      /* device allocation failed                    */
    WSG_ERR_STATE = 5,      /* call out of order (e.g. adjoint before bin) */
    WSG_ERR_CAPACITY = 6,   /* more points than the reserved capacity      */
    WSG_ERR_UNSUPPORTED = 7,/* configuration outside the kernels' limits   */
    WSG_ERR_IO = 8          /* a file could not be opened, read or written
                               (wstack_gb300_io.h)                         */
} wsg_status;

typedef enum {
    WSG_FP64 = 0,   /* FP64 grid, planes and image, within 1e-12 (grid, FFT) and
                       1e-11 (image) of the reference's FP64 arithmetic; the
                       taps, the FFT of power-of-two grids and the w-correction
                       run in 64-bit fixed point inside */
    WSG_FP32C = 1   /* complex64 grid; FP64-exact coordinates and phase
                       argument.  Each tile is summed in int32 fixed point at
                       a per-work-item scale (exact, order-independent sums;
                       one rounding per tap); the partial tiles of a bin cut
                       into several work items are combined with TwoSum */
} wsg_precision;

typedef struct wsg_plan wsg_plan;

typedef struct {
    long long points_in;        /* measurements passed to the last wsg_bin   */
    long long records;          /* (measurement, tile) records written       */
    long long dropped_plane;    /* skipped: w-plane index outside [0, P)      */
    long long dropped_window;   /* skipped: support window entirely off-grid  */
    int bins;                   /* number of (plane, tile) bins              */
    int tile;                   /* tile edge in cells                        */
    int max_bin_records;        /* largest bin                               */
    int ctas;                   /* persistent CTAs launched per kernel       */
} wsg_stats;

/*
 * Creates a plan for a [num_w_planes][grid_size_y][grid_size_x] grid.
 * dx, dw: as passed to wstack() (dx = 1/Nx, dw = 1/P in the reference,
 * init.c:16-17).  w_support: kernel support in cells (odd, 1..15).
 * stream: a cudaStream_t (NULL = the legacy default stream).
 */
WSG_API int wsg_plan_create(wsg_plan **plan, int grid_size_x, int grid_size_y, int num_w_planes,
                    int w_support, double dx, double dw, int precision, void *stream);
WSG_API int wsg_plan_destroy(wsg_plan *plan);
WSG_API int wsg_plan_set_stream(wsg_plan *plan, void *stream);
/* Tile edge (32 or 64 cells), persistent CTA count and split size (records
 * per work item of a bin cut into several; >= 512) -- 0 keeps the current
 * value (ctas 0 = automatic). */
WSG_API int wsg_plan_set_tuning(wsg_plan *plan, int tile, int ctas, int chunk);
/* Layout of the measurements: [dump][baseline] order with rows_per_dump rows
 * per dump, as the reference's measurement sets are written (meta.txt's
 * `baselines`, init.c:293).  An FP32C plan's binning then walks each
 * baseline's consecutive dumps together, so records that share a bin merge
 * their cursor atomics and are written contiguously, and the gridder sums
 * the records of each track as stored instead of sorting them by cell.  A
 * speed hint: the grid is bit-identical when no bin is split into chunks and
 * otherwise differs only by the FP32C rounding of the chunks' partial tiles;
 * a wrong count only changes the speed.  FP64 plans keep the index-order
 * walk; 0 (the default) walks in index order. */
WSG_API int wsg_plan_set_layout(wsg_plan *plan, long rows_per_dump);
/* Reserves device memory for up to max_points measurements so that later
 * calls allocate nothing (required before CUDA-graph capture). */
WSG_API int wsg_plan_reserve(wsg_plan *plan, long max_points);
/* W-correction geometry (phase_correction's resolution, wmin, wmax). */
WSG_API int wsg_plan_set_wcorrection(wsg_plan *plan, double resolution, double wmin, double wmax);
WSG_API int wsg_plan_get_stats(wsg_plan *plan, wsg_stats *stats);
/* Bytes of device memory the plan holds. */
WSG_API long long wsg_plan_device_bytes(wsg_plan *plan);

/* Sort measurements into (w-plane, tile) bins and fold vis*weight over
 * frequency and polarisation (w-stacking.cu:98-112).  Device pointers. */
WSG_API int wsg_bin(wsg_plan *plan, long num_points, long freq_per_chan, long polarizations,
            const double *uu, const double *vv, const double *ww, const float *vis_real,
            const float *vis_img, const float *weight);
/* Grid the binned measurements; grid is overwritten (every cell written). */
WSG_API int wsg_grid(wsg_plan *plan, void *grid);
/* As wsg_grid, but only the tiles that hold measurements are written; the
 * other tiles of `grid` keep their contents.  Those tiles are exactly the ones
 * wsg_fft_wcorrect reads with pruning on a fused FP32C plan, so this pair is
 * the staged form of wsg_image_forward.  On other plans it equals wsg_grid. */
WSG_API int wsg_grid_occupied(wsg_plan *plan, void *grid);
/* Unnormalised per-plane 2D FFT in place; sign +1 = exponent +i
 * (FFTW_BACKWARD, the forward imaging direction), -1 = exponent -i. */
WSG_API int wsg_fft(wsg_plan *plan, void *grid, int sign);
/* image = sum_w planes_w * e^{i phi_w} * dwnorm * sqrt(1-r^2) * scale
 * (phase_correction.cu:36-80); scale = 1/(Nx*Ny) folds in the FFT norm. */
WSG_API int wsg_wcorrect(wsg_plan *plan, const void *planes, void *image, double scale);
/* Adjoint of wsg_wcorrect: planes_w = conj(e^{i phi_w}) * dwnorm *
 * sqrt(1-r^2) * scale * image. */
WSG_API int wsg_wcorrect_adjoint(wsg_plan *plan, const void *image, void *planes, double scale);
/* Adjoint of wsg_grid for the measurements of the last wsg_bin:
 * out[m] = sum over m's support window of kernel weight * grid (complex,
 * plan precision), [num_points] complex, overwritten. */
WSG_API int wsg_degrid(wsg_plan *plan, const void *grid, void *out);

/* Per-plane inverse FFT (exponent +i) of `grid` followed by the w-correction
 * into `image` (scale 1/(Nx*Ny) included); `grid` is overwritten.  With
 * prune = 1 the grid must be the one gridded from the last wsg_bin: tiles
 * without measurements are taken as zero and never read, and for FP32C
 * power-of-two grids the two steps run fused (the transformed planes never
 * reach memory).  prune = 0 transforms every cell. */
WSG_API int wsg_fft_wcorrect(wsg_plan *plan, void *grid, void *image, int prune);
/* Adjoint of wsg_fft_wcorrect: w-correction adjoint, then per-plane FFT
 * (exponent -i), into `grid`.  With prune = 1 only the cells that wsg_degrid
 * reads for the last wsg_bin are guaranteed to be written. */
WSG_API int wsg_wcorrect_adjoint_fft(wsg_plan *plan, const void *image, void *grid, int prune);

/* Forward imaging: bin + grid + FFT + w-correction into image
 * ([Ny][Nx] complex, plan precision).  Uses the plan's resident grid. */
WSG_API int wsg_image_forward(wsg_plan *plan, long num_points, long freq_per_chan, long polarizations,
                      const double *uu, const double *vv, const double *ww,
                      const float *vis_real, const float *vis_img, const float *weight,
                      void *image);
/* Adjoint imaging for the measurements of the last wsg_image_forward/wsg_bin:
 * out[m] (complex, plan precision) = (A^H image)[m]. */
WSG_API int wsg_image_adjoint(wsg_plan *plan, const void *image, void *out);

/* Same as wsg_image_forward / wsg_image_adjoint with HOST buffers; the copies
 * to and from the device are part of the call, which returns when the host
 * outputs are written. */
WSG_API int wsg_image_forward_host(wsg_plan *plan, long num_points, long freq_per_chan,
                           long polarizations, const double *uu, const double *vv,
                           const double *ww, const float *vis_real, const float *vis_img,
                           const float *weight, void *image);
WSG_API int wsg_image_adjoint_host(wsg_plan *plan, const void *image, void *out);

/* Asynchronous forms of the two calls above, for a stream of imaging steps:
 * they return at once, and wsg_plan_synchronize waits for everything
 * submitted.  The inputs of a forward call are uploaded on a copy stream into
 * one of two device slots while the previous call computes; outputs are
 * downloaded on a second copy stream while the next call computes.  Host
 * buffers must stay valid and unchanged (outputs: unread) until
 * wsg_plan_synchronize returns; pinned host memory lets the copies overlap.
 * The image travels on the compute stream, so an adjoint call may take the
 * host image its forward call writes: on FP32C power-of-two plans with a
 * pinned host image the row kernels write and read the image rows in host
 * memory directly; otherwise the image is copied (by a copy kernel when the
 * host image is pinned and 16-byte aligned). */
WSG_API int wsg_image_forward_host_async(wsg_plan *plan, long num_points, long freq_per_chan,
                                         long polarizations, const double *uu, const double *vv,
                                         const double *ww, const float *vis_real,
                                         const float *vis_img, const float *weight, void *image);
WSG_API int wsg_image_adjoint_host_async(wsg_plan *plan, const void *image, void *out);
WSG_API int wsg_plan_synchronize(wsg_plan *plan);

/* Resident cube buffer of the plan ([P][Ny][Nx] complex): the grid after
 * wsg_grid; wsg_image_forward uses it as its work buffer (on fused FP32C plans
 * the tiles without measurements are left unwritten there). */
WSG_API void *wsg_plan_grid(wsg_plan *plan);

/* Times candidate settings of the tile edge, split size and persistent CTA
 * count on these inputs (wsg_image_forward, `iters` timed calls each after
 * one warm-up, searched one parameter at a time) and keeps the fastest.
 * best (optional) receives it; tried (optional, max_tried entries) every
 * candidate timed, *n_tried their number. */
typedef struct {
    int tile, ctas, chunk;   /* as wsg_plan_set_tuning (ctas 0 = automatic) */
    float ms;                /* mean time of one timed call                 */
} wsg_tuning;
WSG_API int wsg_plan_autotune(wsg_plan *plan, long num_points, long freq_per_chan,
                              long polarizations, const double *uu, const double *vv,
                              const double *ww, const float *vis_real, const float *vis_img,
                              const float *weight, void *image, int iters, wsg_tuning *best,
                              wsg_tuning *tried, int max_tried, int *n_tried);

/* ------------------------------------------------------------------ */
/* 3. (channel, polarisation) batches                                   */
/* ------------------------------------------------------------------ */
/*
 * Many channels and polarisations imaged at once; the reference has no such
 * entry point (it folds all freq_per_chan*polarizations into one grid,
 * w-stacking.cu:98-112).  Each (channel, polarisation) pair is one job: the
 * grid, FFT and w-corrected image that wstack() + fftw_data +
 * phase_correction() give for that channel and polarisation alone
 * (freq_per_chan = polarizations = 1).  Jobs share the grid geometry, dx,
 * dw, the support and the w-correction geometry; each channel has its own
 * uvw and measurement count (after flagging).  Layouts:
 *   grids   [channel][pol][P][Ny][Nx] complex64 (job = channel*pols + pol)
 *   images  [channel][pol][Ny][Nx] complex64
 *   vis_out [sum over channels of num_points*pols] complex64, channel after
 *           channel, each [num_points][pols] (wsg_batch_vis_offset)
 * All jobs are binned in one pass and gridded in one persistent launch over a
 * (job, plane, tile) work queue; the whole forward can be replayed as one
 * CUDA graph.  WSG_FP32C only, power-of-two grid edges 256..8192.
 */
typedef struct wsg_batch wsg_batch;
typedef struct {
    long num_points;                   /* measurements of this channel (>= 0) */
    const double *uu, *vv, *ww;        /* [num_points], device               */
    const float *vis_real, *vis_img;   /* [num_points][pols], device          */
    const float *weight;               /* [num_points][pols], device          */
} wsg_channel;

WSG_API int wsg_batch_create(wsg_batch **batch, int grid_size_x, int grid_size_y,
                             int num_w_planes, int w_support, double dx, double dw,
                             int num_channels, int polarizations, void *stream);
WSG_API int wsg_batch_destroy(wsg_batch *batch);
WSG_API int wsg_batch_set_stream(wsg_batch *batch, void *stream);
WSG_API int wsg_batch_set_wcorrection(wsg_batch *batch, double resolution, double wmin,
                                      double wmax);
WSG_API int wsg_batch_set_tuning(wsg_batch *batch, int tile, int ctas, int chunk);
/* Binds the channels' input buffers (num_channels entries; the table is
 * copied, the buffers are not: they must stay allocated while bound, and
 * their contents may change between forwards) and reserves device memory. */
WSG_API int wsg_batch_bind(wsg_batch *batch, const wsg_channel *channels);
/* Forward of every job into images (overwritten).  use_graph = 1 captures
 * bin + grid + FFT + w-correction as one CUDA graph on first use and replays
 * it while the binding, tuning, w-correction and images pointer stay the same. */
WSG_API int wsg_batch_forward(wsg_batch *batch, void *images, int use_graph);
/* Adjoint of the forward for the bound measurements (after a forward):
 * vis_out = A^H images, per visibility as wsg_image_adjoint. */
WSG_API int wsg_batch_adjoint(wsg_batch *batch, const void *images, void *vis_out);
/* As wsg_plan_autotune, timing wsg_batch_forward on the bound inputs. */
WSG_API int wsg_batch_autotune(wsg_batch *batch, void *images, int iters, wsg_tuning *best,
                               wsg_tuning *tried, int max_tried, int *n_tried);
/* First visibility of `channel` in vis_out; channel = num_channels gives the
 * total (-1 before wsg_batch_bind). */
WSG_API long long wsg_batch_vis_offset(wsg_batch *batch, int channel);
/* Resident cube buffer of the batch ([channel][pol][P][Ny][Nx] complex64): the
 * forward's work buffer (column-transformed planes of the occupied tiles). */
WSG_API void *wsg_batch_grids(wsg_batch *batch);
WSG_API int wsg_batch_get_stats(wsg_batch *batch, wsg_stats *stats);
WSG_API long long wsg_batch_device_bytes(wsg_batch *batch);

/*
 * FP64 gridding that allocates no device memory.  It has no counterpart in
 * the reference; it is for callers that cannot call cudaMalloc when they grid
 * (a real-time pipeline that reserves all device memory up front, a host
 * application that owns the device memory and lends a plug-in only its own
 * buffers, code that must not synchronise the device with an allocation).
 * Arguments and results are those of wstack() (FP64, grid overwritten), but
 * every pointer must be device memory and the call is asynchronous on
 * `stream` (a cudaStream_t, NULL = legacy default stream).
 * Its scratch is a fixed 64 MiB static device array per GPU, held until the
 * process exits; a call needing more than
 *     2560 + 36*nbins + 16*ceil(nbins/256) + 161*num_points bytes
 *     (alignment included),
 *     nbins = num_w_planes*ceil(grid_size_y/64)*ceil(grid_size_x/64),
 * fails with WSG_ERR_CAPACITY (about 387,000 measurements on a 4096x4096x32
 * grid).  Each call overwrites the whole grid: a larger set is gridded part by
 * part into separate grids that the caller sums.  All calls share that array: calls whose GPU work may overlap race
 * and must be serialised by the caller.  The first call on a device looks up
 * the array's device address and may load the device code: make it before
 * any stream capture.
 */
WSG_API int wsg_grid_noalloc(int num_w_planes, long num_points, long freq_per_chan,
                             long polarizations, const double *uu, const double *vv,
                             const double *ww, const float *vis_real, const float *vis_img,
                             const float *weight, double dx, double dw, int w_support,
                             int grid_size_x, int grid_size_y, double *grid, void *stream);

/* ------------------------------------------------------------------ */
/* 4. v-slab sectoring (the reference's multi-rank decomposition)      */
/* ------------------------------------------------------------------ */

/*
 * A rank of the reference grids its rows slab by slab: nsectors v-slabs of
 * yaxis grid rows each (nsectors = ranks, yaxis = grid_size_y / nsectors,
 * init.c:24-33).  Row i belongs to slab b = (int)(vv[i]*nsectors), and also
 * to slab b+1 (b-1) when its distance to that slab's edge is below
 * w_supporth = ((w_support-1)/2)*dx (init.c:18), computed exactly as
 * gridding.c:45-55 does.  Each slab's list holds its rows in increasing
 * order; histo_send has nsectors+1 entries (the last slab, b == nsectors, is
 * never gridded).  Rows whose slab index would fall outside [0, nsectors]
 * (the reference indexes histo_send out of bounds for them) fail the call with
 * WSG_ERR_ARG.  Limits: nsectors <= WSG_MAX_SECTORS, n <= 1e9.
 */
#define WSG_MAX_SECTORS 1023

/* Slab list offsets only: offsets[s] = first entry of slab s, offsets[nsectors+1]
   = total entries (histo_send[s] = offsets[s+1] - offsets[s]).  vv and offsets
   are device memory; returns after the work on `stream` has finished. */
WSG_API int wsg_sector_count(const double *vv, long n, long nsectors, int yaxis, double dx,
                             double w_supporth, long *offsets, void *stream);
/* Offsets and the concatenated lists: index[offsets[s] .. offsets[s+1]) is
   sectorarray[s] (gridding.c:58-77).  Device memory; capacity = entries of
   index (at most 3*n are needed), WSG_ERR_CAPACITY when too small. */
WSG_API int wsg_sector_lists(const double *vv, long n, long nsectors, int yaxis, double dx,
                             double w_supporth, long *offsets, long *index, long capacity,
                             void *stream);
/* The composition step of gridding_data() (gridding.c:193-211) for slab
   isector on the device: list = that slab's nsec entries of index; writes
   the slab's rows in reverse list order with vvs = vv - isector*(dx*yaxis),
   ready for wstack() on a yaxis-row grid.  Asynchronous on `stream`. */
WSG_API int wsg_sector_gather(const long *list, long nsec, long isector, int yaxis, double dx,
                              long freq_per_chan, long polarisations, const double *uu,
                              const double *vv, const double *ww, const float *weights,
                              const float *vis_real, const float *vis_img, double *uus,
                              double *vvs, double *wws, float *weightss, float *visreals,
                              float *visimgs, void *stream);
/* Drop-in for initialize_array() (gridding.c:35-86): vv in host or device
   memory; fills histo_send[nsectors+1] and sectorarray[nsectors+1] in host
   memory, each list allocated with malloc() (free() it), on the GPU. */
WSG_API int wsg_initialize_array(const double *vv, long n, long nsectors, int yaxis, double dx,
                                 double w_supporth, long *histo_send, long **sectorarray);

#ifdef __cplusplus
}
#endif
#endif /* WSTACK_GB300_H_ */
