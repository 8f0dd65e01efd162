// Internal declarations shared by the translation units of libwstack_gb300.so.
//
// Data layout in HBM (one plan: J jobs of P planes of Ny x Nx cells, tile
// edge T; a single image is J = 1, a (channel, polarisation) batch has one
// job per pair, stacked along the plane axis):
//   grid      [J*P][Ny][Nx] complex (float2 for FP32C, double2 for FP64),
//             per job the reference's [w][v][u][re,im] layout
//             (w-stacking.cu:90); cube plane = job*P + w
//   bins      (cube plane, tile-row, tile-col) in row-major order,
//             bin = (plane*ntv + tv)*ntu + tu; per-bin record counts, offsets
//   records   structure-of-arrays, grouped by bin, primaries first:
//             rec_cell  u32   (cu + 32768) | (cv + 32768) << 16, the
//                             measurement's cell relative to the tile origin
//             rec_frac  float2/double2   pos - cell (exact in FP64)
//             rec_val   float2/double2   sum_{f,p} weight*vis (the fold of
//                             w-stacking.cu:98-112)
//             rec_idx   u32   original measurement index (batch: index
//                             of the visibility in the concatenated
//                             [channel][measurement][pol] layout)
//   A measurement whose support window touches k tiles has k records
//   (halo duplication, k <= 4); the record in the tile holding its own
//   (clamped) cell is its primary.
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>

#include "wstack_gb300.h"

namespace wsg {

// The reference's pi (w-stacking.h:6), kept for bit-level parity.
constexpr double kRefPi = 3.14159265359;

constexpr int kMaxHalf = 7;          // support up to 15 cells
constexpr int kThreads = 256;        // threads per CTA for tile kernels
constexpr int kScanThreads = 256;    // bin-size scan: threads per CTA
constexpr int kScanPerBlock = 256;   // bin-size scan: bins per CTA (one a thread)
constexpr int kStage = 512;          // records staged in shared memory per pass
constexpr int kDefaultSplit = 4096;      // records per work item of a split bin (FP64)
constexpr int kDefaultSplitF32 = 16384;  // the same for FP32C plans

struct DevCounters {
    unsigned long long records;
    unsigned long long dropped_plane;
    unsigned long long dropped_window;
    unsigned int max_bin;
    unsigned int work_grid;
    unsigned int work_degrid;
    unsigned int error;
    unsigned int nsplit_items;   // work items of split bins (the list `split`)
    unsigned int nslots;         // partial tiles needed by split bins
    unsigned int nwork;          // occupied bins that are not split (the list `work`)
};

// Geometry of the coordinate step (w-stacking.cu:66-77) and the tiling.
struct GeomParams {
    int nx, ny, planes, half, tile, ntu, ntv;   // planes: all jobs' planes
    int tile_shift;                             // tile == 1 << tile_shift
    int wplanes;                                // w-planes of one job
    int u_pow2, w_pow2;   // dx (dw) is an exact power of two: 1/dx == 2^ku
    int ku, kw;
    double dx, dw;
    long long nbins;
    long long rows;       // measurements per dump of a [dump][baseline] layout, 0 = unknown
};

// Work decomposition.  A bin with more than `split` records is cut into
// ceil(n/split) work items of at most `split` records; they are listed in
// `split` (entry = bin | chunk << 32) and processed first.  Every other bin is
// one work item; the occupied ones among them are also listed in `work` (in
// no particular order), for kernels that skip empty bins.
//
// Counting uses nsub sub-counters per bin (nsub = kSub for plans, 1 for the
// no-allocation entry point): a record uses sub-counter (cu mod 4) + 4 (cv mod
// 4) of its measurement's cell (cu, cv), in both passes.  The atomics of a
// crowded bin are then spread over nsub addresses, and all records of one cell
// stay in one sub-range, which keeps each cell's records together in the FP32C
// gridder's sorted stages.  After the scan,
// sub_prim[s][b] / sub_dup[s][b] hold the first record position of sub-range s
// of bin b's primaries / duplicates and the scatter advances them as cursors.
constexpr int kSub = 16;
struct BinBuffers {
    unsigned *sub_prim, *sub_dup;            // [nsub][nbins]
    unsigned *off, *nprim, *ntotal, *is_split, *slot, *done, *work;   // [nbins]
    unsigned long long *part;                // 2 * scan_blocks(nbins) entries
    unsigned long long *split;               // split-item list
    DevCounters *ctr;
    unsigned split_size;
    unsigned nsub;
};

// Records.  FP32C: rec16 (16 B, see k_bin_scatter) + idx.  FP64: cell, frac,
// val (structure of arrays) + idx.
struct RecBuffers {
    uint4 *rec16;
    unsigned *cell;
    void *frac;   // double2
    void *val;    // double2
    unsigned *idx;
    unsigned long long capacity;
    // the [dump][baseline] walk (FP32C): pos[m] = the record of measurement
    // m's primary (0xFFFFFFFF: none); vrec[p] = the degridded value of
    // primary record p, gathered to measurement order afterwards
    unsigned *pos;
    float2 *vrec;
};

// Bytes of BinBuffers storage for nbins bins with nsub sub-counters and at
// most `items` split items (u32 arrays, then the scan partials, then the
// split list; 256-byte aligned): (2*nsub + 7)*4 bytes per bin, 16 per 256
// bins and 8 per split item.
long long scan_blocks(long long nbins);
inline size_t bin_u32_per_bin(unsigned nsub) { return 2 * (size_t)nsub + 7; }
inline size_t bin_buffer_bytes(long long nbins, unsigned long long items, unsigned nsub)
{
    const size_t a = (bin_u32_per_bin(nsub) * nbins * sizeof(unsigned) + 255) & ~(size_t)255;
    const size_t b = ((size_t)scan_blocks(nbins) * 16 + 255) & ~(size_t)255;
    return a + b + (size_t)items * 8;
}
inline void bin_buffer_carve(void *base, long long nbins, unsigned nsub, BinBuffers &b)
{
    unsigned *u = reinterpret_cast<unsigned *>(base);
    b.nsub = nsub;
    b.sub_prim = u;
    b.sub_dup = u + (size_t)nsub * nbins;
    unsigned *v = u + 2 * (size_t)nsub * nbins;
    b.off = v;
    b.nprim = v + nbins;
    b.ntotal = v + 2 * nbins;
    b.is_split = v + 3 * nbins;
    b.slot = v + 4 * nbins;
    b.done = v + 5 * nbins;
    b.work = v + 6 * nbins;
    unsigned char *c = reinterpret_cast<unsigned char *>(base);
    const size_t a = (bin_u32_per_bin(nsub) * nbins * sizeof(unsigned) + 255) & ~(size_t)255;
    const size_t p = ((size_t)scan_blocks(nbins) * 16 + 255) & ~(size_t)255;
    b.part = reinterpret_cast<unsigned long long *>(c + a);
    b.split = reinterpret_cast<unsigned long long *>(c + a + p);
}
// Bytes of the sub-counters (cleared before each binning).
inline size_t bin_counter_bytes(long long nbins, unsigned nsub)
{
    return (size_t)2 * nsub * nbins * sizeof(unsigned);
}
// Upper bounds for `records` records cut into items of `split`: split items
// and partial-tile slots.
inline unsigned long long max_split_items(unsigned long long records, unsigned split)
{
    return 2 * (records / split) + 1;
}
inline unsigned long long max_slots(unsigned long long records, unsigned split)
{
    return records / split + 1;
}

// Pixel-geometry table of the FP32C w-correction (per pixel, planar):
// the phase in cycles for plane w is a + w*b (mod 1), a and b as
// float-float pairs reduced to [-0.5, 0.5]; amp = dwnorm*sqrt(1-r^2).
// FP32C w-screen, per pixel: the phase of plane w in cycles, a + w*b, with a
// and b reduced modulo 1 and stored as Q32 fractions of a cycle (aq, bq), so
// that (aq + w*bq) mod 2^32 is the plane's cycle fraction exactly, by integer
// wrap-around; amp = dwnorm * sqrt(1 - r2) (NaN outside the unit circle).
struct WScreen {
    unsigned *aq, *bq;
    float *amp;
    double *sinx, *siny;
};

// Phase angle of plane w in radians, in [-pi, pi): the Q32 cycle fraction
// (aq + w*bq) mod 2^32 read as a signed fraction of a cycle.
__device__ __forceinline__ float wscreen_angle(unsigned aq, unsigned bq, unsigned w)
{
    const int c = (int)(aq + w * bq);
    return (float)c * 1.46291807926715968e-9f;   // 2 pi / 2^32
}

// ---- launchers (bin.cu) ----
// The single-image binning walks [dump][baseline] tiles (g.rows rows per
// dump) instead of index order.
inline bool rows_walk(const GeomParams &g, long long n) { return g.rows > 1 && g.rows < n; }

cudaError_t launch_bin_count(const GeomParams &g, const double *uu, const double *vv,
                             const double *ww, long long n, const BinBuffers &b,
                             cudaStream_t s);
cudaError_t launch_bin_scan(const GeomParams &g, const BinBuffers &b, cudaStream_t s);
// out[m] = vrec[pos[m]] (zero where pos[m] is 0xFFFFFFFF) along the walk.
cudaError_t launch_walk_gather(const GeomParams &g, long long n, const unsigned *pos,
                               const float2 *vrec, float2 *out, cudaStream_t s);
cudaError_t launch_bin_scatter(const GeomParams &g, int prec, const double *uu,
                               const double *vv, const double *ww, const float *vr,
                               const float *vi, const float *wt, long long n, long long nf,
                               long long np, const BinBuffers &b, const RecBuffers &r,
                               cudaStream_t s);

// One channel of a (channel, polarisation) batch: its measurements are
// global indices [m0, m0 + n) of the concatenated batch; its visibilities
// start at vis0 in the concatenated [channel][measurement][pol] layout.
struct ChanDesc {
    const double *uu, *vv, *ww;
    const float *vr, *vi, *wt;   // [n][pols]
    long long m0, n;
    unsigned long long vis0;
};
constexpr int kMaxChannels = 2048;
struct ChanTable {
    const ChanDesc *ch;           // device array [nch]
    const long long *m0;          // device array [nch]: ch[c].m0
    int nch, pols;
    long long ntot;               // sum of n
};
cudaError_t launch_bin_count_batch(const GeomParams &g, const ChanTable &t, const BinBuffers &b,
                                   cudaStream_t s);
cudaError_t launch_bin_scatter_batch(const GeomParams &g, int prec, const ChanTable &t,
                                     const BinBuffers &b, const RecBuffers &r, cudaStream_t s);

// ---- launchers (grid.cu) ----
// partials: FP32C partial tiles of split bins (max_slots * tile^2 float2),
// unused for FP64.
// sparse: FP32C only; grids the occupied bins alone and leaves the tiles of
// empty bins unwritten (for the fused imaging path, whose column transforms
// read occupied tiles only).  Otherwise every tile of the grid is written.
// tracks: FP32C only; the records were binned by the [dump][baseline] walk
// (rows_walk), so each bin holds tracks in dump order and the stages are
// used as stored instead of sorted by cell (the grid is the same).
cudaError_t launch_grid(const GeomParams &g, int prec, const BinBuffers &b,
                        const RecBuffers &r, void *grid, void *partials, int ctas,
                        cudaStream_t s, bool sparse = false, bool tracks = false);
int grid_max_ctas_per_sm(int prec, int tile, int half);

// ---- launchers (degrid.cu) ----
// walked: the records came from the [dump][baseline] walk (FP32C); the
// values are written in record order (r.vrec) and gathered to measurement
// order along the walk (r.pos), every output written.  Otherwise each value
// is stored at its measurement's index (r.idx) after a memset of `out`.
cudaError_t launch_degrid(const GeomParams &g, int prec, const BinBuffers &b,
                          const RecBuffers &r, const void *grid, void *out, long long n,
                          int ctas, cudaStream_t s, bool walked = false);
int degrid_max_ctas_per_sm(int prec, int tile, int half);

// ---- launchers (wcorrect.cu) ----
struct WcParams {
    int xaxis, yaxis, planes, xaxistot, yaxistot;
    double resolution, wmin, wmax;
    int phase_on;
};
cudaError_t launch_wscreen_tables(const WcParams &p, double *sinx, double *siny,
                                  cudaStream_t s);
cudaError_t launch_wscreen_build(const WcParams &p, const WScreen &ws, cudaStream_t s);
cudaError_t launch_wcorrect_f32c(const WcParams &p, const WScreen &ws, const float2 *planes,
                                 float2 *image, double scale, cudaStream_t s);
cudaError_t launch_wcorrect_adj_f32c(const WcParams &p, const WScreen &ws, const float2 *image,
                                     float2 *planes, double scale, cudaStream_t s);
cudaError_t launch_wcorrect_f64(const WcParams &p, const double *sinx, const double *siny,
                                const double2 *planes, double2 *image, double *image_re,
                                double *image_im, double scale, cudaStream_t s);
cudaError_t launch_wcorrect_adj_f64(const WcParams &p, const double *sinx, const double *siny,
                                    const double2 *image, double2 *planes, double scale,
                                    cudaStream_t s);
cudaError_t launch_scale_f64(double2 *x, long long n, double scale, cudaStream_t s);

// ---- launchers (fft.cu): FP32C per-plane FFTs fused with the w-correction ----
// Tile masks derived from the bin table (u8 arrays).
struct FftMasks {
    unsigned char *occ_tile;    // [P][ntv][ntu] tile holds a measurement (forward input)
    unsigned char *occ_col;     // [P][ntu]      tile column holds one
    unsigned char *plane_occ;   // [P]
    unsigned char *need_tile;   // [P][ntv][ntu] tile read by the degridder (3x3 dilation)
    unsigned char *need_col;    // [P][ntu]
    unsigned char *plane_need;  // [P]
};
bool fft_fused_supported(int nx, int ny, int tile);

// FP64 per-plane 2D FFT on the integer pipe (fft64.cu): power-of-two edges
// 256..8192, up to 65535 planes; twiddles e^{+-2 pi i k / n} in Q62, 2n int4
// entries per axis.  In place, unnormalised, times the exact power of two 2^post.
bool fft64_supported(int nx, int ny, long long planes);
cudaError_t build_twiddles64(int4 *tw, int n, cudaStream_t stream);
// masks (optional, the plan's tile masks of its last binning; tile = 2^tsh;
// used by the adjoint, sign -1): the row pass runs first, then the column
// pass transforms only the tile columns the degridder reads and writes only
// their needed tiles (the other cells of the output are left unspecified).
cudaError_t launch_fft64(double2 *data, int nx, int ny, int planes, int sign,
                         const int4 *twx, const int4 *twy, int post, cudaStream_t stream,
                         const FftMasks *masks = nullptr, int tsh = 0);
cudaError_t launch_twiddles(float2 *tw, int n, cudaStream_t s);
cudaError_t launch_fft_masks(const GeomParams &g, const BinBuffers &b, const FftMasks &m,
                             cudaStream_t s);
cudaError_t launch_image_fwd_fused(const GeomParams &g, float2 *grid, float2 *image,
                                   const float2 *twx, const float2 *twy, const WScreen &ws,
                                   const FftMasks &m, bool phase, double scale, cudaStream_t s);
cudaError_t launch_image_adj_fused(const GeomParams &g, const float2 *image, float2 *grid,
                                   const float2 *twx, const float2 *twy, const WScreen &ws,
                                   const FftMasks &m, bool phase, double scale, cudaStream_t s);
cudaError_t launch_fft2d_plain(const GeomParams &g, float2 *grid, const float2 *twx,
                               const float2 *twy, int sign, cudaStream_t s);
// A column-FFT CTA gave up waiting for its TMA-staged strip (process-wide,
// sticky): its columns were not transformed.
bool fft_tma_timed_out();
// The same for a degridding CTA and its TMA-staged tile.
bool degrid_tma_timed_out();
cudaError_t launch_f64_to_f32(const double2 *in, float2 *out, long long n, cudaStream_t s);
cudaError_t launch_f32_to_f64(const float2 *in, double2 *out, long long n, cudaStream_t s);

int num_sms();
int report_status(int status, const char *msg);

// 2^x from the hardware approximation (PTX ex2.approx: relative error about
// 2^-22); used for the FP32C kernel weights, with x <= 0.
__device__ __forceinline__ float fast_exp2(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

}  // namespace wsg
