// Gridding kernels.  Persistent CTAs take work items from a queue: first the
// items of split bins (bins with more than `split` records, cut into items of
// at most `split` records), then every other (plane, tile) bin.  Each item is
// accumulated in shared memory and its T x T interior written to HBM once with
// coalesced stores.  Every grid cell belongs to exactly one tile, and
// measurements near a tile edge were duplicated into the neighbouring bins by
// the binning pass, so tiles are written with plain stores: no global
// atomics, no memset of the grid.  This replaces convolve_g
// (w-stacking.cu:35-118), whose FP64 global atomics scatter every tap to HBM.
//
// FP32C (k_grid_f32c): see the kernel's comment for the lane layout and the
// fixed-point tile accumulator.  The accumulator's sums are exact integers and
// each item's scale comes from an order-independent bound, so a bin that is
// not split grids to the same bits whatever the order of its records.  An
// item of a split bin writes its partial
// tile (chunk 0 straight into the grid, the others into partial-tile slots);
// the CTA that finishes a split bin's last item combines the bin's partials
// cell by cell with TwoSum (hi + lo), in chunk order, so the error of a cell
// does not grow with the number of measurements that hit it.
//
// FP64 (k_grid_f64): the same work items and partial-tile combination (in
// FP64, chunk order).  The FP64 pipe issues at 1/64 of the integer rate, so
// the weights are factorised (taps64.cuh: four exponentials per record, one
// warp-wide pass for eight records) and the taps are summed as 64-bit
// integers at an order-independent power-of-two scale per item (fixed64.cuh);
// an item above kFixedMaxRecords records, or holding a NaN or an infinity,
// sums in FP64 shared-memory atomics.  A group of G lanes takes a record, lane
// k scattering row k of the window; the tile's pitch T + 2K + 1 puts the rows
// of one window in distinct banks.
#include <cuda_runtime.h>

#include "fixed64.cuh"
#include "taps64.cuh"
#include "wsg_internal.cuh"

namespace wsg {

namespace {

struct GridArgs {
    GeomParams g;
    BinBuffers b;
    RecBuffers r;
    void *grid;
    void *partials;
    int sparse;   // FP32C: occupied bins only (the list b.work)
};

__device__ __forceinline__ void two_sum_acc(float &hi, float &lo, float x)
{
    const float s = hi + x;
    const float z = s - hi;
    const float e = (hi - (s - z)) + (x - z);
    hi = s;
    lo += e;
}

constexpr float kRoundMagic = 12582912.0f;   // 1.5 * 2^23
constexpr int kRoundMagicBits = 0x4B400000;    // its bit pattern

__device__ __forceinline__ void decode_bin(const GeomParams &g, unsigned bin, int &w, int &u0,
                                           int &v0)
{
    const int tu = (int)(bin % (unsigned)g.ntu);
    const unsigned rest = bin / (unsigned)g.ntu;
    const int tv = (int)(rest % (unsigned)g.ntv);
    w = (int)(rest / (unsigned)g.ntv);
    u0 = tu * g.tile;
    v0 = tv * g.tile;
}

// Work item -> (bin, chunk).  Returns false for a bin that is handled by
// split items instead.
__device__ __forceinline__ bool work_item(const BinBuffers &b, unsigned item, unsigned nsplit,
                                          unsigned &bin, unsigned &chunk)
{
    if (item < nsplit) {
        const unsigned long long e = b.split[item];
        bin = (unsigned)(e & 0xFFFFFFFFull);
        chunk = (unsigned)(e >> 32);
        return true;
    }
    bin = item - nsplit;
    chunk = 0;
    return b.is_split[bin] == 0u;
}

// FP32C tile kernel: records sorted by cell in shared memory, taps of
// consecutive records of one cell summed in registers, one shared-memory
// atomic per cell and run of records instead of one per tap (the run-length
// idea of Romein, "An efficient work-distribution strategy for gridding
// radio-telescope data on GPUs", ICS 2012, applied to sorted runs).
//
// An item is processed in stages of at most kStageR records.  A stage is
// loaded into shared memory with coalesced 16-byte loads and counting-sorted
// by the Morton index of its (clamped) tile-relative cell, so the records of
// one cell are consecutive: at 4096^2 x 32 planes and 50M measurements a
// populated cell holds ~14 records, and the binning keeps all records of a
// cell in one sub-range of its bin, so a stage holds whole cells at the bin's
// own density.  The sorted stage is cut into NS contiguous streams, one per
// group of NT = 2K+1 lanes (RPW groups per warp).
//
// Track order (SORTED = false): when the binning walked the measurements
// baseline by baseline (the [dump][baseline] walk), a bin holds each
// baseline's consecutive dumps in consecutive records, and a track crosses a
// cell in ~10 dumps at 4096^2 (a sorted stage gathers ~14 records per cell).
// Stages are then used as stored: no counting sort, two barriers per stage
// instead of six.
//
// Lane k of a group owns window row k of its stream's records and keeps NT
// register accumulators, one per window column.  While consecutive records
// sit in the same cell their windows cover the same cells, so the taps keep
// summing in registers; when the cell changes, and at the end of the stream,
// the accumulators are added to the shared-memory tile (integer atomics at an
// odd pitch, so the NT rows of a window fall in distinct banks; cells outside
// the tile, which only duplicates of neighbouring tiles reach, are skipped).
//
// Tap arithmetic is that of the separable Gaussian: lane k evaluates the row
// weight gv of row k and the column weight gu of column k; the other column
// weights come by shuffles.  Each tap V*gv*gu is rounded to the item's
// fixed-point quantum with one FMA against 1.5*2^23 and summed as an int32, so
// sums are exact and independent of order: an unsplit bin grids to the same
// bits whatever the order of its records and wherever the runs break.  The
// scale 2^f of an item keeps every cell sum below 2^30 (see the bound below;
// a partial sum of a cell is bounded by the same sum of absolute values) and
// every tap below 2^22.

// Threads per CTA of the FP32C gridder: 512 (two CTAs per SM, 64 registers a
// thread) up to support 7; 256 for wider supports, whose 2*(2K+1) register
// accumulators per lane need more registers.
constexpr int f32c_threads(int half) { return half >= 4 ? 256 : 512; }
constexpr int kStageR = 2048;    // records per sorted stage (16-bit indices)

__device__ __forceinline__ unsigned spread6(unsigned x)
{
    x = (x | (x << 4)) & 0x0F0Fu;
    x = (x | (x << 2)) & 0x3333u;
    x = (x | (x << 1)) & 0x5555u;
    return x;
}

// Bytes of the two int32 accumulator tiles (pitch T + 1), 16-byte aligned.
template <int T> constexpr size_t acc_bytes() { return ((size_t)8 * T * (T + 1) + 15) / 16 * 16; }

// Sort key of a record: Morton index of its cell clamped to the tile.
template <int T>
__device__ __forceinline__ unsigned cell_key(const uint4 &q)
{
    const int cu = min(max((int)(q.x >> 24) - 64, 0), T - 1);
    const int cv = min(max((int)(q.y >> 24) - 64, 0), T - 1);
    return spread6((unsigned)cu) | (spread6((unsigned)cv) << 1);
}

template <int T, int K, bool SORTED>
__global__ void __launch_bounds__(f32c_threads(K), 2) k_grid_f32c(GridArgs a)
{
    constexpr int kThreadsR = f32c_threads(K);
    constexpr int NT = 2 * K + 1;
    constexpr int RPW = 32 / NT;
    constexpr int NW = kThreadsR / 32;
    constexpr int NS = NW * RPW;                 // record streams per stage
    constexpr int H = 2 * K;
    constexpr int AW = T + 2 * H;                // area of the bound's blocks
    constexpr int BS = K <= 4 ? 2 : 3;           // bound blocks of 2^BS cells, >= K
    constexpr int NB = (AW + (1 << BS) - 1) >> BS;   // blocks per side
    constexpr int NKEY = T * T;                  // sort buckets
    constexpr int KW = NKEY / 2 / kThreadsR;     // packed bucket words per thread
    constexpr int RPT = kStageR / kThreadsR;     // staged records per thread
    constexpr int CPT = T * T / kThreadsR;
    constexpr int TP = T + 1;                    // accumulator pitch (odd)
    static_assert(KW >= 1 && NKEY / 2 == KW * kThreadsR, "bucket words per thread");
    static_assert(kStageR < 65536, "16-bit record indices and bucket counts");
    extern __shared__ __align__(16) unsigned char smraw[];
    int *are = reinterpret_cast<int *>(smraw);
    int *aim = are + T * TP;
    uint4 *stage = reinterpret_cast<uint4 *>(smraw + acc_bytes<T>());
    unsigned *hist = reinterpret_cast<unsigned *>(stage + kStageR);   // 2 counts per word
    unsigned short *sidx = reinterpret_cast<unsigned short *>(hist + NKEY / 2);
    __shared__ unsigned s_item[2];
    __shared__ int s_last;
    __shared__ float s_part[NW];
    __shared__ float s_vmax[NW];
    __shared__ unsigned s_blk[NB * NB];
    __shared__ unsigned s_wsum[NW];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int grp = lane / NT, k = lane - (lane / NT) * NT;
    const bool lane_on = grp < RPW;
    const float norm = (float)(0.5 / kRefPi);
    const float c2 = -0.72134752044448170368f;   // -0.5 * log2(e)
    const float off1 = (float)(k - K) + 0.5f;
    const uint4 *__restrict__ rec = a.r.rec16;
    float2 *grid = reinterpret_cast<float2 *>(a.grid);
    float2 *parts = reinterpret_cast<float2 *>(a.partials);
    const unsigned nsplit = a.b.ctr->nsplit_items;
    const unsigned nitems = nsplit + (a.sparse ? a.b.ctr->nwork : (unsigned)a.g.nbins);
    const unsigned split = a.b.split_size;

    for (int i = tid; i < 2 * T * TP; i += kThreadsR) are[i] = 0;
    // work items come from a global counter; the next one is fetched while
    // the current one is processed, which hides the atomic's latency
    if (tid == 0) s_item[0] = atomicAdd(&a.b.ctr->work_grid, 1u);
    int slot = 0;

    for (;;) {
        __syncthreads();
        const unsigned item = s_item[slot];
        if (item >= nitems) break;
        if (tid == 0) s_item[slot ^ 1] = atomicAdd(&a.b.ctr->work_grid, 1u);
        slot ^= 1;
        unsigned bin, chunk;
        if (a.sparse && item >= nsplit) {
            bin = a.b.work[item - nsplit];
            chunk = 0;
        } else if (!work_item(a.b, item, nsplit, bin, chunk)) {
            continue;
        }
        int w, u0, v0;
        decode_bin(a.g, bin, w, u0, v0);
        const int tx = min(T, a.g.nx - u0);
        const int ty = min(T, a.g.ny - v0);
        const unsigned total = a.b.ntotal[bin];
        const bool is_split = item < nsplit;
        const unsigned r0 = chunk * split;
        const unsigned r1 = is_split ? min(total, r0 + split) : total;
        const unsigned off = a.b.off[bin];

        // The item's scale.  Sum |Re V| + |Im V| of the records per block of
        // 2^BS x 2^BS cells (2^BS >= K) of the area the records are centred in
        // (records of neighbouring tiles' halos included); a cell's taps all
        // come from records centred within K cells, i.e. in its block or the 8
        // around it, so the largest 3x3-block sum times the peak weight norm
        // bounds every cell of the item, and every partial sum of a cell.  The
        // block sums are integers: each term is rounded up at a scale taken
        // from the item's largest value and record count (sums stay below
        // 2^31), so the bound is an upper bound, independent of the order of
        // the records.
        const unsigned n = r1 - r0;
        // block-sum scale 2^sc: terms <= 2^(31-lb) for n < 2^lb records
        auto sum_scale = [&](float tmax) {
            int ev;
            frexpf(tmax, &ev);                      // |Re V| + |Im V| < 2^(ev+1)
            const int lb = 32 - __clz(n);           // record count < 2^lb
            return min(30 - lb - ev, 126);
        };
        auto add_block = [&](const uint4 &q, float up) {
            const int bx = ((int)(q.x >> 24) - 64 + H) >> BS;
            const int by = ((int)(q.y >> 24) - 64 + H) >> BS;
            const float v = fabsf(__uint_as_float(q.z)) + fabsf(__uint_as_float(q.w));
            // v*up rounded up twice: the product toward +inf, then ceil
            atomicAdd(&s_blk[by * NB + bx], (unsigned)ceilf(__fmul_ru(v, up)));
        };
        // largest 3x3-block sum, reduced over the warp into s_part[warp]
        auto block_max = [&]() {
            unsigned long long bmax = 0ull;
            for (int i = tid; i < NB * NB; i += kThreadsR) {
                const int by = i / NB, bx = i - (i / NB) * NB;
                unsigned long long t = 0ull;
                for (int yy = max(by - 1, 0); yy <= min(by + 1, NB - 1); yy++)
                    for (int xx = max(bx - 1, 0); xx <= min(bx + 1, NB - 1); xx++)
                        t += s_blk[yy * NB + xx];
                bmax = max(bmax, t);
            }
            for (int d = 16; d >= 1; d >>= 1) bmax = max(bmax, __shfl_xor_sync(0xFFFFFFFFu, bmax, d));
            if (lane == 0) s_part[warp] = __ull2float_ru(bmax);
        };
        auto warp_vmax = [&](float vmax) {
            for (int d = 16; d >= 1; d >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xFFFFFFFFu, vmax, d));
            if (lane == 0) s_vmax[warp] = vmax;
        };
        auto cta_max = [&](const float *s) {
            float m = 0.0f;
#pragma unroll
            for (int i = 0; i < NW; i++) m = fmaxf(m, s[i]);
            return m;
        };
        // the staged records' bucket counts (two 16-bit counts per word)
        auto count_keys = [&](const unsigned (&key)[RPT], unsigned cnt) {
#pragma unroll
            for (int t = 0; t < RPT; t++)
                if (tid + t * kThreadsR < cnt)
                    atomicAdd(&hist[key[t] >> 1], (key[t] & 1u) ? 0x10000u : 1u);
        };
        // exclusive scan of the bucket counts, buckets in key order (a cursor
        // never exceeds cnt < 2^16): the warp scans, then (after a barrier)
        // the CTA's prefix and the cursors
        unsigned wv[KW], s_run = 0u, s_incl = 0u;
        auto scan_warps = [&]() {
            s_run = 0u;
#pragma unroll
            for (int t = 0; t < KW; t++) {
                wv[t] = hist[tid * KW + t];
                s_run += (wv[t] & 0xFFFFu) + (wv[t] >> 16);
            }
            s_incl = s_run;
            for (int d = 1; d < 32; d <<= 1) {
                const unsigned y = __shfl_up_sync(0xFFFFFFFFu, s_incl, d);
                if (lane >= d) s_incl += y;
            }
            if (lane == 31) s_wsum[warp] = s_incl;
        };
        auto scan_cursors = [&]() {
            unsigned base = s_incl - s_run;
            for (int i = 0; i < warp; i++) base += s_wsum[i];
#pragma unroll
            for (int t = 0; t < KW; t++) {
                const unsigned lo = wv[t] & 0xFFFFu, hi = wv[t] >> 16;
                hist[tid * KW + t] = base | ((base + lo) << 16);
                base += lo + hi;
            }
        };
        auto place = [&](const unsigned (&key)[RPT], unsigned cnt) {
#pragma unroll
            for (int t = 0; t < RPT; t++) {
                const unsigned i = tid + t * kThreadsR;
                if (i < cnt) {
                    const unsigned old = atomicAdd(&hist[key[t] >> 1], (key[t] & 1u) ? 0x10000u : 1u);
                    sidx[(key[t] & 1u) ? (old >> 16) : (old & 0xFFFFu)] = (unsigned short)i;
                }
            }
        };

        float tapmax = 0.0f, bound = 0.0f;
        unsigned key[RPT];
        const bool one_stage = n <= (unsigned)kStageR;
        if (one_stage) {
            // The whole item fits one stage: its records are read once, and
            // the bound, the sort keys and the bucket counts all come from
            // the staged copy (five barriers instead of ten; three in track
            // order).
            for (int i = tid; i < NB * NB; i += kThreadsR) s_blk[i] = 0u;
            if (SORTED)
                for (int i = tid; i < NKEY / 2; i += kThreadsR) hist[i] = 0u;
            float vmax = 0.0f;
#pragma unroll
            for (int t = 0; t < RPT; t++) {
                const unsigned i = tid + t * kThreadsR;
                key[t] = 0u;
                if (i < n) {
                    const uint4 q = __ldcs(rec + off + r0 + i);
                    stage[i] = q;
                    if (SORTED) key[t] = cell_key<T>(q);
                    vmax = fmaxf(vmax, fmaxf(fabsf(__uint_as_float(q.z)), fabsf(__uint_as_float(q.w))));
                }
            }
            warp_vmax(vmax);
            __syncthreads();
            tapmax = cta_max(s_vmax);
            if (SORTED) count_keys(key, n);
            int sc = 0;
            if (tapmax > 0.0f) {
                sc = sum_scale(tapmax);
                const float up = ldexpf(1.0f, sc);
#pragma unroll
                for (int t = 0; t < RPT; t++) {
                    const unsigned i = tid + t * kThreadsR;
                    if (i < n) add_block(stage[i], up);   // this thread's own records
                }
            }
            __syncthreads();
            if (SORTED) scan_warps();
            if (tapmax > 0.0f) block_max();
            __syncthreads();
            if (SORTED) scan_cursors();
            if (tapmax > 0.0f) bound = ldexpf(cta_max(s_part), -sc);
            if (SORTED) {
                __syncthreads();
                place(key, n);
                __syncthreads();
            }
        } else {
            for (int i = tid; i < NB * NB; i += kThreadsR) s_blk[i] = 0u;
            float vmax = 0.0f;
            for (unsigned i = r0 + tid; i < r1; i += kThreadsR) {
                const uint4 q = __ldcg(rec + off + i);
                vmax = fmaxf(vmax, fmaxf(fabsf(__uint_as_float(q.z)), fabsf(__uint_as_float(q.w))));
            }
            warp_vmax(vmax);
            __syncthreads();
            tapmax = cta_max(s_vmax);
            if (tapmax > 0.0f) {
                const int sc = sum_scale(tapmax);
                const float up = ldexpf(1.0f, sc);
                for (unsigned i = r0 + tid; i < r1; i += kThreadsR) add_block(__ldcg(rec + off + i), up);
                __syncthreads();
                block_max();
                __syncthreads();
                bound = ldexpf(cta_max(s_part), -sc);
            }
        }
        // cell sums stay below 2^30 (+ at most one rounding per term) and
        // every scaled tap below 2^22 (exact rounding with one FMA, below)
        bound = bound * norm * 1.0001f;
        tapmax = tapmax * norm * 1.0001f;
        int fexp = 30;
        if (bound > 0.0f) {
            int e2, e3;
            frexpf(bound, &e2);    // bound < 2^e2
            frexpf(tapmax, &e3);   // tapmax < 2^e3
            fexp = min(min(30 - e2, 22 - e3), 100);
        }
        const float scale = ldexpf(1.0f, fexp);
        const float inv = ldexpf(1.0f, -fexp);
        const float vscale = scale * norm;   // the row weight carries the kernel's norm

        const unsigned nst = one_stage ? 1u : (n + kStageR - 1) / kStageR;
        const unsigned per = nst ? (n + nst - 1) / nst : 0u;
        for (unsigned st = 0; st < nst; st++) {
            const unsigned c0 = r0 + st * per;
            const unsigned cnt = min(per, r1 - c0);
            if (!one_stage) {
                __syncthreads();   // the previous stage's streams are done with stage/sidx
                if (SORTED)
                    for (int i = tid; i < NKEY / 2; i += kThreadsR) hist[i] = 0u;
#pragma unroll
                for (int t = 0; t < RPT; t++) {
                    const unsigned i = tid + t * kThreadsR;
                    key[t] = 0u;
                    if (i < cnt) {
                        const uint4 q = __ldcs(rec + off + c0 + i);
                        stage[i] = q;
                        if (SORTED) key[t] = cell_key<T>(q);
                    }
                }
                __syncthreads();
                if (SORTED) {
                    count_keys(key, cnt);
                    __syncthreads();
                    scan_warps();
                    __syncthreads();
                    scan_cursors();
                    __syncthreads();
                    place(key, cnt);
                    __syncthreads();
                }
            }

            // the streams
            const unsigned len = (cnt + NS - 1) / NS;
            const unsigned sbeg = (unsigned)(warp * RPW + grp) * len;
            int acc_r[NT], acc_i[NT];
#pragma unroll
            for (int j = 0; j < NT; j++) acc_r[j] = acc_i[j] = 0;
            // the run being summed: the cell bytes (bits 24..31) of its
            // records' first two words; all ones before the first record, a
            // cell outside every tile
            unsigned px = 0xFFFFFFFFu, py = 0xFFFFFFFFu;
            for (unsigned t = 0; t < len; t++) {
                const unsigned ri = sbeg + t;
                const bool valid = lane_on && ri < cnt;
                const uint4 q = stage[SORTED ? sidx[valid ? ri : 0u] : (valid ? ri : 0u)];
                const float fu = (float)(q.x & 0xFFFFFFu) * 1.1920928955078125e-7f - 1.0f;
                const float fv = (float)(q.y & 0xFFFFFFu) * 1.1920928955078125e-7f - 1.0f;
                const float du = off1 - fu, dv = off1 - fv;
                const float gu = fast_exp2(du * du * c2);
                const float gv = fast_exp2(dv * dv * c2) * vscale;
                const float ar = valid ? __uint_as_float(q.z) * gv : 0.0f;
                const float ai = valid ? __uint_as_float(q.w) * gv : 0.0f;
                const bool chg = valid && ((q.x ^ px) | (q.y ^ py)) >= (1u << 24);
                if (__any_sync(0xFFFFFFFFu, chg)) {
                    // the run ended: add its window row to the tile, restart
                    const int pcu = (int)(px >> 24) - 64, pcv = (int)(py >> 24) - 64;
                    const int row = pcv - K + k;
                    const int col0 = pcu - K;
                    const bool rin = chg && row >= 0 && row < T;
#pragma unroll
                    for (int j = 0; j < NT; j++) {
                        if (rin && (unsigned)(col0 + j) < (unsigned)T) {
                            atomicAdd(are + row * TP + col0 + j, acc_r[j]);
                            atomicAdd(aim + row * TP + col0 + j, acc_i[j]);
                        }
                        acc_r[j] = chg ? 0 : acc_r[j];
                        acc_i[j] = chg ? 0 : acc_i[j];
                    }
                }
                if (valid) {
                    px = q.x;
                    py = q.y;
                }
#pragma unroll
                for (int j = 0; j < NT; j++) {
                    const float g = __shfl_sync(0xFFFFFFFFu, gu, grp * NT + j);
                    // |ar*g| < 2^22: adding 1.5*2^23 in the same FMA rounds it
                    // to an integer held in the low mantissa bits
                    acc_r[j] += __float_as_int(fmaf(ar, g, kRoundMagic)) - kRoundMagicBits;
                    acc_i[j] += __float_as_int(fmaf(ai, g, kRoundMagic)) - kRoundMagicBits;
                }
            }
            {
                const int pcu = (int)(px >> 24) - 64, pcv = (int)(py >> 24) - 64;
                const int row = pcv - K + k;
                const int col0 = pcu - K;
                if (lane_on && row >= 0 && row < T) {
#pragma unroll
                    for (int j = 0; j < NT; j++) {
                        if ((unsigned)(col0 + j) < (unsigned)T) {
                            atomicAdd(are + row * TP + col0 + j, acc_r[j]);
                            atomicAdd(aim + row * TP + col0 + j, acc_i[j]);
                        }
                    }
                }
            }
        }
        __syncthreads();
        // write the tile (to the grid, or to this item's partial slot) and clear it
        const size_t gbase = (size_t)w * a.g.ny;
        const bool to_grid = !(is_split && chunk > 0);
        float2 *dst = to_grid ? grid
                              : parts + (size_t)(a.b.slot[bin] + chunk - 1) * (size_t)(T * T);
#pragma unroll 4
        for (int i = 0; i < CPT; i++) {
            const int c = tid + i * kThreadsR;
            const int y = c / T, x = c % T;
            const int ac = y * TP + x;
            const float2 v = make_float2((float)are[ac] * inv, (float)aim[ac] * inv);
            are[ac] = 0;
            aim[ac] = 0;
            if (to_grid) {
                if (x < tx && y < ty)
                    __stcg(grid + (gbase + (size_t)(v0 + y)) * a.g.nx + (size_t)(u0 + x), v);
            } else {
                __stcg(dst + c, v);
            }
        }
        if (!is_split) continue;
        // split bin: the CTA finishing its last item combines the partials
        __threadfence();
        __syncthreads();
        const unsigned nchunks = (total + split - 1) / split;
        if (tid == 0) s_last = atomicAdd(&a.b.done[bin], 1u) == nchunks - 1;
        __syncthreads();
        if (!s_last) continue;
        __threadfence();
        const float2 *src = parts + (size_t)a.b.slot[bin] * (size_t)(T * T);
        for (int i = 0; i < CPT; i++) {
            const int c = tid + i * kThreadsR;
            const int y = c / T, x = c % T;
            if (x >= tx || y >= ty) continue;
            float2 *cell = grid + (gbase + (size_t)(v0 + y)) * a.g.nx + (size_t)(u0 + x);
            const float2 g0 = __ldcg(cell);
            float hr = g0.x, lr = 0.f, hi = g0.y, li = 0.f;
            for (unsigned q = 1; q < nchunks; q++) {
                const float2 p = __ldcg(src + (size_t)(q - 1) * (size_t)(T * T) + c);
                two_sum_acc(hr, lr, p.x);
                two_sum_acc(hi, li, p.y);
            }
            __stcg(cell, make_float2(hr + lr, hi + li));
        }
        if (tid == 0) a.b.done[bin] = 0u;   // rearmed for the next launch
    }
}

// Largest work item the FP64 gridder sums in fixed point: the bound below
// costs bitlen(records) bits of the 62, so the error of a cell stays below
// about 2^-49 of the item's largest value times the peak weight, whatever
// the cancellation in the cell.  Larger items (whole bins when there is no
// partial-tile buffer, or a chunk size raised above this) sum in FP64.
constexpr unsigned kFixedMaxRecords = 4096;

// The FP64 gridder's CTA: 512 threads, 64 registers each, two CTAs per SM
// (32 warps; three 256-thread CTAs at 80 registers gave 24).
constexpr int kThreadsG64 = 512;

template <int T, int K>
__global__ void __launch_bounds__(kThreadsG64, 2) k_grid_f64(GridArgs a)
{
    using P = Taps64<K>;
    constexpr int NT = P::NT;
    constexpr int PITCH = T + NT;
    constexpr int NW = kThreadsG64 / 32;
    extern __shared__ long long smd[];
    unsigned long long *sre = reinterpret_cast<unsigned long long *>(smd);
    unsigned long long *sim = sre + T * PITCH;
    __shared__ unsigned s_item, s_exp;
    __shared__ int s_last;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int grp = lane / P::G, row = lane % P::G;
    const double2 *__restrict__ fr_all = reinterpret_cast<const double2 *>(a.r.frac);
    const double2 *__restrict__ val_all = reinterpret_cast<const double2 *>(a.r.val);
    double2 *grid = reinterpret_cast<double2 *>(a.grid);
    double2 *parts = reinterpret_cast<double2 *>(a.partials);
    const unsigned nsplit = a.b.ctr->nsplit_items;
    const unsigned nitems = nsplit + (unsigned)a.g.nbins;
    const unsigned split = a.b.split_size;
    double nt_u, t_v;
    taps64_consts<K>(lane, 0.5 / kRefPi, nt_u, t_v);
    const long long nt_uq = to_fixed(__double_as_longlong(nt_u), 62);
    const long long t_vq = to_fixed(__double_as_longlong(t_v), 62);

    for (int i = tid; i < 2 * T * PITCH; i += kThreadsG64) smd[i] = 0;

    for (;;) {
        __syncthreads();
        if (tid == 0) {
            s_item = atomicAdd(&a.b.ctr->work_grid, 1u);
            s_exp = 0u;
        }
        __syncthreads();
        const unsigned item = s_item;
        if (item >= nitems) break;
        unsigned bin, chunk;
        if (!work_item(a.b, item, nsplit, bin, chunk)) continue;
        // without a partial-tile buffer, the first item of a split bin takes
        // the whole bin
        if (!parts && chunk != 0) continue;
        const bool is_split = parts && item < nsplit;
        int w, u0, v0;
        decode_bin(a.g, bin, w, u0, v0);
        const int tx = min(T, a.g.nx - u0);
        const int ty = min(T, a.g.ny - v0);
        const unsigned total = a.b.ntotal[bin];
        const unsigned r0 = is_split ? chunk * split : 0u;
        const unsigned r1 = is_split ? min(total, r0 + split) : total;
        const unsigned off = a.b.off[bin] + r0;
        const unsigned n = r1 - r0;

        // The item's scale, from the largest exponent of its values (an
        // order-independent bound): every |tap| <= norm * max|V| < 2^(e - 1024)
        // and a cell takes at most n taps, so with
        //   f = 64 - max(bitlen(n), 4) - (e - 1022)
        // a tap's value times 2^f is below 2^(62 - bitlen(n)) and every
        // partial sum of a cell below 2^62; the values enter as V 2^(f+2),
        // below 2^62.  An item holding a NaN or an infinity (e = 2047) sums in
        // FP64 atomics instead, which propagate as the reference's do.
        unsigned ex = 0u;
        for (unsigned rr = tid; rr < n; rr += kThreadsG64) {
            const double2 v = __ldg(val_all + off + rr);
            ex = max(ex, max(exp_field(v.x), exp_field(v.y)));
        }
        ex = __reduce_max_sync(0xFFFFFFFFu, ex);
        if (lane == 0) atomicMax(&s_exp, ex);
        __syncthreads();
        const int e = (int)s_exp;
        const bool fixed = e < 2047 && n <= kFixedMaxRecords;
        const int f = min(64 - max(32 - __clz((int)n), 4) - (e - 1022), 1018);

        for (unsigned base = warp * P::RE; base < n; base += NW * P::RE) {
            const unsigned cnt = min((unsigned)P::RE, n - base);
            const Exps64 E = taps64_exps(fr_all + off + base, cnt, lane);
            const Exps64Q EQ = taps64_exps_q60(E);
#pragma unroll
            for (int s = 0; s < P::SUB; s++) {
                const int r = s * P::R + grp;
                unsigned cell = 0;
                double2 v = make_double2(0.0, 0.0);
                if ((unsigned)r < cnt) {
                    cell = __ldg(a.r.cell + off + base + r);
                    v = __ldg(val_all + off + base + r);
                }
                // window origin; lane `row` scatters row `row` of the window
                const int cu = (int)(cell & 0xFFFFu) - 32768 - K;
                const int y = (int)(cell >> 16) - 32768 - K + row;
                const bool on = (unsigned)r < cnt && row < NT && (unsigned)y < (unsigned)ty;
                if (fixed) {
                    long long guq, gvq;
                    taps64_factors_q<K>(EQ, r, lane, nt_uq, t_vq, guq, gvq);
                    // (V 2^(f+2)) (gu 2^62) / 2^64 = gu V 2^f, then times
                    // (gv 2^62) / 2^64: the cell sums carry 2^(f-2)
                    const Half64 gq = split64(guq);
                    const Half64 ar =
                        split64(mulhi_bal(split64(to_fixed(__double_as_longlong(v.x), f + 2)), gq));
                    const Half64 ai =
                        split64(mulhi_bal(split64(to_fixed(__double_as_longlong(v.y), f + 2)), gq));
                    const Half64 g = split64(gvq);
#pragma unroll
                    for (int j = 0; j < NT; j++) {
                        const int src = grp * P::G + j;
                        const Half64 tr = {__shfl_sync(0xFFFFFFFFu, ar.h, src),
                                           __shfl_sync(0xFFFFFFFFu, ar.l, src)};
                        const Half64 ti = {__shfl_sync(0xFFFFFFFFu, ai.h, src),
                                           __shfl_sync(0xFFFFFFFFu, ai.l, src)};
                        const int x = cu + j;
                        if (on && (unsigned)x < (unsigned)tx) {
                            atomicAdd(sre + y * PITCH + x, (unsigned long long)mulhi_bal(tr, g));
                            atomicAdd(sim + y * PITCH + x, (unsigned long long)mulhi_bal(ti, g));
                        }
                    }
                } else {
                    double gu, gv;
                    taps64_factors<K>(E, r, lane, nt_u, t_v, gu, gv);
                    const double au = gu * v.x, bu = gu * v.y;
#pragma unroll
                    for (int j = 0; j < NT; j++) {
                        const double tr = __shfl_sync(0xFFFFFFFFu, au, grp * P::G + j);
                        const double ti = __shfl_sync(0xFFFFFFFFu, bu, grp * P::G + j);
                        const int x = cu + j;
                        if (on && (unsigned)x < (unsigned)tx) {
                            atomicAdd(reinterpret_cast<double *>(sre + y * PITCH + x), tr * gv);
                            atomicAdd(reinterpret_cast<double *>(sim + y * PITCH + x), ti * gv);
                        }
                    }
                }
            }
        }
        __syncthreads();
        // write the interior (to the grid, or to this item's partial slot) and clear it
        const size_t gbase = (size_t)w * a.g.ny;
        const bool to_grid = !(is_split && chunk > 0);
        double2 *slot = to_grid ? nullptr
                                : parts + (size_t)(a.b.slot[bin] + chunk - 1) * (size_t)(T * T);
        for (int c = tid; c < T * T; c += kThreadsG64) {
            const int y = c / T, x = c % T;
            const int idx = y * PITCH + x;
            const long long br = (long long)sre[idx], bi = (long long)sim[idx];
            const double2 v =
                fixed ? make_double2(__longlong_as_double(from_fixed(br, 2 - f)),
                                     __longlong_as_double(from_fixed(bi, 2 - f)))
                      : make_double2(__longlong_as_double(br), __longlong_as_double(bi));
            sre[idx] = 0ull;
            sim[idx] = 0ull;
            if (to_grid) {
                if (x < tx && y < ty)
                    grid[(gbase + (size_t)(v0 + y)) * a.g.nx + (size_t)(u0 + x)] = v;
            } else {
                __stcg(slot + c, v);
            }
        }
        if (!is_split) continue;
        // split bin: the CTA finishing its last item adds the partials in
        // chunk order and rearms the bin's counter for the next launch
        __threadfence();
        __syncthreads();
        const unsigned nchunks = (total + split - 1) / split;
        if (tid == 0) s_last = atomicAdd(&a.b.done[bin], 1u) == nchunks - 1;
        __syncthreads();
        if (!s_last) continue;
        __threadfence();
        const double2 *src = parts + (size_t)a.b.slot[bin] * (size_t)(T * T);
        for (int c = tid; c < T * T; c += kThreadsG64) {
            const int y = c / T, x = c % T;
            if (x >= tx || y >= ty) continue;
            double2 *cell = grid + (gbase + (size_t)(v0 + y)) * a.g.nx + (size_t)(u0 + x);
            double2 acc = __ldcg(cell);
            for (unsigned q = 1; q < nchunks; q++) {
                const double2 p = __ldcg(src + (size_t)(q - 1) * (size_t)(T * T) + c);
                acc.x += p.x;
                acc.y += p.y;
            }
            __stcg(cell, acc);
        }
        if (tid == 0) a.b.done[bin] = 0u;
    }
}

template <int T, int K> size_t grid_smem(int prec)
{
    if (prec == WSG_FP64) return (size_t)2 * T * (T + 2 * K + 1) * sizeof(double);
    return acc_bytes<T>() + (size_t)kStageR * sizeof(uint4) + (size_t)T * T / 2 * 4 +
           (size_t)kStageR * sizeof(unsigned short);
}

template <int T, int K> const void *grid_kernel(int prec, bool tracks)
{
    if (prec == WSG_FP64) return (const void *)k_grid_f64<T, K>;
    return tracks ? (const void *)k_grid_f32c<T, K, false> : (const void *)k_grid_f32c<T, K, true>;
}

template <int T>
const void *grid_select(int prec, int half, bool tracks, size_t &smem)
{
    switch (half) {
#define WSG_CASE(KK)                           \
    case KK:                                   \
        smem = grid_smem<T, KK>(prec);         \
        return grid_kernel<T, KK>(prec, tracks);
        WSG_CASE(0) WSG_CASE(1) WSG_CASE(2) WSG_CASE(3)
        WSG_CASE(4) WSG_CASE(5) WSG_CASE(6) WSG_CASE(7)
#undef WSG_CASE
    }
    return nullptr;
}

const void *grid_pick(int prec, int tile, int half, bool tracks, size_t &smem)
{
    if (tile == 32) return grid_select<32>(prec, half, tracks, smem);
    if (tile == 64) return grid_select<64>(prec, half, tracks, smem);
    return nullptr;
}

}  // namespace

int grid_max_ctas_per_sm(int prec, int tile, int half)
{
    size_t smem = 0;
    const void *k = grid_pick(prec, tile, half, false, smem);
    if (!k) return 0;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &nb, k, prec == WSG_FP64 ? kThreadsG64 : f32c_threads(half), smem) != cudaSuccess)
        return 0;
    return nb;
}

cudaError_t launch_grid(const GeomParams &g, int prec, const BinBuffers &b, const RecBuffers &r,
                        void *grid, void *partials, int ctas, cudaStream_t s, bool sparse,
                        bool tracks)
{
    size_t smem = 0;
    const void *k = grid_pick(prec, g.tile, g.half, tracks, smem);
    if (!k) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    GridArgs a{g, b, r, grid, partials, (sparse && prec == WSG_FP32C) ? 1 : 0};
    void *args[] = {&a};
    return cudaLaunchKernel(k, dim3(ctas), dim3(prec == WSG_FP64 ? kThreadsG64 : f32c_threads(g.half)), args,
                            smem, s);
}

}  // namespace wsg
