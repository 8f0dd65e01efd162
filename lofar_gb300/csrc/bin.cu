// Binning: a counting sort of measurements into (w-plane, tile) bins.
//
// Replaces the reference's per-rank v-slab decomposition (gridding.c:35-86)
// with a device-side sort whose key reuses the reference's own coordinate
// step (w-stacking.cu:66-77), so every measurement lands on exactly the cells
// and plane the reference would use.  Five short kernels:
//   k_bin_count    one pass over uvw: per-bin record counts (primary/duplicate)
//   k_bin_scan_a   per-CTA sums of bin sizes and of split work items
//   k_bin_scan_b   one CTA: scan of the per-CTA sums
//   k_bin_scan_c   per-bin record offsets; bins above the split size are cut
//                  into work items of at most that many records
//   k_bin_scatter  second pass over all inputs: writes the records
// k_bin_count_batch / k_bin_scatter_batch replace the two passes for a
// (channel, polarisation) batch, whose jobs are stacked along the plane axis.
// The tile kernels take the split items first, then every other bin, so no
// work item holds more than `split` records and the load stays balanced.
#include <cuda_runtime.h>

#include <type_traits>

#include "coord.cuh"
#include "wsg_internal.cuh"

namespace wsg {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;

struct MGeom {
    int gu, gv, gw;
    int tu0, tu1, tv0, tv1;   // tiles touched by the clipped window
    int tup, tvp;             // primary tile (holds the clamped centre cell)
};

// Status: 0 gridded, 1 plane outside [0,P) (reference writes out of bounds),
// 2 support window entirely off the grid (reference writes nothing).
template <bool UP2, bool WP2, typename F>
__device__ __forceinline__ int measure(const GeomParams &g, double x, double y, double z,
                                       MGeom &o, F &fu, F &fv)
{
    const Cell<F> cu = coord_step<UP2, F>(x, g.ku, g.dx);
    const Cell<F> cv = coord_step<UP2, F>(y, g.ku, g.dx);
    const Cell<float> cw = coord_step<WP2, float>(z, g.kw, g.dw);
    fu = cu.frac;
    fv = cv.frac;
    if (!cu.ok || !cv.ok) return 2;
    const int K = g.half;
    // clipped window (w-stacking.cu:74-77): [max(c-K,0), min(c+K,N-1)]
    const int ju0 = max(cu.g - K, 0), ju1 = min(cu.g + K, g.nx - 1);
    const int jv0 = max(cv.g - K, 0), jv1 = min(cv.g + K, g.ny - 1);
    if (ju0 > ju1 || jv0 > jv1) return 2;
    if (!cw.ok || cw.g < 0 || cw.g >= g.wplanes) return 1;
    o.gu = cu.g;
    o.gv = cv.g;
    o.gw = cw.g;
    // tile indices of non-negative cells: the tile edge is a power of two
    o.tu0 = ju0 >> g.tile_shift;
    o.tu1 = ju1 >> g.tile_shift;
    o.tv0 = jv0 >> g.tile_shift;
    o.tv1 = jv1 >> g.tile_shift;
    o.tup = min(max(cu.g, 0), g.nx - 1) >> g.tile_shift;
    o.tvp = min(max(cv.g, 0), g.ny - 1) >> g.tile_shift;
    return 0;
}

// measure() without the fractions: the status and the geometry only.
template <bool UP2, bool WP2>
__device__ __forceinline__ int measure_cells(const GeomParams &g, double x, double y, double z,
                                             MGeom &o)
{
    bool oku, okv, okw;
    const int cu = coord_cell<UP2>(x, g.ku, g.dx, oku);
    const int cv = coord_cell<UP2>(y, g.ku, g.dx, okv);
    const int cw = coord_cell<WP2>(z, g.kw, g.dw, okw);
    if (!oku || !okv) return 2;
    const int K = g.half;
    const int ju0 = max(cu - K, 0), ju1 = min(cu + K, g.nx - 1);
    const int jv0 = max(cv - K, 0), jv1 = min(cv + K, g.ny - 1);
    if (ju0 > ju1 || jv0 > jv1) return 2;
    if (!okw || cw < 0 || cw >= g.wplanes) return 1;
    o.gu = cu;
    o.gv = cv;
    o.gw = cw;
    o.tu0 = ju0 >> g.tile_shift;
    o.tu1 = ju1 >> g.tile_shift;
    o.tv0 = jv0 >> g.tile_shift;
    o.tv1 = jv1 >> g.tile_shift;
    o.tup = min(max(cu, 0), g.nx - 1) >> g.tile_shift;
    o.tvp = min(max(cv, 0), g.ny - 1) >> g.tile_shift;
    return 0;
}

__device__ __forceinline__ unsigned bin_index(const GeomParams &g, int w, int tv, int tu)
{
    return (unsigned)(((long long)w * g.ntv + tv) * g.ntu + tu);
}


// Sub-range of a record within its bin: the measurement's cell modulo 4 in
// each axis; one range when nsub < 16.  Every record of one cell falls in
// one sub-range, so the tile kernels' sorted stages keep each cell's records
// together, and the atomics of a crowded region of the grid are spread over
// 16 counters.
__device__ __forceinline__ unsigned sub_key(unsigned nsub, int cell_u, int cell_v)
{
    return nsub >= 16u ? ((unsigned)cell_u & 3u) | (((unsigned)cell_v & 3u) << 2) : 0u;
}

// Both passes give each thread IT measurements per tile of 256*IT: item i of
// thread t of tile q is measurement 256*IT*q + 256*i + t (coalesced loads).
template <int IT>
__device__ __forceinline__ long long tile_m(long long q, int i)
{
    return q * (256 * IT) + (long long)i * 256 + threadIdx.x;
}

// The counters of a measurement's records, one per tile of its window's 2x2
// tile block (d: du = d & 1, dv = d >> 1 from (tu0, tv0)): indices into the
// counter array sub_prim, which sub_dup follows (primaries, then duplicates);
// kFull where the window has no tile.  dp: the primary's d.
// Sub-range by position (walks along tracks): the 4x4 block (T/4 cells
// square, Morton order) of the measurement's clamped cell in its primary
// tile.  A track stays in one block for many dumps, so the records of a
// baseline's consecutive dumps share counters; each cell still falls in one
// sub-range.
__device__ __forceinline__ unsigned block_key(const GeomParams &g, unsigned nsub, const MGeom &o)
{
    if (nsub < 16u) return 0u;
    const int bs = g.tile_shift - 2;
    const unsigned bx = (unsigned)(min(max(o.gu, 0), g.nx - 1) - (o.tup << g.tile_shift)) >> bs;
    const unsigned by = (unsigned)(min(max(o.gv, 0), g.ny - 1) - (o.tvp << g.tile_shift)) >> bs;
    return (bx & 1u) | ((by & 1u) << 1) | ((bx & 2u) << 1) | ((by & 2u) << 2);
}

template <bool SPATIAL>
__device__ __forceinline__ void rec_keys(const GeomParams &g, const BinBuffers &b, const MGeom &o,
                                         int st, unsigned nb, unsigned key[4], int &dp)
{
    dp = 0;
    if (st != 0) {
        key[0] = key[1] = key[2] = key[3] = kFull;
        return;
    }
    const unsigned sub = SPATIAL ? block_key(g, b.nsub, o) : sub_key(b.nsub, o.gu, o.gv);
    const unsigned b0 = ((unsigned)o.gw * (unsigned)g.ntv + (unsigned)o.tv0) * (unsigned)g.ntu +
                        (unsigned)o.tu0 + sub * nb;
    const bool two_u = o.tu1 > o.tu0, two_v = o.tv1 > o.tv0;
    dp = (o.tup - o.tu0) | ((o.tvp - o.tv0) << 1);
    const unsigned dupbase = b.nsub * nb;
#pragma unroll
    for (int d = 0; d < 4; d++) {
        const int du = d & 1, dv = d >> 1;
        const bool has = (du == 0 || two_u) && (dv == 0 || two_v);
        key[d] = has ? (d == dp ? 0u : dupbase) + b0 + (unsigned)(dv * g.ntu + du) : kFull;
    }
}

// Runs of equal keys in consecutive lanes: the run's first lane (`lead`), its
// length (`cnt`, valid at the lead) and this lane's rank in it.  A key that
// recurs after a different one starts a new run, so runs are exact and each
// run takes its own cursor atomic.
__device__ __forceinline__ void warp_runs(unsigned key, int lane, int &lead, unsigned &cnt,
                                          unsigned &rank)
{
    const unsigned prev = __shfl_up_sync(kFull, key, 1);
    const unsigned heads = __ballot_sync(kFull, lane == 0 || prev != key);
    const unsigned upto = lane == 31 ? kFull : ((2u << lane) - 1u);
    lead = 31 - __clz(heads & upto);
    const unsigned after = heads & ~upto;
    const int next = after ? __ffs(after) - 1 : 32;
    cnt = (unsigned)(next - lane);   // run length when lane == lead
    rank = (unsigned)(lane - lead);
}

constexpr int kItemsCount = 4;     // measurements a thread per tile, counting pass
constexpr int kItemsScatter = 1;   // the same, scatter pass (registers, occupancy)

// Counting pass.  Primaries take one atomic per run of equal counters in
// consecutive lanes (crowded bins near the uv origin are hit by neighbouring
// measurements); duplicates, which lie along tile edges, one atomic each.
template <bool UP2, bool WP2>
__global__ void __launch_bounds__(256)
k_bin_count(GeomParams g, const double *__restrict__ uu, const double *__restrict__ vv,
            const double *__restrict__ ww, long long n, long long tiles, BinBuffers b)
{
    constexpr int IT = kItemsCount;
    const int lane = threadIdx.x & 31;
    const unsigned nb = (unsigned)g.nbins;
    for (long long q = blockIdx.x; q < tiles; q += gridDim.x) {
        double x[IT], y[IT], z[IT];
#pragma unroll
        for (int i = 0; i < IT; i++) {
            const long long m = tile_m<IT>(q, i);
            x[i] = m < n ? __ldcs(uu + m) : 0.0;
            y[i] = m < n ? __ldcs(vv + m) : 0.0;
            z[i] = m < n ? __ldcs(ww + m) : 0.0;
        }
        int ndp = 0, ndw = 0;
#pragma unroll
        for (int i = 0; i < IT; i++) {
            const long long m = tile_m<IT>(q, i);
            MGeom o;
            const int st = m < n ? measure_cells<UP2, WP2>(g, x[i], y[i], z[i], o) : 3;
            ndp += st == 1;
            ndw += st == 2;
            unsigned key[4];
            int dp;
            rec_keys<false>(g, b, o, st, nb, key, dp);
            unsigned kp = kFull;
#pragma unroll
            for (int d = 0; d < 4; d++) kp = d == dp ? key[d] : kp;
            int lead;
            unsigned cnt, rank;
            warp_runs(kp, lane, lead, cnt, rank);
            if (kp != kFull && lane == lead) atomicAdd(&b.sub_prim[kp], cnt);
#pragma unroll
            for (int d = 0; d < 4; d++)
                if (d != dp && key[d] != kFull) atomicAdd(&b.sub_prim[key[d]], 1u);
        }
        for (int d = 16; d >= 1; d >>= 1) {
            ndp += __shfl_xor_sync(kFull, ndp, d);
            ndw += __shfl_xor_sync(kFull, ndw, d);
        }
        if (lane == 0) {
            if (ndp) atomicAdd(&b.ctr->dropped_plane, (unsigned long long)ndp);
            if (ndw) atomicAdd(&b.ctr->dropped_window, (unsigned long long)ndw);
        }
    }
}

template <typename S>
__device__ __forceinline__ void fold_value(const float *__restrict__ vr,
                                           const float *__restrict__ vi,
                                           const float *__restrict__ wt, long long m,
                                           long long nf, long long np, S &re, S &im)
{
    // the fold of w-stacking.cu:98-112 taken out of the tap loop: weight*vis
    // is a float product; entries whose real part is NaN are skipped
    re = 0;
    im = 0;
    const long long vb = m * nf * np;
    const long long wb = m * np;
    for (long long f = 0; f < nf; f++) {
        for (long long p = 0; p < np; p++) {
            const float a = __ldcs(vr + vb + f * np + p);
            if (!isnan(a)) {
                const float w = __ldcs(wt + wb + p);
                const float c = __ldcs(vi + vb + f * np + p);
                re += (S)(w * a);
                im += (S)(w * c);
            }
        }
    }
}

// The FP32C record (16 bytes): per axis one word, the tile-relative cell in
// the top 8 bits (biased by 64) and (frac + 1) * 2^23 in the low 24 bits,
// then the folded value as two floats.
__device__ __forceinline__ unsigned pack_axis(int c, float f)
{
    unsigned q = (unsigned)__float2int_rn((f + 1.0f) * 8388608.0f);
    q = min(q, 0xFFFFFFu);
    return ((unsigned)(c + 64) << 24) | q;
}

template <bool UP2, bool WP2, int PREC>
__global__ void __launch_bounds__(256)
k_bin_scatter(GeomParams g, const double *__restrict__ uu, const double *__restrict__ vv,
              const double *__restrict__ ww, const float *__restrict__ vr,
              const float *__restrict__ vi, const float *__restrict__ wt, long long n,
              long long tiles, long long nf, long long np, BinBuffers b, RecBuffers r)
{
    using S = typename std::conditional<PREC == WSG_FP64, double, float>::type;
    constexpr int IT = kItemsScatter;
    const int lane = threadIdx.x & 31;
    const unsigned nb = (unsigned)g.nbins;
    // one frequency and one polarisation (the usual case): the value is one
    // float product, and its inputs are loaded with the coordinates so that
    // their latency overlaps the cursor atomics
    const bool single = nf == 1 && np == 1;
    for (long long q = blockIdx.x; q < tiles; q += gridDim.x) {
        double x[IT], y[IT], z[IT];
        float a_re[IT], a_im[IT], a_wt[IT];
#pragma unroll
        for (int i = 0; i < IT; i++) {
            const long long m = tile_m<IT>(q, i);
            x[i] = m < n ? __ldcs(uu + m) : 0.0;
            y[i] = m < n ? __ldcs(vv + m) : 0.0;
            z[i] = m < n ? __ldcs(ww + m) : 0.0;
            a_re[i] = (single && m < n) ? __ldcs(vr + m) : 0.0f;
            a_im[i] = (single && m < n) ? __ldcs(vi + m) : 0.0f;
            a_wt[i] = (single && m < n) ? __ldcs(wt + m) : 0.0f;
        }
        // record positions first: every cursor atomic of the tile is issued
        // before the first result is used.  Primaries take one atomic per run
        // of equal counters in consecutive lanes, duplicates one each.
        unsigned pos[IT][4];   // duplicates (the primary's entry unused)
        unsigned ppos[IT];     // primary: the run's base at the lead lane, then its position
        unsigned lr[IT];
        int dpi[IT];
#pragma unroll
        for (int i = 0; i < IT; i++) {
            const long long m = tile_m<IT>(q, i);
            MGeom o;
            const int st = m < n ? measure_cells<UP2, WP2>(g, x[i], y[i], z[i], o) : 3;
            unsigned key[4];
            rec_keys<false>(g, b, o, st, nb, key, dpi[i]);
            unsigned kp = kFull;
#pragma unroll
            for (int d = 0; d < 4; d++) kp = d == dpi[i] ? key[d] : kp;
            int lead;
            unsigned cnt, rank;
            warp_runs(kp, lane, lead, cnt, rank);
            lr[i] = ((unsigned)lead << 8) | rank;
            ppos[i] = (kp != kFull && lane == lead) ? atomicAdd(&b.sub_prim[kp], cnt) : 0u;
            if (kp == kFull) lr[i] |= 0x80000000u;   // no record
#pragma unroll
            for (int d = 0; d < 4; d++)
                pos[i][d] = (d != dpi[i] && key[d] != kFull) ? atomicAdd(&b.sub_prim[key[d]], 1u)
                                                              : kFull;
        }
        // the primary's run base comes from its lead lane
#pragma unroll
        for (int i = 0; i < IT; i++) {
            const unsigned base = __shfl_sync(kFull, ppos[i], (int)((lr[i] >> 8) & 31u));
            ppos[i] = (lr[i] & 0x80000000u) ? kFull : base + (lr[i] & 0xFFu);
        }
#pragma unroll
        for (int i = 0; i < IT; i++) {
            if (ppos[i] == kFull) continue;   // a measurement with records has a primary
            const long long m = tile_m<IT>(q, i);
            MGeom o;
            S fu = 0, fv = 0;
            unsigned qu = 0u, qv = 0u;
            if (PREC == WSG_FP64) {
                measure<UP2, WP2, S>(g, x[i], y[i], z[i], o, fu, fv);
            } else {
                measure_cells<UP2, WP2>(g, x[i], y[i], z[i], o);
                bool ok;
                coord_cell_q24<UP2>(x[i], g.ku, g.dx, qu, ok);
                coord_cell_q24<UP2>(y[i], g.ku, g.dx, qv, ok);
            }
            S re, im;
            if (single) {
                // the fold of w-stacking.cu:98-112 with one entry
                re = isnan(a_re[i]) ? (S)0 : (S)(a_wt[i] * a_re[i]);
                im = isnan(a_re[i]) ? (S)0 : (S)(a_wt[i] * a_im[i]);
            } else {
                fold_value<S>(vr, vi, wt, m, nf, np, re, im);
            }
#pragma unroll
            for (int d = 0; d < 4; d++) {
                const unsigned p = d == dpi[i] ? ppos[i] : pos[i][d];
                if (p == kFull) continue;
                const int tu = o.tu0 + (d & 1), tv = o.tv0 + (d >> 1);
                const int cu = o.gu - (tu << g.tile_shift);
                const int cv = o.gv - (tv << g.tile_shift);
                if (PREC == WSG_FP64) {
                    r.cell[p] = (unsigned)(cu + 32768) | ((unsigned)(cv + 32768) << 16);
                    reinterpret_cast<double2 *>(r.frac)[p] = make_double2(fu, fv);
                    reinterpret_cast<double2 *>(r.val)[p] = make_double2(re, im);
                } else {
                    r.rec16[p] = make_uint4(((unsigned)(cu + 64) << 24) | qu,
                                            ((unsigned)(cv + 64) << 24) | qv,
                                            __float_as_uint((float)re), __float_as_uint((float)im));
                }
                // only the degridder reads idx, and only of primaries
                if (tu == o.tup && tv == o.tvp) r.idx[p] = (unsigned)m;
            }
        }
    }
}

// ---- the [dump][baseline] walk --------------------------------------------
//
// The reference's measurement sets hold their rows dump by dump, `baselines`
// rows each (meta.txt, init.c:293).  Told that count (rows = B), the two
// passes walk tiles of 32 dumps x 8 baselines (256 measurements, one a
// thread): each dump's 8 baselines are loaded as one contiguous segment and
// transposed through shared memory, so that warp w holds baseline 8 bb + w at
// 32 consecutive dumps, lane l dump 32 tb + l.  A baseline's track moves by a
// fraction of a cell per dump, so consecutive lanes mostly share the counters
// of their records (the sub-ranges are then 4x4 blocks of the tile, which a
// track crosses rarely): one cursor atomic per run of equal counters, for the
// duplicates too, and a run's records land in consecutive positions, written
// by consecutive lanes.
struct RowsWalk {
    long long n, rows;
    unsigned nbb;       // blocks of 8 baselines
    long long tiles;
};

__device__ __forceinline__ long long rows_m(const RowsWalk &w, unsigned tb, unsigned bb, int t,
                                            int j)
{
    const long long bl = (long long)bb * 8 + j;
    const long long m = ((long long)tb * 32 + t) * w.rows + bl;
    return (bl < w.rows && m < w.n) ? m : -1;
}

// Walk tile q = tb * nbb + bb (tb: block of 32 dumps, bb: block of 8
// baselines).  A CTA's tiles advance by the grid stride, one division ahead
// of the loop and none in it.
struct WalkPos {
    unsigned tb, bb;
};
__device__ __forceinline__ WalkPos walk_pos(const RowsWalk &w, unsigned q)
{
    const unsigned tb = q / w.nbb;
    return {tb, q - tb * w.nbb};
}
__device__ __forceinline__ void walk_advance(const RowsWalk &w, WalkPos &p, const WalkPos &step)
{
    p.tb += step.tb;
    p.bb += step.bb;
    if (p.bb >= w.nbb) {
        p.bb -= w.nbb;
        p.tb += 1u;
    }
}

// Loads the coordinates of dump t, baseline j of walk tile p (zeros outside
// the measurements); returns the measurement's index, or -1.
__device__ __forceinline__ long long rows_load3(const RowsWalk &w, const WalkPos &p, int t, int j,
                                               const double *__restrict__ uu,
                                               const double *__restrict__ vv,
                                               const double *__restrict__ ww, double &u, double &v,
                                               double &x)
{
    const long long m = rows_m(w, p.tb, p.bb, t, j);
    u = m >= 0 ? __ldcs(uu + m) : 0.0;
    v = m >= 0 ? __ldcs(vv + m) : 0.0;
    x = m >= 0 ? __ldcs(ww + m) : 0.0;
    return m;
}

template <bool UP2, bool WP2>
__global__ void __launch_bounds__(256)
k_bin_count_rows(GeomParams g, const double *__restrict__ uu, const double *__restrict__ vv,
                 const double *__restrict__ ww, RowsWalk wk, BinBuffers b)
{
    __shared__ double su[32][9], sv[32][9], sw[32][9];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int lt = tid >> 3, lj = tid & 7;   // this thread's load: dump lt, baseline lj
    const unsigned nb = (unsigned)g.nbins;
    // the next tile's coordinates are loaded into registers while the
    // current tile is processed
    double pu = 0.0, pv = 0.0, pw = 0.0;
    const WalkPos step = walk_pos(wk, gridDim.x);
    WalkPos cur = walk_pos(wk, blockIdx.x), nxt = cur;
    walk_advance(wk, nxt, step);
    if ((long long)blockIdx.x < wk.tiles) rows_load3(wk, cur, lt, lj, uu, vv, ww, pu, pv, pw);
    int ndp = 0, ndw = 0;   // this thread's measurements outside the planes / the grid
    for (long long q = blockIdx.x; q < wk.tiles; q += gridDim.x) {
        su[lt][lj] = pu;
        sv[lt][lj] = pv;
        sw[lt][lj] = pw;
        __syncthreads();
        if (q + gridDim.x < wk.tiles) rows_load3(wk, nxt, lt, lj, uu, vv, ww, pu, pv, pw);
        const long long m = rows_m(wk, cur.tb, cur.bb, lane, warp);
        MGeom o;
        const int st = m >= 0 ? measure_cells<UP2, WP2>(g, su[lane][warp], sv[lane][warp],
                                                         sw[lane][warp], o)
                              : 3;
        unsigned key[4];
        int dp;
        rec_keys<true>(g, b, o, st, nb, key, dp);
#pragma unroll
        for (int d = 0; d < 4; d++) {
            if (!__any_sync(kFull, key[d] != kFull)) continue;
            int lead;
            unsigned cnt, rank;
            warp_runs(key[d], lane, lead, cnt, rank);
            if (key[d] != kFull && lane == lead) atomicAdd(&b.sub_prim[key[d]], cnt);
        }
        ndp += st == 1;
        ndw += st == 2;
        __syncthreads();   // the tile's inputs are read before the next tile's land
        cur = nxt;
        walk_advance(wk, nxt, step);
    }
    for (int d = 16; d >= 1; d >>= 1) {
        ndp += __shfl_xor_sync(kFull, ndp, d);
        ndw += __shfl_xor_sync(kFull, ndw, d);
    }
    if (lane == 0) {
        if (ndp) atomicAdd(&b.ctr->dropped_plane, (unsigned long long)ndp);
        if (ndw) atomicAdd(&b.ctr->dropped_window, (unsigned long long)ndw);
    }
}

template <bool UP2, bool WP2, int PREC>
__global__ void __launch_bounds__(256)
k_bin_scatter_rows(GeomParams g, const double *__restrict__ uu, const double *__restrict__ vv,
                   const double *__restrict__ ww, const float *__restrict__ vr,
                   const float *__restrict__ vi, const float *__restrict__ wt, RowsWalk wk,
                   long long nf, long long np, BinBuffers b, RecBuffers r)
{
    static_assert(PREC == WSG_FP32C, "the walk serves FP32C plans");
    __shared__ double su[32][9], sv[32][9], sw[32][9];
    __shared__ float sr[32][9], si[32][9], st_[32][9];
    __shared__ unsigned spos[32][9];   // each measurement's primary record, transposed back
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned nb = (unsigned)g.nbins;
    const bool single = nf == 1 && np == 1;
    const int lt = tid >> 3, lj = tid & 7;   // this thread's load: dump lt, baseline lj
    // the next tile's inputs are loaded into registers while the current tile
    // is processed
    double pu = 0.0, pv = 0.0, pw = 0.0;
    float pr = 0.0f, pi = 0.0f, pt = 0.0f;
    auto load = [&](const WalkPos &pp) {
        const long long mm = rows_load3(wk, pp, lt, lj, uu, vv, ww, pu, pv, pw);
        pr = (single && mm >= 0) ? __ldcs(vr + mm) : 0.0f;
        pi = (single && mm >= 0) ? __ldcs(vi + mm) : 0.0f;
        pt = (single && mm >= 0) ? __ldcs(wt + mm) : 0.0f;
    };
    const WalkPos step = walk_pos(wk, gridDim.x);
    WalkPos cur = walk_pos(wk, blockIdx.x), nxt = cur;
    walk_advance(wk, nxt, step);
    if ((long long)blockIdx.x < wk.tiles) load(cur);
    for (long long q = blockIdx.x; q < wk.tiles; q += gridDim.x) {
        su[lt][lj] = pu;
        sv[lt][lj] = pv;
        sw[lt][lj] = pw;
        sr[lt][lj] = pr;
        si[lt][lj] = pi;
        st_[lt][lj] = pt;
        __syncthreads();
        if (q + gridDim.x < wk.tiles) load(nxt);
        const long long m = rows_m(wk, cur.tb, cur.bb, lane, warp);
        const double x = su[lane][warp], y = sv[lane][warp], z = sw[lane][warp];
        MGeom o;
        const int st = m >= 0 ? measure_cells<UP2, WP2>(g, x, y, z, o) : 3;
        unsigned key[4];
        int dp;
        rec_keys<true>(g, b, o, st, nb, key, dp);
        // every cursor atomic of the tile is issued before the first result
        // is used: one per run of equal counters
        unsigned got[4], lr[4];
#pragma unroll
        for (int d = 0; d < 4; d++) {
            got[d] = 0u;
            lr[d] = 0u;
            if (!__any_sync(kFull, key[d] != kFull)) continue;
            int lead;
            unsigned cnt, rank;
            warp_runs(key[d], lane, lead, cnt, rank);
            if (key[d] != kFull && lane == lead) got[d] = atomicAdd(&b.sub_prim[key[d]], cnt);
            lr[d] = ((unsigned)lead << 8) | rank;
        }
        unsigned pos[4];
#pragma unroll
        for (int d = 0; d < 4; d++) {
            const unsigned base = __shfl_sync(kFull, got[d], (int)(lr[d] >> 8));
            pos[d] = key[d] != kFull ? base + (lr[d] & 0xFFu) : kFull;
        }
        if (st == 0) {
            unsigned qu = 0u, qv = 0u;
            bool ok;
            coord_cell_q24<UP2>(x, g.ku, g.dx, qu, ok);
            coord_cell_q24<UP2>(y, g.ku, g.dx, qv, ok);
            float re, im;
            if (single) {
                // the fold of w-stacking.cu:98-112 with one entry
                const float a = sr[lane][warp], w = st_[lane][warp];
                re = isnan(a) ? 0.0f : w * a;
                im = isnan(a) ? 0.0f : w * si[lane][warp];
            } else {
                fold_value<float>(vr, vi, wt, m, nf, np, re, im);
            }
#pragma unroll
            for (int d = 0; d < 4; d++) {
                const unsigned p = pos[d];
                if (p == kFull) continue;
                const int tu = o.tu0 + (d & 1), tv = o.tv0 + (d >> 1);
                const int cu = o.gu - (tu << g.tile_shift);
                const int cv = o.gv - (tv << g.tile_shift);
                r.rec16[p] = make_uint4(((unsigned)(cu + 64) << 24) | qu,
                                        ((unsigned)(cv + 64) << 24) | qv, __float_as_uint(re),
                                        __float_as_uint(im));
            }
        }
        // the degridder writes its values in record order and the walk
        // gathers them back: the map measurement -> primary record
        unsigned pp = kFull;
#pragma unroll
        for (int d = 0; d < 4; d++) pp = (st == 0 && d == dp) ? pos[d] : pp;
        spos[lane][warp] = pp;
        __syncthreads();   // the tile's inputs are read before the next tile's land
        {
            const long long mo = rows_m(wk, cur.tb, cur.bb, lt, lj);
            if (mo >= 0) r.pos[mo] = spos[lt][lj];
        }
        cur = nxt;
        walk_advance(wk, nxt, step);
    }
}

// out[m] = vrec[pos[m]] along the walk: a tile's map entries are loaded by
// dump segments, the values read by baseline (consecutive dumps of a track
// sit in consecutive records) and written back by dump segments.  A CTA
// takes kGatherTiles tiles at a time, so that every thread has as many
// independent loads in flight.
constexpr int kGatherTiles = 4;

__global__ void __launch_bounds__(256)
k_walk_gather(RowsWalk wk, const unsigned *__restrict__ pos, const float2 *__restrict__ vrec,
              float2 *__restrict__ out)
{
    constexpr int G = kGatherTiles;
    __shared__ unsigned sp[G][32][9];
    __shared__ float2 so[G][32][9];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int lt = tid >> 3, lj = tid & 7;
    const WalkPos step = walk_pos(wk, gridDim.x);
    WalkPos cur = walk_pos(wk, blockIdx.x);
    for (long long q = blockIdx.x; q < wk.tiles; q += (long long)G * gridDim.x) {
        long long mo[G];
        WalkPos at = cur;
#pragma unroll
        for (int k = 0; k < G; k++) {
            const bool in = q + (long long)k * gridDim.x < wk.tiles;
            mo[k] = in ? rows_m(wk, at.tb, at.bb, lt, lj) : -1;
            sp[k][lt][lj] = mo[k] >= 0 ? __ldcs(pos + mo[k]) : kFull;
            walk_advance(wk, at, step);
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < G; k++) {
            const unsigned p = sp[k][lane][warp];
            so[k][lane][warp] = p != kFull ? __ldcs(vrec + p) : make_float2(0.f, 0.f);
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < G; k++)
            if (mo[k] >= 0) out[mo[k]] = so[k][lt][lj];
        cur = at;
    }
}

// ---- (channel, polarisation) batches ----------------------------------------
//
// One pass over the concatenated measurements of all channels.  A
// measurement's coordinates are computed once; each polarisation p gives its
// own records, in the bins of job c*pols + p (cube plane job*P + w).  Every
// job is what the reference's wstack() computes for that channel and
// polarisation alone (freq_per_chan = polarizations = 1, w-stacking.cu:98-112
// with one entry): the record value is the float product weight*vis, zero
// where vis_real is NaN.

// Largest c with m0[c] <= m: the channel holding global measurement m (empty
// channels share their successor's m0 and are skipped).
__device__ __forceinline__ int chan_of(const long long *s_m0, int nch, long long m)
{
    int lo = 0, hi = nch - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_m0[mid] <= m) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

struct BatchPoint {
    const float *vr, *vi, *wt;
    long long e0;                 // [m][pols] index of polarisation 0
    unsigned long long vis0;
    int c;
};

template <bool UP2, bool WP2, typename F>
__device__ __forceinline__ int batch_point(const GeomParams &g, const ChanTable &t,
                                           const long long *s_m0, long long m, MGeom &o,
                                           F &fu, F &fv, BatchPoint &bp)
{
    if (m >= t.ntot) return 3;
    const int c = chan_of(s_m0, t.nch, m);
    const ChanDesc *d = t.ch + c;
    const long long ml = m - s_m0[c];
    bp.c = c;
    bp.vr = d->vr;
    bp.vi = d->vi;
    bp.wt = d->wt;
    bp.e0 = ml * t.pols;
    bp.vis0 = d->vis0;
    return measure<UP2, WP2, F>(g, __ldcs(d->uu + ml), __ldcs(d->vv + ml), __ldcs(d->ww + ml), o,
                                fu, fv);
}

template <bool UP2, bool WP2>
__global__ void __launch_bounds__(256) k_bin_count_batch(GeomParams g, ChanTable t, BinBuffers b)
{
    __shared__ long long s_m0[kMaxChannels];
    for (int i = threadIdx.x; i < t.nch; i += blockDim.x) s_m0[i] = t.m0[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long nb = g.nbins;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < t.ntot; base += stride) {
        const long long m = base + threadIdx.x;
        MGeom o;
        float fu, fv;
        BatchPoint bp;
        const int st = batch_point<UP2, WP2, float>(g, t, s_m0, m, o, fu, fv, bp);
        const unsigned psub = st == 0 ? sub_key(b.nsub, o.gu, o.gv) : 0u;
        for (int p = 0; p < t.pols; p++) {
            const int plane = (bp.c * t.pols + p) * g.wplanes + o.gw;
            const unsigned prim = (st == 0) ? psub * nb + bin_index(g, plane, o.tvp, o.tup) : kFull;
            const unsigned peers = __match_any_sync(kFull, prim);
            if (st == 0) {
                if (lane == __ffs(peers) - 1) atomicAdd(&b.sub_prim[prim], (unsigned)__popc(peers));
                for (int tv = o.tv0; tv <= o.tv1; tv++)
                    for (int tu = o.tu0; tu <= o.tu1; tu++)
                        if (tv != o.tvp || tu != o.tup)
                            atomicAdd(&b.sub_dup[sub_key(b.nsub, o.gu, o.gv) * nb +
                                                 bin_index(g, plane, tv, tu)], 1u);
            }
        }
        int ndp = st == 1, ndw = st == 2;
        for (int d = 16; d >= 1; d >>= 1) {
            ndp += __shfl_xor_sync(kFull, ndp, d);
            ndw += __shfl_xor_sync(kFull, ndw, d);
        }
        if (lane == 0) {
            if (ndp) atomicAdd(&b.ctr->dropped_plane, (unsigned long long)ndp);
            if (ndw) atomicAdd(&b.ctr->dropped_window, (unsigned long long)ndw);
        }
    }
}

template <bool UP2, bool WP2, int PREC>
__global__ void __launch_bounds__(256)
k_bin_scatter_batch(GeomParams g, ChanTable t, BinBuffers b, RecBuffers r)
{
    using S = typename std::conditional<PREC == WSG_FP64, double, float>::type;
    __shared__ long long s_m0[kMaxChannels];
    for (int i = threadIdx.x; i < t.nch; i += blockDim.x) s_m0[i] = t.m0[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long nb = g.nbins;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < t.ntot; base += stride) {
        const long long m = base + threadIdx.x;
        MGeom o;
        S fu, fv;
        BatchPoint bp;
        const int st = batch_point<UP2, WP2, S>(g, t, s_m0, m, o, fu, fv, bp);
        const unsigned psub = st == 0 ? sub_key(b.nsub, o.gu, o.gv) : 0u;
        for (int p = 0; p < t.pols; p++) {
            const int plane = (bp.c * t.pols + p) * g.wplanes + o.gw;
            const unsigned prim = (st == 0) ? psub * nb + bin_index(g, plane, o.tvp, o.tup) : kFull;
            const unsigned peers = __match_any_sync(kFull, prim);
            const int leader = __ffs(peers) - 1;
            unsigned got = 0;
            if (st == 0 && lane == leader) got = atomicAdd(&b.sub_prim[prim], (unsigned)__popc(peers));
            const unsigned basep = __shfl_sync(kFull, got, leader);
            if (st != 0) continue;
            const unsigned ppos = basep + (unsigned)__popc(peers & lt_mask);
            const long long e = bp.e0 + p;
            const float a = __ldcs(bp.vr + e);
            S re = 0, im = 0;
            if (!isnan(a)) {
                const float w = __ldcs(bp.wt + e);
                re = (S)(w * a);
                im = (S)(w * __ldcs(bp.vi + e));
            }
            const unsigned idx = (unsigned)(bp.vis0 + (unsigned long long)e);
            for (int tv = o.tv0; tv <= o.tv1; tv++) {
                for (int tu = o.tu0; tu <= o.tu1; tu++) {
                    const bool primary = tv == o.tvp && tu == o.tup;
                    const unsigned pos =
                        primary ? ppos
                                : atomicAdd(&b.sub_dup[sub_key(b.nsub, o.gu, o.gv) * nb +
                                                       bin_index(g, plane, tv, tu)], 1u);
                    const int cu = o.gu - (tu << g.tile_shift);
                    const int cv = o.gv - (tv << g.tile_shift);
                    if (PREC == WSG_FP64) {
                        r.cell[pos] = (unsigned)(cu + 32768) | ((unsigned)(cv + 32768) << 16);
                        reinterpret_cast<double2 *>(r.frac)[pos] = make_double2(fu, fv);
                        reinterpret_cast<double2 *>(r.val)[pos] = make_double2(re, im);
                    } else {
                        r.rec16[pos] = make_uint4(pack_axis(cu, (float)fu), pack_axis(cv, (float)fv),
                                                  __float_as_uint((float)re),
                                                  __float_as_uint((float)im));
                    }
                    if (primary) r.idx[pos] = idx;   // read for primaries only
                }
            }
        }
    }
}

// ---- scan of the bin sizes and the work decomposition ----------------------

__device__ __forceinline__ unsigned split_items(unsigned t, unsigned split)
{
    return t > split ? (t + split - 1) / split : 0u;
}

// per-CTA partials: part[2*blk] = records, part[2*blk+1] = items | slots << 32
__global__ void __launch_bounds__(kScanThreads) k_bin_scan_a(long long nbins, BinBuffers b)
{
    __shared__ unsigned long long s_rec[kScanThreads / 32], s_pk[kScanThreads / 32];
    __shared__ unsigned s_max;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_max = 0;
    __syncthreads();
    const long long beg = (long long)blockIdx.x * kScanPerBlock;
    unsigned long long rec = 0, pk = 0;
    unsigned lmax = 0;
    for (int k = 0; k < kScanPerBlock / kScanThreads; k++) {
        const long long i = beg + (long long)k * kScanThreads + tid;
        if (i < nbins) {
            unsigned t = 0;
#pragma unroll
            for (unsigned q = 0; q < b.nsub; q++) t += b.sub_prim[q * nbins + i] + b.sub_dup[q * nbins + i];
            const unsigned it = split_items(t, b.split_size);
            rec += t;
            pk += (unsigned long long)it | ((unsigned long long)(it ? it - 1 : 0) << 32);
            lmax = max(lmax, t);
        }
    }
    for (int d = 16; d >= 1; d >>= 1) {
        rec += __shfl_xor_sync(kFull, rec, d);
        pk += __shfl_xor_sync(kFull, pk, d);
    }
    if (lane == 0) {
        s_rec[warp] = rec;
        s_pk[warp] = pk;
    }
    atomicMax(&s_max, lmax);
    __syncthreads();
    if (tid == 0) {
        unsigned long long r = 0, q = 0;
        for (int w = 0; w < kScanThreads / 32; w++) {
            r += s_rec[w];
            q += s_pk[w];
        }
        b.part[2 * blockIdx.x] = r;
        b.part[2 * blockIdx.x + 1] = q;
        atomicMax(&b.ctr->max_bin, s_max);
    }
}

// One CTA: exclusive scan of the per-CTA partials (both words).
__global__ void __launch_bounds__(1024) k_bin_scan_b(int nblk, BinBuffers b)
{
    __shared__ unsigned long long s_w0[32], s_w1[32];
    __shared__ unsigned long long s_c0, s_c1;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_c0 = s_c1 = 0;
    __syncthreads();
    for (int c0 = 0; c0 < nblk; c0 += 1024) {
        const int i = c0 + tid;
        const unsigned long long v0 = i < nblk ? b.part[2 * i] : 0ull;
        const unsigned long long v1 = i < nblk ? b.part[2 * i + 1] : 0ull;
        unsigned long long a0 = v0, a1 = v1;
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long t0 = __shfl_up_sync(kFull, a0, d);
            const unsigned long long t1 = __shfl_up_sync(kFull, a1, d);
            if (lane >= d) {
                a0 += t0;
                a1 += t1;
            }
        }
        if (lane == 31) {
            s_w0[warp] = a0;
            s_w1[warp] = a1;
        }
        __syncthreads();
        if (warp == 0) {
            unsigned long long w0 = s_w0[lane], w1 = s_w1[lane];
            for (int d = 1; d < 32; d <<= 1) {
                const unsigned long long t0 = __shfl_up_sync(kFull, w0, d);
                const unsigned long long t1 = __shfl_up_sync(kFull, w1, d);
                if (lane >= d) {
                    w0 += t0;
                    w1 += t1;
                }
            }
            s_w0[lane] = w0;
            s_w1[lane] = w1;
        }
        __syncthreads();
        if (i < nblk) {
            b.part[2 * i] = s_c0 + a0 - v0 + (warp ? s_w0[warp - 1] : 0ull);
            b.part[2 * i + 1] = s_c1 + a1 - v1 + (warp ? s_w1[warp - 1] : 0ull);
        }
        __syncthreads();
        if (tid == 0) {
            s_c0 += s_w0[31];
            s_c1 += s_w1[31];
        }
        __syncthreads();
    }
    if (tid == 0) {
        b.ctr->records = s_c0;
        b.ctr->nsplit_items = (unsigned)(s_c1 & 0xFFFFFFFFull);
        b.ctr->nslots = (unsigned)(s_c1 >> 32);
    }
}

// Per bin: record offset, split flag, first partial-tile slot, split items.
__global__ void __launch_bounds__(kScanThreads) k_bin_scan_c(long long nbins, BinBuffers b)
{
    __shared__ unsigned long long s_w0[kScanThreads / 32], s_w1[kScanThreads / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long long beg = (long long)blockIdx.x * kScanPerBlock;
    constexpr int PER = kScanPerBlock / kScanThreads;   // consecutive bins per thread
    unsigned long long l0 = 0, l1 = 0;
    unsigned tt[PER];
#pragma unroll
    for (int k = 0; k < PER; k++) {
        const long long i = beg + (long long)tid * PER + k;
        unsigned t = 0;
        if (i < nbins) {
#pragma unroll
            for (unsigned q = 0; q < b.nsub; q++) t += b.sub_prim[q * nbins + i] + b.sub_dup[q * nbins + i];
        }
        tt[k] = t;
        const unsigned it = split_items(t, b.split_size);
        l0 += t;
        l1 += (unsigned long long)it | ((unsigned long long)(it ? it - 1 : 0) << 32);
    }
    unsigned long long a0 = l0, a1 = l1;
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long t0 = __shfl_up_sync(kFull, a0, d);
        const unsigned long long t1 = __shfl_up_sync(kFull, a1, d);
        if (lane >= d) {
            a0 += t0;
            a1 += t1;
        }
    }
    if (lane == 31) {
        s_w0[warp] = a0;
        s_w1[warp] = a1;
    }
    __syncthreads();
    if (warp == 0) {
        unsigned long long w0 = lane < kScanThreads / 32 ? s_w0[lane] : 0ull;
        unsigned long long w1 = lane < kScanThreads / 32 ? s_w1[lane] : 0ull;
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long t0 = __shfl_up_sync(kFull, w0, d);
            const unsigned long long t1 = __shfl_up_sync(kFull, w1, d);
            if (lane >= d) {
                w0 += t0;
                w1 += t1;
            }
        }
        if (lane < kScanThreads / 32) {
            s_w0[lane] = w0;
            s_w1[lane] = w1;
        }
    }
    __syncthreads();
    unsigned long long r0 = b.part[2 * blockIdx.x] + a0 - l0 + (warp ? s_w0[warp - 1] : 0ull);
    unsigned long long r1 = b.part[2 * blockIdx.x + 1] + a1 - l1 + (warp ? s_w1[warp - 1] : 0ull);
    for (int k = 0; k < PER; k++) {
        const long long i = beg + (long long)tid * PER + k;
        if (i >= nbins) break;
        const unsigned t = tt[k];
        const unsigned it = split_items(t, b.split_size);
        // sub-range starts: primaries of sub 0..nsub-1, then duplicates
        unsigned run = (unsigned)r0;
        for (unsigned q = 0; q < b.nsub; q++) {
            const unsigned c = b.sub_prim[q * nbins + i];
            b.sub_prim[q * nbins + i] = run;
            run += c;
        }
        b.nprim[i] = run - (unsigned)r0;
        for (unsigned q = 0; q < b.nsub; q++) {
            const unsigned c = b.sub_dup[q * nbins + i];
            b.sub_dup[q * nbins + i] = run;
            run += c;
        }
        b.ntotal[i] = t;
        b.off[i] = (unsigned)r0;
        b.is_split[i] = it ? 1u : 0u;
        if (t && !it) b.work[atomicAdd(&b.ctr->nwork, 1u)] = (unsigned)i;
        b.slot[i] = (unsigned)(r1 >> 32);
        b.done[i] = 0u;
        const unsigned first = (unsigned)(r1 & 0xFFFFFFFFull);
        for (unsigned c = 0; c < it; c++)
            b.split[first + c] = (unsigned long long)i | ((unsigned long long)c << 32);
        r0 += t;
        r1 += (unsigned long long)it | ((unsigned long long)(it ? it - 1 : 0) << 32);
    }
}

RowsWalk make_rows_walk(long long n, long long rows)
{
    const long long dumps = (n + rows - 1) / rows;
    RowsWalk w{n, rows, (unsigned)((rows + 7) / 8), 0};
    w.tiles = (dumps + 31) / 32 * (long long)w.nbb;
    return w;
}

int tile_grid(long long tiles)
{
    return (int)max(1ll, min(tiles, (long long)num_sms() * 8));
}

}  // namespace

long long scan_blocks(long long nbins) { return (nbins + kScanPerBlock - 1) / kScanPerBlock; }

cudaError_t launch_walk_gather(const GeomParams &g, long long n, const unsigned *pos,
                               const float2 *vrec, float2 *out, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const RowsWalk w = make_rows_walk(n, g.rows);
    k_walk_gather<<<tile_grid(w.tiles), 256, 0, s>>>(w, pos, vrec, out);
    return cudaGetLastError();
}

cudaError_t launch_bin_count(const GeomParams &g, const double *uu, const double *vv,
                             const double *ww, long long n, const BinBuffers &b, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    if (rows_walk(g, n)) {
        const RowsWalk w = make_rows_walk(n, g.rows);
        const int blocks = tile_grid(w.tiles);
        if (g.u_pow2 && g.w_pow2) k_bin_count_rows<true, true><<<blocks, 256, 0, s>>>(g, uu, vv, ww, w, b);
        else if (g.u_pow2) k_bin_count_rows<true, false><<<blocks, 256, 0, s>>>(g, uu, vv, ww, w, b);
        else if (g.w_pow2) k_bin_count_rows<false, true><<<blocks, 256, 0, s>>>(g, uu, vv, ww, w, b);
        else k_bin_count_rows<false, false><<<blocks, 256, 0, s>>>(g, uu, vv, ww, w, b);
        return cudaGetLastError();
    }
    const long long tiles = (n + 256 * kItemsCount - 1) / (256 * kItemsCount);
    const int blocks = tile_grid(tiles);
    if (g.u_pow2 && g.w_pow2) k_bin_count<true, true><<<blocks, 256, 0, s>>>(g, uu, vv, ww, n, tiles, b);
    else if (g.u_pow2) k_bin_count<true, false><<<blocks, 256, 0, s>>>(g, uu, vv, ww, n, tiles, b);
    else if (g.w_pow2) k_bin_count<false, true><<<blocks, 256, 0, s>>>(g, uu, vv, ww, n, tiles, b);
    else k_bin_count<false, false><<<blocks, 256, 0, s>>>(g, uu, vv, ww, n, tiles, b);
    return cudaGetLastError();
}

cudaError_t launch_bin_scan(const GeomParams &g, const BinBuffers &b, cudaStream_t s)
{
    const long long nblk = scan_blocks(g.nbins);
    k_bin_scan_a<<<(unsigned)nblk, kScanThreads, 0, s>>>(g.nbins, b);
    k_bin_scan_b<<<1, 1024, 0, s>>>((int)nblk, b);
    k_bin_scan_c<<<(unsigned)nblk, kScanThreads, 0, s>>>(g.nbins, b);
    return cudaGetLastError();
}

template <int PREC>
static void scatter_dispatch(const GeomParams &g, const double *uu, const double *vv,
                             const double *ww, const float *vr, const float *vi,
                             const float *wt, long long n, long long nf, long long np,
                             const BinBuffers &b, const RecBuffers &r, cudaStream_t s)
{
    // FP32C plans only (the plan keeps g.rows at 0 for FP64)
    if constexpr (PREC != WSG_FP64) {
        if (rows_walk(g, n)) {
            const RowsWalk w = make_rows_walk(n, g.rows);
            const int blocks = tile_grid(w.tiles);
            if (g.u_pow2 && g.w_pow2)
                k_bin_scatter_rows<true, true, PREC><<<blocks, 256, 0, s>>>(g, uu, vv, ww, vr, vi, wt, w, nf, np, b, r);
            else if (g.u_pow2)
                k_bin_scatter_rows<true, false, PREC><<<blocks, 256, 0, s>>>(g, uu, vv, ww, vr, vi, wt, w, nf, np, b, r);
            else if (g.w_pow2)
                k_bin_scatter_rows<false, true, PREC><<<blocks, 256, 0, s>>>(g, uu, vv, ww, vr, vi, wt, w, nf, np, b, r);
            else
                k_bin_scatter_rows<false, false, PREC><<<blocks, 256, 0, s>>>(g, uu, vv, ww, vr, vi, wt, w, nf, np, b, r);
            return;
        }
    }
    const long long tiles = (n + 256 * kItemsScatter - 1) / (256 * kItemsScatter);
    const int blocks = tile_grid(tiles);
    if (g.u_pow2 && g.w_pow2)
        k_bin_scatter<true, true, PREC><<<blocks, 256, 0, s>>>(g, uu, vv, ww, vr, vi, wt, n, tiles, nf, np, b, r);
    else if (g.u_pow2)
        k_bin_scatter<true, false, PREC><<<blocks, 256, 0, s>>>(g, uu, vv, ww, vr, vi, wt, n, tiles, nf, np, b, r);
    else if (g.w_pow2)
        k_bin_scatter<false, true, PREC><<<blocks, 256, 0, s>>>(g, uu, vv, ww, vr, vi, wt, n, tiles, nf, np, b, r);
    else
        k_bin_scatter<false, false, PREC><<<blocks, 256, 0, s>>>(g, uu, vv, ww, vr, vi, wt, n, tiles, nf, np, b, r);
}

cudaError_t launch_bin_scatter(const GeomParams &g, int prec, const double *uu, const double *vv,
                               const double *ww, const float *vr, const float *vi,
                               const float *wt, long long n, long long nf, long long np,
                               const BinBuffers &b, const RecBuffers &r, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    if (prec == WSG_FP64) scatter_dispatch<WSG_FP64>(g, uu, vv, ww, vr, vi, wt, n, nf, np, b, r, s);
    else scatter_dispatch<WSG_FP32C>(g, uu, vv, ww, vr, vi, wt, n, nf, np, b, r, s);
    return cudaGetLastError();
}

template <int PREC>
static void scatter_batch_dispatch(const GeomParams &g, const ChanTable &t, const BinBuffers &b,
                                   const RecBuffers &r, int blocks, cudaStream_t s)
{
    if (g.u_pow2 && g.w_pow2) k_bin_scatter_batch<true, true, PREC><<<blocks, 256, 0, s>>>(g, t, b, r);
    else if (g.u_pow2) k_bin_scatter_batch<true, false, PREC><<<blocks, 256, 0, s>>>(g, t, b, r);
    else if (g.w_pow2) k_bin_scatter_batch<false, true, PREC><<<blocks, 256, 0, s>>>(g, t, b, r);
    else k_bin_scatter_batch<false, false, PREC><<<blocks, 256, 0, s>>>(g, t, b, r);
}

static int batch_blocks(long long n)
{
    const long long want = (n + 255) / 256;
    return (int)max(1ll, min(want, (long long)num_sms() * 8));
}

cudaError_t launch_bin_count_batch(const GeomParams &g, const ChanTable &t, const BinBuffers &b,
                                   cudaStream_t s)
{
    if (t.ntot <= 0) return cudaSuccess;
    if (t.nch <= 0 || t.nch > kMaxChannels) return cudaErrorInvalidValue;
    const int blocks = batch_blocks(t.ntot);
    if (g.u_pow2 && g.w_pow2) k_bin_count_batch<true, true><<<blocks, 256, 0, s>>>(g, t, b);
    else if (g.u_pow2) k_bin_count_batch<true, false><<<blocks, 256, 0, s>>>(g, t, b);
    else if (g.w_pow2) k_bin_count_batch<false, true><<<blocks, 256, 0, s>>>(g, t, b);
    else k_bin_count_batch<false, false><<<blocks, 256, 0, s>>>(g, t, b);
    return cudaGetLastError();
}

cudaError_t launch_bin_scatter_batch(const GeomParams &g, int prec, const ChanTable &t,
                                     const BinBuffers &b, const RecBuffers &r, cudaStream_t s)
{
    if (t.ntot <= 0) return cudaSuccess;
    if (t.nch <= 0 || t.nch > kMaxChannels) return cudaErrorInvalidValue;
    const int blocks = batch_blocks(t.ntot);
    if (prec == WSG_FP64) scatter_batch_dispatch<WSG_FP64>(g, t, b, r, blocks, s);
    else scatter_batch_dispatch<WSG_FP32C>(g, t, b, r, blocks, s);
    return cudaGetLastError();
}

}  // namespace wsg
