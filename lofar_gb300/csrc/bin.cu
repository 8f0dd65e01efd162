// Binning: a counting sort of measurements into (w-plane, tile) bins.
//
// Replaces the reference's per-rank v-slab decomposition (gridding.c:35-86)
// with a device-side sort whose key reuses the reference's own coordinate
// step (w-stacking.cu:66-77), so every measurement lands on exactly the cells
// and plane the reference would use.  Three kernels, all HBM-streaming:
//   k_bin_count   one pass over uvw: per-bin record counts (primary/duplicate)
//   k_bin_scan    exclusive scan of the counts + a longest-first bin order
//   k_bin_scatter second pass over all inputs: writes the SoA records
#include <cuda_runtime.h>

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
    if (!cw.ok || cw.g < 0 || cw.g >= g.planes) return 1;
    o.gu = cu.g;
    o.gv = cv.g;
    o.gw = cw.g;
    o.tu0 = ju0 / g.tile;
    o.tu1 = ju1 / g.tile;
    o.tv0 = jv0 / g.tile;
    o.tv1 = jv1 / g.tile;
    o.tup = min(max(cu.g, 0), g.nx - 1) / g.tile;
    o.tvp = min(max(cv.g, 0), g.ny - 1) / g.tile;
    return 0;
}

__device__ __forceinline__ unsigned bin_index(const GeomParams &g, int w, int tv, int tu)
{
    return (unsigned)(((long long)w * g.ntv + tv) * g.ntu + tu);
}

template <bool UP2, bool WP2>
__global__ void __launch_bounds__(256)
k_bin_count(GeomParams g, const double *__restrict__ uu, const double *__restrict__ vv,
            const double *__restrict__ ww, long long n, BinBuffers b)
{
    const int lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < n; base += stride) {
        const long long m = base + threadIdx.x;
        int st = 3;
        MGeom o;
        if (m < n) {
            float fu, fv;
            st = measure<UP2, WP2, float>(g, __ldg(uu + m), __ldg(vv + m), __ldg(ww + m), o, fu,
                                          fv);
        }
        const unsigned dp = __ballot_sync(kFull, st == 1);
        const unsigned dwn = __ballot_sync(kFull, st == 2);
        if (lane == 0) {
            if (dp) atomicAdd(&b.ctr->dropped_plane, (unsigned long long)__popc(dp));
            if (dwn) atomicAdd(&b.ctr->dropped_window, (unsigned long long)__popc(dwn));
        }
        const unsigned prim = (st == 0) ? bin_index(g, o.gw, o.tvp, o.tup) : kFull;
        const unsigned peers = __match_any_sync(kFull, prim);
        if (st == 0) {
            if (lane == __ffs(peers) - 1) atomicAdd(&b.cnt_prim[prim], (unsigned)__popc(peers));
            for (int tv = o.tv0; tv <= o.tv1; tv++)
                for (int tu = o.tu0; tu <= o.tu1; tu++)
                    if (tv != o.tvp || tu != o.tup)
                        atomicAdd(&b.cnt_dup[bin_index(g, o.gw, tv, tu)], 1u);
        }
    }
}

template <typename F2> struct Vec2;
template <> struct Vec2<float2> {
    using S = float;
    static __device__ __forceinline__ float2 make(float a, float b) { return make_float2(a, b); }
};
template <> struct Vec2<double2> {
    using S = double;
    static __device__ __forceinline__ double2 make(double a, double b)
    {
        return make_double2(a, b);
    }
};

// The fold of w-stacking.cu:98-112 taken out of the tap loop: the product
// weight*vis is formed in float (float*float), entries whose real part is
// NaN are skipped; the FP64 form sums the promoted products in double.
template <typename S>
__device__ __forceinline__ void fold_value(const float *__restrict__ vr,
                                           const float *__restrict__ vi,
                                           const float *__restrict__ wt, long long m,
                                           long long nf, long long np, S &re, S &im)
{
    re = 0;
    im = 0;
    const long long vb = m * nf * np;
    const long long wb = m * np;
    for (long long f = 0; f < nf; f++) {
        for (long long p = 0; p < np; p++) {
            const float a = __ldg(vr + vb + f * np + p);
            if (!isnan(a)) {
                const float w = __ldg(wt + wb + p);
                const float b = __ldg(vi + vb + f * np + p);
                re += (S)(w * a);
                im += (S)(w * b);
            }
        }
    }
}

template <bool UP2, bool WP2, typename F2>
__global__ void __launch_bounds__(256)
k_bin_scatter(GeomParams g, const double *__restrict__ uu, const double *__restrict__ vv,
              const double *__restrict__ ww, const float *__restrict__ vr,
              const float *__restrict__ vi, const float *__restrict__ wt, long long n,
              long long nf, long long np, BinBuffers b, RecBuffers r)
{
    using S = typename Vec2<F2>::S;
    F2 *frac = reinterpret_cast<F2 *>(r.frac);
    F2 *val = reinterpret_cast<F2 *>(r.val);
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < n; base += stride) {
        const long long m = base + threadIdx.x;
        int st = 3;
        MGeom o;
        S fu = 0, fv = 0;
        if (m < n) st = measure<UP2, WP2, S>(g, __ldg(uu + m), __ldg(vv + m), __ldg(ww + m), o, fu, fv);
        const unsigned prim = (st == 0) ? bin_index(g, o.gw, o.tvp, o.tup) : kFull;
        const unsigned peers = __match_any_sync(kFull, prim);
        const int leader = __ffs(peers) - 1;
        unsigned got = 0;
        if (st == 0 && lane == leader) got = atomicAdd(&b.cur_prim[prim], (unsigned)__popc(peers));
        const unsigned basep = __shfl_sync(kFull, got, leader);
        if (st != 0) continue;

        S re, im;
        fold_value<S>(vr, vi, wt, m, nf, np, re, im);
        const F2 fr = Vec2<F2>::make(fu, fv);
        const F2 vv2 = Vec2<F2>::make(re, im);
        for (int tv = o.tv0; tv <= o.tv1; tv++) {
            for (int tu = o.tu0; tu <= o.tu1; tu++) {
                const unsigned bin = bin_index(g, o.gw, tv, tu);
                unsigned pos;
                if (tv == o.tvp && tu == o.tup) {
                    pos = b.off[bin] + basep + (unsigned)__popc(peers & lt_mask);
                } else {
                    const unsigned tot = b.cnt_prim[bin] + b.cnt_dup[bin];
                    pos = b.off[bin] + tot - 1u - atomicAdd(&b.cur_dup[bin], 1u);
                }
                const int cu = o.gu - tu * g.tile;
                const int cv = o.gv - tv * g.tile;
                r.cell[pos] = (unsigned)(cu + 32768) | ((unsigned)(cv + 32768) << 16);
                frac[pos] = fr;
                val[pos] = vv2;
                r.idx[pos] = (unsigned)m;
            }
        }
    }
}

// Single-CTA exclusive scan of the bin sizes and a longest-first bin order
// (bins bucketed by floor(log2(size)), largest bucket first) for the
// persistent tile kernels.
__global__ void __launch_bounds__(1024) k_bin_scan(long long nbins, BinBuffers b)
{
    __shared__ unsigned long long s_warp[32];
    __shared__ unsigned s_hist[33];
    __shared__ unsigned s_cur[33];
    __shared__ unsigned s_max;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid < 33) s_hist[tid] = 0;
    if (tid == 0) s_max = 0;
    __syncthreads();
    const long long per = (nbins + 1023) / 1024;
    const long long beg = min((long long)tid * per, nbins);
    const long long end = min(beg + per, nbins);
    unsigned long long local = 0;
    unsigned lmax = 0;
    for (long long i = beg; i < end; i++) {
        const unsigned t = b.cnt_prim[i] + b.cnt_dup[i];
        local += t;
        lmax = max(lmax, t);
        atomicAdd(&s_hist[t ? 32 - __clz(t) : 0], 1u);
    }
    // block-wide exclusive scan of `local`
    unsigned long long incl = local;
    for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long v = __shfl_up_sync(kFull, incl, d);
        if (lane >= d) incl += v;
    }
    if (lane == 31) s_warp[warp] = incl;
    atomicMax(&s_max, lmax);
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = s_warp[lane];
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned long long v = __shfl_up_sync(kFull, w, d);
            if (lane >= d) w += v;
        }
        s_warp[lane] = w;  // inclusive warp prefix
    }
    __syncthreads();
    unsigned long long run = incl - local + (warp ? s_warp[warp - 1] : 0ull);
    for (long long i = beg; i < end; i++) {
        b.off[i] = (unsigned)run;
        run += b.cnt_prim[i] + b.cnt_dup[i];
    }
    if (tid == 0) {
        unsigned acc = 0;
        for (int c = 32; c >= 0; c--) {
            s_cur[c] = acc;
            acc += s_hist[c];
        }
        b.ctr->records = s_warp[31];
        b.ctr->max_bin = s_max;
    }
    __syncthreads();
    for (long long i = beg; i < end; i++) {
        const unsigned t = b.cnt_prim[i] + b.cnt_dup[i];
        const unsigned pos = atomicAdd(&s_cur[t ? 32 - __clz(t) : 0], 1u);
        b.order[pos] = (unsigned)i;
    }
}

int stream_grid(long long n, int threads)
{
    const long long want = (n + threads - 1) / threads;
    const long long cap = (long long)num_sms() * 8;
    return (int)max(1ll, min(want, cap));
}

}  // namespace

cudaError_t launch_bin_count(const GeomParams &g, const double *uu, const double *vv,
                             const double *ww, long long n, const BinBuffers &b, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const int blocks = stream_grid(n, 256);
    if (g.u_pow2 && g.w_pow2) k_bin_count<true, true><<<blocks, 256, 0, s>>>(g, uu, vv, ww, n, b);
    else if (g.u_pow2) k_bin_count<true, false><<<blocks, 256, 0, s>>>(g, uu, vv, ww, n, b);
    else if (g.w_pow2) k_bin_count<false, true><<<blocks, 256, 0, s>>>(g, uu, vv, ww, n, b);
    else k_bin_count<false, false><<<blocks, 256, 0, s>>>(g, uu, vv, ww, n, b);
    return cudaGetLastError();
}

cudaError_t launch_bin_scan(const GeomParams &g, const BinBuffers &b, cudaStream_t s)
{
    k_bin_scan<<<1, 1024, 0, s>>>(g.nbins, b);
    return cudaGetLastError();
}

template <typename F2>
static void scatter_dispatch(const GeomParams &g, const double *uu, const double *vv,
                             const double *ww, const float *vr, const float *vi,
                             const float *wt, long long n, long long nf, long long np,
                             const BinBuffers &b, const RecBuffers &r, cudaStream_t s)
{
    const int blocks = stream_grid(n, 256);
    if (g.u_pow2 && g.w_pow2)
        k_bin_scatter<true, true, F2><<<blocks, 256, 0, s>>>(g, uu, vv, ww, vr, vi, wt, n, nf, np, b, r);
    else if (g.u_pow2)
        k_bin_scatter<true, false, F2><<<blocks, 256, 0, s>>>(g, uu, vv, ww, vr, vi, wt, n, nf, np, b, r);
    else if (g.w_pow2)
        k_bin_scatter<false, true, F2><<<blocks, 256, 0, s>>>(g, uu, vv, ww, vr, vi, wt, n, nf, np, b, r);
    else
        k_bin_scatter<false, false, F2><<<blocks, 256, 0, s>>>(g, uu, vv, ww, vr, vi, wt, n, nf, np, b, r);
}

cudaError_t launch_bin_scatter(const GeomParams &g, int prec, const double *uu, const double *vv,
                               const double *ww, const float *vr, const float *vi,
                               const float *wt, long long n, long long nf, long long np,
                               const BinBuffers &b, const RecBuffers &r, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    if (prec == WSG_FP64) scatter_dispatch<double2>(g, uu, vv, ww, vr, vi, wt, n, nf, np, b, r, s);
    else scatter_dispatch<float2>(g, uu, vv, ww, vr, vi, wt, n, nf, np, b, r, s);
    return cudaGetLastError();
}

}  // namespace wsg
