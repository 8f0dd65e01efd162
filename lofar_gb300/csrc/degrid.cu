// Degridding (the adjoint of the gridder; the reference has none).
//
// For every measurement m gridded by the last binning,
//     out[m] = sum_{(j,k) in window(m)} c_m(j,k) * grid[plane(m)][k][j]
// with the gridder's clipped window and real Gaussian weights c_m, which is
// exactly the transpose of the map V_m -> grid of w-stacking.cu:59-117.
//
// It reuses the gridder's sort: a persistent CTA takes a (plane, tile) bin,
// stages the tile plus its K-cell halo from HBM into shared memory once
// (cells off the grid read as zero), then each warp gathers one primary
// measurement: lanes take taps, a shuffle tree sums them, lane 0 stores the
// complex result at the measurement's original index.  Duplicate records of
// the bin are not visited: the halo makes every primary's window local.
#include <cuda_runtime.h>

#include "wsg_internal.cuh"

namespace wsg {

namespace {

struct DegridArgs {
    GeomParams g;
    BinBuffers b;
    RecBuffers r;
    const void *grid;
    void *out;
};

__device__ __forceinline__ void decode_bin_d(const GeomParams &g, unsigned bin, int &w, int &u0,
                                             int &v0)
{
    const int tu = (int)(bin % (unsigned)g.ntu);
    const unsigned rest = bin / (unsigned)g.ntu;
    const int tv = (int)(rest % (unsigned)g.ntv);
    w = (int)(rest / (unsigned)g.ntv);
    u0 = tu * g.tile;
    v0 = tv * g.tile;
}

template <typename T2> struct Cx;
template <> struct Cx<float2> {
    using S = float;
    static __device__ __forceinline__ float2 zero() { return make_float2(0.f, 0.f); }
};
template <> struct Cx<double2> {
    using S = double;
    static __device__ __forceinline__ double2 zero() { return make_double2(0.0, 0.0); }
};

__device__ __forceinline__ float gauss1d(float d) { return __expf(-0.5f * (d * d)); }
__device__ __forceinline__ double gauss1d(double d) { return exp(-(d * d) * 0.5); }

template <int T, int K, typename C2>
__global__ void __launch_bounds__(kThreads) k_degrid(DegridArgs a)
{
    using S = typename Cx<C2>::S;
    constexpr int NT = 2 * K + 1;
    constexpr int NTAP = NT * NT;
    constexpr int ROUNDS = (NTAP + 31) / 32;
    constexpr int HW = T + 2 * K;      // tile + halo
    constexpr int SP = T + NT;         // smem pitch (== HW + 1)
    constexpr int NW = kThreads / 32;
    extern __shared__ unsigned char smraw[];
    C2 *tile = reinterpret_cast<C2 *>(smraw);
    __shared__ unsigned s_item;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const S norm = (S)(0.5 / kRefPi);
    const C2 *__restrict__ grid = reinterpret_cast<const C2 *>(a.grid);
    const C2 *__restrict__ fr_all = reinterpret_cast<const C2 *>(a.r.frac);
    C2 *out = reinterpret_cast<C2 *>(a.out);

    int odj[ROUNDS], odk[ROUNDS];
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
        const int l = lane + 32 * r;
        odk[r] = (l < NTAP) ? l / NT : 4096;
        odj[r] = l % NT;
    }
    const bool is_u = lane < NT;
    const bool is_v = lane >= NT && lane < 2 * NT;
    const S off1d = (S)((is_u ? lane : lane - NT) - K) + (S)0.5;

    for (;;) {
        __syncthreads();
        if (tid == 0) s_item = atomicAdd(&a.b.ctr->work_degrid, 1u);
        __syncthreads();
        const unsigned item = s_item;
        if ((long long)item >= a.g.nbins) break;
        const unsigned bin = a.b.order[item];
        const unsigned nprim = a.b.cnt_prim[bin];
        if (nprim == 0) continue;
        int w, u0, v0;
        decode_bin_d(a.g, bin, w, u0, v0);
        const unsigned off = a.b.off[bin];
        const size_t plane = (size_t)w * a.g.ny;
        for (int i = tid; i < HW * HW; i += kThreads) {
            const int y = i / HW, x = i - (i / HW) * HW;
            const int gy = v0 - K + y, gx = u0 - K + x;
            C2 val = Cx<C2>::zero();
            if (gx >= 0 && gx < a.g.nx && gy >= 0 && gy < a.g.ny)
                val = grid[(plane + (size_t)gy) * a.g.nx + (size_t)gx];
            tile[y * SP + x] = val;
        }
        __syncthreads();
        for (unsigned rr = warp; rr < nprim; rr += NW) {
            const unsigned cell = __ldg(a.r.cell + off + rr);
            const C2 fr = fr_all[off + rr];
            const unsigned idx = __ldg(a.r.idx + off + rr);
            // window origin in halo-tile coordinates: (cell - K) - (-K) = cell
            const int cu = (int)(cell & 0xFFFFu) - 32768;
            const int cv = (int)(cell >> 16) - 32768;
            // separable Gaussian: lanes [0,NT) hold norm*exp(-du^2/2) for
            // column j, lanes [NT,2NT) exp(-dv^2/2) for row k
            S e = 0;
            if (is_u) e = norm * gauss1d(off1d - fr.x);
            else if (is_v) e = gauss1d(off1d - fr.y);
            S sr = 0, si = 0;
#pragma unroll
            for (int r = 0; r < ROUNDS; r++) {
                const S gu = __shfl_sync(0xFFFFFFFFu, e, odj[r]);
                const S gv = __shfl_sync(0xFFFFFFFFu, e, (NT + odk[r]) & 31);
                const int x = cu + odj[r];
                const int y = cv + odk[r];
                if ((unsigned)x < (unsigned)HW && (unsigned)y < (unsigned)HW) {
                    const S wgt = gu * gv;
                    const C2 g = tile[y * SP + x];
                    sr += wgt * g.x;
                    si += wgt * g.y;
                }
            }
#pragma unroll
            for (int d = 16; d >= 1; d >>= 1) {
                sr += __shfl_xor_sync(0xFFFFFFFFu, sr, d);
                si += __shfl_xor_sync(0xFFFFFFFFu, si, d);
            }
            if (lane == 0) {
                C2 o;
                o.x = sr;
                o.y = si;
                out[idx] = o;
            }
        }
    }
}

template <int T, int K> size_t degrid_smem(int prec)
{
    return (size_t)(T + 2 * K) * (T + 2 * K + 1) *
           (prec == WSG_FP64 ? sizeof(double2) : sizeof(float2));
}

template <int T, int K> const void *degrid_kernel(int prec)
{
    return prec == WSG_FP64 ? (const void *)k_degrid<T, K, double2>
                            : (const void *)k_degrid<T, K, float2>;
}

template <int T>
const void *degrid_select(int prec, int half, size_t &smem)
{
    switch (half) {
#define WSG_CASE(KK)                           \
    case KK:                                   \
        smem = degrid_smem<T, KK>(prec);       \
        return degrid_kernel<T, KK>(prec);
        WSG_CASE(0) WSG_CASE(1) WSG_CASE(2) WSG_CASE(3)
        WSG_CASE(4) WSG_CASE(5) WSG_CASE(6) WSG_CASE(7)
#undef WSG_CASE
    }
    return nullptr;
}

const void *degrid_pick(int prec, int tile, int half, size_t &smem)
{
    if (tile == 32) return degrid_select<32>(prec, half, smem);
    if (tile == 64) return degrid_select<64>(prec, half, smem);
    return nullptr;
}

}  // namespace

int degrid_max_ctas_per_sm(int prec, int tile, int half)
{
    size_t smem = 0;
    const void *k = degrid_pick(prec, tile, half, smem);
    if (!k) return 0;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, kThreads, smem) != cudaSuccess)
        return 0;
    return nb;
}

cudaError_t launch_degrid(const GeomParams &g, int prec, const BinBuffers &b, const RecBuffers &r,
                          const void *grid, void *out, long long n, int ctas, cudaStream_t s)
{
    size_t smem = 0;
    const void *k = degrid_pick(prec, g.tile, g.half, smem);
    if (!k) return cudaErrorInvalidValue;
    const size_t esz = prec == WSG_FP64 ? sizeof(double2) : sizeof(float2);
    cudaError_t e = cudaMemsetAsync(out, 0, (size_t)n * esz, s);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    DegridArgs a{g, b, r, grid, out};
    void *args[] = {&a};
    return cudaLaunchKernel(k, dim3(ctas), dim3(kThreads), args, smem, s);
}

}  // namespace wsg
