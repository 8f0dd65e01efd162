// Gridding kernels: one persistent CTA per SM slot walks the (plane, tile)
// bins longest-first and accumulates each tile in shared memory, then writes
// it to HBM once with coalesced stores.  Every cell of the grid belongs to
// exactly one tile, and measurements near a tile edge were duplicated into
// the neighbouring bins by the binning pass, so tiles are written with plain
// stores: no global atomics, no memset of the grid.
//
// Work inside a tile (replaces convolve_g, w-stacking.cu:35-118, whose FP64
// global atomics scatter each tap to HBM): a warp takes one measurement and
// its lanes take the (2K+1)^2 taps of the support window.  The tile's
// shared-memory pitch is T + 2K + 1, congruent to the window width modulo 32,
// so the taps of one window fall in distinct banks: the tap scatter is
// conflict-free.
//
// FP32C: taps are added with shared-memory float atomics into an FP32
// chunk accumulator; after every `chunk` measurements each thread folds the
// cells it owns into a register-resident two-float (hi + lo, TwoSum) master
// tile and clears them.  The grid therefore carries compensated sums whose
// error does not grow with the number of measurements in a cell.
//
// FP64: taps are added with FP64 shared-memory atomics; the separable
// Gaussian exp(-du^2/2)*exp(-dv^2/2) is evaluated once per row/column
// (2(2K+1) FP64 exponentials per measurement instead of (2K+1)^2).
#include <cuda_runtime.h>

#include "wsg_internal.cuh"

namespace wsg {

namespace {

struct GridArgs {
    GeomParams g;
    BinBuffers b;
    RecBuffers r;
    void *grid;
    int chunk;
};

__device__ __forceinline__ void two_sum_acc(float &hi, float &lo, float x)
{
    const float s = hi + x;
    const float z = s - hi;
    const float e = (hi - (s - z)) + (x - z);
    hi = s;
    lo += e;
}

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

template <int T, int K>
__global__ void __launch_bounds__(kThreads) k_grid_f32c(GridArgs a)
{
    constexpr int NT = 2 * K + 1;
    constexpr int NTAP = NT * NT;
    constexpr int ROUNDS = (NTAP + 31) / 32;
    constexpr int PITCH = T + NT;
    constexpr int NW = kThreads / 32;
    constexpr int CPT = T * T / kThreads;
    extern __shared__ float sm[];
    float *sre = sm;
    float *sim = sm + T * PITCH;
    __shared__ unsigned s_item;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const float norm = (float)(0.5 / kRefPi);
    const float2 *__restrict__ fr_all = reinterpret_cast<const float2 *>(a.r.frac);
    const float2 *__restrict__ val_all = reinterpret_cast<const float2 *>(a.r.val);
    float2 *grid = reinterpret_cast<float2 *>(a.grid);

    int odj[ROUNDS], odk[ROUNDS];
    float offu[ROUNDS], offv[ROUNDS];
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
        const int l = lane + 32 * r;
        odk[r] = (l < NTAP) ? l / NT : 4096;
        odj[r] = l % NT;
        offu[r] = (float)(odj[r] - K) + 0.5f;
        offv[r] = (float)(odk[r] - K) + 0.5f;
    }
    for (int i = tid; i < 2 * T * PITCH; i += kThreads) sm[i] = 0.0f;

    for (;;) {
        __syncthreads();
        if (tid == 0) s_item = atomicAdd(&a.b.ctr->work_grid, 1u);
        __syncthreads();
        const unsigned item = s_item;
        if ((long long)item >= a.g.nbins) break;
        const unsigned bin = a.b.order[item];
        int w, u0, v0;
        decode_bin(a.g, bin, w, u0, v0);
        const int tx = min(T, a.g.nx - u0);
        const int ty = min(T, a.g.ny - v0);
        const unsigned off = a.b.off[bin];
        const unsigned n = a.b.cnt_prim[bin] + a.b.cnt_dup[bin];

        float mhr[CPT], mlr[CPT], mhi[CPT], mli[CPT];
#pragma unroll
        for (int i = 0; i < CPT; i++) mhr[i] = mlr[i] = mhi[i] = mli[i] = 0.0f;

        for (unsigned c0 = 0; c0 < n; c0 += (unsigned)a.chunk) {
            const unsigned c1 = min(n, c0 + (unsigned)a.chunk);
            for (unsigned rr = c0 + warp; rr < c1; rr += NW) {
                const unsigned cell = __ldg(a.r.cell + off + rr);
                const float2 fr = __ldg(fr_all + off + rr);
                const float2 v = __ldg(val_all + off + rr);
                const int cu = (int)(cell & 0xFFFFu) - 32768 - K;
                const int cv = (int)(cell >> 16) - 32768 - K;
#pragma unroll
                for (int r = 0; r < ROUNDS; r++) {
                    const int x = cu + odj[r];
                    const int y = cv + odk[r];
                    if ((unsigned)x < (unsigned)tx && (unsigned)y < (unsigned)ty) {
                        const float du = offu[r] - fr.x;
                        const float dv = offv[r] - fr.y;
                        const float wgt = norm * __expf(-0.5f * (du * du + dv * dv));
                        atomicAdd(sre + y * PITCH + x, wgt * v.x);
                        atomicAdd(sim + y * PITCH + x, wgt * v.y);
                    }
                }
            }
            __syncthreads();
#pragma unroll
            for (int i = 0; i < CPT; i++) {
                const int c = tid + i * kThreads;
                const int idx = (c / T) * PITCH + (c % T);
                const float xr = sre[idx];
                const float xi = sim[idx];
                sre[idx] = 0.0f;
                sim[idx] = 0.0f;
                two_sum_acc(mhr[i], mlr[i], xr);
                two_sum_acc(mhi[i], mli[i], xi);
            }
            __syncthreads();
        }

#pragma unroll
        for (int i = 0; i < CPT; i++) {
            const int c = tid + i * kThreads;
            const int y = c / T, x = c % T;
            if (x < tx && y < ty)
                grid[((size_t)w * a.g.ny + (size_t)(v0 + y)) * a.g.nx + (size_t)(u0 + x)] =
                    make_float2(mhr[i] + mlr[i], mhi[i] + mli[i]);
        }
    }
}

template <int T, int K>
__global__ void __launch_bounds__(kThreads) k_grid_f64(GridArgs a)
{
    constexpr int NT = 2 * K + 1;
    constexpr int NTAP = NT * NT;
    constexpr int ROUNDS = (NTAP + 31) / 32;
    constexpr int PITCH = T + NT;
    constexpr int NW = kThreads / 32;
    extern __shared__ double smd[];
    double *sre = smd;
    double *sim = smd + T * PITCH;
    __shared__ unsigned s_item;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const double norm = 0.5 / kRefPi;
    const double2 *__restrict__ fr_all = reinterpret_cast<const double2 *>(a.r.frac);
    const double2 *__restrict__ val_all = reinterpret_cast<const double2 *>(a.r.val);
    double2 *grid = reinterpret_cast<double2 *>(a.grid);

    int odj[ROUNDS], odk[ROUNDS];
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
        const int l = lane + 32 * r;
        odk[r] = (l < NTAP) ? l / NT : 4096;
        odj[r] = l % NT;
    }
    // lanes [0,NT) evaluate the u-factors, lanes [NT,2NT) the v-factors
    const bool is_u = lane < NT;
    const bool is_v = lane >= NT && lane < 2 * NT;
    const double off1d = (double)((is_u ? lane : lane - NT) - K) + 0.5;

    for (int i = tid; i < 2 * T * PITCH; i += kThreads) smd[i] = 0.0;

    for (;;) {
        __syncthreads();
        if (tid == 0) s_item = atomicAdd(&a.b.ctr->work_grid, 1u);
        __syncthreads();
        const unsigned item = s_item;
        if ((long long)item >= a.g.nbins) break;
        const unsigned bin = a.b.order[item];
        int w, u0, v0;
        decode_bin(a.g, bin, w, u0, v0);
        const int tx = min(T, a.g.nx - u0);
        const int ty = min(T, a.g.ny - v0);
        const unsigned off = a.b.off[bin];
        const unsigned n = a.b.cnt_prim[bin] + a.b.cnt_dup[bin];

        for (unsigned rr = warp; rr < n; rr += NW) {
            const unsigned cell = __ldg(a.r.cell + off + rr);
            const double2 fr = __ldg(fr_all + off + rr);
            const double2 v = __ldg(val_all + off + rr);
            const int cu = (int)(cell & 0xFFFFu) - 32768 - K;
            const int cv = (int)(cell >> 16) - 32768 - K;
            // j + 0.5 - pos == (j - cell) + 0.5 - frac, the same rounded value
            // as the reference's u_dist (w-stacking.cu:85,89)
            double e = 0.0;
            if (is_u) {
                const double d = off1d - fr.x;
                e = norm * exp(-(d * d) * 0.5);
            } else if (is_v) {
                const double d = off1d - fr.y;
                e = exp(-(d * d) * 0.5);
            }
#pragma unroll
            for (int r = 0; r < ROUNDS; r++) {
                const double gu = __shfl_sync(0xFFFFFFFFu, e, odj[r]);
                const double gv = __shfl_sync(0xFFFFFFFFu, e, (NT + odk[r]) & 31);
                const int x = cu + odj[r];
                const int y = cv + odk[r];
                if ((unsigned)x < (unsigned)tx && (unsigned)y < (unsigned)ty) {
                    const double wgt = gu * gv;
                    atomicAdd(sre + y * PITCH + x, wgt * v.x);
                    atomicAdd(sim + y * PITCH + x, wgt * v.y);
                }
            }
        }
        __syncthreads();
        for (int c = tid; c < T * T; c += kThreads) {
            const int y = c / T, x = c % T;
            const int idx = y * PITCH + x;
            if (x < tx && y < ty)
                grid[((size_t)w * a.g.ny + (size_t)(v0 + y)) * a.g.nx + (size_t)(u0 + x)] =
                    make_double2(sre[idx], sim[idx]);
            sre[idx] = 0.0;
            sim[idx] = 0.0;
        }
    }
}

template <int T, int K> size_t grid_smem(int prec)
{
    return (size_t)2 * T * (T + 2 * K + 1) * (prec == WSG_FP64 ? sizeof(double) : sizeof(float));
}

template <int T, int K> const void *grid_kernel(int prec)
{
    return prec == WSG_FP64 ? (const void *)k_grid_f64<T, K> : (const void *)k_grid_f32c<T, K>;
}

template <int T>
const void *grid_select(int prec, int half, size_t &smem)
{
    switch (half) {
#define WSG_CASE(KK)                           \
    case KK:                                   \
        smem = grid_smem<T, KK>(prec);         \
        return grid_kernel<T, KK>(prec);
        WSG_CASE(0) WSG_CASE(1) WSG_CASE(2) WSG_CASE(3)
        WSG_CASE(4) WSG_CASE(5) WSG_CASE(6) WSG_CASE(7)
#undef WSG_CASE
    }
    return nullptr;
}

const void *grid_pick(int prec, int tile, int half, size_t &smem)
{
    if (tile == 32) return grid_select<32>(prec, half, smem);
    if (tile == 64) return grid_select<64>(prec, half, smem);
    return nullptr;
}

}  // namespace

int grid_max_ctas_per_sm(int prec, int tile, int half)
{
    size_t smem = 0;
    const void *k = grid_pick(prec, tile, half, smem);
    if (!k) return 0;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, kThreads, smem) != cudaSuccess)
        return 0;
    return nb;
}

cudaError_t launch_grid(const GeomParams &g, int prec, const BinBuffers &b, const RecBuffers &r,
                        void *grid, int ctas, int chunk, cudaStream_t s)
{
    size_t smem = 0;
    const void *k = grid_pick(prec, g.tile, g.half, smem);
    if (!k) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    GridArgs a{g, b, r, grid, chunk};
    void *args[] = {&a};
    return cudaLaunchKernel(k, dim3(ctas), dim3(kThreads), args, smem, s);
}

}  // namespace wsg
