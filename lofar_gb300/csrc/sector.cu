// v-slab sectoring on the device: the reference's initialize_array()
// (gridding.c:35-86) and the per-sector gather of gridding_data()
// (gridding.c:167-211).  Declared in include/wstack_gb300.h (section 4).
//
// A measurement with v coordinate vv belongs to slab b = (int)(vv*nsectors),
// and also to b+1 (b-1) when it lies within w_supporth of that slab's edge.
// Each slab's list holds its measurements in increasing row order, as the
// reference's second pass appends them.  Here:
//
//   pass 1   each warp takes a chunk of 32*R consecutive rows; per round of 32
//            rows it finds, with ballots, the lanes of each slab (the slab's
//            own rows, plus the rows below it flagged "up" and the rows above
//            it flagged "down") and keeps a per-slab running count in shared
//            memory; at the end it writes count[slab][chunk].
//   scan     one exclusive scan over count[][] flattened slab-major gives
//            every (slab, chunk) its first position in the concatenated
//            lists: slabs in order, chunks in row order within a slab.
//   pass 2   the same rounds again; a row's position in a slab's list is the
//            chunk's start plus the running count plus the number of lower
//            lanes of the same slab in this round.  Stable, hence identical to
//            the reference's lists.
//
// The slab arithmetic is the reference's, operation for operation and
// without contraction (__dmul_rn / __dsub_rn), so membership at a slab edge
// is bit-identical.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "plan.cuh"
#include "wstack_gb300.h"

using namespace wsg;

namespace {

constexpr int kWarps = 8;                       // warps per block
constexpr long long kMaxCounts = 1ll << 26;     // count[][] entries (256 MiB)
constexpr int kScanThreads = 1024, kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

struct SecGeom {
    long long n;       // rows
    int S;             // nsectors
    int yaxis;         // rows of the grid per slab
    double dx, wsh;    // cell size, w_supporth
    int R;             // rounds of 32 rows per warp chunk
    long long T;       // chunks
};

// Slab of one row, and its "up"/"down" flags (gridding.c:45-55).  bad: the
// reference would index histo_send outside [0, nsectors].
__device__ __forceinline__ int slab_of(double v, const SecGeom &g, bool &up, bool &down, bool &bad)
{
    up = down = bad = false;
    const double x = __dmul_rn(v, (double)g.S);
    if (!(x > -1.0 && x < (double)g.S + 1.0)) {   // NaN, or (int) outside [0, S]
        bad = true;
        return 0;
    }
    const int b = (int)x;
    const double updist = __dsub_rn(__dmul_rn((double)((b + 1) * g.yaxis), g.dx), v);
    const double downdist = __dsub_rn(v, __dmul_rn((double)(b * g.yaxis), g.dx));
    up = updist < g.wsh && updist >= 0.0;
    down = downdist < g.wsh && b > 0 && downdist >= 0.0;
    if (up && b + 1 > g.S) {   // histo_send[nsectors + 1]
        bad = true;
        up = false;
    }
    return b;
}

// Lane masks of the slabs this lane's row belongs to: mself (slab b), mup
// (b+1, valid when up), mdown (b-1, valid when down).
struct SlabMasks {
    int b;
    bool valid, up, down;
    unsigned mself, mup, mdown;
};

__device__ __forceinline__ SlabMasks warp_slabs(const double *__restrict__ vv, long long i,
                                                const SecGeom &g, int *bad_flag)
{
    SlabMasks m;
    bool bad = false;
    m.valid = i < g.n;
    m.b = -1;
    m.up = m.down = false;
    if (m.valid) {
        m.b = slab_of(vv[i], g, m.up, m.down, bad);
        if (bad) {
            m.valid = false;
            m.up = m.down = false;
            atomicExch(bad_flag, 1);
        }
    }
    const unsigned full = 0xffffffffu;
    // A[k] = lanes whose slab is b + k - 2
    unsigned a0 = 0, a1 = 0, a2 = 0, a3 = 0, a4 = 0;
    unsigned pending = __ballot_sync(full, m.valid);
    while (pending) {
        const int leader = __ffs(pending) - 1;
        const int x = __shfl_sync(full, m.b, leader);
        const unsigned ax = __ballot_sync(full, m.valid && m.b == x);
        pending &= ~ax;
        const int d = x - m.b;
        a0 = d == -2 ? ax : a0;
        a1 = d == -1 ? ax : a1;
        a2 = d == 0 ? ax : a2;
        a3 = d == 1 ? ax : a3;
        a4 = d == 2 ? ax : a4;
    }
    const unsigned up = __ballot_sync(full, m.up), dn = __ballot_sync(full, m.down);
    m.mself = a2 | (a1 & up) | (a3 & dn);
    m.mup = a3 | (a2 & up) | (a4 & dn);
    m.mdown = a1 | (a0 & up) | (a2 & dn);
    return m;
}

__device__ __forceinline__ bool last_lane(unsigned mask, int lane)
{
    return lane == 31 - __clz(mask);
}

// PASS = 1: count[slab * T + chunk]; PASS = 2: index[] from the scanned counts.
template <int PASS>
__global__ void __launch_bounds__(kWarps * 32)
k_sector(const double *__restrict__ vv, SecGeom g, unsigned *__restrict__ counts,
         long long *__restrict__ index, int *bad_flag)
{
    extern __shared__ unsigned s_cnt[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long chunk = (long long)blockIdx.x * kWarps + warp;
    if (chunk >= g.T) return;   // whole warps only: no later block-wide barrier
    unsigned *cnt = s_cnt + (size_t)warp * (g.S + 1);
    for (int s = lane; s <= g.S; s += 32) cnt[s] = PASS == 1 ? 0u : counts[(long long)s * g.T + chunk];
    __syncwarp();
    const unsigned lt = (1u << lane) - 1u;
    const long long first = chunk * 32ll * g.R;
    for (int r = 0; r < g.R; ++r) {
        const long long i = first + (long long)r * 32 + lane;
        if (first + (long long)r * 32 >= g.n) break;   // warp-uniform
        const SlabMasks m = warp_slabs(vv, i, g, bad_flag);
        if (PASS == 2 && m.valid) {
            index[cnt[m.b] + __popc(m.mself & lt)] = i;
            if (m.up) index[cnt[m.b + 1] + __popc(m.mup & lt)] = i;
            if (m.down) index[cnt[m.b - 1] + __popc(m.mdown & lt)] = i;
        }
        __syncwarp();
        if (m.valid) {
            if (last_lane(m.mself, lane)) cnt[m.b] += __popc(m.mself);
            if (m.up && last_lane(m.mup, lane)) cnt[m.b + 1] += __popc(m.mup);
            if (m.down && last_lane(m.mdown, lane)) cnt[m.b - 1] += __popc(m.mdown);
        }
        __syncwarp();
    }
    if (PASS == 1)
        for (int s = lane; s <= g.S; s += 32) counts[(long long)s * g.T + chunk] = cnt[s];
}

// ---- exclusive scan of unsigned counts (three kernels) -----------------------

__device__ __forceinline__ unsigned block_exclusive_scan(unsigned v, unsigned *s_warp,
                                                         unsigned &total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned w = lane < (int)(blockDim.x >> 5) ? s_warp[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        s_warp[lane] = w;   // inclusive warp totals
    }
    __syncthreads();
    total = s_warp[(blockDim.x >> 5) - 1];
    const unsigned before = warp ? s_warp[warp - 1] : 0u;
    __syncthreads();   // s_warp is reused by the next call
    return before + x - v;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const unsigned *__restrict__ a,
                                                               long long n, unsigned *sums)
{
    __shared__ unsigned s_warp[32];
    const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
    unsigned v = 0;
    for (int k = 0; k < kScanItems; ++k) v += base + k < n ? a[base + k] : 0u;
    unsigned total;
    block_exclusive_scan(v, s_warp, total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_sums(unsigned *sums, int nblocks,
                                                             unsigned *grand_total)
{
    __shared__ unsigned s_warp[32];
    const int per = (nblocks + kScanThreads - 1) / kScanThreads;
    const int b0 = threadIdx.x * per;
    unsigned v = 0;
    for (int k = 0; k < per; ++k) v += b0 + k < nblocks ? sums[b0 + k] : 0u;
    unsigned total;
    unsigned run = block_exclusive_scan(v, s_warp, total);
    for (int k = 0; k < per; ++k)
        if (b0 + k < nblocks) {
            const unsigned t = sums[b0 + k];
            sums[b0 + k] = run;
            run += t;
        }
    if (threadIdx.x == 0) *grand_total = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(unsigned *__restrict__ a, long long n,
                                                              const unsigned *__restrict__ sums)
{
    __shared__ unsigned s_warp[32];
    const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
    unsigned v[kScanItems], t = 0;
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < n ? a[base + k] : 0u;
        t += v[k];
    }
    unsigned total;
    unsigned run = sums[blockIdx.x] + block_exclusive_scan(t, s_warp, total);
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < n) {
            a[base + k] = run;
            run += v[k];
        }
}

// offsets[s] = start of slab s in the lists (s <= S), offsets[S+1] = total
__global__ void k_offsets(const unsigned *__restrict__ scanned, const unsigned *total, SecGeom g,
                          long *__restrict__ offsets)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s <= g.S) offsets[s] = g.T > 0 ? (long)scanned[(long long)s * g.T] : 0;
    if (s == g.S + 1) offsets[s] = (long)*total;
}

// gridding.c:193-211: the slab's rows in reverse list order, v shifted to the slab
__global__ void k_gather(const long *__restrict__ list, long nsec, double vshift, long np, long nfp,
                         const double *__restrict__ uu, const double *__restrict__ vv,
                         const double *__restrict__ ww, const float *__restrict__ wt,
                         const float *__restrict__ vr, const float *__restrict__ vi,
                         double *__restrict__ uus, double *__restrict__ vvs,
                         double *__restrict__ wws, float *__restrict__ wts,
                         float *__restrict__ vrs, float *__restrict__ vis)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < nsec; j += stride) {
        const long long src = list[nsec - 1 - j];
        uus[j] = uu[src];
        vvs[j] = __dsub_rn(vv[src], vshift);
        wws[j] = ww[src];
        for (long p = 0; p < np; ++p) wts[j * np + p] = wt[src * np + p];
        for (long q = 0; q < nfp; ++q) {
            vrs[j * nfp + q] = vr[src * nfp + q];
            vis[j * nfp + q] = vi[src * nfp + q];
        }
    }
}

int check_geometry(long n, long nsectors, int yaxis, double dx, double wsh)
{
    if (n < 0) return set_error(WSG_ERR_ARG, "negative row count");
    if (n > 1000000000L) return set_error(WSG_ERR_UNSUPPORTED, "more than 1e9 rows");
    if (nsectors < 1 || nsectors > WSG_MAX_SECTORS)
        return set_error(WSG_ERR_UNSUPPORTED, "nsectors %ld outside [1, %d]", nsectors,
                         WSG_MAX_SECTORS);
    if (yaxis < 1 || (long long)(nsectors + 1) * yaxis > 2147483647ll)
        return set_error(WSG_ERR_ARG, "yaxis %d invalid for %ld sectors", yaxis, nsectors);
    if (!(dx > 0.0) || !(wsh >= 0.0) || dx != dx || wsh != wsh)
        return set_error(WSG_ERR_ARG, "dx must be positive and w_supporth non-negative");
    return WSG_OK;
}

SecGeom make_geom(long n, long nsectors, int yaxis, double dx, double wsh)
{
    SecGeom g;
    g.n = n;
    g.S = (int)nsectors;
    g.yaxis = yaxis;
    g.dx = dx;
    g.wsh = wsh;
    // rounds per warp chunk: enough that count[][] stays within kMaxCounts,
    // and about 64 K chunks otherwise (fewer counts to write and scan, still
    // several chunks per resident warp)
    const long long r_counts = ((long long)n * (nsectors + 1) + 32ll * kMaxCounts - 1) /
                               (32ll * kMaxCounts);
    const long long r_par = std::min<long long>(64, (long long)n / (32ll * 65536));
    g.R = (int)std::max<long long>(1, std::max(r_counts, r_par));
    g.T = (n + 32ll * g.R - 1) / (32ll * g.R);
    return g;
}

// Pass 1 + scan (+ pass 2 when index != nullptr) into caller's device arrays.
// Scratch: count[][] and the scan's block sums, stream-ordered.
int sector_run(const double *vv, const SecGeom &g, long *offsets, long long *index,
               long capacity, cudaStream_t s)
{
    const long long L = (long long)(g.S + 1) * g.T;
    const int nblk = (int)((L + kScanTile - 1) / kScanTile);
    void *scratch = nullptr;
    const size_t bytes = sizeof(unsigned) * ((size_t)std::max(L, 1ll) + (size_t)nblk + 2) +
                         sizeof(int) * 2;
    WSG_CUDA(cudaMallocAsync(&scratch, bytes, s));
    unsigned *counts = static_cast<unsigned *>(scratch);
    unsigned *sums = counts + std::max(L, 1ll);
    unsigned *total = sums + nblk;
    int *bad = reinterpret_cast<int *>(total + 2);
    cudaError_t e = cudaMemsetAsync(total, 0, sizeof(unsigned) * 2 + sizeof(int) * 2, s);
    const size_t smem = sizeof(unsigned) * kWarps * (size_t)(g.S + 1);
    const unsigned grid = (unsigned)((g.T + kWarps - 1) / kWarps);
    if (e == cudaSuccess && g.T > 0) {
        k_sector<1><<<grid, kWarps * 32, smem, s>>>(vv, g, counts, nullptr, bad);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && L > 0) {
        k_scan_reduce<<<nblk, kScanThreads, 0, s>>>(counts, L, sums);
        k_scan_sums<<<1, kScanThreads, 0, s>>>(sums, nblk, total);
        k_scan_apply<<<nblk, kScanThreads, 0, s>>>(counts, L, sums);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_offsets<<<(g.S + 2 + 255) / 256, 256, 0, s>>>(counts, total, g, offsets);
        e = cudaGetLastError();
    }
    unsigned h_total = 0;
    int h_bad = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_total, total, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    int st = WSG_OK;
    if (e != cudaSuccess)
        st = set_error(WSG_ERR_CUDA, "sectoring: %s", cudaGetErrorString(e));
    else if (h_bad)
        st = set_error(WSG_ERR_ARG, "a v coordinate puts a row outside slabs [0, nsectors] "
                                    "(the reference would index histo_send out of bounds)");
    else if (index && (long long)h_total > capacity)
        st = set_error(WSG_ERR_CAPACITY, "sector lists need %u entries, capacity %ld", h_total,
                       capacity);
    if (st == WSG_OK && index && g.T > 0) {
        k_sector<2><<<grid, kWarps * 32, smem, s>>>(vv, g, counts, index, bad);
        e = cudaGetLastError();
        if (e != cudaSuccess) st = set_error(WSG_ERR_CUDA, "sectoring: %s", cudaGetErrorString(e));
    }
    cudaFreeAsync(scratch, s);
    return st;
}

}  // namespace

extern "C" {

int wsg_sector_count(const double *vv, long n, long nsectors, int yaxis, double dx,
                     double w_supporth, long *offsets, void *stream)
{
    clear_error();
    WSG_TRY(check_geometry(n, nsectors, yaxis, dx, w_supporth));
    if (!offsets || (n > 0 && !vv)) return set_error(WSG_ERR_ARG, "NULL argument");
    const SecGeom g = make_geom(n, nsectors, yaxis, dx, w_supporth);
    return sector_run(vv, g, offsets, nullptr, 0, (cudaStream_t)stream);
}

int wsg_sector_lists(const double *vv, long n, long nsectors, int yaxis, double dx,
                     double w_supporth, long *offsets, long *index, long capacity, void *stream)
{
    clear_error();
    WSG_TRY(check_geometry(n, nsectors, yaxis, dx, w_supporth));
    if (!offsets || (n > 0 && (!vv || (!index && capacity > 0))))
        return set_error(WSG_ERR_ARG, "NULL argument");
    static_assert(sizeof(long) == sizeof(long long), "LP64 is assumed");
    const SecGeom g = make_geom(n, nsectors, yaxis, dx, w_supporth);
    return sector_run(vv, g, offsets, reinterpret_cast<long long *>(index), capacity,
                      (cudaStream_t)stream);
}

int wsg_sector_gather(const long *list, long nsec, long isector, int yaxis, double dx,
                      long freq_per_chan, long polarisations, const double *uu, const double *vv,
                      const double *ww, const float *weights, const float *vis_real,
                      const float *vis_img, double *uus, double *vvs, double *wws,
                      float *weightss, float *visreals, float *visimgs, void *stream)
{
    clear_error();
    if (nsec < 0 || isector < 0 || yaxis < 1 || freq_per_chan < 1 || polarisations < 1)
        return set_error(WSG_ERR_ARG, "invalid sizes");
    if (nsec == 0) return WSG_OK;
    if (!list || !uu || !vv || !ww || !weights || !vis_real || !vis_img || !uus || !vvs || !wws ||
        !weightss || !visreals || !visimgs)
        return set_error(WSG_ERR_ARG, "NULL argument");
    // shift = (double)(dx*yaxis) (gridding.c:91); vvs = vv - isector*shift (:197)
    const double shift = dx * (double)yaxis;
    const double vshift = (double)isector * shift;
    const int threads = 256;
    const int blocks = (int)std::min<long long>((nsec + threads - 1) / threads, 152ll * 16);
    k_gather<<<blocks, threads, 0, (cudaStream_t)stream>>>(
        list, nsec, vshift, polarisations, freq_per_chan * polarisations, uu, vv, ww, weights,
        vis_real, vis_img, uus, vvs, wws, weightss, visreals, visimgs);
    WSG_CUDA(cudaGetLastError());
    return WSG_OK;
}

int wsg_initialize_array(const double *vv, long n, long nsectors, int yaxis, double dx,
                         double w_supporth, long *histo_send, long **sectorarray)
{
    clear_error();
    WSG_TRY(check_geometry(n, nsectors, yaxis, dx, w_supporth));
    if (!histo_send || !sectorarray || (n > 0 && !vv)) return set_error(WSG_ERR_ARG, "NULL argument");
    for (long s = 0; s <= nsectors; ++s) sectorarray[s] = nullptr;
    cudaStream_t s = nullptr;
    WSG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    const bool dev_in = n > 0 && device_accessible(vv);
    double *d_vv = nullptr;
    long *d_off = nullptr, *d_idx = nullptr;
    int st = WSG_OK;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&d_off), sizeof(long) * (nsectors + 2), s);
    if (e == cudaSuccess && n > 0 && !dev_in) {
        e = cudaMallocAsync(reinterpret_cast<void **>(&d_vv), sizeof(double) * n, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_vv, vv, sizeof(double) * n, cudaMemcpyHostToDevice, s);
    }
    const double *src = dev_in ? vv : d_vv;
    std::vector<long> off((size_t)nsectors + 2, 0);
    if (e != cudaSuccess) st = set_error(WSG_ERR_CUDA, "wsg_initialize_array: %s", cudaGetErrorString(e));
    if (st == WSG_OK) {
        const SecGeom g = make_geom(n, nsectors, yaxis, dx, w_supporth);
        // at most 3 entries per row
        const long cap = 3 * n;
        e = cudaMallocAsync(reinterpret_cast<void **>(&d_idx), sizeof(long) * std::max(cap, 1l), s);
        if (e != cudaSuccess) st = set_error(WSG_ERR_CUDA, "wsg_initialize_array: %s", cudaGetErrorString(e));
        if (st == WSG_OK)
            st = sector_run(src, g, d_off, reinterpret_cast<long long *>(d_idx), cap, s);
        if (st == WSG_OK) {
            e = cudaMemcpyAsync(off.data(), d_off, sizeof(long) * (nsectors + 2),
                                cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) st = set_error(WSG_ERR_CUDA, "wsg_initialize_array: %s", cudaGetErrorString(e));
        }
        for (long k = 0; st == WSG_OK && k <= nsectors; ++k) {
            const long cnt = off[k + 1] - off[k];
            histo_send[k] = cnt;
            sectorarray[k] = static_cast<long *>(malloc(sizeof(long) * (cnt > 0 ? cnt : 1)));
            if (!sectorarray[k]) {
                st = set_error(WSG_ERR_NOMEM, "malloc of a sector list");
                break;
            }
            if (cnt > 0) {
                e = cudaMemcpyAsync(sectorarray[k], d_idx + off[k], sizeof(long) * cnt,
                                    cudaMemcpyDeviceToHost, s);
                if (e != cudaSuccess) st = set_error(WSG_ERR_CUDA, "wsg_initialize_array: %s", cudaGetErrorString(e));
            }
        }
        if (st == WSG_OK) {
            e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) st = set_error(WSG_ERR_CUDA, "wsg_initialize_array: %s", cudaGetErrorString(e));
        }
    }
    if (d_idx) cudaFreeAsync(d_idx, s);
    if (d_vv) cudaFreeAsync(d_vv, s);
    if (d_off) cudaFreeAsync(d_off, s);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (st != WSG_OK)
        for (long k = 0; k <= nsectors; ++k) {
            free(sectorarray[k]);
            sectorarray[k] = nullptr;
        }
    return st;
}

}  // extern "C"
