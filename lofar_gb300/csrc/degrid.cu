// Degridding (the adjoint of the gridder; the reference has none).
//
// For every measurement m gridded by the last binning,
//     out[m] = sum_{(j,k) in window(m)} c_m(j,k) * grid[plane(m)][k][j]
// with the gridder's clipped window and real Gaussian weights c_m, which is
// exactly the transpose of the map V_m -> grid of w-stacking.cu:59-117.
//
// It reuses the gridder's sort: a persistent CTA takes a (plane, tile) bin,
// stages the tile plus a halo from HBM into shared memory once (cells off the
// grid read as zero), then gathers the bin's primary records.  Duplicate
// records of the bin are not visited: the halo makes every primary's window
// local.
//   FP32C: the tile + halo arrives by TMA (below; plain loads on odd-width
//   grids), records are staged kStageD at a time; a group of 8 (or 16) lanes
//   takes a contiguous stream of the stage, one record at a time, lane k its
//   row k: the row sum over the NT columns uses the column weights shuffled
//   from the group's lanes and the window row, kept in registers while the
//   records stay in one cell; the row weight is applied once, and a shuffle
//   tree over the group sums the rows.  Records binned by the [dump][baseline]
//   walk get their values stored in record order (vrec) and gathered back to
//   measurement order by the walk (k_walk_gather); others are stored at
//   their measurement's index.
//   FP64: the same group-per-record layout, with the FP64 weights of
//   taps64.cuh (several records per warp-wide exponential pass).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstring>

#include "fixed64.cuh"
#include "taps64.cuh"
#include "wsg_internal.cuh"

namespace wsg {

namespace {

// Records staged per pass: 384 (with the TMA-staged tile of support 7, four
// CTAs fit an SM, against three with 512).
constexpr int kStageD = 384;

struct DegridArgs {
    GeomParams g;
    BinBuffers b;
    RecBuffers r;
    const void *grid;
    void *out;
};

// ---- TMA staging of the tile + halo -------------------------------------
//
// FP32C on grids of even width: one thread loads the tile and its halo as one
// 3D box (the tensor memory accelerator zero-fills the cells off the grid) and
// the CTA waits on an mbarrier with a bounded try_wait loop; the per-cell
// loads, bounds tests and shared-memory stores of the plain staging go away.

// Set when a CTA gave up waiting for its tile (read by degrid_tma_timed_out).
__device__ int g_degrid_tma_timeout;
constexpr long kDegridWaitLimit = 1l << 22;

__device__ __forceinline__ unsigned smem_u32d(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ bool mbar_try_wait_d(unsigned long long *bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32d(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Shared-memory pitch (complex values) of the TMA-staged tile: even (a TMA
// box row is a multiple of 16 bytes) and 2 mod 4, so that the rows of one
// record's window start in distinct 8-byte banks for up to 8 rows.  An even
// pitch cannot separate more rows, so supports above 7 (9..15 rows) keep the
// plain staging and its odd pitch: measured, TMA with the even pitch made
// support 9 14 % slower.
template <int AW> __host__ __device__ constexpr int tma_pitch() { return (AW % 4 == 2) ? AW : AW + (AW % 2 ? 1 : 2 + (AW % 4 == 0 ? 0 : 2)); }

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


// Work item -> (bin, primaries [p0, p1)): the split items, then the occupied
// bins that are not split (empty bins hold no primaries to degrid).
__device__ __forceinline__ bool work_item_d(const BinBuffers &b, unsigned item, unsigned nsplit,
                                            unsigned &bin, unsigned &p0, unsigned &p1)
{
    unsigned chunk = 0;
    if (item < nsplit) {
        const unsigned long long e = b.split[item];
        bin = (unsigned)(e & 0xFFFFFFFFull);
        chunk = (unsigned)(e >> 32);
    } else {
        bin = b.work[item - nsplit];   // occupied bins that are not split
    }
    const unsigned nprim = b.nprim[bin];
    if (item < nsplit) {
        p0 = min(nprim, chunk * b.split_size);
        p1 = min(nprim, p0 + b.split_size);
    } else {
        p0 = 0;
        p1 = nprim;
    }
    return p1 > p0;
}

template <int T, int K, bool TMA>
__global__ void __launch_bounds__(kThreads) k_degrid_f32c(DegridArgs a, const __grid_constant__ CUtensorMap tmap)
{
    constexpr int NT = 2 * K + 1;
    constexpr int GS = NT <= 8 ? 8 : 16;   // lanes per record (power of two)
    constexpr int RPW = 32 / GS;
    constexpr int H = 2 * K;
    constexpr int AW = T + 2 * H;
    constexpr int PW = tma_pitch<AW>();
    constexpr int AP0 = AW | 1;
    constexpr int NW = kThreads / 32;
    constexpr int NS = NW * RPW;           // record streams per stage
    constexpr int AP = TMA ? PW : AP0;
    constexpr int TB = TMA ? (AW * PW * 8 + 127) / 128 * 128 : (AW * AP0 * 8 + 15) / 16 * 16;
    extern __shared__ __align__(TMA ? 128 : 16) unsigned char smraw[];
    float2 *tile = reinterpret_cast<float2 *>(smraw);
    uint4 *stage = reinterpret_cast<uint4 *>(smraw + TB);
    unsigned *sidx = reinterpret_cast<unsigned *>(smraw + TB + kStageD * sizeof(uint4));
    __shared__ unsigned s_item;
    __shared__ __align__(8) unsigned long long s_bar;
    unsigned phase = 0;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int grp = lane / GS, k = lane % GS;
    const bool on = k < NT;
    const int kk = on ? k : NT - 1;
    const float norm = (float)(0.5 / kRefPi);
    const float c2 = -0.72134752044448170368f;   // -0.5 * log2(e)
    const float off1 = (float)(kk - K) + 0.5f;
    const float2 *__restrict__ grid = reinterpret_cast<const float2 *>(a.grid);
    float2 *out = reinterpret_cast<float2 *>(a.out);
    float2 *vrec = a.r.vrec;   // set: values in record order (the walk gathers them)
    const unsigned nsplit = a.b.ctr->nsplit_items;
    const unsigned nitems = nsplit + a.b.ctr->nwork;
    if (TMA && tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32d(&s_bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }

    for (;;) {
        __syncthreads();
        if (tid == 0) s_item = atomicAdd(&a.b.ctr->work_degrid, 1u);
        __syncthreads();
        const unsigned item = s_item;
        if (item >= nitems) break;
        unsigned bin, p0, p1;
        if (!work_item_d(a.b, item, nsplit, bin, p0, p1)) continue;
        int w, u0, v0;
        decode_bin_d(a.g, bin, w, u0, v0);
        const unsigned off = a.b.off[bin];
        const size_t plane = (size_t)w * a.g.ny;
        if constexpr (TMA) {
            // one box: PW x AW values at (u0 - H, v0 - H) of plane w; cells
            // off the grid read as zero
            if (tid == 0) {
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                                 smem_u32d(&s_bar)),
                             "r"((unsigned)(PW * AW * 8))
                             : "memory");
                asm volatile(
                    "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
                    "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32d(tile)),
                    "l"(reinterpret_cast<unsigned long long>(&tmap)), "r"(u0 - H), "r"(v0 - H), "r"(w),
                    "r"(smem_u32d(&s_bar))
                    : "memory");
            }
            bool done = false;
            for (long it = 0; it < kDegridWaitLimit && !done; ++it) done = mbar_try_wait_d(&s_bar, phase);
            if (!done) {
                atomicExch(&g_degrid_tma_timeout, 1);
                for (long it = 0; it < kDegridWaitLimit && !done; ++it) done = mbar_try_wait_d(&s_bar, phase);
            }
            phase ^= 1u;
            if (__syncthreads_or(!done)) return;   // the whole CTA gives up together
        } else {
            for (int i = tid; i < AW * AW; i += kThreads) {
                const int y = i / AW, x = i - (i / AW) * AW;
                const int gy = v0 - H + y, gx = u0 - H + x;
                float2 val = make_float2(0.f, 0.f);
                if (gx >= 0 && gx < a.g.nx && gy >= 0 && gy < a.g.ny)
                    val = grid[(plane + (size_t)gy) * a.g.nx + (size_t)gx];
                tile[y * AP + x] = val;
            }
        }
        for (unsigned c0 = p0; c0 < p1; c0 += kStageD) {
            const unsigned cnt = min((unsigned)kStageD, p1 - c0);
            __syncthreads();
            for (unsigned i = tid; i < cnt; i += kThreads) {
                stage[i] = __ldcs(a.r.rec16 + off + c0 + i);
                if (!vrec) sidx[i] = __ldcs(a.r.idx + off + c0 + i);
            }
            __syncthreads();
            // each group takes a contiguous stream of the stage; lane k keeps
            // row k of its record's window in registers and reloads it only
            // when the cell changes (records of one track share cells)
            const unsigned len = (cnt + NS - 1) / NS;
            const unsigned sbeg = (unsigned)(warp * RPW + grp) * len;
            float2 win[NT];
            int wrow = -1;   // tile offset of the row held in win
            for (unsigned t = 0; t < len; t++) {
                const unsigned r = sbeg + t;
                const bool valid = r < cnt;
                const uint4 q = stage[valid ? r : 0];
                const int cu = (int)(q.x >> 24) - 64;
                const int cv = (int)(q.y >> 24) - 64;
                const float fu = (float)(q.x & 0xFFFFFFu) * 1.1920928955078125e-7f - 1.0f;
                const float fv = (float)(q.y & 0xFFFFFFu) * 1.1920928955078125e-7f - 1.0f;
                const float du = off1 - fu, dv = off1 - fv;
                const float gu = norm * fast_exp2(du * du * c2);
                const float gv = on ? fast_exp2(dv * dv * c2) : 0.0f;
                const int row = (cv - K + kk + H) * AP + (cu - K + H);
                if (row != wrow) {
#pragma unroll
                    for (int j = 0; j < NT; j++) win[j] = tile[row + j];
                    wrow = row;
                }
                float sr = 0.f, si = 0.f;
#pragma unroll
                for (int j = 0; j < NT; j++) {
                    const float g = __shfl_sync(0xFFFFFFFFu, gu, grp * GS + j);
                    sr = fmaf(g, win[j].x, sr);
                    si = fmaf(g, win[j].y, si);
                }
                sr *= gv;
                si *= gv;
#pragma unroll
                for (int d = GS / 2; d >= 1; d >>= 1) {
                    sr += __shfl_xor_sync(0xFFFFFFFFu, sr, d);
                    si += __shfl_xor_sync(0xFFFFFFFFu, si, d);
                }
                if (k == 0 && valid) {
                    if (vrec) vrec[off + c0 + r] = make_float2(sr, si);   // record order
                    else out[sidx[r]] = make_float2(sr, si);
                }
            }
        }
    }
}

// The FP64 degridder's CTA: 512 threads, so that the two CTAs whose
// (T + 2K)^2 complex128 tiles fit an SM keep 32 warps resident.
constexpr int kThreadsD64 = 512;

template <int T, int K>
__global__ void __launch_bounds__(kThreadsD64, 2) k_degrid_f64(DegridArgs a)
{
    using P = Taps64<K>;
    constexpr int NT = P::NT;
    constexpr int HW = T + 2 * K;      // tile + halo
    constexpr int SP = T + NT;         // smem pitch (== HW + 1)
    constexpr int NW = kThreadsD64 / 32;
    extern __shared__ unsigned char smraw[];
    double2 *tile = reinterpret_cast<double2 *>(smraw);
    int4 *tfix = reinterpret_cast<int4 *>(smraw);   // the same cells in fixed point
    __shared__ unsigned s_item, s_exp;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int grp = lane / P::G, row = lane % P::G;
    const double2 *__restrict__ grid = reinterpret_cast<const double2 *>(a.grid);
    const double2 *__restrict__ fr_all = reinterpret_cast<const double2 *>(a.r.frac);
    double2 *out = reinterpret_cast<double2 *>(a.out);
    const unsigned nsplit = a.b.ctr->nsplit_items;
    const unsigned nitems = nsplit + a.b.ctr->nwork;
    double nt_u, t_v;
    taps64_consts<K>(lane, 0.5 / kRefPi, nt_u, t_v);
    const long long nt_uq = to_fixed(__double_as_longlong(nt_u), 62);
    const long long t_vq = to_fixed(__double_as_longlong(t_v), 62);

    for (;;) {
        __syncthreads();
        if (tid == 0) {
            s_item = atomicAdd(&a.b.ctr->work_degrid, 1u);
            s_exp = 0u;
        }
        __syncthreads();
        const unsigned item = s_item;
        if (item >= nitems) break;
        unsigned bin, p0, p1;
        if (!work_item_d(a.b, item, nsplit, bin, p0, p1)) continue;
        int w, u0, v0;
        decode_bin_d(a.g, bin, w, u0, v0);
        const unsigned off = a.b.off[bin];
        const size_t plane = (size_t)w * a.g.ny;
        unsigned ex = 0u;
        for (int i = tid; i < HW * HW; i += kThreadsD64) {
            const int y = i / HW, x = i - (i / HW) * HW;
            const int gy = v0 - K + y, gx = u0 - K + x;
            double2 val = make_double2(0.0, 0.0);
            if (gx >= 0 && gx < a.g.nx && gy >= 0 && gy < a.g.ny)
                val = grid[(plane + (size_t)gy) * a.g.nx + (size_t)gx];
            tile[y * SP + x] = val;
            ex = max(ex, max(exp_field(val.x), exp_field(val.y)));
        }
        ex = __reduce_max_sync(0xFFFFFFFFu, ex);
        if (lane == 0) atomicMax(&s_exp, ex);
        __syncthreads();
        // The tile's scale: every |cell| < 2^(e - 1022), so cells times 2^s,
        // s = 61 - (e - 1022), are below 2^61; a tile holding a NaN or an
        // infinity (e = 2047) is gathered in FP64 instead.
        const int e = (int)s_exp;
        const bool fixed = e < 2047;
        const int sc = min(61 - (e - 1022), 1020);
        if (fixed) {
            for (int i = tid; i < HW * HW; i += kThreadsD64) {
                const int y = i / HW, x = i - (i / HW) * HW;
                const double2 val = tile[y * SP + x];
                const Half64 hr = split64(to_fixed(__double_as_longlong(val.x), sc));
                const Half64 hi = split64(to_fixed(__double_as_longlong(val.y), sc));
                tfix[y * SP + x] = make_int4(hr.h, hr.l, hi.h, hi.l);
            }
            __syncthreads();
        }
        for (unsigned base = p0 + warp * P::RE; base < p1; base += NW * P::RE) {
            const unsigned cnt = min((unsigned)P::RE, p1 - base);
            const Exps64 E = taps64_exps(fr_all + off + base, cnt, lane);
            const Exps64Q EQ = taps64_exps_q60(E);
#pragma unroll
            for (int s = 0; s < P::SUB; s++) {
                const int r = s * P::R + grp;
                unsigned cell = 0, idx = 0;
                if ((unsigned)r < cnt) {
                    cell = __ldg(a.r.cell + off + base + r);
                    idx = __ldg(a.r.idx + off + base + r);
                }
                // window origin in halo-tile coordinates: (cell - K) - (-K) = cell;
                // lane `row` sums row `row` of the window
                const int cu = (int)(cell & 0xFFFFu) - 32768;
                const int y = (int)(cell >> 16) - 32768 + row;
                const bool on = (unsigned)r < cnt && row < NT && (unsigned)y < (unsigned)HW;
                double2 o;
                if (fixed) {
                    // sum_j (cell 2^s)(gu 2^62) / 2^64, times (gv 2^62) / 2^64:
                    // the result carries 2^(s-4); partial sums stay below 2^63
                    long long guq, gvq;
                    taps64_factors_q<K>(EQ, r, lane, nt_uq, t_vq, guq, gvq);
                    const Half64 u = split64(guq);
                    const Half64 g = split64(gvq);
                    long long sr = 0, si = 0;
#pragma unroll
                    for (int j = 0; j < NT; j++) {
                        const int src = grp * P::G + j;
                        const Half64 uj = {__shfl_sync(0xFFFFFFFFu, u.h, src),
                                           __shfl_sync(0xFFFFFFFFu, u.l, src)};
                        const int x = cu + j;
                        if (on && (unsigned)x < (unsigned)HW) {
                            const int4 t = tfix[y * SP + x];
                            sr += mulhi_bal({t.x, t.y}, uj);
                            si += mulhi_bal({t.z, t.w}, uj);
                        }
                    }
                    sr = mulhi_bal(split64(sr), g);
                    si = mulhi_bal(split64(si), g);
#pragma unroll
                    for (int d = P::G / 2; d >= 1; d >>= 1) {
                        sr += __shfl_xor_sync(0xFFFFFFFFu, sr, d);
                        si += __shfl_xor_sync(0xFFFFFFFFu, si, d);
                    }
                    o = make_double2(__longlong_as_double(from_fixed(sr, 4 - sc)),
                                     __longlong_as_double(from_fixed(si, 4 - sc)));
                } else {
                    double gu, gv;
                    taps64_factors<K>(E, r, lane, nt_u, t_v, gu, gv);
                    double sr = 0.0, si = 0.0;
#pragma unroll
                    for (int j = 0; j < NT; j++) {
                        const double gj = __shfl_sync(0xFFFFFFFFu, gu, grp * P::G + j);
                        const int x = cu + j;
                        if (on && (unsigned)x < (unsigned)HW) {
                            const double2 t = tile[y * SP + x];
                            sr = fma(gj, t.x, sr);
                            si = fma(gj, t.y, si);
                        }
                    }
                    sr *= gv;
                    si *= gv;
#pragma unroll
                    for (int d = P::G / 2; d >= 1; d >>= 1) {
                        sr += __shfl_xor_sync(0xFFFFFFFFu, sr, d);
                        si += __shfl_xor_sync(0xFFFFFFFFu, si, d);
                    }
                    o = make_double2(sr, si);
                }
                if (row == 0 && (unsigned)r < cnt) out[idx] = o;
            }
        }
    }
}

// TMA staging serves supports up to 7 (window rows in distinct banks).
constexpr int kDegridTmaMaxHalf = 3;

template <int T, int K> size_t degrid_smem(int prec, bool tma)
{
    if (prec == WSG_FP64) return (size_t)(T + 2 * K) * (T + 2 * K + 1) * sizeof(double2);
    constexpr int AW = T + 4 * K;
    constexpr int AP = AW | 1;
    constexpr int PW = tma_pitch<AW>();
    const size_t tile = tma ? ((size_t)AW * PW * 8 + 127) / 128 * 128
                            : ((size_t)AW * AP * 8 + 15) / 16 * 16;
    return tile + (size_t)kStageD * (sizeof(uint4) + sizeof(unsigned));
}

template <int T, int K> const void *degrid_kernel(int prec, bool tma)
{
    if (prec == WSG_FP64) return (const void *)k_degrid_f64<T, K>;
    if constexpr (K <= kDegridTmaMaxHalf)
        if (tma) return (const void *)k_degrid_f32c<T, K, true>;
    return (const void *)k_degrid_f32c<T, K, false>;
}

template <int T>
const void *degrid_select(int prec, int half, bool tma, size_t &smem)
{
    tma = tma && prec != WSG_FP64 && half <= kDegridTmaMaxHalf;
    switch (half) {
#define WSG_CASE(KK)                           \
    case KK:                                   \
        smem = degrid_smem<T, KK>(prec, tma);  \
        return degrid_kernel<T, KK>(prec, tma);
        WSG_CASE(0) WSG_CASE(1) WSG_CASE(2) WSG_CASE(3)
        WSG_CASE(4) WSG_CASE(5) WSG_CASE(6) WSG_CASE(7)
#undef WSG_CASE
    }
    return nullptr;
}

const void *degrid_pick(int prec, int tile, int half, bool tma, size_t &smem)
{
    if (tile == 32) return degrid_select<32>(prec, half, tma, smem);
    if (tile == 64) return degrid_select<64>(prec, half, tma, smem);
    return nullptr;
}

PFN_cuTensorMapEncodeTiled_v12000 degrid_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = []() {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// The complex64 cube as a 3D tensor with a (tile + halo) box; false when the
// grid cannot be described (odd width, unaligned base): the kernel then
// stages with plain loads.
bool degrid_tensor_map(const GeomParams &g, const void *grid, CUtensorMap *m)
{
    PFN_cuTensorMapEncodeTiled_v12000 enc = degrid_encoder();
    if (!enc || (g.nx % 2) || ((size_t)grid & 15)) return false;
    const int aw = g.tile + 4 * g.half;
    int pw = aw;
    switch (g.tile * 1000 + g.half) {   // tma_pitch<AW>() of the instantiated kernels
#define WSG_PW(T, K) case T * 1000 + K: pw = tma_pitch<T + 4 * K>(); break;
        WSG_PW(32, 0) WSG_PW(32, 1) WSG_PW(32, 2) WSG_PW(32, 3) WSG_PW(32, 4) WSG_PW(32, 5)
        WSG_PW(32, 6) WSG_PW(32, 7) WSG_PW(64, 0) WSG_PW(64, 1) WSG_PW(64, 2) WSG_PW(64, 3)
        WSG_PW(64, 4) WSG_PW(64, 5) WSG_PW(64, 6) WSG_PW(64, 7)
#undef WSG_PW
    default: return false;
    }
    if (pw > 256 || aw > 256) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)g.nx, (cuuint64_t)g.ny, (cuuint64_t)g.planes};
    const cuuint64_t strides[2] = {(cuuint64_t)g.nx * 8, (cuuint64_t)g.nx * g.ny * 8};
    const cuuint32_t box[3] = {(cuuint32_t)pw, (cuuint32_t)aw, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<void *>(grid), dims, strides, box,
               estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

int degrid_max_ctas_per_sm(int prec, int tile, int half)
{
    size_t smem = 0;
    const void *k = degrid_pick(prec, tile, half, true, smem);
    if (!k) return 0;
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
        return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &nb, k, prec == WSG_FP64 ? kThreadsD64 : kThreads, smem) != cudaSuccess)
        return 0;
    return nb;
}

bool degrid_tma_timed_out()
{
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_degrid_tma_timeout, sizeof(v)) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return v != 0;
}

cudaError_t launch_degrid(const GeomParams &g, int prec, const BinBuffers &b, const RecBuffers &r,
                          const void *grid, void *out, long long n, int ctas, cudaStream_t s,
                          bool walked)
{
    walked = walked && prec != WSG_FP64 && r.pos && r.vrec;
    CUtensorMap m;
    memset(&m, 0, sizeof(m));
    const bool tma = prec != WSG_FP64 && g.half <= kDegridTmaMaxHalf &&
                     degrid_tensor_map(g, grid, &m);
    size_t smem = 0;
    const void *k = degrid_pick(prec, g.tile, g.half, tma, smem);
    if (!k) return cudaErrorInvalidValue;
    const size_t esz = prec == WSG_FP64 ? sizeof(double2) : sizeof(float2);
    cudaError_t e = cudaSuccess;
    // the walk's gather writes every output; otherwise measurements without
    // a record (dropped) read zero
    if (!walked) e = cudaMemsetAsync(out, 0, (size_t)n * esz, s);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    DegridArgs a{g, b, r, grid, out};
    if (!walked) a.r.vrec = nullptr;
    if (prec == WSG_FP64) {
        void *args[] = {&a};
        return cudaLaunchKernel(k, dim3(ctas), dim3(kThreadsD64), args, smem, s);
    }
    void *args[] = {&a, &m};
    e = cudaLaunchKernel(k, dim3(ctas), dim3(kThreads), args, smem, s);
    if (e != cudaSuccess || !walked) return e;
    return launch_walk_gather(g, n, r.pos, r.vrec, reinterpret_cast<float2 *>(out), s);
}

}  // namespace wsg
