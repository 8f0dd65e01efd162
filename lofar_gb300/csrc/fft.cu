// Per-plane 2D FFTs of the FP32C form, fused with the w-correction.
//
// The reference transforms every plane with FFTW (fourier_transform.c:25-59)
// and then applies the w-term phase and sums the planes
// (phase_correction.cu:36-80).  A generic 2D FFT reads and writes every plane
// several times; here the transforms are shaped by what the gridder knows:
//
//   forward (grid -> image):
//     k_cols<FWD>   column FFTs (exponent +i) of each plane; tiles that
//                   received no measurement are zero and are not read; a
//                   plane's columns whose tile column is empty stay zero and
//                   are skipped;
//     k_rows_wc     for one image row, all planes in turn: row FFT, then the
//                   w-term phase and the plane sum in registers (the next
//                   plane's row is prefetched meanwhile); the image row is
//                   written once.  The FFT'd planes never reach HBM.
//   adjoint (image -> grid):
//     k_rows_wc_adj for one image row, all planes in turn: conjugate phase,
//                   row FFT (exponent -i), and only the columns that the
//                   degridder will read are written;
//     k_cols<ADJ>   column FFTs of those columns; only the tiles the
//                   degridder reads (tiles with measurements and their
//                   neighbours) are written.
//
// 1D transforms run in shared memory: Stockham passes of radix 16 (a 4x4
// decomposition in registers) and one final radix-2/4/8 pass, lengths
// 256..8192.  Shared-memory index i is stored at i + i/16 so that the
// butterfly strides hit distinct banks.  Twiddles come from a per-plan table
// of e^{2 pi i m/N} computed in FP64 and rounded once to float.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstring>

#include "wsg_internal.cuh"

namespace wsg {

namespace {

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// a * (s i): s = +1 (exponent +i) or -1
template <int S> __device__ __forceinline__ float2 mul_si(float2 a)
{
    return S > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// 4-point DFT in place, X[k] = sum a[n] e^{S 2 pi i nk/4}
template <int S> __device__ __forceinline__ void dft4(float2 &a0, float2 &a1, float2 &a2, float2 &a3)
{
    const float2 t0 = cadd(a0, a2), t1 = csub(a0, a2);
    const float2 t2 = cadd(a1, a3), t3 = mul_si<S>(csub(a1, a3));
    a0 = cadd(t0, t2);
    a2 = csub(t0, t2);
    a1 = cadd(t1, t3);
    a3 = csub(t1, t3);
}

template <int S> __device__ __forceinline__ void dft2(float2 &a0, float2 &a1)
{
    const float2 t = a0;
    a0 = cadd(t, a1);
    a1 = csub(t, a1);
}

// e^{S 2 pi i m / 16}, m = 0..15 (cos/sin of multiples of 22.5 degrees)
template <int S> __device__ __forceinline__ float2 w16(int m)
{
    const float c1 = 0.92387953251128675613f, s1 = 0.38268343236508977173f,
                r2 = 0.70710678118654752440f;
    float c, s;
    switch (m & 15) {
    case 0: c = 1.f; s = 0.f; break;
    case 1: c = c1; s = s1; break;
    case 2: c = r2; s = r2; break;
    case 3: c = s1; s = c1; break;
    case 4: c = 0.f; s = 1.f; break;
    case 5: c = -s1; s = c1; break;
    case 6: c = -r2; s = r2; break;
    case 7: c = -c1; s = s1; break;
    case 8: c = -1.f; s = 0.f; break;
    case 9: c = -c1; s = -s1; break;
    case 10: c = -r2; s = -r2; break;
    case 11: c = -s1; s = -c1; break;
    case 12: c = 0.f; s = -1.f; break;
    case 13: c = s1; s = -c1; break;
    case 14: c = r2; s = -r2; break;
    default: c = c1; s = -s1; break;
    }
    return make_float2(c, S > 0 ? s : -s);
}

// 16-point DFT in registers: n = 4 n1 + n2, k = k1 + 4 k2.
template <int S> __device__ __forceinline__ void dft16(float2 (&x)[16])
{
#pragma unroll
    for (int n2 = 0; n2 < 4; n2++) dft4<S>(x[n2], x[4 + n2], x[8 + n2], x[12 + n2]);
    // now x[4 k1 + n2] = y[n2][k1]; apply W16^{n2 k1}
#pragma unroll
    for (int n2 = 1; n2 < 4; n2++)
#pragma unroll
        for (int k1 = 1; k1 < 4; k1++) x[4 * k1 + n2] = cmul(x[4 * k1 + n2], w16<S>(n2 * k1));
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) dft4<S>(x[4 * k1], x[4 * k1 + 1], x[4 * k1 + 2], x[4 * k1 + 3]);
    // x[4 k1 + k2] = X[k1 + 4 k2]: transpose the 4x4 index to natural order
    float2 t[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++)
#pragma unroll
        for (int k2 = 0; k2 < 4; k2++) t[k1 + 4 * k2] = x[4 * k1 + k2];
#pragma unroll
    for (int i = 0; i < 16; i++) x[i] = t[i];
}

template <int S, int R> __device__ __forceinline__ void dft_small(float2 (&x)[16])
{
    if constexpr (R == 2) {
        dft2<S>(x[0], x[1]);
    } else if constexpr (R == 4) {
        dft4<S>(x[0], x[1], x[2], x[3]);
    } else if constexpr (R == 8) {
        // 8 = 2 x 4: n = 2 n1 + n2, k = k1 + 4 k2
        dft4<S>(x[0], x[2], x[4], x[6]);
        dft4<S>(x[1], x[3], x[5], x[7]);
        const float r2 = 0.70710678118654752440f;
        const float2 w1 = make_float2(r2, S > 0 ? r2 : -r2);
        x[3] = cmul(x[3], w1);
        x[5] = mul_si<S>(x[5]);
        x[7] = cmul(x[7], make_float2(-r2, S > 0 ? r2 : -r2));
        // pairs (y[0][k1], y[1][k1]) are (x[2 k1], x[2 k1 + 1])
        float2 t[8];
#pragma unroll
        for (int k1 = 0; k1 < 4; k1++) {
            float2 a = x[2 * k1], b = x[2 * k1 + 1];
            dft2<S>(a, b);
            t[k1] = a;
            t[k1 + 4] = b;
        }
#pragma unroll
        for (int i = 0; i < 8; i++) x[i] = t[i];
    }
}

__device__ __forceinline__ int pidx(int i) { return i + (i >> 4); }

template <int N> struct FftPlan {
    static constexpr int L16 = N >= 4096 ? 3 : (N >= 256 ? 2 : 1);
    static constexpr int R = N / (L16 == 3 ? 4096 : (L16 == 2 ? 256 : 16));   // last radix
    static constexpr int PAD = N + N / 16;
};

// One length-N transform in shared memory buf (padded), with the T threads
// t0..t0+T-1 of the CTA (T <= N/16, a divisor of it).  Sign S of the exponent.
// Caller synchronises before (data in buf) and after (results in buf).
template <int N, int S, int T>
__device__ __forceinline__ void fft_smem(float2 *buf, int t, const float2 *__restrict__ tw)
{
    constexpr int L16 = FftPlan<N>::L16;
    constexpr int R = FftPlan<N>::R;
    int ns = 1;
#pragma unroll
    for (int p = 0; p < L16; p++) {
        float2 x[16][N / 16 / T];
#pragma unroll
        for (int b = 0; b < N / 16 / T; b++) {
            const int j = t + b * T;
            const int k = j % ns;
#pragma unroll
            for (int r = 0; r < 16; r++) x[r][b] = buf[pidx(j + r * (N / 16))];
            if (ns > 1) {
                // W^{r k} for r = 1..15 from one table entry W^k: powers by a
                // product tree of depth <= 4 (a few ulp), instead of 15 loads
                float2 w1 = __ldg(tw + k * (N / (16 * ns)));
                if (S < 0) w1.y = -w1.y;
                float2 wp[16];
                wp[1] = w1;
                wp[2] = cmul(w1, w1);
                wp[3] = cmul(wp[2], w1);
                wp[4] = cmul(wp[2], wp[2]);
#pragma unroll
                for (int r = 5; r < 8; r++) wp[r] = cmul(wp[4], wp[r - 4]);
                wp[8] = cmul(wp[4], wp[4]);
#pragma unroll
                for (int r = 9; r < 12; r++) wp[r] = cmul(wp[8], wp[r - 8]);
                wp[12] = cmul(wp[8], wp[4]);
#pragma unroll
                for (int r = 13; r < 16; r++) wp[r] = cmul(wp[12], wp[r - 12]);
#pragma unroll
                for (int r = 1; r < 16; r++) x[r][b] = cmul(x[r][b], wp[r]);
            }
        }
        __syncthreads();
#pragma unroll
        for (int b = 0; b < N / 16 / T; b++) {
            const int j = t + b * T;
            const int k = j % ns;
            float2 y[16];
#pragma unroll
            for (int r = 0; r < 16; r++) y[r] = x[r][b];
            dft16<S>(y);
            const int base = (j / ns) * ns * 16 + k;
#pragma unroll
            for (int r = 0; r < 16; r++) buf[pidx(base + r * ns)] = y[r];
        }
        __syncthreads();
        ns *= 16;
    }
    if constexpr (R > 1) {
        constexpr int NB = N / R;   // butterflies of the last pass
        constexpr int BPT = (NB + T - 1) / T;
        float2 x[R][BPT];
#pragma unroll
        for (int b = 0; b < BPT; b++) {
            const int j = t + b * T;
            if (j < NB) {
                const int k = j % ns;
                const int step = N / (R * ns);
#pragma unroll
                for (int r = 0; r < R; r++) {
                    float2 v = buf[pidx(j + r * NB)];
                    if (r > 0) {
                        float2 w = __ldg(tw + (r * k * step) % N);
                        if (S < 0) w.y = -w.y;
                        v = cmul(v, w);
                    }
                    x[r][b] = v;
                }
            }
        }
        __syncthreads();
#pragma unroll
        for (int b = 0; b < BPT; b++) {
            const int j = t + b * T;
            if (j < NB) {
                const int k = j % ns;
                float2 y[16];
#pragma unroll
                for (int r = 0; r < R; r++) y[r] = x[r][b];
                dft_small<S, R>(y);
                const int base = (j / ns) * ns * R + k;
#pragma unroll
                for (int r = 0; r < R; r++) buf[pidx(base + r * ns)] = y[r];
            }
        }
        __syncthreads();
    }
}


// Twiddle powers W^{r k}, r = 0..15, of one table entry W^k (a product tree
// of depth <= 4, a few ulp).
template <int S> __device__ __forceinline__ void twiddle_powers(float2 w1, float2 (&wp)[16])
{
    if (S < 0) w1.y = -w1.y;
    wp[0] = make_float2(1.f, 0.f);
    wp[1] = w1;
    wp[2] = cmul(w1, w1);
    wp[3] = cmul(wp[2], w1);
    wp[4] = cmul(wp[2], wp[2]);
#pragma unroll
    for (int r = 5; r < 8; r++) wp[r] = cmul(wp[4], wp[r - 4]);
    wp[8] = cmul(wp[4], wp[4]);
#pragma unroll
    for (int r = 9; r < 12; r++) wp[r] = cmul(wp[8], wp[r - 8]);
    wp[12] = cmul(wp[8], wp[4]);
#pragma unroll
    for (int r = 13; r < 16; r++) wp[r] = cmul(wp[12], wp[r - 12]);
}

// The same transform for a CTA of T threads whose thread t holds the values
// of indices t + q*T (q < N/T) in registers: with IN_REGS the first radix-16
// pass takes its inputs from v (butterfly j = t + b*T reads indices
// j + r*N/16, i.e. q = b + r*(N/16)/T), and with OUT_REGS the last pass leaves
// its outputs in v in the same layout; shared memory then carries only the
// passes in between.  Without IN_REGS the input is in buf (caller
// synchronises before); without OUT_REGS the output is in buf.  The caller
// synchronises before a call whose first pass writes buf while other threads
// may still read it.
template <int N, int S, int T, bool IN_REGS, bool OUT_REGS>
__device__ __forceinline__ void fft_row(float2 (&v)[N / T], float2 *buf, int t,
                                        const float2 *__restrict__ tw)
{
    constexpr int L16 = FftPlan<N>::L16;
    constexpr int R = FftPlan<N>::R;
    constexpr int NB = N / 16;
    constexpr int BPT = NB / T;
    static_assert(BPT * T == NB, "T divides the butterfly count");
    int ns = 1;
#pragma unroll
    for (int p = 0; p < L16; p++) {
        const bool from_regs = IN_REGS && p == 0;
        const bool to_regs = OUT_REGS && R == 1 && p == L16 - 1;
        float2 x[16][BPT];
#pragma unroll
        for (int b = 0; b < BPT; b++) {
            const int j = t + b * T;
            const int k = j % ns;
#pragma unroll
            for (int r = 0; r < 16; r++) x[r][b] = from_regs ? v[b + r * BPT] : buf[pidx(j + r * NB)];
            if (ns > 1) {
                float2 wp[16];
                twiddle_powers<S>(__ldg(tw + k * (N / (16 * ns))), wp);
#pragma unroll
                for (int r = 1; r < 16; r++) x[r][b] = cmul(x[r][b], wp[r]);
            }
        }
        if (!from_regs && !to_regs) __syncthreads();
#pragma unroll
        for (int b = 0; b < BPT; b++) {
            const int j = t + b * T;
            const int k = j % ns;
            float2 y[16];
#pragma unroll
            for (int r = 0; r < 16; r++) y[r] = x[r][b];
            dft16<S>(y);
            if (to_regs) {
                // ns = N/16: outputs j + r*N/16
#pragma unroll
                for (int r = 0; r < 16; r++) v[b + r * BPT] = y[r];
            } else {
                const int base = (j / ns) * ns * 16 + k;
#pragma unroll
                for (int r = 0; r < 16; r++) buf[pidx(base + r * ns)] = y[r];
            }
        }
        if (!to_regs) __syncthreads();
        ns *= 16;
    }
    if constexpr (R > 1) {
        // ns = N/R: butterflies j < N/R, outputs j + r*N/R
        constexpr int NBR = N / R;
        constexpr int BPR = NBR / T;
        static_assert(BPR * T == NBR, "T divides the last pass");
        float2 x[R][BPR];
#pragma unroll
        for (int b = 0; b < BPR; b++) {
            const int j = t + b * T;
#pragma unroll
            for (int r = 0; r < R; r++) {
                float2 u = buf[pidx(j + r * NBR)];
                if (r > 0) {
                    float2 wv = __ldg(tw + r * j);
                    if (S < 0) wv.y = -wv.y;
                    u = cmul(u, wv);
                }
                x[r][b] = u;
            }
        }
        if (!OUT_REGS) __syncthreads();
#pragma unroll
        for (int b = 0; b < BPR; b++) {
            const int j = t + b * T;
            float2 y[16];
#pragma unroll
            for (int r = 0; r < R; r++) y[r] = x[r][b];
            dft_small<S, R>(y);
#pragma unroll
            for (int r = 0; r < R; r++) {
                if (OUT_REGS) v[b + r * BPR] = y[r];
                else buf[pidx(j + r * NBR)] = y[r];
            }
        }
        if (!OUT_REGS) __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

enum { kColsFwd = 0, kColsAdj = 1, kColsPlain = 2 };

template <int N> __host__ __device__ constexpr int fft_threads() { return N / 16 < 512 ? N / 16 : 512; }
template <int N> __host__ __device__ constexpr int col_group() { return 2; }
// stride between the column buffers: congruent to 16/COLS modulo 16 so that
// the transposing loads (COLS columns of consecutive rows) hit distinct banks
template <int N> __host__ __device__ constexpr int col_stride()
{
    constexpr int pad = FftPlan<N>::PAD;
    constexpr int want = 16 / col_group<N>();
    return pad + ((want - pad % 16) + 16) % 16;
}

struct ColArgs {
    float2 *grid;
    const float2 *tw;
    int nx, ny, tile, ntu, ntv, tsh;   // tsh = log2(tile)
    FftMasks m;
};

// ---- TMA staging of a column strip ---------------------------------------

// Set when a CTA gave up waiting for its strip (the wait is bounded); read
// by fft_tma_timed_out().
__device__ int g_cols_tma_timeout;

constexpr long kTmaWaitLimit = 1l << 22;

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// box {2 complex, rows, 1 plane} at (x, y, z) into shared memory
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z,
                                            unsigned long long *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

// Shared-memory writes of the generic proxy made visible to the tensor memory
// accelerator (each writing thread, before the barrier that precedes a store).
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// box {2 complex, rows, 1 plane} from shared memory to (x, y, z)
__device__ __forceinline__ void tma_store_3d(const CUtensorMap *map, const void *src, int x, int y,
                                             int z)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(
            reinterpret_cast<unsigned long long>(map)),
        "r"(smem_u32(src)), "r"(x), "r"(y), "r"(z)
        : "memory");
}
// Commits this thread's bulk stores and waits until they have read shared memory.
__device__ __forceinline__ void tma_store_commit_and_wait_read()
{
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

// Threads of a column-strip CTA: one per radix-16 butterfly of a column.
template <int N> __host__ __device__ constexpr int col_threads() { return N / 16 < 512 ? N / 16 : 512; }

// 16 complex values of both columns of a strip row: one 16-byte access.
__device__ __forceinline__ float4 ld_row2(const float2 *p) { return __ldcg(reinterpret_cast<const float4 *>(p)); }
__device__ __forceinline__ void st_row2(float2 *p, float2 a, float2 b)
{
    __stcg(reinterpret_cast<float4 *>(p), make_float4(a.x, a.y, b.x, b.y));
}

// Columns per column-FFT CTA (1 or 2).
constexpr int kColsPerCta = 2;

// The transformed strip goes back through shared memory with
// tensor-memory-accelerator stores (one box per tile row written; the adjoint
// writes the tiles the degridder reads) instead of 16-byte stores from every
// thread.
constexpr bool kTmaStoreFwd = true;
constexpr bool kTmaStoreAdj = true;
template <int MODE> __host__ __device__ constexpr bool tma_store_cols()
{
    return MODE == kColsFwd ? kTmaStoreFwd : kTmaStoreAdj;
}

// Column FFTs of a strip of kColsPerCta adjacent columns of one plane (grid: x =
// strip, y = plane).  Thread t owns butterfly t of every radix-16 pass of both
// columns (same twiddles).  The last pass writes its 16 (or R) outputs straight
// back to HBM.  The first pass takes its 16 inputs (rows t + r*N/16):
//   forward   straight from HBM, rows of tiles without measurements being zero
//             and not read;
//   adjoint, plain   from the strip staged in shared memory by the tensor
//             memory accelerator: one thread issues one tile-high box per
//             tile row, the CTA waits on an mbarrier (bounded), and the 16-byte
//             row gathers of the direct loads leave the load/store pipeline.
//             (Staging the sparse forward strips this way measured slower.)
//             The staged kernels run three CTAs per SM (at most 80 registers,
//             a few spilled), the forward two: measured, three made the
//             forward slower and the staged adjoint faster.
// Adjoint: only rows of tiles the degridder reads are written.
template <int N, int S, int MODE>
__global__ void __launch_bounds__(col_threads<N>(), col_threads<N>() <= 256 ? (MODE == kColsFwd ? 2 : 3) : 1) k_cols(ColArgs a, const __grid_constant__ CUtensorMap tmap)
{
    constexpr bool kStaged = MODE != kColsFwd;
    constexpr int NC = kColsPerCta;
    constexpr int T = col_threads<N>();
    constexpr int L16 = FftPlan<N>::L16;
    constexpr int R = FftPlan<N>::R;
    constexpr int NB = N / 16;
    static_assert(NB == T, "one radix-16 butterfly per thread");
    static_assert(L16 >= 2, "at least two radix-16 passes");
    constexpr int SC = col_stride<N>();
    extern __shared__ __align__(128) float2 cbuf[];
    __shared__ __align__(8) unsigned long long s_bar;
    float2 *ca = cbuf, *cb = cbuf + SC;
    const int w = blockIdx.y;
    const int x0 = blockIdx.x * NC;
    const int tu = x0 >> a.tsh;
    if (MODE == kColsFwd && !a.m.occ_col[w * a.ntu + tu]) return;   // strip stays zero
    if (MODE == kColsAdj && !a.m.need_col[w * a.ntu + tu]) return;  // never read
    // this strip's tile-row mask (forward: tiles read; adjoint: tiles written)
    __shared__ unsigned char s_rows[N / 16];
    const int t = threadIdx.x;
    static_assert(!kStaged || NC == 2, "a staged strip is two columns wide");
    if (MODE != kColsPlain)
        for (int tv = t; tv < a.ntv; tv += T)
            s_rows[tv] = MODE == kColsFwd ? a.m.occ_tile[((size_t)w * a.ntv + tv) * a.ntu + tu]
                                          : a.m.need_tile[((size_t)w * a.ntv + tv) * a.ntu + tu];
    if (kStaged && t == 0) mbar_init(&s_bar);
    __syncthreads();
    float2 *col = a.grid + (size_t)w * a.ny * a.nx + x0;
    const size_t pitch = (size_t)a.nx;
    float4 *stage = reinterpret_cast<float4 *>(cbuf);   // row r at stage[r]

    if constexpr (kStaged) {
        const int nbox = N >> a.tsh;
        if (t == 0) {
            mbar_expect_tx(&s_bar, (unsigned)(nbox * a.tile) * 16u);
            for (int b = 0; b < nbox; b++)
                tma_load_3d(stage + b * a.tile, &tmap, x0, b * a.tile, w, &s_bar);
        }
        bool done = false;
        for (long it = 0; it < kTmaWaitLimit && !done; ++it) done = mbar_try_wait(&s_bar, 0);
        if (!done) {
            atomicExch(&g_cols_tma_timeout, 1);
            // the copies may still be in flight: wait for them (bounded) before leaving
            for (long it = 0; it < kTmaWaitLimit && !done; ++it) done = mbar_try_wait(&s_bar, 0);
        }
        if (__syncthreads_or(!done)) return;   // the whole CTA gives up together
    }

    // pass 0 (no twiddles): rows t + r*NB, outputs to 16t + r
    {
        float2 xa[16], xb[16];
#pragma unroll
        for (int r = 0; r < 16; r++) {
            const int row = t + r * NB;
            if (kStaged) {
                const float4 v = stage[row];
                xa[r] = make_float2(v.x, v.y);
                xb[r] = make_float2(v.z, v.w);
            } else if (NC == 2) {
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (s_rows[row >> a.tsh]) v = ld_row2(col + (size_t)row * pitch);
                xa[r] = make_float2(v.x, v.y);
                xb[r] = make_float2(v.z, v.w);
            } else {
                xa[r] = make_float2(0.f, 0.f);
                if (s_rows[row >> a.tsh]) xa[r] = __ldcg(col + (size_t)row * pitch);
            }
        }
        dft16<S>(xa);
        if (NC == 2) dft16<S>(xb);
        if (kStaged) __syncthreads();   // the strip is read: ca/cb overwrite it
#pragma unroll
        for (int r = 0; r < 16; r++) {
            ca[pidx(16 * t + r)] = xa[r];
            if (NC == 2) cb[pidx(16 * t + r)] = xb[r];
        }
    }
    __syncthreads();
    int ns = 16;
#pragma unroll
    for (int p = 1; p < L16; p++) {
        const bool last = (p == L16 - 1) && R == 1;
        const int k = t % ns;
        float2 xa[16], xb[16], wp[16];
        twiddle_powers<S>(__ldg(a.tw + k * (N / (16 * ns))), wp);
#pragma unroll
        for (int r = 0; r < 16; r++) {
            xa[r] = cmul(ca[pidx(t + r * NB)], wp[r]);
            if (NC == 2) xb[r] = cmul(cb[pidx(t + r * NB)], wp[r]);
        }
        dft16<S>(xa);
        if (NC == 2) dft16<S>(xb);
        if (last) {
            // t / ns == 0: outputs go to rows t + r*ns = t + r*NB
            if constexpr (tma_store_cols<MODE>() && NC == 2) {
                __syncthreads();   // every thread has read ca/cb, which the strip overwrites
#pragma unroll
                for (int r = 0; r < 16; r++)
                    stage[t + r * NB] = make_float4(xa[r].x, xa[r].y, xb[r].x, xb[r].y);
                fence_proxy_async_smem();
                __syncthreads();
                if (t == 0) {
                    const int nbox = N >> a.tsh;
                    for (int b = 0; b < nbox; b++)
                        if (MODE != kColsAdj || s_rows[b])
                            tma_store_3d(&tmap, stage + b * a.tile, x0, b * a.tile, w);
                    tma_store_commit_and_wait_read();
                }
            } else {
#pragma unroll
                for (int r = 0; r < 16; r++) {
                    const int row = t + r * NB;
                    if (MODE != kColsAdj || s_rows[row >> a.tsh]) {
                        if (NC == 2) st_row2(col + (size_t)row * pitch, xa[r], xb[r]);
                        else __stcg(col + (size_t)row * pitch, xa[r]);
                    }
                }
            }
        } else {
            __syncthreads();
            const int base = (t / ns) * ns * 16 + k;
#pragma unroll
            for (int r = 0; r < 16; r++) {
                ca[pidx(base + r * ns)] = xa[r];
                if (NC == 2) cb[pidx(base + r * ns)] = xb[r];
            }
            __syncthreads();
        }
        ns *= 16;
    }
    if constexpr (R > 1) {
        // last pass, radix R: ns = N/R, butterflies j < N/R, outputs to rows j + r*N/R
        constexpr int NBR = N / R;
        constexpr int BPT = NBR / T;
#pragma unroll
        for (int b = 0; b < BPT; b++) {
            const int j = t + b * T;
            float2 xa[16], xb[16];
#pragma unroll
            for (int r = 0; r < R; r++) {
                float2 va = ca[pidx(j + r * NBR)];
                float2 vb = NC == 2 ? cb[pidx(j + r * NBR)] : make_float2(0.f, 0.f);
                if (r > 0) {
                    float2 wv = __ldg(a.tw + r * j);   // W_N^{r j}: k = j, step 1
                    if (S < 0) wv.y = -wv.y;
                    va = cmul(va, wv);
                    if (NC == 2) vb = cmul(vb, wv);
                }
                xa[r] = va;
                xb[r] = vb;
            }
            dft_small<S, R>(xa);
            if (NC == 2) dft_small<S, R>(xb);
#pragma unroll
            for (int r = 0; r < R; r++) {
                const int row = j + r * NBR;
                if (MODE != kColsAdj || s_rows[row >> a.tsh]) {
                    if (NC == 2) st_row2(col + (size_t)row * pitch, xa[r], xb[r]);
                    else __stcg(col + (size_t)row * pitch, xa[r]);
                }
            }
        }
    }
}

struct RowArgs {
    float2 *grid;     // [jobs][P][ny][nx]
    float2 *image;    // [jobs][ny][nx]
    const float2 *tw;
    int nx, ny, planes, tile, ntu, phase, tsh;   // planes: P, of one job
    WScreen ws;
    float scale;
    FftMasks m;
};

// Forward: one image row.  For every plane: row FFT (exponent +i), w-term
// phase, plane sum.  Grid: y = image row.
template <int N>
__global__ void __launch_bounds__(fft_threads<N>()) k_rows_wc(RowArgs a)
{
    constexpr int T = fft_threads<N>();
    constexpr int Q = N / T;   // pixels per thread
    extern __shared__ __align__(16) unsigned char rsm[];
    float2 *buf = reinterpret_cast<float2 *>(rsm);
    // the row's w-screen: Q32 cycle fractions (aq, bq) per pixel
    uint2 *wq = reinterpret_cast<uint2 *>(rsm + ((FftPlan<N>::PAD * 8 + 15) / 16) * 16);
    const int y = blockIdx.x, t = threadIdx.x;
    const size_t prow = (size_t)y * N;
    // job blockIdx.y: its planes, masks and image
    const size_t jp = (size_t)blockIdx.y * a.planes;
    const float2 *gridj = a.grid + jp * a.ny * N;
    const unsigned char *plane_occ = a.m.plane_occ + jp;
    float2 *image = a.image + (size_t)blockIdx.y * a.ny * N;
    if (a.phase)
        for (int x = t; x < N; x += T) wq[x] = make_uint2(a.ws.aq[prow + x], a.ws.bq[prow + x]);
    unsigned char *smask = reinterpret_cast<unsigned char *>(wq + N);   // [planes][ntu]
    for (int i = t; i < a.planes * a.ntu; i += T) smask[i] = a.m.occ_col[jp * a.ntu + i];
    __syncthreads();
    float sr[Q], si[Q];
#pragma unroll
    for (int q = 0; q < Q; q++) sr[q] = si[q] = 0.f;
    // the next occupied plane's row is loaded into registers while the
    // current one is transformed
    int w = 0;
    while (w < a.planes && !plane_occ[w]) w++;
    float2 nxt[Q];
    auto fetch = [&](int ww) {
        const float2 *src = gridj + ((size_t)ww * a.ny + y) * N;
#pragma unroll
        for (int q = 0; q < Q; q++) {
            const int x = t + q * T;
            nxt[q] = smask[ww * a.ntu + (x >> a.tsh)] ? __ldcs(src + x) : make_float2(0.f, 0.f);
        }
    };
    if (w < a.planes) fetch(w);
    while (w < a.planes) {
        float2 fv[Q];
#pragma unroll
        for (int q = 0; q < Q; q++) fv[q] = nxt[q];
        int wn = w + 1;
        while (wn < a.planes && !plane_occ[wn]) wn++;
        if (wn < a.planes) fetch(wn);
        __syncthreads();   // the previous plane's last pass has read buf
        fft_row<N, +1, T, true, true>(fv, buf, t, a.tw);   // the row in and out of registers
#pragma unroll
        for (int q = 0; q < Q; q++) {
            const int x = t + q * T;
            const float2 v = fv[q];
            if (a.phase) {
                const uint2 c = wq[x];
                float sn, cs;
                __sincosf(wscreen_angle(c.x, c.y, (unsigned)w), &sn, &cs);
                sr[q] += v.x * cs - v.y * sn;
                si[q] += v.x * sn + v.y * cs;
            } else {
                sr[q] += v.x;
                si[q] += v.y;
            }
        }
        w = wn;
    }
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const int x = t + q * T;
        const float amp = a.phase ? a.ws.amp[prow + x] * a.scale : a.scale;
        image[prow + x] = make_float2(sr[q] * amp, si[q] * amp);
    }
}

// Adjoint: one image row.  For every plane the degridder reads: conjugate
// phase, row FFT (exponent -i), store the columns it reads.
template <int N>
__global__ void __launch_bounds__(fft_threads<N>()) k_rows_wc_adj(RowArgs a)
{
    constexpr int T = fft_threads<N>();
    constexpr int Q = N / T;
    extern __shared__ __align__(16) unsigned char rsm[];
    float2 *buf = reinterpret_cast<float2 *>(rsm);
    // the row's w-screen: Q32 cycle fractions (aq, bq) per pixel
    uint2 *wq = reinterpret_cast<uint2 *>(rsm + ((FftPlan<N>::PAD * 8 + 15) / 16) * 16);
    const int y = blockIdx.x, t = threadIdx.x;
    const size_t prow = (size_t)y * N;
    const size_t jp = (size_t)blockIdx.y * a.planes;
    float2 *gridj = a.grid + jp * a.ny * N;
    const unsigned char *plane_need = a.m.plane_need + jp;
    const float2 *image = a.image + (size_t)blockIdx.y * a.ny * N;
    if (a.phase)
        for (int x = t; x < N; x += T) wq[x] = make_uint2(a.ws.aq[prow + x], a.ws.bq[prow + x]);
    unsigned char *smask = reinterpret_cast<unsigned char *>(wq + N);   // [planes][ntu]
    for (int i = t; i < a.planes * a.ntu; i += T) smask[i] = a.m.need_col[jp * a.ntu + i];
    float2 im[Q];
#pragma unroll
    for (int q = 0; q < Q; q++) {
        const int x = t + q * T;
        const float2 v = image[prow + x];
        float amp = a.phase ? a.ws.amp[prow + x] * a.scale : a.scale;
        if (!(amp == amp)) {
            // pixels where the forward is NaN are excluded: zero value (the
            // image may hold NaN there) and a zero phase (their w-screen
            // entries are NaN too)
            im[q] = make_float2(0.f, 0.f);
            if (a.phase) wq[x] = make_uint2(0u, 0u);
        } else {
            im[q] = make_float2(v.x * amp, v.y * amp);
        }
    }
    __syncthreads();   // shared w-screen and masks loaded
    for (int w = 0; w < a.planes; w++) {
        if (!plane_need[w]) continue;
        float2 fv[Q];   // the phased row, then (in place) its transform
#pragma unroll
        for (int q = 0; q < Q; q++) {
            const int x = t + q * T;
            float2 v = im[q];
            if (a.phase) {
                const uint2 c = wq[x];
                float sn, cs;
                __sincosf(wscreen_angle(c.x, c.y, (unsigned)w), &sn, &cs);
                v = make_float2(cs * im[q].x + sn * im[q].y, cs * im[q].y - sn * im[q].x);
            }
            fv[q] = v;
        }
        __syncthreads();   // the previous plane's last pass has read buf
        fft_row<N, -1, T, true, true>(fv, buf, t, a.tw);
        float2 *dst = gridj + ((size_t)w * a.ny + y) * N;
#pragma unroll
        for (int q = 0; q < Q; q++) {
            const int x = t + q * T;
            if (smask[w * a.ntu + (x >> a.tsh)]) __stcg(dst + x, fv[q]);
        }
    }
}

// Plain row FFTs of every row of every plane (grid: x = row, y = plane).
template <int N, int S>
__global__ void __launch_bounds__(fft_threads<N>()) k_rows_plain(float2 *grid, const float2 *tw,
                                                                  int ny)
{
    constexpr int T = fft_threads<N>();
    extern __shared__ __align__(16) float2 pbuf[];
    float2 *row = grid + ((size_t)blockIdx.y * ny + blockIdx.x) * N;
    for (int x = threadIdx.x; x < N; x += T) pbuf[pidx(x)] = __ldcg(row + x);
    __syncthreads();
    fft_smem<N, S, T>(pbuf, threadIdx.x, tw);
    for (int x = threadIdx.x; x < N; x += T) __stcg(row + x, pbuf[pidx(x)]);
}

// Tile masks from the bin table, one CTA per plane.
__global__ void k_fft_masks(BinBuffers b, int ntu, int ntv, FftMasks m)
{
    extern __shared__ unsigned char msm[];
    unsigned char *occ = msm, *prim = msm + ntu * ntv;
    __shared__ int s_any_occ, s_any_need;
    const int w = blockIdx.x, tid = threadIdx.x;
    const int nt = ntu * ntv;
    if (tid == 0) s_any_occ = s_any_need = 0;
    for (int i = tid; i < nt; i += blockDim.x) {
        const size_t bin = (size_t)w * nt + i;
        occ[i] = b.ntotal[bin] > 0;
        prim[i] = b.nprim[bin] > 0;
        m.occ_tile[bin] = occ[i];
    }
    __syncthreads();
    for (int i = tid; i < nt; i += blockDim.x) {
        const int tv = i / ntu, tu = i % ntu;
        unsigned char nd = 0;
        for (int dv = -1; dv <= 1; dv++)
            for (int du = -1; du <= 1; du++) {
                const int v = tv + dv, u = tu + du;
                if (v >= 0 && v < ntv && u >= 0 && u < ntu && prim[v * ntu + u]) nd = 1;
            }
        m.need_tile[(size_t)w * nt + i] = nd;
        if (nd) s_any_need = 1;
        if (occ[i]) s_any_occ = 1;
    }
    __syncthreads();
    for (int tu = tid; tu < ntu; tu += blockDim.x) {
        unsigned char o = 0, nd = 0;
        for (int tv = 0; tv < ntv; tv++) {
            o |= occ[tv * ntu + tu];
            nd |= m.need_tile[(size_t)w * nt + tv * ntu + tu];
        }
        m.occ_col[w * ntu + tu] = o;
        m.need_col[w * ntu + tu] = nd;
    }
    if (tid == 0) {
        m.plane_occ[w] = (unsigned char)s_any_occ;
        m.plane_need[w] = (unsigned char)s_any_need;
    }
}

__global__ void k_twiddles(float2 *tw, int n)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m < n) {
        double s, c;
        sincospi(2.0 * (double)m / (double)n, &s, &c);
        tw[m] = make_float2((float)c, (float)s);
    }
}

template <int N> size_t col_smem() { return (size_t)kColsPerCta * col_stride<N>() * sizeof(float2); }
template <int N> size_t row_smem(int planes, int ntu)
{
    return ((FftPlan<N>::PAD * 8 + 15) / 16) * 16 + (size_t)N * sizeof(uint2) +
           (size_t)planes * ntu;
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
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

// The cube [planes][ny][nx] of 8-byte complex values as a 3D tensor; a box is
// 2 values (16 bytes) wide, one tile high, one plane deep.
cudaError_t cols_tensor_map(const ColArgs &a, int planes, CUtensorMap *m)
{
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return cudaErrorNotSupported;
    if (a.nx % 2 || ((unsigned long long)(size_t)a.grid & 15) || a.tile > 256)
        return cudaErrorInvalidValue;
    const cuuint64_t dims[3] = {(cuuint64_t)a.nx, (cuuint64_t)a.ny, (cuuint64_t)planes};
    const cuuint64_t strides[2] = {(cuuint64_t)a.nx * 8, (cuuint64_t)a.nx * a.ny * 8};
    const cuuint32_t box[3] = {2, (cuuint32_t)a.tile, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, a.grid, dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

template <int N, int S, int MODE>
cudaError_t run_cols(const ColArgs &a, int planes, cudaStream_t s)
{
    const size_t smem = col_smem<N>();
    cudaError_t e = cudaFuncSetAttribute(k_cols<N, S, MODE>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    CUtensorMap m;
    memset(&m, 0, sizeof(m));   // unused by a forward without tensor stores
    if (MODE != kColsFwd || kTmaStoreFwd) {
        e = cols_tensor_map(a, planes, &m);
        if (e != cudaSuccess) return e;
    }
    k_cols<N, S, MODE><<<dim3(a.nx / kColsPerCta, planes), col_threads<N>(),
                         smem, s>>>(a, m);
    return cudaGetLastError();
}

template <int N> cudaError_t run_rows_wc(const RowArgs &a, int jobs, bool adjoint, cudaStream_t s)
{
    const size_t smem = row_smem<N>(a.planes, a.ntu);
    const void *k = adjoint ? (const void *)k_rows_wc_adj<N> : (const void *)k_rows_wc<N>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    RowArgs ra = a;
    void *args[] = {&ra};
    return cudaLaunchKernel(k, dim3(a.ny, jobs), dim3(fft_threads<N>()), args, smem, s);
}

template <int N, int S> cudaError_t run_rows_plain(float2 *grid, const float2 *tw, int ny,
                                                   int planes, cudaStream_t s)
{
    const size_t smem = ((FftPlan<N>::PAD * 8 + 15) / 16) * 16;
    cudaError_t e = cudaFuncSetAttribute(k_rows_plain<N, S>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_rows_plain<N, S><<<dim3(ny, planes), fft_threads<N>(), smem, s>>>(grid, tw, ny);
    return cudaGetLastError();
}

int tile_shift(int tile)
{
    int sh = 0;
    while ((1 << sh) < tile) sh++;
    return sh;
}

#define WSG_FFT_SIZES(X) X(256) X(512) X(1024) X(2048) X(4096) X(8192)

template <int S, int MODE> cudaError_t cols_dispatch(int n, const ColArgs &a, int planes,
                                                     cudaStream_t s)
{
    switch (n) {
#define WSG_C(NN) case NN: return run_cols<NN, S, MODE>(a, planes, s);
        WSG_FFT_SIZES(WSG_C)
#undef WSG_C
    }
    return cudaErrorInvalidValue;
}

cudaError_t rows_wc_dispatch(int n, const RowArgs &a, int jobs, bool adjoint, cudaStream_t s)
{
    switch (n) {
#define WSG_C(NN) case NN: return run_rows_wc<NN>(a, jobs, adjoint, s);
        WSG_FFT_SIZES(WSG_C)
#undef WSG_C
    }
    return cudaErrorInvalidValue;
}

template <int S> cudaError_t rows_plain_dispatch(int n, float2 *grid, const float2 *tw, int ny,
                                                 int planes, cudaStream_t s)
{
    switch (n) {
#define WSG_C(NN) case NN: return run_rows_plain<NN, S>(grid, tw, ny, planes, s);
        WSG_FFT_SIZES(WSG_C)
#undef WSG_C
    }
    return cudaErrorInvalidValue;
}

}  // namespace

bool fft_fused_supported(int nx, int ny, int tile)
{
    auto ok = [](int n) { return n >= 256 && n <= 8192 && (n & (n - 1)) == 0; };
    return ok(nx) && ok(ny) && tile > 0 && (tile & (tile - 1)) == 0 && nx % tile == 0 &&
           ny % tile == 0;
}

cudaError_t launch_twiddles(float2 *tw, int n, cudaStream_t s)
{
    k_twiddles<<<(n + 255) / 256, 256, 0, s>>>(tw, n);
    return cudaGetLastError();
}

cudaError_t launch_fft_masks(const GeomParams &g, const BinBuffers &b, const FftMasks &m,
                             cudaStream_t s)
{
    const size_t smem = (size_t)2 * g.ntu * g.ntv;
    cudaError_t e = cudaFuncSetAttribute(k_fft_masks, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    k_fft_masks<<<g.planes, 512, smem, s>>>(b, g.ntu, g.ntv, m);
    return cudaGetLastError();
}

cudaError_t launch_image_fwd_fused(const GeomParams &g, float2 *grid, float2 *image,
                                   const float2 *twx, const float2 *twy, const WScreen &ws,
                                   const FftMasks &m, bool phase, double scale, cudaStream_t s)
{
    ColArgs c{grid, twy, g.nx, g.ny, g.tile, g.ntu, g.ntv, tile_shift(g.tile), m};
    cudaError_t e = cols_dispatch<+1, kColsFwd>(g.ny, c, g.planes, s);
    if (e != cudaSuccess) return e;
    RowArgs r{grid, image, twx, g.nx, g.ny, g.wplanes, g.tile, g.ntu, phase ? 1 : 0,
              tile_shift(g.tile), ws, (float)scale, m};
    return rows_wc_dispatch(g.nx, r, g.planes / g.wplanes, false, s);
}

cudaError_t launch_image_adj_fused(const GeomParams &g, const float2 *image, float2 *grid,
                                   const float2 *twx, const float2 *twy, const WScreen &ws,
                                   const FftMasks &m, bool phase, double scale, cudaStream_t s)
{
    RowArgs r{grid, const_cast<float2 *>(image), twx, g.nx, g.ny, g.wplanes, g.tile, g.ntu,
              phase ? 1 : 0, tile_shift(g.tile), ws, (float)scale, m};
    cudaError_t e = rows_wc_dispatch(g.nx, r, g.planes / g.wplanes, true, s);
    if (e != cudaSuccess) return e;
    ColArgs c{grid, twy, g.nx, g.ny, g.tile, g.ntu, g.ntv, tile_shift(g.tile), m};
    return cols_dispatch<-1, kColsAdj>(g.ny, c, g.planes, s);
}

cudaError_t launch_fft2d_plain(const GeomParams &g, float2 *grid, const float2 *twx,
                               const float2 *twy, int sign, cudaStream_t s)
{
    FftMasks none{};
    ColArgs c{grid, twy, g.nx, g.ny, g.tile, g.ntu, g.ntv, tile_shift(g.tile), none};
    cudaError_t e = sign > 0 ? cols_dispatch<+1, kColsPlain>(g.ny, c, g.planes, s)
                             : cols_dispatch<-1, kColsPlain>(g.ny, c, g.planes, s);
    if (e != cudaSuccess) return e;
    return sign > 0 ? rows_plain_dispatch<+1>(g.nx, grid, twx, g.ny, g.planes, s)
                    : rows_plain_dispatch<-1>(g.nx, grid, twx, g.ny, g.planes, s);
}

bool fft_tma_timed_out()
{
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_cols_tma_timeout, sizeof(v)) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return v != 0;
}

}  // namespace wsg
