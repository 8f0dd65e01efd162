// FP64-accurate per-plane 2D FFT on the integer pipe (power-of-two edges
// 256..8192): the FP64 form's replacement for a Z2Z library FFT, which on
// this part is bound by the FP64 issue rate.
//
// Each 1D transform (a column, then a row) is block floating point:
//   * the transform is staged in shared memory and its largest component
//     fixes a power of two 2^s that brings every component below 2^61; the
//     values are converted to signed 64-bit integers (round to nearest);
//   * Stockham autosort passes (one radix-2 pass first when log2 N is odd,
//     then radix-4 passes; Govindaraju et al., "High performance discrete
//     Fourier transforms on graphics processors", SC 2008) run on the
//     integers with twiddles in Q62; a radix-2 pass halves and a radix-4
//     pass quarters its inputs (rounded), so the modulus of every value
//     stays below 2^61.5 and nothing overflows;
//   * the result is converted back to FP64 and scaled by the exact power of
//     two 2^(log2 N - s).
// Every transform keeps about 50 significant bits relative to its largest
// output (the largest output is at least the largest input times 2^-log2 N
// of the block scale), which is within the FP64 form's 1e-12 bar.
// A transform holding a NaN or an infinity is written as NaN, as every
// output of a DFT of such an input is non-finite.  An all-zero transform is
// left in place untouched (its DFT is zero).
//
// The FFT is unnormalised, like FFTW's: sign +1 is exponent +i.
#include <cuda_runtime.h>

#include "fixed64.cuh"
#include "wsg_internal.cuh"

namespace wsg {
namespace {

template <int N> struct Fft64Shape {
    static constexpr int L = N == 256 ? 8 : N == 512 ? 9 : N == 1024 ? 10 : N == 2048 ? 11
                           : N == 4096 ? 12 : 13;
    static constexpr int IPT = 2;                       // radix-4 items per thread
    static constexpr int TPT = N / (4 * IPT);           // threads per transform
    static constexpr int NTR = N >= 4096 ? 1 : 4096 / N;   // transforms per CTA
    static constexpr int THREADS = TPT * NTR;
    static constexpr int MINB = 65536 / (THREADS * 64);     // CTAs per SM at 64 registers
    static constexpr bool R2 = (L & 1) != 0;            // leading radix-2 pass
    static constexpr int NP = NTR > 1 ? N + 1 : N;      // padded stride between transforms
    static constexpr size_t SMEM = (size_t)NTR * NP * sizeof(longlong2);
};

// (x * w) / 4 for the Q62 twiddle w = c + i s, stored as balanced 32-bit
// halves {ch, cl, sh, sl} (c = ch 2^32 + cl, cl in [-2^31, 2^31)).  With x
// split the same way, x w / 2^64 = xh wh + (xh wl + xl wh) / 2^32 + xl wl / 2^64:
// the last term (below 1/4) is dropped and the middle sums of both parts are
// rounded, so the error is below one unit and unbiased.  For moduli below
// 2^61.5 the middle sums stay below 2^62.6.  Six 32x32->64 multiply-adds
// per part instead of four 64-bit high products.
__device__ __forceinline__ longlong2 cmul_quarter(longlong2 x, int4 w)
{
    const int rl = (int)(unsigned)x.x, il = (int)(unsigned)x.y;
    const int rh = (int)(x.x >> 32) + (int)((unsigned)x.x >> 31);
    const int ih = (int)(x.y >> 32) + (int)((unsigned)x.y >> 31);
    const long long mre = (1ll << 31) + (long long)rh * w.y + (long long)rl * w.x -
                          (long long)ih * w.w - (long long)il * w.z;
    const long long mim = (1ll << 31) + (long long)rh * w.w + (long long)rl * w.z +
                          (long long)ih * w.y + (long long)il * w.x;
    return make_longlong2((long long)rh * w.x - (long long)ih * w.z + (mre >> 32),
                          (long long)rh * w.z + (long long)ih * w.x + (mim >> 32));
}

__device__ __forceinline__ longlong2 add2(longlong2 a, longlong2 b)
{
    return make_longlong2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ longlong2 sub2(longlong2 a, longlong2 b)
{
    return make_longlong2(a.x - b.x, a.y - b.y);
}
// a / 2^K rounded to nearest (ties up)
template <int K> __device__ __forceinline__ longlong2 shr2(longlong2 a)
{
    return make_longlong2((a.x + (1ll << (K - 1))) >> K, (a.y + (1ll << (K - 1))) >> K);
}

// Radix-4 Stockham pass over the transform `a` (N values) with span NS:
// item j takes a[j + r N/4], r = 0..3, twiddles e^{SIGN 2 pi i r k / (4 NS)}
// with k = j mod NS, and writes a[(j / NS) 4 NS + k + q NS].  The thread
// takes items lt + m TPT, m = 0..IPT-1.  Scales by 1/4, on the inputs (the Q62
// twiddle product is x w / 4; the untwiddled inputs are shifted): moduli
// below 2^61.5 stay below 2^61.5, and the partial sums below 2^62.  `tw`
// holds the twiddles of this transform's sign.
template <int N, int NS, int SIGN>
__device__ __forceinline__ void pass4(longlong2 *a, int lt, const int4 *__restrict__ tw)
{
    using S = Fft64Shape<N>;
    longlong2 x[4 * S::IPT];
#pragma unroll
    for (int m = 0; m < S::IPT; m++)
#pragma unroll
        for (int r = 0; r < 4; r++) x[4 * m + r] = a[lt + m * S::TPT + r * (N / 4)];
    __syncthreads();
#pragma unroll
    for (int m = 0; m < S::IPT; m++) {
        const int j = lt + m * S::TPT;
        const int k = j % NS;
        longlong2 y0 = shr2<2>(x[4 * m]), y1, y2, y3;
        if (NS == 1) {
            y1 = shr2<2>(x[4 * m + 1]);
            y2 = shr2<2>(x[4 * m + 2]);
            y3 = shr2<2>(x[4 * m + 3]);
        } else {
            constexpr int STEP = N / (4 * NS);
            y1 = cmul_quarter(x[4 * m + 1], __ldg(tw + k * STEP));
            y2 = cmul_quarter(x[4 * m + 2], __ldg(tw + 2 * k * STEP));
            y3 = cmul_quarter(x[4 * m + 3], __ldg(tw + 3 * k * STEP));
        }
        const longlong2 a0 = add2(y0, y2), a1 = sub2(y0, y2);
        const longlong2 a2 = add2(y1, y3), a3 = sub2(y1, y3);
        // SIGN i a3
        const longlong2 ia3 = SIGN > 0 ? make_longlong2(-a3.y, a3.x) : make_longlong2(a3.y, -a3.x);
        x[4 * m] = add2(a0, a2);
        x[4 * m + 1] = add2(a1, ia3);
        x[4 * m + 2] = sub2(a0, a2);
        x[4 * m + 3] = sub2(a1, ia3);
    }
#pragma unroll
    for (int m = 0; m < S::IPT; m++) {
        const int j = lt + m * S::TPT;
        const int d = (j / NS) * 4 * NS + j % NS;
#pragma unroll
        for (int q = 0; q < 4; q++) a[d + q * NS] = x[4 * m + q];
    }
    __syncthreads();
}

// Leading radix-2 pass (span 1, no twiddles): item j takes a[j], a[j + N/2]
// and writes a[2j], a[2j + 1].  Scales by 1/2.
template <int N>
__device__ __forceinline__ void pass2_first(longlong2 *a, int lt)
{
    using S = Fft64Shape<N>;
    longlong2 x[4 * S::IPT];
#pragma unroll
    for (int m = 0; m < 2 * S::IPT; m++) {
        x[2 * m] = a[lt + m * S::TPT];
        x[2 * m + 1] = a[lt + m * S::TPT + N / 2];
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < 2 * S::IPT; m++) {
        const int j = lt + m * S::TPT;
        a[2 * j] = shr2<1>(add2(x[2 * m], x[2 * m + 1]));
        a[2 * j + 1] = shr2<1>(sub2(x[2 * m], x[2 * m + 1]));
    }
    __syncthreads();
}

template <int N, int NS, int SIGN>
__device__ __forceinline__ void passes4(longlong2 *a, int lt, const int4 *__restrict__ tw)
{
    if constexpr (NS < N) {
        pass4<N, NS, SIGN>(a, lt, tw);
        passes4<N, NS * 4, SIGN>(a, lt, tw);
    }
}

// Element f of the CTA's staging order: transform tt, index i, offset g in
// the plane.  COLS: consecutive f walk along a row (NTR columns), else along
// a row of the transform.
template <int N, bool COLS>
__device__ __forceinline__ void fft64_elem(int f, int first, int nx, int &tt, int &i, size_t &g)
{
    using S = Fft64Shape<N>;
    if (COLS) {
        i = f / S::NTR;
        tt = f - i * S::NTR;
        g = (size_t)i * nx + (size_t)(first + tt);
    } else {
        tt = f / N;
        i = f - tt * N;
        g = (size_t)(first + tt) * nx + (size_t)i;
    }
}

// Block exponent s of a transform from the upper word of its largest |component|.
__device__ __forceinline__ int fft64_shift(unsigned hi)
{
    const int e = (int)(hi >> 20);          // biased exponent: max < 2^(e - 1022)
    return min(61 - (e - 1022), 1000);
}

// One CTA: NTR transforms of length N of plane blockIdx.y.  COLS: columns
// blockIdx.x * NTR + t (element stride nx); else rows (contiguous).  The
// output is scaled by the exact power of two 2^post.
// Tile masks of the adjoint's column pass (the last): only the tiles with
// tile[] set are written, and a tile column with col[] clear is skipped.
struct ColMasks64 {
    const unsigned char *tile;   // [planes][ntv][ntu]
    const unsigned char *col;    // [planes][ntu]
    int ntu, ntv, tsh;
    bool on;
};

template <int N, int SIGN, bool COLS>
__global__ void __launch_bounds__(Fft64Shape<N>::THREADS, Fft64Shape<N>::MINB)
    k_fft64(double2 *__restrict__ data, int nx, int ny, const int4 *__restrict__ tw, int post,
            ColMasks64 mk)
{
    using S = Fft64Shape<N>;
    extern __shared__ longlong2 sm64[];
    __shared__ unsigned s_hi[S::NTR];
    __shared__ int s_any;
    // the column's tile mask (a CTA's NTR <= 16 columns share one tile column)
    __shared__ unsigned char s_tm[N / 16];
    const int tid = threadIdx.x;
    const int t = tid / S::TPT, lt = tid - t * S::TPT;
    const int first = blockIdx.x * S::NTR;
    double2 *base = data + (size_t)blockIdx.y * (size_t)nx * (size_t)ny;
    const bool masked = COLS && mk.on;
    if (masked) {
        const int tu = first >> mk.tsh;
        if (!mk.col[(size_t)blockIdx.y * mk.ntu + tu]) return;   // a column nobody reads
        for (int tv = tid; tv < mk.ntv; tv += S::THREADS)
            s_tm[tv] = mk.tile[((size_t)blockIdx.y * mk.ntv + tv) * mk.ntu + tu];
    }

    if (tid < S::NTR) s_hi[tid] = 0u;
    if (tid == 0) s_any = 0;
    __syncthreads();
    // global -> shared (raw FP64 bits), and each transform's largest |component|
    // (upper words order like the magnitudes at exponent granularity; a
    // biased exponent of 2047 marks NaN and infinity).  Every thread runs
    // 4 IPT iterations.
    unsigned hi = 0u;
    constexpr int PER = N * S::NTR / S::THREADS;   // 4 IPT elements per thread
    double2 ld[PER];
#pragma unroll
    for (int q = 0; q < PER; q++) {   // all loads in flight before the first use
        int tt, i;
        size_t g;
        fft64_elem<N, COLS>(tid + q * S::THREADS, first, nx, tt, i, g);
        ld[q] = base[g];
    }
#pragma unroll
    for (int q = 0; q < PER; q++) {
        int tt, i;
        size_t g;
        fft64_elem<N, COLS>(tid + q * S::THREADS, first, nx, tt, i, g);
        const double2 v = ld[q];
        sm64[tt * S::NP + i] = make_longlong2(__double_as_longlong(v.x), __double_as_longlong(v.y));
        const unsigned h = max((unsigned)(__double_as_longlong(v.x) >> 32) & 0x7FFFFFFFu,
                               (unsigned)(__double_as_longlong(v.y) >> 32) & 0x7FFFFFFFu);
        if (COLS) {
            hi = max(hi, h);   // the thread's elements all belong to transform tid % NTR
        } else {
            // the 32 elements of a warp's iteration belong to one transform
            const unsigned wm = __reduce_max_sync(0xFFFFFFFFu, h);
            if ((tid & 31) == 0) atomicMax(&s_hi[tt], wm);
        }
    }
    if (COLS) {
        // lanes l and l ^ d (d >= NTR) hold the same transform
#pragma unroll
        for (int d = 16; d >= S::NTR; d >>= 1) hi = max(hi, __shfl_xor_sync(0xFFFFFFFFu, hi, d));
        if ((tid & 31) < S::NTR) atomicMax(&s_hi[tid % S::NTR], hi);
    }
    __syncthreads();
    if (tid < S::NTR && s_hi[tid] != 0u) atomicOr(&s_any, 1);
    __syncthreads();
    if (!s_any) return;   // every transform of the CTA is zero: nothing to write

    // FP64 -> integers scaled by 2^s, in place
    const unsigned my_hi = s_hi[t];
    longlong2 *a = sm64 + t * S::NP;
    if (my_hi != 0u && (my_hi >> 20) != 2047u) {
        const int sh = fft64_shift(my_hi);
        for (int i = lt; i < N; i += S::TPT) {
            const longlong2 r = a[i];
            a[i] = make_longlong2(to_fixed(r.x, sh), to_fixed(r.y, sh));
        }
    }
    __syncthreads();

    if constexpr (S::R2) {
        pass2_first<N>(a, lt);
        passes4<N, 2, SIGN>(a, lt, tw);
    } else {
        passes4<N, 1, SIGN>(a, lt, tw);
    }

    // shared -> global in FP64, times 2^(log2 N - s + post)
    for (int f = tid; f < N * S::NTR; f += S::THREADS) {
        int tt, i;
        size_t g;
        fft64_elem<N, COLS>(f, first, nx, tt, i, g);
        const unsigned th = s_hi[tt];
        if (th == 0u) continue;   // zero transform: already zero in place
        if (masked && !s_tm[i >> mk.tsh]) continue;   // a tile nobody reads
        double2 o;
        if ((th >> 20) == 2047u) {
            o.x = o.y = __longlong_as_double(0x7FF8000000000000ll);
        } else {
            const int k = S::L - fft64_shift(th) + post;
            const longlong2 r = sm64[tt * S::NP + i];
            o = make_double2(__longlong_as_double(from_fixed(r.x, k)),
                             __longlong_as_double(from_fixed(r.y, k)));
        }
        base[g] = o;
    }
}

// tw[k] (sign +1) and tw[n + k] (sign -1): e^{+-2 pi i k / n} in Q62 as
// balanced halves {ch, cl, sh, sl}.
__global__ void k_tw64(int4 *tw, int n)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double s, c;
    sincospi(2.0 * (double)k / (double)n, &s, &c);
    const double q = 4611686018427387904.0;   // 2^62
    auto split = [](long long v, int &h, int &l) {
        l = (int)(unsigned)v;
        h = (int)((v - (long long)l) >> 32);
    };
    int ch, cl, sh, sl, nh, nl;
    split(__double2ll_rn(c * q), ch, cl);
    split(__double2ll_rn(s * q), sh, sl);
    split(-__double2ll_rn(s * q), nh, nl);
    tw[k] = make_int4(ch, cl, sh, sl);
    tw[n + k] = make_int4(ch, cl, nh, nl);
}

template <int N, int SIGN, bool COLS>
cudaError_t launch_n(double2 *data, int nx, int ny, int planes, const int4 *tw, int post,
                     cudaStream_t stream, const ColMasks64 &mk)
{
    using S = Fft64Shape<N>;
    auto kern = k_fft64<N, SIGN, COLS>;
    // set on every launch: the attribute belongs to the current device
    const cudaError_t e =
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM);
    if (e != cudaSuccess) return e;
    const int count = COLS ? nx : ny;
    const dim3 grid(count / S::NTR, planes);
    kern<<<grid, S::THREADS, S::SMEM, stream>>>(data, nx, ny, SIGN > 0 ? tw : tw + N, post, mk);
    return cudaGetLastError();
}

template <int SIGN, bool COLS>
cudaError_t launch_dir(double2 *data, int nx, int ny, int planes, const int4 *tw, int post,
                       cudaStream_t stream, const ColMasks64 &mk = ColMasks64{})
{
    switch (COLS ? ny : nx) {
    case 256: return launch_n<256, SIGN, COLS>(data, nx, ny, planes, tw, post, stream, mk);
    case 512: return launch_n<512, SIGN, COLS>(data, nx, ny, planes, tw, post, stream, mk);
    case 1024: return launch_n<1024, SIGN, COLS>(data, nx, ny, planes, tw, post, stream, mk);
    case 2048: return launch_n<2048, SIGN, COLS>(data, nx, ny, planes, tw, post, stream, mk);
    case 4096: return launch_n<4096, SIGN, COLS>(data, nx, ny, planes, tw, post, stream, mk);
    case 8192: return launch_n<8192, SIGN, COLS>(data, nx, ny, planes, tw, post, stream, mk);
    }
    return cudaErrorInvalidValue;
}

}  // namespace

bool fft64_supported(int nx, int ny, long long planes)
{
    auto ok = [](int n) { return n >= 256 && n <= 8192 && (n & (n - 1)) == 0; };
    return ok(nx) && ok(ny) && planes >= 1 && planes <= 65535;   // planes on grid.y
}

cudaError_t build_twiddles64(int4 *tw, int n, cudaStream_t stream)
{
    k_tw64<<<(n + 255) / 256, 256, 0, stream>>>(tw, n);
    return cudaGetLastError();
}

cudaError_t launch_fft64(double2 *data, int nx, int ny, int planes, int sign,
                         const int4 *twx, const int4 *twy, int post, cudaStream_t stream,
                         const FftMasks *masks, int tsh)
{
    ColMasks64 mk{};
    if (masks) {
        mk.ntu = nx >> tsh;
        mk.ntv = ny >> tsh;
        mk.tsh = tsh;
        // a CTA's columns must share one tile column
        if ((1 << tsh) < 16 || mk.ntv > ny / 16) return cudaErrorInvalidValue;
    }
    cudaError_t e;
    if (sign > 0) {
        // (reading only the occupied tiles saved nothing here: the pass is
        // bound by its integer arithmetic, and empty columns are skipped anyway)
        e = launch_dir<1, true>(data, nx, ny, planes, twy, 0, stream);
        if (e == cudaSuccess) e = launch_dir<1, false>(data, nx, ny, planes, twx, post, stream);
    } else if (masks) {
        // rows first, so that the column pass, last, writes only what is read
        mk.tile = masks->need_tile;
        mk.col = masks->need_col;
        mk.on = true;
        e = launch_dir<-1, false>(data, nx, ny, planes, twx, 0, stream);
        if (e == cudaSuccess) e = launch_dir<-1, true>(data, nx, ny, planes, twy, post, stream, mk);
    } else {
        e = launch_dir<-1, true>(data, nx, ny, planes, twy, 0, stream);
        if (e == cudaSuccess) e = launch_dir<-1, false>(data, nx, ny, planes, twx, post, stream);
    }
    return e;
}

}  // namespace wsg
