// Fused 2-D FFT stages between images and CAS images (one launch each way).
//
// The reference turns images into CAS images with a pad, an fftshift, a
// forward 2-D FFT, another fftshift and Re+Im (gpuGridder.cpp:520-596), and
// back with FromCAS, shifts, an inverse FFT, a crop and 1/M^2
// (gpuGridder.cpp:432-518).  The general path here runs these as a stage
// kernel, a batched cuFFT and another stage kernel; for power-of-two M <= 256
// and N <= M/2 these kernels do the whole thing per image in shared memory,
// reading the images (or CAS images) once and writing the CAS images (or
// images) once.
//
// Per image (one CTA, 16 warps):
//   images -> CAS images: the N nonzero columns of the shifted, padded image
//     are transformed in pairs (z = a + i b, one complex FFT per pair) along
//     y; then each of the M/2+1 rows v <= M/2 is transformed along x, with
//     the pair split back (A = (Z(v) + conj Z(M-v))/2, B = (Z(v) - conj
//     Z(M-v))/2i), giving F(., v); that writes CAS row shift(v) (Re+Im) and,
//     by Hermitian symmetry, CAS row shift(M-v) (Re-Im of the mirrored
//     entries).
//   CAS images -> images: rows v <= M/2 of the Hermitian spectrum (built from
//     the CAS image as FromCAS does) are inverse-transformed along x, keeping
//     the N output columns of the crop; then pairs of output columns are
//     inverse-transformed along y (the missing rows v > M/2 are conjugates),
//     keeping the N output rows, scaled by 1/M^2.
// Inputs are staged with cp.async: the next image while the rows of the
// current one are transformed, and each warp's next two CAS rows while it
// transforms the current spectrum row.
//
// Each M-point FFT runs on one warp: M = R * 32, lane l holding elements
// R*l .. R*l+R-1.  A 32-point decimation-in-frequency FFT across the lanes
// (shuffles) for each of the R sub-sequences, the twiddle W_M^(n1*k2), then an
// R-point FFT in registers; element br5(l) + 32*k1 ends in lane l, register
// k1.  Twiddles are cos/sin of 2*pi*m/256 evaluated in FP64 on the host (exact
// zeros and ones at the quarter turns) and rounded to FP32.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

#include "gg_common.cuh"
#include "gg_internal.h"

namespace gg {

constexpr int kFftThreads = 512;
constexpr int kFftMaxM = 256;

// e^(-2 pi i m / 256), m = 0..255
struct FftTwiddles {
    float2 w[kFftMaxM];
};

__device__ __forceinline__ int br5(int l) { return (int)(__brev((unsigned)l) >> 27); }

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ float2 tw_at(const FftTwiddles &t, int m, bool inv)
{
    const float2 w = t.w[m];
    return inv ? make_float2(w.x, -w.y) : w;
}

// Per-lane twiddles of warp_fft.
template <int R>
struct LaneTw {
    float2 stage[5]; // W_(2h)^(lane & (h-1)) for h = 16, 8, 4, 2, 1 on the upper lanes, 1 on the lower
    float sign[5];   // -1 on the upper lanes (lane & h), +1 on the lower
    float2 step[R];  // W_M^(n1 * br5(lane))
    float2 reg[R / 2 > 0 ? R / 2 : 1]; // W_R^m, m < R/2 (uniform)
};

template <int R, bool INV>
__device__ __forceinline__ void lane_twiddles(LaneTw<R> &lt, const FftTwiddles &t, int lane)
{
    constexpr int M = R * 32;
#pragma unroll
    for (int st = 0; st < 5; st++) {
        const int h = 16 >> st;
        const bool upper = (lane & h) != 0;
        lt.stage[st] = upper ? tw_at(t, (lane & (h - 1)) * (128 / h), INV) : make_float2(1.0f, 0.0f);
        lt.sign[st] = upper ? -1.0f : 1.0f;
    }
    const int k2 = br5(lane);
#pragma unroll
    for (int n1 = 0; n1 < R; n1++) lt.step[n1] = tw_at(t, n1 * k2 * (kFftMaxM / M), INV);
#pragma unroll
    for (int m = 0; m < (R / 2 > 0 ? R / 2 : 1); m++) lt.reg[m] = tw_at(t, m * (kFftMaxM / R), INV);
}

// R-point FFT in registers: radix-2 decimation in frequency, natural order in
// and out.  Multiplications by 1 are skipped and by -i (+i inverse) are swaps.
template <int R, bool INV>
__device__ __forceinline__ void reg_fft(float2 (&x)[R], const float2 *wr)
{
#pragma unroll
    for (int half = R / 2; half >= 1; half >>= 1) {
#pragma unroll
        for (int blk = 0; blk < R; blk += 2 * half) {
#pragma unroll
            for (int j = 0; j < half; j++) {
                const float2 a = x[blk + j], b = x[blk + j + half];
                x[blk + j] = make_float2(a.x + b.x, a.y + b.y);
                const float2 d = make_float2(a.x - b.x, a.y - b.y);
                const int m = j * (R / (2 * half)); // W_R^m
                if (m == 0) {
                    x[blk + j + half] = d;
                } else if (4 * m == R) {
                    // W_R^(R/4) = -i forward, +i inverse
                    x[blk + j + half] = INV ? make_float2(-d.y, d.x) : make_float2(d.y, -d.x);
                } else {
                    x[blk + j + half] = cmul(d, wr[m]);
                }
            }
        }
    }
    // bit-reversed -> natural order
#pragma unroll
    for (int i = 0; i < R; i++) {
        int r = 0;
#pragma unroll
        for (int b = 1, q = R >> 1; b < R; b <<= 1, q >>= 1)
            if (i & b) r |= q;
        if (r > i) {
            const float2 tmp = x[i];
            x[i] = x[r];
            x[r] = tmp;
        }
    }
}

// M = 32 R point FFT across one warp (forward: W = e^(-2 pi i / M); INV: the
// unnormalised inverse).  In: x[n1] = element R*lane + n1.  Out: x[k1] =
// element br5(lane) + 32*k1.
template <int R, bool INV>
__device__ __forceinline__ void warp_fft(float2 (&x)[R], const LaneTw<R> &lt, int lane)
{
    // lower lane: x + other; upper lane: (other - x) * W.  Both as
    // fma(sign, x, other) (rounds as the add or subtract) times the lane's
    // twiddle, which is exactly 1 on the lower lanes.
#pragma unroll
    for (int st = 0; st < 5; st++) {
        const int h = 16 >> st;
        const float2 w = lt.stage[st];
        const float sg = lt.sign[st];
#pragma unroll
        for (int n1 = 0; n1 < R; n1++) {
            const float ox = __shfl_xor_sync(0xffffffffu, x[n1].x, h);
            const float oy = __shfl_xor_sync(0xffffffffu, x[n1].y, h);
            x[n1] = cmul(make_float2(fmaf(sg, x[n1].x, ox), fmaf(sg, x[n1].y, oy)), w);
        }
    }
#pragma unroll
    for (int n1 = 1; n1 < R; n1++) x[n1] = cmul(x[n1], lt.step[n1]);
    reg_fft<R, INV>(x, lt.reg);
}

// Index of the N x N image row/column held at index q of the shifted M-point
// axis (the image centred and wrapped: q < N/2 and q >= M - N/2), or -1.
__device__ __forceinline__ int wrap_src(int q, int N, int M)
{
    return q < N / 2 ? q + N / 2 : (q >= M - N / 2 ? q - (M - N / 2) : -1);
}

// Asynchronous 4-byte global -> shared copies (cp.async), to stage the next
// image while the current one is transformed.
__device__ __forceinline__ void cp_async4(float *dst, const float *src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_group() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Row r of an N-row block stored at row (r mod R) * (N / R) + r / R: the rows
// R apart that one gather of a warp touches land in consecutive rows.
template <int R>
__device__ __forceinline__ int spread(int r, int rows)
{
    return (r % R) * (rows / R) + r / R;
}

// ---- images -> CAS images ----------------------------------------------------
// ADJ: the adjoint form used by the gradient (first CAS row and column zero,
// times `post`).
template <int M, typename T, bool ADJ>
__global__ void __launch_bounds__(kFftThreads, 1)
fft_images_to_cas_kernel(const float *__restrict__ img, int N, int n, T *__restrict__ cas, float post,
                         const FftTwiddles tw)
{
    constexpr int R = M / 32;
    extern __shared__ float sm[];
    const int H = N / 2, NP = N + 1, ZP = H + 1;
    float *simg = sm;             // N rows (spread) of NP
    float *zre = simg + N * NP;   // Z of the column pairs: M rows of ZP (pair index spread)
    float *zim = zre + M * ZP;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    LaneTw<R> lt;
    lane_twiddles<R, false>(lt, tw, lane);
    // image a -> simg (rows spread), asynchronously
    auto stage = [&](int a) {
        const float *im = img + (size_t)a * N * N;
        for (int r = warp; r < N; r += nw) {
            float *dst = simg + spread<R>(r, N) * NP;
            for (int c = lane; c < N; c += 32) cp_async4(dst + c, im + (size_t)r * N + c);
        }
        cp_async_commit();
    };
    if ((int)blockIdx.x < n) stage(blockIdx.x);

    for (int a = blockIdx.x; a < n; a += gridDim.x) {
        cp_async_wait_all();
        __syncthreads(); // image a is in simg

        // columns k and k + H of the image, along y
        for (int k = warp; k < H; k += nw) {
            float2 x[R];
#pragma unroll
            for (int n1 = 0; n1 < R; n1++) {
                const int r = wrap_src(R * lane + n1, N, M);
                x[n1] = make_float2(0.f, 0.f);
                if (r >= 0) {
                    const float *row = simg + spread<R>(r, N) * NP;
                    x[n1] = make_float2(row[k], row[k + H]);
                }
            }
            warp_fft<R, false>(x, lt, lane);
            const int s = spread<R>(k, H);
#pragma unroll
            for (int k1 = 0; k1 < R; k1++) {
                const int v = br5(lane) + 32 * k1;
                zre[v * ZP + s] = x[k1].x;
                zim[v * ZP + s] = x[k1].y;
            }
        }
        __syncthreads();
        // simg is free: the next image loads while the rows are transformed
        if (a + (int)gridDim.x < n) stage(a + gridDim.x);

        // rows v = 0 .. M/2, along x
        for (int v = warp; v <= M / 2; v += nw) {
            const int vm = (M - v) & (M - 1);
            float2 x[R];
#pragma unroll
            for (int n1 = 0; n1 < R; n1++) {
                const int c = wrap_src(R * lane + n1, N, M);
                x[n1] = make_float2(0.f, 0.f);
                if (c >= 0) {
                    const int s = spread<R>(c < H ? c : c - H, H);
                    const float ax = zre[v * ZP + s], ay = zim[v * ZP + s];
                    const float bx = zre[vm * ZP + s], by = zim[vm * ZP + s];
                    // column a: (Z(v) + conj Z(M-v)) / 2; column b: (Z(v) - conj Z(M-v)) / 2i
                    x[n1] = c < H ? make_float2(0.5f * (ax + bx), 0.5f * (ay - by))
                                  : make_float2(0.5f * (ay + by), 0.5f * (bx - ax));
                }
            }
            warp_fft<R, false>(x, lt, lane);
            const int j = (v + M / 2) & (M - 1), jm = (vm + M / 2) & (M - 1);
            T *rowd = cas + ((size_t)a * M + j) * M;
            T *rowm = cas + ((size_t)a * M + jm) * M;
            const bool mirror = v != 0 && v != M / 2;
#pragma unroll
            for (int k1 = 0; k1 < R; k1++) {
                const int u = br5(lane) + 32 * k1;
                const int i = (u + M / 2) & (M - 1), imr = (M / 2 - u) & (M - 1); // shift(u), shift(M - u)
                float d = x[k1].x + x[k1].y, e = x[k1].x - x[k1].y;
                if (ADJ) {
                    d = (i == 0 || j == 0) ? 0.0f : d * post;
                    e = (imr == 0 || jm == 0) ? 0.0f : e * post;
                }
                rowd[i] = from_f32<T>(d);
                if (mirror) rowm[imr] = from_f32<T>(e);
            }
        }
        __syncthreads();
    }
}

// ---- CAS images -> images ----------------------------------------------------
// A staged CAS row (M floats) holds column c at (c mod R) * (M/R + 32/R) +
// c / R: lanes that read columns R apart, or write consecutive ones, hit
// distinct banks.  A staged row takes M + 32 floats.
template <int R>
__device__ __forceinline__ int row_slot(int c, int M)
{
    return (c % R) * (M / R + 32 / R) + c / R;
}

template <int M>
__global__ void __launch_bounds__(kFftThreads, 1)
fft_cas_to_images_kernel(const float *__restrict__ cas, int N, int n, float *__restrict__ img, const FftTwiddles tw)
{
    constexpr int R = M / 32;
    constexpr int GR = (M / 2) / R + 1; // rows of G per residue class
    extern __shared__ float sm[];
    const int H = N / 2, GP = N + 1, OP = N + 1;
    float *gre = sm;                 // g(p, v), v <= M/2 (spread), N output columns of GP
    float *gim = gre + R * GR * GP;
    float *sout = gim + R * GR * GP; // N x OP output image; during the row pass, the warps'
                                     // staged CAS rows (2 buffers x 2 rows x (M + 32), row_slot)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const float scale = 1.0f / ((float)M * (float)M);
    LaneTw<R> lt;
    lane_twiddles<R, true>(lt, tw, lane);

    for (int a = blockIdx.x; a < n; a += gridDim.x) {
        const float *ca = cas + (size_t)a * M * M;
        // rows v = 0 .. M/2 of the spectrum, along u, keeping the cropped p.
        // Each warp stages CAS rows shift(v) and M - shift(v) of its next v
        // while it transforms the current one.
        constexpr int RL = M + 32; // staged row length
        float *stg = sout + warp * (4 * RL);
        auto fetch = [&](int v, int buf) {
            const int j = (v + M / 2) & (M - 1), jm = (M - j) & (M - 1);
            const float *rj = ca + (size_t)j * M, *rjm = ca + (size_t)jm * M;
            float *b = stg + buf * (2 * RL);
            for (int c = lane; c < M; c += 32) {
                const int sc = row_slot<R>(c, M);
                cp_async4(b + sc, rj + c);
                cp_async4(b + RL + sc, rjm + c);
            }
            cp_async_commit();
        };
        fetch(warp, 0);
        for (int v = warp, it = 0; v <= M / 2; v += nw, it++) {
            const bool more = v + nw <= M / 2;
            if (more) {
                fetch(v + nw, (it + 1) & 1);
                cp_async_wait_group<1>();
            } else {
                cp_async_wait_group<0>();
            }
            __syncwarp(); // row v is staged
            const int j = (v + M / 2) & (M - 1);
            const float *b = stg + (it & 1) * (2 * RL);
            float2 x[R];
#pragma unroll
            for (int n1 = 0; n1 < R; n1++) {
                const int u = R * lane + n1;
                const int i = (u + M / 2) & (M - 1), im = (M - i) & (M - 1);
                x[n1] = make_float2(0.f, 0.f);
                if (i != 0 && j != 0) {
                    const float c1 = b[row_slot<R>(i, M)], c2 = b[RL + row_slot<R>(im, M)];
                    x[n1] = make_float2(0.5f * (c1 + c2), 0.5f * (c1 - c2));
                }
            }
            __syncwarp(); // the buffer may be refilled two rows later
            warp_fft<R, true>(x, lt, lane);
            const int gs = (v % R) * GR + v / R;
#pragma unroll
            for (int k1 = 0; k1 < R; k1++) {
                const int o = wrap_src(br5(lane) + 32 * k1, N, M);
                if (o >= 0) {
                    gre[gs * GP + o] = x[k1].x;
                    gim[gs * GP + o] = x[k1].y;
                }
            }
        }
        __syncthreads();

        // output columns k and k + H, along v (rows v > M/2 are conjugates)
        for (int k = warp; k < H; k += nw) {
            float2 x[R];
#pragma unroll
            for (int n1 = 0; n1 < R; n1++) {
                const int v = R * lane + n1;
                const bool lo = v <= M / 2;
                const int vv = lo ? v : M - v;
                const int gs = (vv % R) * GR + vv / R;
                const float arx = gre[gs * GP + k], ary = gim[gs * GP + k];
                const float brx = gre[gs * GP + k + H], bry = gim[gs * GP + k + H];
                const float2 ga = lo ? make_float2(arx, ary) : make_float2(arx, -ary);
                const float2 gb = lo ? make_float2(brx, bry) : make_float2(brx, -bry);
                x[n1] = make_float2(ga.x - gb.y, ga.y + gb.x); // ga + i gb
            }
            warp_fft<R, true>(x, lt, lane);
#pragma unroll
            for (int k1 = 0; k1 < R; k1++) {
                const int o = wrap_src(br5(lane) + 32 * k1, N, M);
                if (o >= 0) {
                    sout[o * OP + k] = x[k1].x * scale;
                    sout[o * OP + k + H] = x[k1].y * scale;
                }
            }
        }
        __syncthreads();
        float *out = img + (size_t)a * N * N;
        for (int r = warp; r < N; r += nw)
            for (int c = lane; c < N; c += 32) out[(size_t)r * N + c] = sout[r * OP + c];
        __syncthreads();
    }
}

// ---- host side -----------------------------------------------------------------

static const FftTwiddles &twiddles()
{
    static const FftTwiddles t = [] {
        FftTwiddles r;
        const double pi = 3.14159265358979323846;
        for (int m = 0; m < kFftMaxM; m++) {
            // exact values at the quarter turns, each octant from [0, pi/4]
            const int q = m / 64, o = m % 64;
            double c, s;
            if (o <= 32) {
                c = std::cos(2 * pi * o / kFftMaxM);
                s = std::sin(2 * pi * o / kFftMaxM);
            } else {
                c = std::sin(2 * pi * (64 - o) / kFftMaxM);
                s = std::cos(2 * pi * (64 - o) / kFftMaxM);
            }
            if (o == 0) {
                c = 1.0;
                s = 0.0;
            }
            // rotate by q quarter turns: (c, s) -> (-s, c)
            for (int k = 0; k < q; k++) {
                const double t2 = c;
                c = -s;
                s = t2;
            }
            r.w[m] = make_float2((float)c, (float)-s); // e^(-i theta)
        }
        return r;
    }();
    return t;
}

static size_t fwd_smem(int N, int M) { return ((size_t)N * (N + 1) + 2 * (size_t)M * (N / 2 + 1)) * sizeof(float); }

static size_t inv_smem(int N, int M)
{
    const int R = M / 32, GR = (M / 2) / R + 1;
    const size_t out = (size_t)N * (N + 1), stage = (size_t)(kFftThreads / 32) * 4 * (M + 32);
    return (2 * (size_t)R * GR * (N + 1) + (out > stage ? out : stage)) * sizeof(float);
}

bool fft2_fused_ok(int N, int M)
{
    if (M != 64 && M != 128 && M != 256) return false;
    const int R = M / 32;
    if (N <= 0 || N > M / 2 || N % (2 * R) != 0) return false;
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return false;
    return fwd_smem(N, M) <= (size_t)optin && inv_smem(N, M) <= (size_t)optin;
}

static int fft_grid(int n)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
    return n < sms ? n : sms;
}

template <int M, typename T, bool ADJ>
static cudaError_t launch_fwd_t(const float *d_img, int N, int n, T *d_cas, float post, cudaStream_t s)
{
    const size_t smem = fwd_smem(N, M);
    auto kern = fft_images_to_cas_kernel<M, T, ADJ>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<fft_grid(n), kFftThreads, smem, s>>>(d_img, N, n, d_cas, post, twiddles());
    count_launches(1);
    return cudaGetLastError();
}

template <int M>
static cudaError_t launch_fwd_m(const float *d_img, int N, int n, void *d_cas, int prec, bool adjoint, cudaStream_t s)
{
    const float post = 1.0f / ((float)M * (float)M);
    if (adjoint) return launch_fwd_t<M, float, true>(d_img, N, n, (float *)d_cas, post, s);
    if (prec == kBF16) return launch_fwd_t<M, __nv_bfloat16, false>(d_img, N, n, (__nv_bfloat16 *)d_cas, 1.0f, s);
    return launch_fwd_t<M, float, false>(d_img, N, n, (float *)d_cas, 1.0f, s);
}

cudaError_t launch_images_to_cas_fused(const float *d_img, int N, int M, int n, void *d_cas, int prec, bool adjoint,
                                       cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    if (prec == kF16 || (adjoint && prec != kF32)) return cudaErrorInvalidValue;
    if (M == 64) return launch_fwd_m<64>(d_img, N, n, d_cas, prec, adjoint, s);
    if (M == 128) return launch_fwd_m<128>(d_img, N, n, d_cas, prec, adjoint, s);
    if (M == 256) return launch_fwd_m<256>(d_img, N, n, d_cas, prec, adjoint, s);
    return cudaErrorInvalidValue;
}

template <int M>
static cudaError_t launch_inv_m(const float *d_cas, int N, int n, float *d_img, cudaStream_t s)
{
    const size_t smem = inv_smem(N, M);
    auto kern = fft_cas_to_images_kernel<M>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<fft_grid(n), kFftThreads, smem, s>>>(d_cas, N, n, d_img, twiddles());
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_cas_to_images_fused(const float *d_cas, int M, int N, int n, float *d_img, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    if (M == 64) return launch_inv_m<64>(d_cas, N, n, d_img, s);
    if (M == 128) return launch_inv_m<128>(d_cas, N, n, d_img, s);
    if (M == 256) return launch_inv_m<256>(d_cas, N, n, d_img, s);
    return cudaErrorInvalidValue;
}

} // namespace gg
