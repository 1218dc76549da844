// CAS ("cosine and sine") conversions around the FFTs, for GB300 (sm_103a).
//
// The reference chains separate element-wise kernels around cuFFT C2C calls
// (pad, real->complex, fftshift, FFT, fftshift, complex->CAS, ...;
// src/Gridders/gpuGridder.cpp:432-596, src/Matlab/utils/CASFromVol_Gridder.m,
// volFromCAS_Gridder.m).  Here each chain is one pre-kernel and one
// post-kernel around a real-to-complex or complex-to-real cuFFT transform:
//   * the fftshifts (even sizes) become index remaps, folded into the loads
//     and stores of the neighbouring kernel;
//   * FromCAS yields an exactly Hermitian spectrum (c[-k] = conj(c[k]), the
//     Nyquist row/column/slice zeroed), so the inverse transform is C2R and
//     "take the real part" is free;
//   * a real input makes the forward transform R2C; the other half of the
//     spectrum is read through conjugate symmetry when forming Re+Im.
#include <stdint.h>

#include <cmath>

#include "gg_common.cuh"
#include "gg_internal.h"
#include "../../include/gg_gridder.h"

namespace gg {

static inline unsigned grid_for(size_t count, int threads)
{
    size_t g = (count + threads - 1) / threads;
    if (g > 0x7fffffffull) g = 0x7fffffffull;
    return (unsigned)(g ? g : 1);
}

__device__ __forceinline__ int shift_idx(int q, int M) { return q + M / 2 >= M ? q + M / 2 - M : q + M / 2; }

// ---- 3-D: volume -> CAS volume --------------------------------------------

// x[q] = (zero-padded volume * precomp^3)[(q + M/2) mod M] per axis.
__global__ void vol_to_fft_input_kernel(const float *__restrict__ vol, int N, int M,
                                        const double *__restrict__ pc, float *__restrict__ x)
{
    const size_t total = (size_t)M * M * M;
    const int b = M / 2 - N / 2;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int qi = (int)(e % M), qj = (int)((e / M) % M), qk = (int)(e / ((size_t)M * M));
        const int i = shift_idx(qi, M), j = shift_idx(qj, M), k = shift_idx(qk, M);
        const int oi = i - b, oj = j - b, ok = k - b;
        float v = 0.0f;
        if ((unsigned)oi < (unsigned)N && (unsigned)oj < (unsigned)N && (unsigned)ok < (unsigned)N) {
            const float f = (float)(pc[i] * pc[j] * pc[k]);
            v = vol[(size_t)ok * N * N + (size_t)oj * N + oi] * f;
        }
        x[e] = v;
    }
}

// CAS[pad+k][pad+j][pad+i] = Re+Im of fftshift(Y)[k][j][i]; border zero.
template <typename T>
__global__ void spectrum_to_cas_volume_kernel(const cufftComplex *__restrict__ spec, int M, int V, T *__restrict__ cas,
                                              const float *__restrict__ d_scale)
{
    const float inv_scale = d_scale ? 1.0f / *d_scale : 1.0f;
    const size_t total = (size_t)V * V * V;
    const int pad = V / 2 - M / 2;
    const int H = M / 2 + 1;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int ci = (int)(e % V), cj = (int)((e / V) % V), ck = (int)(e / ((size_t)V * V));
        const int i = ci - pad, j = cj - pad, k = ck - pad;
        float out = 0.0f;
        if ((unsigned)i < (unsigned)M && (unsigned)j < (unsigned)M && (unsigned)k < (unsigned)M) {
            const int u = shift_idx(i, M), v = shift_idx(j, M), w = shift_idx(k, M);
            if (u <= M / 2) {
                const cufftComplex c = spec[((size_t)w * M + v) * H + u];
                out = c.x + c.y;
            } else {  // conjugate symmetry: Y[w][v][u] = conj(Y[-w][-v][-u])
                const int w2 = w ? M - w : 0, v2 = v ? M - v : 0, u2 = M - u;
                const cufftComplex c = spec[((size_t)w2 * M + v2) * H + u2];
                out = c.x - c.y;
            }
        }
        cas[e] = from_f32<T>(out * inv_scale);
    }
}

// ---- 3-D: CAS volume -> volume ---------------------------------------------

// H[w][v][u] = FromCAS(crop(cas))[(w+M/2)%M][(v+M/2)%M][(u+M/2)%M], u <= M/2.
__global__ void cas_volume_to_spectrum_kernel(const float *__restrict__ cas, int V, int M, cufftComplex *__restrict__ spec)
{
    const int H = M / 2 + 1;
    const size_t total = (size_t)M * M * H;
    const int b = V / 2 - M / 2;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int u = (int)(e % H), v = (int)((e / H) % M), w = (int)(e / ((size_t)H * M));
        const int i = shift_idx(u, M), j = shift_idx(v, M), k = shift_idx(w, M);
        cufftComplex c;
        c.x = 0.0f;
        c.y = 0.0f;
        if (i != 0 && j != 0 && k != 0) {
            const float r1 = cas[((size_t)(k + b) * V + (j + b)) * V + (i + b)];
            const float r2 = cas[((size_t)(M - k + b) * V + (M - j + b)) * V + (M - i + b)];
            c.x = 0.5f * (r1 + r2);
            c.y = 0.5f * (r1 - r2);
        }
        spec[e] = c;
    }
}

// vol[k][j][i] = y[(k+ob+M/2)%M]... / M^3 * precomp, centred crop.
__global__ void fft_output_to_vol_kernel(const float *__restrict__ y, int M, int N, const double *__restrict__ pc,
                                         float *__restrict__ vol)
{
    const size_t total = (size_t)N * N * N;
    const int ob = M / 2 - N / 2;
    const double inv = 1.0 / ((double)M * M * M);
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int oi = (int)(e % N), oj = (int)((e / N) % N), ok = (int)(e / ((size_t)N * N));
        const int i = oi + ob, j = oj + ob, k = ok + ob;
        const float val = y[((size_t)shift_idx(k, M) * M + shift_idx(j, M)) * M + shift_idx(i, M)];
        vol[e] = (float)((double)val * inv * pc[i] * pc[j] * pc[k]);
    }
}

// ---- 2-D: CAS images -> images (forward-projection output path) -----------

// Per-image row kernels: a (kRowX, kRowY) block covers kRowY rows of one
// image, blockIdx.y walks the images; each thread takes kRowU columns kRowX
// apart per chunk and issues its loads before its stores (more bytes in
// flight than one element per thread, and no per-element division).
constexpr int kRowX = 64, kRowY = 4, kRowU = 4;

static inline dim3 row_grid(int rows, int n)
{
    return dim3((unsigned)((rows + kRowY - 1) / kRowY), (unsigned)(n < 65535 ? n : 65535));
}

__global__ void __launch_bounds__(kRowX *kRowY)
cas_images_to_spectrum_kernel(const float *__restrict__ cas, int M, int n, cufftComplex *__restrict__ spec)
{
    const int H = M / 2 + 1;
    const int v = blockIdx.x * kRowY + threadIdx.y;
    if (v >= M) return;
    const int j = shift_idx(v, M);
    for (int a = blockIdx.y; a < n; a += gridDim.y) {
        const float *img = cas + (size_t)a * M * M;
        const float *r1 = img + (size_t)j * M, *r2 = img + (size_t)(M - j) * M;
        cufftComplex *out = spec + ((size_t)a * M + v) * H;
        for (int u0 = threadIdx.x; u0 < H; u0 += kRowX * kRowU) {
            float x1[kRowU], x2[kRowU];
#pragma unroll
            for (int k = 0; k < kRowU; k++) {
                const int u = u0 + k * kRowX;
                const int i = u < H ? shift_idx(u, M) : 0;
                const bool live = u < H && i != 0 && j != 0;
                x1[k] = live ? __ldg(r1 + i) : 0.0f;
                x2[k] = live ? __ldg(r2 + (M - i)) : 0.0f;
            }
#pragma unroll
            for (int k = 0; k < kRowU; k++) {
                const int u = u0 + k * kRowX;
                if (u < H) {
                    cufftComplex c;
                    c.x = 0.5f * (x1[k] + x2[k]);
                    c.y = 0.5f * (x1[k] - x2[k]);
                    out[u] = c;
                }
            }
        }
    }
}

__global__ void __launch_bounds__(kRowX *kRowY)
fft_output_to_images_kernel(const float *__restrict__ y, int M, int N, int n, float *__restrict__ img)
{
    const int ob = (M - N) / 2;
    const float scale = 1.0f / ((float)M * (float)M);
    const int oj = blockIdx.x * kRowY + threadIdx.y;
    if (oj >= N) return;
    const int j = shift_idx(oj + ob, M);
    for (int a = blockIdx.y; a < n; a += gridDim.y) {
        const float *yr = y + ((size_t)a * M + j) * M;
        float *ir = img + ((size_t)a * N + oj) * N;
        for (int o0 = threadIdx.x; o0 < N; o0 += kRowX * kRowU) {
            float v[kRowU];
#pragma unroll
            for (int k = 0; k < kRowU; k++) {
                const int oi = o0 + k * kRowX;
                v[k] = oi < N ? __ldg(yr + shift_idx(oi + ob, M)) : 0.0f;
            }
#pragma unroll
            for (int k = 0; k < kRowU; k++) {
                const int oi = o0 + k * kRowX;
                if (oi < N) ir[oi] = v[k] * scale;
            }
        }
    }
}

// ---- 2-D: images -> CAS images (back-projection input path) --------------

__global__ void __launch_bounds__(kRowX *kRowY)
images_to_fft_input_kernel(const float *__restrict__ img, int N, int M, int n, float *__restrict__ x)
{
    const int b = (M - N) / 2;
    const int qj = blockIdx.x * kRowY + threadIdx.y;
    if (qj >= M) return;
    const int oj = shift_idx(qj, M) - b;
    const bool row_in = (unsigned)oj < (unsigned)N;
    for (int a = blockIdx.y; a < n; a += gridDim.y) {
        const float *ir = img + ((size_t)a * N + (row_in ? oj : 0)) * N;
        float *xr = x + ((size_t)a * M + qj) * M;
        for (int q0 = threadIdx.x; q0 < M; q0 += kRowX * kRowU) {
            float v[kRowU];
#pragma unroll
            for (int k = 0; k < kRowU; k++) {
                const int qi = q0 + k * kRowX;
                const int oi = qi < M ? shift_idx(qi, M) - b : -1;
                v[k] = row_in && (unsigned)oi < (unsigned)N ? __ldg(ir + oi) : 0.0f;
            }
#pragma unroll
            for (int k = 0; k < kRowU; k++) {
                const int qi = q0 + k * kRowX;
                if (qi < M) xr[qi] = v[k];
            }
        }
    }
}

// Row j of CAS image a from the half spectrum: Re+Im at (u, v) = the shifted
// (i, j) for u <= M/2, else Re-Im at the Hermitian mirror.  ADJ: the adjoint
// form (first row and column zero, times `post`).
template <typename T, bool ADJ>
__global__ void __launch_bounds__(kRowX *kRowY)
spectrum_to_cas_images_kernel(const cufftComplex *__restrict__ spec, int M, int n, T *__restrict__ cas,
                              const float *__restrict__ d_scale, float post)
{
    const float mul = ADJ ? post : (d_scale ? 1.0f / *d_scale : 1.0f);
    const int H = M / 2 + 1;
    const int j = blockIdx.x * kRowY + threadIdx.y;
    if (j >= M) return;
    const int v = shift_idx(j, M), v2 = v ? M - v : 0;
    for (int a = blockIdx.y; a < n; a += gridDim.y) {
        const cufftComplex *s = spec + (size_t)a * M * H;
        const cufftComplex *r1 = s + (size_t)v * H, *r2 = s + (size_t)v2 * H;
        T *cr = cas + ((size_t)a * M + j) * M;
        for (int i0 = threadIdx.x; i0 < M; i0 += kRowX * kRowU) {
            float o[kRowU];
#pragma unroll
            for (int k = 0; k < kRowU; k++) {
                const int i = i0 + k * kRowX;
                float out = 0.0f;
                if (i < M && (!ADJ || (i != 0 && j != 0))) {
                    const int u = shift_idx(i, M);
                    if (u <= M / 2) {
                        const cufftComplex c = r1[u];
                        out = c.x + c.y;
                    } else {
                        const cufftComplex c = r2[M - u];
                        out = c.x - c.y;
                    }
                }
                o[k] = out;
            }
#pragma unroll
            for (int k = 0; k < kRowU; k++) {
                const int i = i0 + k * kRowX;
                if (i < M) cr[i] = from_f32<T>(o[k] * mul);
            }
        }
    }
}

// ---- adjoint of the whole forward operator ----------------------------------
// Gradient of images -> CAS images: the adjoint of (FromCAS, shift, inverse
// FFT / M^2, shift, real part, crop).  For the FFT of a real image FromCAS^T
// equals Re+Im, so this is spectrum_to_cas_images with the first row and
// column (zeroed by FromCAS) dropped and the 1/M^2 applied (the ADJ form).

// Gradient of the CAS volume -> volume, first half: crop V^3 to the inner M^3
// and fftshift (the adjoint of the zero-pad and of the output fftshift).
__global__ void cas_volume_adjoint_input_kernel(const float *__restrict__ g, int V, int M, float *__restrict__ x)
{
    const size_t total = (size_t)M * M * M;
    const int b = V / 2 - M / 2;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int qi = (int)(e % M), qj = (int)((e / M) % M), qk = (int)(e / ((size_t)M * M));
        const int i = shift_idx(qi, M), j = shift_idx(qj, M), k = shift_idx(qk, M);
        x[e] = g[((size_t)(k + b) * V + (j + b)) * V + (i + b)];
    }
}

// Second half: Re+Im of fftshift(FFT), times the precomp, centred crop to N^3.
// (The adjoint of ToCAS maps g to g + i g; with the unnormalised FFT's adjoint
// M^3 * ifft of a real input equal to conj(fft), Re((1+i) conj(F)) = Re F + Im F.)
__global__ void spectrum_to_vol_adjoint_kernel(const cufftComplex *__restrict__ spec, int M, int N,
                                               const double *__restrict__ pc, float *__restrict__ vol)
{
    const size_t total = (size_t)N * N * N;
    const int ob = M / 2 - N / 2;
    const int H = M / 2 + 1;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int oi = (int)(e % N), oj = (int)((e / N) % N), ok = (int)(e / ((size_t)N * N));
        const int i = oi + ob, j = oj + ob, k = ok + ob;
        const int u = shift_idx(i, M), v = shift_idx(j, M), w = shift_idx(k, M);
        float val;
        if (u <= M / 2) {
            const cufftComplex c = spec[((size_t)w * M + v) * H + u];
            val = c.x + c.y;
        } else {
            const int w2 = w ? M - w : 0, v2 = v ? M - v : 0;
            const cufftComplex c = spec[((size_t)w2 * M + v2) * H + (M - u)];
            val = c.x - c.y;
        }
        vol[e] = (float)((double)val * pc[i] * pc[j] * pc[k]);
    }
}

__global__ void divide_plane_density_kernel(float *__restrict__ a, const float *__restrict__ b, size_t count, float eps)
{
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x)
        a[e] = a[e] / (b[e] + eps);
}

template <typename T>
__global__ void convert_kernel(const float *__restrict__ in, T *__restrict__ out, size_t count, const float *__restrict__ d_scale)
{
    const float inv_scale = d_scale ? 1.0f / *d_scale : 1.0f;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x)
        out[e] = from_f32<T>(in[e] * inv_scale);
}

template <typename T>
__global__ void pitch_volume_kernel(const float *__restrict__ cas, int V, int P, T *__restrict__ out,
                                    const float *__restrict__ d_scale, int layout)
{
    const float inv_scale = d_scale ? 1.0f / *d_scale : 1.0f;
    const size_t total = (size_t)V * V * P, VV = (size_t)V * V;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const size_t row = e / P;
        const size_t c = e - row * P, b = row % V, a = row / V; // out[a][b][c]
        float v = 0.0f;
        if (c < (size_t)V) {
            // layout 0: [z][y][x]; 1: [z][x][y]; 2: [y][x][z]
            const size_t x = layout == 0 ? c : b, y = layout == 0 ? b : layout == 1 ? c : a,
                         z = layout == 2 ? c : a;
            v = cas[z * VV + y * V + x] * inv_scale;
        }
        out[e] = from_f32<T>(v);
    }
}

__global__ void transpose_volume_kernel(const float *__restrict__ in, int V, float *__restrict__ out, int layout)
{
    const size_t VV = (size_t)V * V, total = VV * V;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const size_t c = e % V, b = (e / V) % V, a = e / VV; // out[a][b][c]
        // layout 1: [z][x][y] -> (x, y, z) = (b, c, a); layout 2: [y][x][z] -> (b, a, c)
        const size_t x = b, y = layout == 1 ? c : a, z = layout == 1 ? a : c;
        out[e] = in[z * VV + y * V + x];
    }
}

// Weak-phase CTF at each CAS-image pixel, r2 = |(i, j) - M/2|^2 (an exact
// integer): chi = r2 (alpha df) - r2^2 beta with alpha = pi lambda / (M px)^2,
// beta = pi/2 Cs lambda^3 / (M px)^4; CTF = -(sqrt(1 - A^2) sin chi + A cos chi).
// chi reaches hundreds of radians, so it is formed in float-float arithmetic
// (Dekker's error-free products through fmaf, Knuth's two-sum) and reduced
// mod 2 pi by Cody and Waite's method with 2 pi split into three parts (the
// first two short enough that k * part is exact); sincosf then sees |r| <= pi.
// A real, even CTF multiplies Re and Im alike, so it applies to CAS images
// directly.  d_mul (optional) *= CTF^mul_power; d_gen (optional) = CTF^gen_power.
// ASTIG: per-image astigmatism, defocus_v and astig (radians, from the x
// axis) given.  The defocus at angle theta is df_m + df_d cos 2(theta - phi)
// with df_m, df_d the mean and half-difference of defocus U and V; with
// (dx, dy) the pixel's offset from DC, alpha df s^2 becomes
// alpha (df_m r2 + df_d ((dx^2 - dy^2) cos 2phi + 2 dx dy sin 2phi)), no
// division.  alpha df_m, alpha df_d, cos 2phi and sin 2phi are formed in FP64
// once per image and row and split into float pairs; the per-pixel terms
// stay float-float as above.
template <bool ASTIG>
__global__ void __launch_bounds__(kRowX *kRowY)
ctf_kernel(float *__restrict__ d_mul, float *__restrict__ d_gen, int M, int n, const float *__restrict__ defocus,
           const float *__restrict__ defocus_v, const float *__restrict__ astig, CtfConsts k, int mul_power,
           int gen_power)
{
    const int j = blockIdx.x * kRowY + threadIdx.y;
    if (j >= M) return;
    const int dj = j - M / 2;
    for (int a = blockIdx.y; a < n; a += gridDim.y) {
        float c_hi, c_lo, e_hi = 0.0f, e_lo = 0.0f, c2_hi = 0.0f, c2_lo = 0.0f, s2_hi = 0.0f, s2_lo = 0.0f;
        if (!ASTIG) {
            const float df = defocus[a];
            // c = alpha * df as hi + lo (the rounded products are __fmul_rn so
            // that no FMA contraction changes them: the error terms below
            // assume each one rounded on its own)
            c_hi = __fmul_rn(k.a_hi, df);
            c_lo = fmaf(k.a_hi, df, -c_hi) + k.a_lo * df;
        } else {
            const double du = defocus[a], dv = defocus_v[a];
            const double cm = k.alpha * (0.5 * (du + dv)), cd = k.alpha * (0.5 * (du - dv));
            double sn2, cs2;
            sincos(2.0 * (double)astig[a], &sn2, &cs2);
            c_hi = (float)cm;
            c_lo = (float)(cm - (double)c_hi);
            e_hi = (float)cd;
            e_lo = (float)(cd - (double)e_hi);
            c2_hi = (float)cs2;
            c2_lo = (float)(cs2 - (double)c2_hi);
            s2_hi = (float)sn2;
            s2_lo = (float)(sn2 - (double)s2_hi);
        }
        const size_t row = ((size_t)a * M + j) * M;
        for (int i = threadIdx.x; i < M; i += kRowX) {
            const int di = i - M / 2;
            const float r2 = (float)(di * di + dj * dj);
            // t1 = r2 * c
            float t1_hi = __fmul_rn(r2, c_hi);
            float t1_lo = fmaf(r2, c_hi, -t1_hi) + r2 * c_lo;
            if (ASTIG) {
                // g = (dx^2 - dy^2) cos 2phi + 2 dx dy sin 2phi, then t1 += e g
                const float G1 = (float)(di * di - dj * dj), G2 = (float)(2 * di * dj);
                const float p1 = __fmul_rn(G1, c2_hi), p2 = __fmul_rn(G2, s2_hi);
                const float e1 = fmaf(G1, c2_hi, -p1) + G1 * c2_lo, e2 = fmaf(G2, s2_hi, -p2) + G2 * s2_lo;
                const float g_hi = __fadd_rn(p1, p2);
                const float gb = __fsub_rn(g_hi, p1), ga = __fsub_rn(g_hi, gb);
                const float g_lo = ((p1 - ga) + (p2 - gb)) + (e1 + e2);
                const float t3_hi = __fmul_rn(e_hi, g_hi);
                const float t3_lo = fmaf(e_hi, g_hi, -t3_hi) + e_hi * g_lo + e_lo * g_hi;
                const float u_hi = __fadd_rn(t1_hi, t3_hi);
                const float ub = __fsub_rn(u_hi, t1_hi), ua = __fsub_rn(u_hi, ub);
                t1_lo = ((t1_hi - ua) + (t3_hi - ub)) + (t1_lo + t3_lo);
                t1_hi = u_hi;
            }
            // t2 = r2^2 * beta
            const float q_hi = __fmul_rn(r2, r2), q_lo = fmaf(r2, r2, -q_hi);
            const float t2_hi = __fmul_rn(q_hi, k.b_hi);
            const float t2_lo = fmaf(q_hi, k.b_hi, -t2_hi) + q_hi * k.b_lo + q_lo * k.b_hi;
            // chi = t1 - t2 (two-sum of the high parts)
            const float d_hi = t1_hi - t2_hi;
            const float bb = d_hi - t1_hi, aa = d_hi - bb;
            const float d_lo = ((t1_hi - aa) + (-t2_hi - bb)) + (t1_lo - t2_lo);
            // reduction mod 2 pi
            const float kk = rintf(d_hi * k.inv_2pi);
            float red = fmaf(-kk, k.p1, d_hi);
            red = fmaf(-kk, k.p2, red);
            red = fmaf(-kk, k.p3, red) + d_lo;
            float sn, cs;
            sincosf(red, &sn, &cs);
            const float ctf = -(k.w_sin * sn + k.w_cos * cs);
            if (d_mul) d_mul[row + i] *= mul_power == 2 ? ctf * ctf : ctf;
            if (d_gen) d_gen[row + i] = gen_power == 2 ? ctf * ctf : ctf;
        }
    }
}

// Non-negative floats order like their bit patterns, so an unsigned atomicMax
// on the bits of |x| finds the largest magnitude.
__global__ void max_abs_kernel(const float *__restrict__ x, size_t count, unsigned int *out)
{
    float m = 0.0f;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(x[e]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

__global__ void scale_from_max_kernel(unsigned int *work, float target, float *d_scale)
{
    const float m = __uint_as_float(*work);
    float sc = 1.0f;
    while (sc < 1e30f && m / sc > target) sc *= 2.0f;
    *d_scale = sc;
    *work = 0u;  // ready for the next use
}

// ---- launchers -------------------------------------------------------------

constexpr int kT = 256;

cudaError_t launch_vol_to_fft_input(const float *d_vol, int N, int M, const double *d_precomp, float *d_x, cudaStream_t s)
{
    vol_to_fft_input_kernel<<<grid_for((size_t)M * M * M, kT), kT, 0, s>>>(d_vol, N, M, d_precomp, d_x);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_spectrum_to_cas_volume(const cufftComplex *d_spec, int M, int V, void *d_cas, int prec,
                                          const float *d_scale, cudaStream_t s)
{
    const unsigned g = grid_for((size_t)V * V * V, kT);
    if (prec == kF32) spectrum_to_cas_volume_kernel<float><<<g, kT, 0, s>>>(d_spec, M, V, (float *)d_cas, d_scale);
    else if (prec == kF16) spectrum_to_cas_volume_kernel<__half><<<g, kT, 0, s>>>(d_spec, M, V, (__half *)d_cas, d_scale);
    else spectrum_to_cas_volume_kernel<__nv_bfloat16><<<g, kT, 0, s>>>(d_spec, M, V, (__nv_bfloat16 *)d_cas, d_scale);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_cas_volume_to_spectrum(const float *d_cas, int V, int M, cufftComplex *d_spec, cudaStream_t s)
{
    cas_volume_to_spectrum_kernel<<<grid_for((size_t)M * M * (M / 2 + 1), kT), kT, 0, s>>>(d_cas, V, M, d_spec);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_fft_output_to_vol(const float *d_y, int M, int N, const double *d_precomp, float *d_vol, cudaStream_t s)
{
    fft_output_to_vol_kernel<<<grid_for((size_t)N * N * N, kT), kT, 0, s>>>(d_y, M, N, d_precomp, d_vol);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_cas_images_to_spectrum(const float *d_cas, int M, int n, cufftComplex *d_spec, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    cas_images_to_spectrum_kernel<<<row_grid(M, n), dim3(kRowX, kRowY), 0, s>>>(d_cas, M, n, d_spec);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_fft_output_to_images(const float *d_y, int M, int N, int n, float *d_img, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    fft_output_to_images_kernel<<<row_grid(N, n), dim3(kRowX, kRowY), 0, s>>>(d_y, M, N, n, d_img);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_images_to_fft_input(const float *d_img, int N, int M, int n, float *d_x, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    images_to_fft_input_kernel<<<row_grid(M, n), dim3(kRowX, kRowY), 0, s>>>(d_img, N, M, n, d_x);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_spectrum_to_cas_images(const cufftComplex *d_spec, int M, int n, void *d_cas, int prec,
                                          const float *d_scale, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const dim3 g = row_grid(M, n), b(kRowX, kRowY);
    if (prec == kF32)
        spectrum_to_cas_images_kernel<float, false><<<g, b, 0, s>>>(d_spec, M, n, (float *)d_cas, d_scale, 1.0f);
    else if (prec == kF16)
        spectrum_to_cas_images_kernel<__half, false><<<g, b, 0, s>>>(d_spec, M, n, (__half *)d_cas, d_scale, 1.0f);
    else
        spectrum_to_cas_images_kernel<__nv_bfloat16, false><<<g, b, 0, s>>>(d_spec, M, n, (__nv_bfloat16 *)d_cas,
                                                                             d_scale, 1.0f);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_spectrum_to_cas_images_adjoint(const cufftComplex *d_spec, int M, int n, float *d_cas, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    spectrum_to_cas_images_kernel<float, true><<<row_grid(M, n), dim3(kRowX, kRowY), 0, s>>>(
        d_spec, M, n, d_cas, nullptr, 1.0f / ((float)M * (float)M));
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_cas_volume_adjoint_input(const float *d_g, int V, int M, float *d_x, cudaStream_t s)
{
    cas_volume_adjoint_input_kernel<<<grid_for((size_t)M * M * M, kT), kT, 0, s>>>(d_g, V, M, d_x);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_spectrum_to_vol_adjoint(const cufftComplex *d_spec, int M, int N, const double *d_precomp, float *d_vol,
                                           cudaStream_t s)
{
    spectrum_to_vol_adjoint_kernel<<<grid_for((size_t)N * N * N, kT), kT, 0, s>>>(d_spec, M, N, d_precomp, d_vol);
    count_launches(1);
    return cudaGetLastError();
}

__global__ void fill_kernel(float *__restrict__ d, size_t count, float value)
{
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x)
        d[e] = value;
}

cudaError_t launch_fill(float *d, size_t count, float value, cudaStream_t s)
{
    fill_kernel<<<grid_for(count, kT), kT, 0, s>>>(d, count, value);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_divide_plane_density(float *d_a, const float *d_b, size_t count, float eps, cudaStream_t s)
{
    divide_plane_density_kernel<<<grid_for(count, kT), kT, 0, s>>>(d_a, d_b, count, eps);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_convert(const float *d_in, void *d_out, int prec, size_t count, const float *d_scale, cudaStream_t s)
{
    const unsigned g = grid_for(count, kT);
    if (prec == kF32) convert_kernel<float><<<g, kT, 0, s>>>(d_in, (float *)d_out, count, d_scale);
    else if (prec == kF16) convert_kernel<__half><<<g, kT, 0, s>>>(d_in, (__half *)d_out, count, d_scale);
    else convert_kernel<__nv_bfloat16><<<g, kT, 0, s>>>(d_in, (__nv_bfloat16 *)d_out, count, d_scale);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_pitch_volume(const float *d_cas, int V, int P, void *d_out, int prec, const float *d_scale,
                                cudaStream_t s, int layout)
{
    const unsigned g = grid_for((size_t)V * V * P, kT);
    if (prec == kF32) pitch_volume_kernel<float><<<g, kT, 0, s>>>(d_cas, V, P, (float *)d_out, d_scale, layout);
    else if (prec == kF16) pitch_volume_kernel<__half><<<g, kT, 0, s>>>(d_cas, V, P, (__half *)d_out, d_scale, layout);
    else pitch_volume_kernel<__nv_bfloat16><<<g, kT, 0, s>>>(d_cas, V, P, (__nv_bfloat16 *)d_out, d_scale, layout);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_transpose_volume(const float *d_in, int V, float *d_out, int layout, cudaStream_t s)
{
    transpose_volume_kernel<<<grid_for((size_t)V * V * V, kT), kT, 0, s>>>(d_in, V, d_out, layout);
    count_launches(1);
    return cudaGetLastError();
}

static void split_f(double x, float *hi, float *lo)
{
    *hi = (float)x;
    *lo = (float)(x - (double)*hi);
}

// 2 pi to `bits` significant bits (towards zero), so that k * part is exact
// in FP32 for |k| < 2^(24 - bits).
static double leading_bits(double x, int bits)
{
    int ex;
    const double m = std::frexp(x, &ex);
    return std::ldexp(std::trunc(std::ldexp(m, bits)), ex - bits);
}

cudaError_t launch_ctf(float *d_mul, int mul_power, float *d_gen, int gen_power, int M, int n, const float *d_defocus,
                       const float *d_defocus_v, const float *d_astig, const CtfParams &c, cudaStream_t s)
{
    if (n <= 0 || (!d_mul && !d_gen)) return cudaSuccess;
    // electron wavelength (Å) at the accelerating voltage, relativistic
    const double U = (double)c.voltage_kv * 1e3;
    const double lambda = 12.2643247 / std::sqrt(U * (1.0 + 0.978466e-6 * U));
    const double pi = 3.14159265358979323846;
    const double q = 1.0 / (((double)M * c.pixel_size) * ((double)M * c.pixel_size));
    const double alpha = pi * lambda * q, beta = 0.5 * pi * ((double)c.cs_mm * 1e7) * lambda * lambda * lambda * q * q;
    CtfConsts k;
    k.alpha = alpha;
    split_f(alpha, &k.a_hi, &k.a_lo);
    split_f(beta, &k.b_hi, &k.b_lo);
    const double p1 = leading_bits(2 * pi, 12), p2 = leading_bits(2 * pi - p1, 12);
    k.p1 = (float)p1;
    k.p2 = (float)p2;
    k.p3 = (float)(2 * pi - p1 - p2);
    k.inv_2pi = (float)(1.0 / (2 * pi));
    const double A = c.amp_contrast;
    k.w_sin = (float)std::sqrt(1.0 - A * A);
    k.w_cos = (float)A;
    if (d_defocus_v && d_astig)
        ctf_kernel<true><<<row_grid(M, n), dim3(kRowX, kRowY), 0, s>>>(d_mul, d_gen, M, n, d_defocus, d_defocus_v,
                                                                        d_astig, k, mul_power, gen_power);
    else
        ctf_kernel<false><<<row_grid(M, n), dim3(kRowX, kRowY), 0, s>>>(d_mul, d_gen, M, n, d_defocus, nullptr,
                                                                         nullptr, k, mul_power, gen_power);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_storage_scale(const float *d_x, size_t count, float target, unsigned int *d_work, float *d_scale,
                                 cudaStream_t s)
{
    // d_work is left at zero by the previous use (and by the allocator's memset)
    unsigned g = grid_for(count, kT);
    if (g > 4096) g = 4096;
    max_abs_kernel<<<g, kT, 0, s>>>(d_x, count, d_work);
    scale_from_max_kernel<<<1, 1, 0, s>>>(d_work, target, d_scale);
    count_launches(2);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// The reference's filters (src/Filters/*.cu) as building blocks.
// Slices are size x size; n_slices = 0 means a size^3 volume.
// ---------------------------------------------------------------------------

__global__ void f_complex_to_cas(const float2 *__restrict__ c, float *__restrict__ r, size_t count)
{
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x)
        r[e] = c[e].x + c[e].y;
}

__global__ void f_cas_to_complex(const float *__restrict__ r, float2 *__restrict__ c, int size, int nsl, bool vol3)
{
    const size_t per = (size_t)size * size;
    const size_t count = per * nsl;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % size), j = (int)((e / size) % size), k = (int)(e / per);
        float2 out = make_float2(0.f, 0.f);
        if (i != 0 && j != 0 && (!vol3 || k != 0)) {
            const int k2 = vol3 ? size - k : k;
            const float a = r[e], b = r[(size_t)k2 * per + (size_t)(size - j) * size + (size - i)];
            out = make_float2(0.5f * (a + b), 0.5f * (a - b));
        }
        c[e] = out;
    }
}

template <typename T>
__global__ void f_fftshift_2d(T *d, int size, int nsl)
{
    // swap quadrant pairs: each thread owns one element of the top half
    const int h = size / 2;
    const size_t per_half = (size_t)size * h;
    const size_t count = per_half * nsl;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x) {
        const size_t s = e / per_half;
        const int rem = (int)(e - s * per_half);
        const int i = rem % size, j = rem / size;  // j < h
        T *img = d + s * size * size;
        const size_t p = (size_t)j * size + i;
        const size_t q = (size_t)(j + h) * size + (i + h) % size;
        T tmp = img[p];
        img[p] = img[q];
        img[q] = tmp;
    }
}

template <typename T>
__global__ void f_fftshift_3d(T *d, int size)
{
    const int h = size / 2;
    const size_t per = (size_t)size * size;
    const size_t count = per * h;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % size), j = (int)((e / size) % size), k = (int)(e / per);  // k < h
        const size_t p = (size_t)k * per + (size_t)j * size + i;
        const size_t q = (size_t)(k + h) * per + (size_t)((j + h) % size) * size + (i + h) % size;
        T tmp = d[p];
        d[p] = d[q];
        d[q] = tmp;
    }
}

__global__ void f_pad(const float *__restrict__ in, float *__restrict__ out, int ix, int iy, int iz, int px, int py, int pz)
{
    const int ox = ix + 2 * px, oy = iy + 2 * py, oz = iz + 2 * pz;
    const size_t count = (size_t)ox * oy * oz;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % ox) - px, j = (int)((e / ox) % oy) - py, k = (int)(e / ((size_t)ox * oy)) - pz;
        float v = 0.f;
        if ((unsigned)i < (unsigned)ix && (unsigned)j < (unsigned)iy && (unsigned)k < (unsigned)iz)
            v = in[((size_t)k * iy + j) * ix + i];
        out[e] = v;
    }
}

__global__ void f_crop(const float *__restrict__ in, float *__restrict__ out, int ix, int iy, int iz, int cx, int cy, int cz)
{
    const int ox = ix - 2 * cx, oy = iy - 2 * cy, oz = iz - 2 * cz;
    const size_t count = (size_t)ox * oy * oz;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % ox), j = (int)((e / ox) % oy), k = (int)(e / ((size_t)ox * oy));
        out[e] = in[((size_t)(k + cz) * iy + (j + cy)) * ix + (i + cx)];
    }
}

__global__ void f_divide_volumes(float *a, const float *__restrict__ b, size_t count)
{
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x)
        a[e] = (a[e] != 0.f && b[e] != 0.f) ? a[e] / b[e] : 0.f;
}

__global__ void f_multiply(float *a, const float *__restrict__ b, size_t count, bool a_complex)
{
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x) {
        if (a_complex) {
            a[2 * e] *= b[e];
            a[2 * e + 1] *= b[e];
        } else {
            a[e] *= b[e];
        }
    }
}

__global__ void f_add(float *a, const float *__restrict__ b, size_t count)
{
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x)
        a[e] += b[e];
}

__global__ void f_div_scalar(float *a, float s, size_t count)
{
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x)
        a[e] = a[e] / s;
}

__global__ void f_real_to_complex(const float *__restrict__ r, float2 *__restrict__ c, size_t count)
{
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x)
        c[e] = make_float2(r[e], 0.f);
}

__global__ void f_complex_to_real(const float2 *__restrict__ c, float *__restrict__ r, size_t count)
{
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x)
        r[e] = c[e].x;
}

} // namespace gg

using namespace gg;

static size_t slice_count(int size, int n_slices) { return (size_t)size * size * (size_t)(n_slices > 0 ? n_slices : size); }

#define GG_FILTER_RET()                                                \
    count_launches(1);                                                 \
    return cudaGetLastError() == cudaSuccess ? GG_OK : GG_ERR_CUDA

extern "C" int gg_filter_complex_to_cas(const float *d_complex, float *d_cas, int size, int n_slices, void *stream)
{
    if (size <= 0 || n_slices < 0 || !d_complex || !d_cas) return GG_ERR_INVALID_ARG;
    const size_t c = slice_count(size, n_slices);
    f_complex_to_cas<<<grid_for(c, kT), kT, 0, (cudaStream_t)stream>>>((const float2 *)d_complex, d_cas, c);
    GG_FILTER_RET();
}

extern "C" int gg_filter_cas_to_complex(const float *d_cas, float *d_complex, int size, int n_slices, void *stream)
{
    if (size <= 0 || n_slices < 0 || !d_complex || !d_cas) return GG_ERR_INVALID_ARG;
    const bool vol3 = n_slices == 0;
    const int nsl = vol3 ? size : n_slices;
    f_cas_to_complex<<<grid_for(slice_count(size, nsl), kT), kT, 0, (cudaStream_t)stream>>>(d_cas, (float2 *)d_complex, size, nsl, vol3);
    GG_FILTER_RET();
}

extern "C" int gg_filter_fftshift_2d(float *d_data, int complex_elems, int size, int n_slices, void *stream)
{
    if (size <= 0 || (size & 1) || n_slices <= 0 || !d_data) return GG_ERR_INVALID_ARG;
    const unsigned g = grid_for((size_t)size * (size / 2) * n_slices, kT);
    if (complex_elems) f_fftshift_2d<float2><<<g, kT, 0, (cudaStream_t)stream>>>((float2 *)d_data, size, n_slices);
    else f_fftshift_2d<float><<<g, kT, 0, (cudaStream_t)stream>>>(d_data, size, n_slices);
    GG_FILTER_RET();
}

extern "C" int gg_filter_fftshift_3d(float *d_data, int complex_elems, int size, void *stream)
{
    if (size <= 0 || (size & 1) || !d_data) return GG_ERR_INVALID_ARG;
    const unsigned g = grid_for((size_t)size * size * (size / 2), kT);
    if (complex_elems) f_fftshift_3d<float2><<<g, kT, 0, (cudaStream_t)stream>>>((float2 *)d_data, size);
    else f_fftshift_3d<float><<<g, kT, 0, (cudaStream_t)stream>>>(d_data, size);
    GG_FILTER_RET();
}

extern "C" int gg_filter_pad_volume(const float *d_in, float *d_out, int in_x, int in_y, int in_z, int pad_x, int pad_y,
                                    int pad_z, void *stream)
{
    if (in_x <= 0 || in_y <= 0 || in_z <= 0 || pad_x < 0 || pad_y < 0 || pad_z < 0 || !d_in || !d_out) return GG_ERR_INVALID_ARG;
    const size_t c = (size_t)(in_x + 2 * pad_x) * (in_y + 2 * pad_y) * (in_z + 2 * pad_z);
    f_pad<<<grid_for(c, kT), kT, 0, (cudaStream_t)stream>>>(d_in, d_out, in_x, in_y, in_z, pad_x, pad_y, pad_z);
    GG_FILTER_RET();
}

extern "C" int gg_filter_crop_volume(const float *d_in, float *d_out, int in_x, int in_y, int in_z, int crop_x, int crop_y,
                                     int crop_z, void *stream)
{
    if (in_x <= 0 || in_y <= 0 || in_z <= 0 || crop_x < 0 || crop_y < 0 || crop_z < 0 || 2 * crop_x >= in_x ||
        2 * crop_y >= in_y || 2 * crop_z >= in_z || !d_in || !d_out)
        return GG_ERR_INVALID_ARG;
    const size_t c = (size_t)(in_x - 2 * crop_x) * (in_y - 2 * crop_y) * (in_z - 2 * crop_z);
    f_crop<<<grid_for(c, kT), kT, 0, (cudaStream_t)stream>>>(d_in, d_out, in_x, in_y, in_z, crop_x, crop_y, crop_z);
    GG_FILTER_RET();
}

extern "C" int gg_filter_divide_volumes(float *d_a, const float *d_b, int size, int n_slices, void *stream)
{
    if (size <= 0 || n_slices < 0 || !d_a || !d_b) return GG_ERR_INVALID_ARG;
    const size_t c = slice_count(size, n_slices);
    f_divide_volumes<<<grid_for(c, kT), kT, 0, (cudaStream_t)stream>>>(d_a, d_b, c);
    GG_FILTER_RET();
}

extern "C" int gg_filter_multiply_volumes(float *d_a, const float *d_b, int a_complex, int size, int n_slices, void *stream)
{
    if (size <= 0 || n_slices < 0 || !d_a || !d_b) return GG_ERR_INVALID_ARG;
    const size_t c = slice_count(size, n_slices);
    f_multiply<<<grid_for(c, kT), kT, 0, (cudaStream_t)stream>>>(d_a, d_b, c, a_complex != 0);
    GG_FILTER_RET();
}

extern "C" int gg_filter_add_volumes(float *d_a, const float *d_b, int size, int n_slices, void *stream)
{
    if (size <= 0 || n_slices < 0 || !d_a || !d_b) return GG_ERR_INVALID_ARG;
    const size_t c = slice_count(size, n_slices);
    f_add<<<grid_for(c, kT), kT, 0, (cudaStream_t)stream>>>(d_a, d_b, c);
    GG_FILTER_RET();
}

extern "C" int gg_filter_divide_scalar(float *d_a, float scalar, int size, int n_slices, void *stream)
{
    if (size <= 0 || n_slices < 0 || !d_a) return GG_ERR_INVALID_ARG;
    const size_t c = slice_count(size, n_slices);
    f_div_scalar<<<grid_for(c, kT), kT, 0, (cudaStream_t)stream>>>(d_a, scalar, c);
    GG_FILTER_RET();
}

extern "C" int gg_filter_real_to_complex(const float *d_real, float *d_complex, int size, int n_slices, void *stream)
{
    if (size <= 0 || n_slices < 0 || !d_real || !d_complex) return GG_ERR_INVALID_ARG;
    const size_t c = slice_count(size, n_slices);
    f_real_to_complex<<<grid_for(c, kT), kT, 0, (cudaStream_t)stream>>>(d_real, (float2 *)d_complex, c);
    GG_FILTER_RET();
}

extern "C" int gg_filter_complex_to_real(const float *d_complex, float *d_real, int size, int n_slices, void *stream)
{
    if (size <= 0 || n_slices < 0 || !d_real || !d_complex) return GG_ERR_INVALID_ARG;
    const size_t c = slice_count(size, n_slices);
    f_complex_to_real<<<grid_for(c, kT), kT, 0, (cudaStream_t)stream>>>((const float2 *)d_complex, d_real, c);
    GG_FILTER_RET();
}

extern "C" int gg_filter_apply_ctf(float *d_cas_images, int cas_img_size, int n_images, const float *d_defocus,
                                   const float *d_defocus_v, const float *d_astig_angle, float voltage_kv, float cs_mm,
                                   float amp_contrast, float pixel_size, int power, int generate, void *stream)
{
    if (cas_img_size <= 0 || n_images < 0 || (n_images > 0 && (!d_cas_images || !d_defocus)) ||
        (power != 1 && power != 2) || !(voltage_kv > 0.0f) || !(pixel_size > 0.0f) ||
        !(amp_contrast >= 0.0f && amp_contrast <= 1.0f) || !std::isfinite(cs_mm) ||
        ((d_defocus_v == nullptr) != (d_astig_angle == nullptr)))
        return GG_ERR_INVALID_ARG;
    const CtfParams c{voltage_kv, cs_mm, amp_contrast, pixel_size};
    return launch_ctf(generate ? nullptr : d_cas_images, power, generate ? d_cas_images : nullptr, power,
                      cas_img_size, n_images, d_defocus, d_defocus_v, d_astig_angle, c, (cudaStream_t)stream) ==
                   cudaSuccess
               ? GG_OK
               : GG_ERR_CUDA;
}
