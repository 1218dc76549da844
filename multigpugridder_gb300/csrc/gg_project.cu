// Kaiser-Bessel Fourier-slice projection kernels for GB300 (sm_103a).
//
//   forward projection   CAS volume -> CAS images (pixel-driven gather)
//   back projection      CAS images -> CAS volume, reference window rule
//   adjoint projection   exact adjoint of the forward projection
//
// Conventions follow the reference kernels (src/Projection/gpuForwardProject.cu,
// src/Projection/gpuBackProject.cu): x fastest, CAS-volume centre V/2, image
// centre M/2, nearest-index lookup into the KB table, int mask radius.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "gg_common.cuh"
#include "gg_internal.h"

namespace gg {

// ---------------------------------------------------------------------------
// Shared pieces
// ---------------------------------------------------------------------------

// Sample point of pixel (di, dj) (offsets from the image centre) in the CAS
// volume frame: the reference's nx*di + ny*dj + volCenter
// (gpuForwardProject.cu:53-55) as its build evaluates it, fma(nx, di, ny*dj) +
// vc, written with round-to-nearest intrinsics so the grouping cannot change.
// Shared by the forward and adjoint kernels so both see identical bits.
__device__ __forceinline__ float sample_coord(float n_x, float n_y, int di, int dj, int vc)
{
    return __fadd_rn(__fmaf_rn(n_x, (float)di, __fmul_rn(n_y, (float)dj)), (float)vc);
}

// A voxel's image-frame coordinate (gpuBackProject.cu:62-64),
// fma(a2, n2, fma(a0, n0, a1*n1)); every grouping of the three products gave
// the same results against the reference kernel, this one is fixed here.
__device__ __forceinline__ float voxel_proj(float a0, float a1, float a2, float n0, float n1, float n2)
{
    return __fmaf_rn(a2, n2, __fmaf_rn(a0, n0, __fmul_rn(a1, n1)));
}

// Table lookup of the reference's nearest-index KB rule,
// ker[roundf(fma(r, kerScale, kerCenter))], as floor(fma(r, kerScale,
// kerCenter + 1/2)): equal for every float r in [-2, 2] (checked
// exhaustively) and one conversion instead of a roundf and a conversion.
// Callers pass r in [-2, 2]; the clamp only keeps a NaN or infinite
// coordinate (bad axes) inside the table.  Entry k is read at sker[k * rep]
// (rep interleaved copies).
__device__ __forceinline__ float kb_weight(const float *sker, float r, float kerScale, float kerCenterHalf, int kerSize,
                                           int rep = 1)
{
    return sker[min(max(__float2int_rd(__fmaf_rn(r, kerScale, kerCenterHalf)), 0), kerSize - 1) * rep];
}

__device__ __forceinline__ void load_table(float *sker, const float *ker, int kerSize)
{
    for (int t = threadIdx.x; t < kerSize; t += blockDim.x) sker[t] = __ldg(ker + t);
}

// An attribute of the current device, cached per device ordinal (a process
// may drive GPUs of different kinds).  cache[] starts at zero; a racing
// first read stores the same value twice.
constexpr int kAttrCacheDevices = 64;

static int device_attr(cudaDeviceAttr attr, std::atomic<int> *cache, int fallback)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return fallback;
    }
    const bool cached = dev >= 0 && dev < kAttrCacheDevices;
    if (cached) {
        const int v = cache[dev].load(std::memory_order_relaxed);
        if (v > 0) return v;
    }
    int v = 0;
    if (cudaDeviceGetAttribute(&v, attr, dev) != cudaSuccess || v <= 0) {
        cudaGetLastError();
        return fallback;
    }
    if (cached) cache[dev].store(v, std::memory_order_relaxed);
    return v;
}

static int num_sms()
{
    static std::atomic<int> cache[kAttrCacheDevices];
    return device_attr(cudaDevAttrMultiProcessorCount, cache, 1);
}

// ---------------------------------------------------------------------------
// Forward projection
// ---------------------------------------------------------------------------
// One CTA = a 16x16 pixel tile of one direction; persistent grid-stride loop
// over (direction, tile) items, direction-major so that the CTAs resident at
// any time read the same few slabs of the volume.  Warps cover 8x4 pixel
// blocks, which keeps a warp's tap addresses compact in the volume.
//
// With a KB table whose first and last entries are zero (getKernelFiltTable
// forces both, getKernelFiltTable.m:12-13), only the 4 taps floor(f)-1 ..
// floor(f)+2 per axis can carry weight: of the reference's 5 taps around
// round(f) (gpuForwardProject.cu:63-98) the fifth always has |r| >= 2, is
// clamped to the table edge and weighs exactly zero.  TAPS = 5 keeps the
// reference's full window for tables without zero edges.
//
// The volume may be stored with a row pitch P >= V (plane pitch P*V; the
// reference's dense layout is P = V).  VEC (2-byte storage, 4 taps, P a
// multiple of 8, P >= V + 4): each row of 4 taps is read as the 8 elements from the 4-aligned
// x at or below floor(f) - 1 in two aligned vector loads, and the 4 x weights
// are placed at their offsets in an 8-wide weight vector (zeros elsewhere) once
// per pixel.  The extra terms are exact zeros, so the sums are those of the
// 4 scalar taps, bit for bit, for a finite volume.
constexpr int kFpTile = 16;
constexpr int kFpThreads = 256;

__device__ __forceinline__ void ld8(const float *p, float v[8])
{
    const float4 a = __ldg(reinterpret_cast<const float4 *>(p));
    const float4 b = __ldg(reinterpret_cast<const float4 *>(p) + 1);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}

__device__ __forceinline__ void ld8(const __half *p, float v[8])
{
    const uint2 a = __ldg(reinterpret_cast<const uint2 *>(p));
    const uint2 b = __ldg(reinterpret_cast<const uint2 *>(p) + 1);
    const unsigned w[4] = {a.x, a.y, b.x, b.y};
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const float2 f = __half22float2(*reinterpret_cast<const __half2 *>(&w[q]));
        v[2 * q] = f.x;
        v[2 * q + 1] = f.y;
    }
}

__device__ __forceinline__ void ld8(const __nv_bfloat16 *p, float v[8])
{
    const uint2 a = __ldg(reinterpret_cast<const uint2 *>(p));
    const uint2 b = __ldg(reinterpret_cast<const uint2 *>(p) + 1);
    const unsigned w[4] = {a.x, a.y, b.x, b.y};
#pragma unroll
    for (int q = 0; q < 4; q++) {
        v[2 * q] = __uint_as_float(w[q] << 16);
        v[2 * q + 1] = __uint_as_float(w[q] & 0xFFFF0000u);
    }
}

// The copy a TR forward projection reads for a direction (layout 0: x,
// 1: y, 2: z contiguous): the one whose contiguous axis is the most
// perpendicular to the viewing direction (ax + 6 .. ax + 8).
__device__ __forceinline__ int fp_copy_of(const float *ax)
{
    const float nz0 = fabsf(__ldg(ax + 6)), nz1 = fabsf(__ldg(ax + 7)), nz2 = fabsf(__ldg(ax + 8));
    return (nz1 < nz0 && nz1 <= nz2) ? 1 : (nz2 < nz0 && nz2 < nz1) ? 2 : 0;
}

// Directions of a TR launch grouped by the copy they read: order[] lists the
// directions reading copy 0, then copy 1, then copy 2, each group in
// direction order (a stable partition).  The forward projection runs its
// work in this order, so that at any time the directions in flight read one
// copy of the volume (72 MB at 128^3) instead of all three (216 MB, more
// than the 126 MB L2).  One CTA: counts, then each chunk of 1,024
// directions scattered with warp ballots and the running offsets.
constexpr int kOrdThreads = 1024;

__global__ void __launch_bounds__(kOrdThreads) fp_order_kernel(const float *__restrict__ axes, int n, int *__restrict__ order)
{
    __shared__ int cnt[3], base[3];
    __shared__ int wcnt[kOrdThreads / 32][3];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x < 3) cnt[threadIdx.x] = 0;
    __syncthreads();
    int c[3] = {0, 0, 0};
    for (int a = threadIdx.x; a < n; a += kOrdThreads) c[fp_copy_of(axes + 9 * (size_t)a)]++;
#pragma unroll
    for (int l = 0; l < 3; l++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c[l] += __shfl_xor_sync(0xffffffffu, c[l], o);
        if (lane == 0) atomicAdd(&cnt[l], c[l]);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        base[0] = 0;
        base[1] = cnt[0];
        base[2] = cnt[0] + cnt[1];
    }
    __syncthreads();
    const unsigned lt = (1u << lane) - 1u;
    for (int c0 = 0; c0 < n; c0 += kOrdThreads) {
        const int a = c0 + threadIdx.x;
        const int l = a < n ? fp_copy_of(axes + 9 * (size_t)a) : 3;
        unsigned m[3];
#pragma unroll
        for (int k = 0; k < 3; k++) m[k] = __ballot_sync(0xffffffffu, l == k);
        if (lane < 3) wcnt[warp][lane] = __popc(m[lane]);
        __syncthreads();
        if (l < 3) {
            int pos = base[l] + __popc(m[l] & lt);
            for (int w = 0; w < warp; w++) pos += wcnt[w][l];
            order[pos] = a;
        }
        __syncthreads();
        if (threadIdx.x < 3) {
            int t = 0;
            for (int w = 0; w < kOrdThreads / 32; w++) t += wcnt[w][threadIdx.x];
            base[threadIdx.x] += t;
        }
        __syncthreads();
    }
}

// TR: two more copies of the volume with y and z as the contiguous axis
// (volY[z][x][y], volZ[y][x][z]).  A warp's 8x4 pixels touch about
// 32 |n . e_c| + (perimeter) distinct volume rows per gather, e_c the
// contiguous axis and n the viewing direction, so each direction reads the
// copy whose contiguous axis is the most perpendicular to n.  FP32 (dense
// copies): each thread still sums its taps in the same order, so the results
// are identical.  VEC (pitched 2-byte copies): the rows of taps are read along
// the copy's contiguous axis, which changes only the order of the sums.
template <typename TV, int TAPS, bool VEC, bool TR = false>
__global__ void __launch_bounds__(kFpThreads)
fp_kernel(const TV *__restrict__ vol, int V, int P, float *__restrict__ img, int M,
          const float *__restrict__ axes, int maskR, const float *__restrict__ ker, int kerSize,
          float kerHW, int tilesX, long long nItems, const float *__restrict__ d_scale,
          const TV *__restrict__ volY, const TV *__restrict__ volZ, const int *__restrict__ order)
{
    const float outScale = d_scale ? *d_scale : 1.0f;
    __shared__ float sker[kMaxKerSize];
    load_table(sker, ker, kerSize);
    __syncthreads();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // 8x4 warp tiles (2 x 4 per CTA), or with TR 4x8 tiles (4 x 2) when the
    // copy's contiguous axis advances more per image row than per column, so
    // that the eight-pixel side of a warp runs along the volume's rows
    const int ic = M / 2, vc = V / 2;
    const float kerCenter = ((float)kerSize - 1) / 2;
    const float kerScale = kerCenter / kerHW;
    const float kerCenterHalf = kerCenter + 0.5f;
    const float convW = (float)(int)roundf(kerHW);
    const long long R2 = (long long)maskR * maskR;
    const int tilesPerImg = tilesX * tilesX;
    const size_t VV = (size_t)V * V, PV = (size_t)P * V;
    const long long V3 = (long long)VV * V;

    const bool items32 = nItems <= 0x7fffffffLL; // 32-bit division per item whenever it fits
    for (long long item = blockIdx.x; item < nItems; item += gridDim.x) {
        const int slot = items32 ? (int)((unsigned)item / (unsigned)tilesPerImg) : (int)(item / tilesPerImg);
        const int t = (int)(item - (long long)slot * tilesPerImg);
        const int a = order ? __ldg(order + slot) : slot; // the direction (and image) of this work slot
        const float *ax = axes + 9 * (size_t)a;
        // the copy (layout 0: x, 1: y, 2: z contiguous) whose contiguous axis
        // is the most perpendicular to the direction
        int lay = 0;
        bool tall = false;
        if (TR) {
            lay = fp_copy_of(ax);
            tall = fabsf(__ldg(ax + 3 + lay)) > fabsf(__ldg(ax + lay));
        }
        const int lx = tall ? (lane >> 3) | ((warp & 3) << 2) : (lane & 7) | ((warp & 1) << 3);
        const int ly = tall ? (lane & 7) | ((warp >> 2) << 3) : (lane >> 3) | ((warp >> 1) << 2);
        const int i = (t % tilesX) * kFpTile + lx;
        const int j = (t / tilesX) * kFpTile + ly;
        if (i >= M || j >= M) continue;
        float *out = img + (size_t)a * M * M + (size_t)j * M + i;
        const int di = i - ic, dj = j - ic;
        if ((long long)di * di + (long long)dj * dj > R2) {
            *out = 0.0f;
            continue;
        }
        const float nx0 = __ldg(ax + 0), nx1 = __ldg(ax + 1), nx2 = __ldg(ax + 2);
        const float ny0 = __ldg(ax + 3), ny1 = __ldg(ax + 4), ny2 = __ldg(ax + 5);
        const float fi = sample_coord(nx0, ny0, di, dj, vc);
        const float fj = sample_coord(nx1, ny1, di, dj, vc);
        const float fk = sample_coord(nx2, ny2, di, dj, vc);

        int b0, b1, b2;
        float wi[TAPS], wj[TAPS], wk[TAPS];
        if (TAPS == 4) {
            b0 = (int)floorf(fi) - 1;
            b1 = (int)floorf(fj) - 1;
            b2 = (int)floorf(fk) - 1;
#pragma unroll
            for (int d = 0; d < TAPS; d++) {
                // r lies in (-2, 2] for these taps: no clamp needed
                wi[d] = kb_weight(sker, (float)(b0 + d) - fi, kerScale, kerCenterHalf, kerSize);
                wj[d] = kb_weight(sker, (float)(b1 + d) - fj, kerScale, kerCenterHalf, kerSize);
                wk[d] = kb_weight(sker, (float)(b2 + d) - fk, kerScale, kerCenterHalf, kerSize);
            }
        } else {
            b0 = (int)roundf(fi) - 2;
            b1 = (int)roundf(fj) - 2;
            b2 = (int)roundf(fk) - 2;
#pragma unroll
            for (int d = 0; d < TAPS; d++) {
                wi[d] = kb_weight(sker, fminf(fmaxf((float)(b0 + d) - fi, -convW), convW), kerScale, kerCenterHalf, kerSize);
                wj[d] = kb_weight(sker, fminf(fmaxf((float)(b1 + d) - fj, -convW), convW), kerScale, kerCenterHalf, kerSize);
                wk[d] = kb_weight(sker, fminf(fmaxf((float)(b2 + d) - fk, -convW), convW), kerScale, kerCenterHalf, kerSize);
            }
        }

        float acc = 0.0f;
        const bool inside = b0 >= 0 && b1 >= 0 && b2 >= 0 && b0 + TAPS <= V && b1 + TAPS <= V && b2 + TAPS <= V;
        if (VEC && inside) {
            // the copy's axes, fastest first
            const int bc = lay == 0 ? b0 : lay == 1 ? b1 : b2;       // contiguous axis
            const int bb = lay == 0 ? b1 : b0;                        // middle axis
            const int ba = lay == 2 ? b1 : b2;                        // outer axis
            float wc[TAPS], wb[TAPS], wa[TAPS];
#pragma unroll
            for (int d = 0; d < TAPS; d++) {
                wc[d] = lay == 0 ? wi[d] : lay == 1 ? wj[d] : wk[d];
                wb[d] = lay == 0 ? wj[d] : wi[d];
                wa[d] = lay == 2 ? wj[d] : wk[d];
            }
            const int sft = bc & 3;
            float w8[8];
#pragma unroll
            for (int t = 0; t < 8; t++)
                w8[t] = t == sft ? wc[0] : t == sft + 1 ? wc[1] : t == sft + 2 ? wc[2] : t == sft + 3 ? wc[3] : 0.0f;
            const TV *base = (lay == 0 ? vol : lay == 1 ? volY : volZ) + (size_t)ba * PV + (size_t)bb * P + (bc - sft);
#pragma unroll
            for (int dk = 0; dk < TAPS; dk++) {
#pragma unroll
                for (int dj2 = 0; dj2 < TAPS; dj2++) {
                    float v[8];
                    ld8(base + (size_t)dk * PV + (size_t)dj2 * P, v);
                    float s = 0.0f;
#pragma unroll
                    for (int t = 0; t < 8; t++) s = fmaf(w8[t], v[t], s);
                    acc = fmaf(wb[dj2] * wa[dk], s, acc);
                }
            }
        } else if (TR && inside) {
            // element strides of x, y, z in the chosen copy
            const size_t sx = lay == 0 ? 1 : (size_t)V;
            const size_t sy = lay == 0 ? (size_t)V : lay == 1 ? 1 : VV;
            const size_t sz = lay == 2 ? 1 : VV;
            const TV *base = (lay == 0 ? vol : lay == 1 ? volY : volZ) + b0 * sx + b1 * sy + b2 * sz;
#pragma unroll
            for (int dk = 0; dk < TAPS; dk++) {
#pragma unroll
                for (int dj2 = 0; dj2 < TAPS; dj2++) {
                    const TV *p = base + dk * sz + dj2 * sy;
                    float s = 0.0f;
#pragma unroll
                    for (int d = 0; d < TAPS; d++) s = fmaf(wi[d], ld_f32(p + d * sx), s);
                    acc = fmaf(wj[dj2] * wk[dk], s, acc);
                }
            }
        } else if (inside) {
            const TV *base = vol + (size_t)b2 * PV + (size_t)b1 * P + b0;
#pragma unroll
            for (int dk = 0; dk < TAPS; dk++) {
#pragma unroll
                for (int dj2 = 0; dj2 < TAPS; dj2++) {
                    const TV *p = base + (size_t)dk * PV + (size_t)dj2 * P;
                    float s = 0.0f;
#pragma unroll
                    for (int d = 0; d < TAPS; d++) s = fmaf(wi[d], ld_f32(p + d), s);
                    acc = fmaf(wj[dj2] * wk[dk], s, acc);
                }
            }
        } else {
            // Near the volume edge: the reference's linear-index test on the
            // dense layout (gpuForwardProject.cu:90), plus a lower bound.
            for (int dk = 0; dk < TAPS; dk++)
                for (int dj2 = 0; dj2 < TAPS; dj2++)
                    for (int d = 0; d < TAPS; d++) {
                        const long long lin = (long long)(b2 + dk) * (long long)VV + (long long)(b1 + dj2) * V + (b0 + d);
                        if (lin >= 0 && lin < V3) {
                            const long long row = lin / V;
                            acc = fmaf(wi[d] * wj[dj2] * wk[dk], ld_f32(vol + row * P + (lin - row * V)), acc);
                        }
                    }
        }
        *out = acc * outScale;
    }
}

template <typename TV, int TAPS, bool VEC, bool TR = false>
static cudaError_t launch_fp_t(const TV *vol, int P, float *img, const float *ker, const float *axes, int n,
                               const Geom &g, const float *scale, cudaStream_t s, const TV *volY = nullptr,
                               const TV *volZ = nullptr, int *order = nullptr)
{
    const int tilesX = (g.M + kFpTile - 1) / kFpTile;
    const long long nItems = (long long)n * tilesX * tilesX;
    if (nItems == 0) return cudaSuccess;
    if (!TR) order = nullptr;
    if (order) {
        fp_order_kernel<<<1, kOrdThreads, 0, s>>>(axes, n, order);
        count_launches(1);
    }
    int perSm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, fp_kernel<TV, TAPS, VEC, TR>, kFpThreads, 0);
    if (perSm <= 0) perSm = 1;
    long long grid = (long long)num_sms() * perSm;
    if (grid > nItems) grid = nItems;
    fp_kernel<TV, TAPS, VEC, TR><<<(unsigned)grid, kFpThreads, 0, s>>>(vol, g.V, P, img, g.M, axes, g.mask_radius,
                                                                        ker, g.ker_size, g.ker_hw, tilesX, nItems,
                                                                        scale, volY, volZ, order);
    count_launches(1);
    return cudaGetLastError();
}

template <typename TV>
static cudaError_t launch_fp_p(const void *d_vol, int P, float *d_img, const float *d_ker, const float *d_axes, int n,
                               const Geom &g, bool five_taps, const float *scale, cudaStream_t s,
                               const void *d_vol_y, const void *d_vol_z, int *d_order)
{
    const TV *v = (const TV *)d_vol;
    if (five_taps) return launch_fp_t<TV, 5, false>(v, P, d_img, d_ker, d_axes, n, g, scale, s);
    const TV *vy = (const TV *)d_vol_y, *vz = (const TV *)d_vol_z;
    if (sizeof(TV) == 4 && vy && vz && P == g.V)
        return launch_fp_t<TV, 4, false, true>(v, P, d_img, d_ker, d_axes, n, g, scale, s, vy, vz, d_order);
    // 2-byte storage only: with FP32 the 8-element rows double the bytes each
    // tap row moves through L1, which costs more than the loads it saves
    const bool vec = sizeof(TV) == 2 && P % 8 == 0 && P >= g.V + 4 && ((size_t)d_vol & 15) == 0;
    const bool aligned = ((size_t)vy & 15) == 0 && ((size_t)vz & 15) == 0;
    if (vec && vy && vz && aligned)
        return launch_fp_t<TV, 4, true, true>(v, P, d_img, d_ker, d_axes, n, g, scale, s, vy, vz, d_order);
    if (vec) return launch_fp_t<TV, 4, true>(v, P, d_img, d_ker, d_axes, n, g, scale, s);
    return launch_fp_t<TV, 4, false>(v, P, d_img, d_ker, d_axes, n, g, scale, s);
}

cudaError_t launch_forward_project(const void *d_vol, int vprec, int pitch, float *d_img, const float *d_ker,
                                   const float *d_axes, int n, const Geom &g, bool five_taps, const float *scale,
                                   cudaStream_t s, const void *d_vol_y, const void *d_vol_z, int *d_order)
{
    if (vprec == kF32)
        return launch_fp_p<float>(d_vol, pitch, d_img, d_ker, d_axes, n, g, five_taps, scale, s, d_vol_y, d_vol_z,
                                  d_order);
    if (vprec == kF16)
        return launch_fp_p<__half>(d_vol, pitch, d_img, d_ker, d_axes, n, g, five_taps, scale, s, d_vol_y, d_vol_z,
                                   d_order);
    return launch_fp_p<__nv_bfloat16>(d_vol, pitch, d_img, d_ker, d_axes, n, g, five_taps, scale, s, d_vol_y, d_vol_z,
                                      d_order);
}

// ---------------------------------------------------------------------------
// Back projection: the reference window and shared constants
// ---------------------------------------------------------------------------
// Directions are staged through shared memory in chunks of kBpChunk, two per
// thread of a brick group for the cull.
constexpr int kBpChunk = 512;

// Conservative reach of the slab test: fp32 rounding of f_imgk is far below this.
constexpr float kCullEps = 1e-2f;

struct RefWindow {
    float nx0, nx1, nx2, ny0, ny1, ny2; // direction columns x, y
    float vi, vj, vk;                   // voxel coordinates
    float vc;                           // volume centre
    float kerScale, kerCenterHalf;      // index = floor(r*kerScale + kerCenter + 1/2)
};

// Pixel (i1, j1)'s position along one volume axis, as the reference's build
// evaluates `(i1 - imgCenter) * nx + (j1 - imgCenter) * ny + volCenter`
// (gpuBackProject.cu:77,84,91): fma(pi, nx, pj*ny) + vc, identified by
// replaying the reference kernel's outputs.  Written with round-to-nearest
// intrinsics so no unrolling or hoisting can change which product is fused.
__device__ __forceinline__ float ref_pixel_pos(float pi, float pj, float n_x, float n_y, float vc)
{
    return __fadd_rn(__fmaf_rn(pi, n_x, __fmul_rn(pj, n_y)), vc);
}

// One voxel's 5x5 pixel window under the reference rule (gpuBackProject.cu:74-104),
// unrolled.  The table index floor(fma(r, kerScale, kerCenter + 1/2)) equals
// the reference's roundf(fma(r, kerScale, kerCenter)) for every float r in
// [-2, 2] (checked exhaustively): both round the same exact value once.
// INSIDE: the whole window lies in the image, so the reference's
// linear-index test always passes.  Table entry k is read at sker[k * rep].
// DW: cumW sums img2 * w (a second image back-projected in the same pass,
// fused as cumSum is) instead of w.
template <typename TI, bool ONES, bool DENS, bool INSIDE, bool DW = false>
__device__ __forceinline__ void ref_window(const RefWindow &q, const float *sker, int rep, const TI *__restrict__ img_ptr,
                                           int M, int imgi, int imgj, int imgCenter, float &cumSum, float &cumW,
                                           const float *__restrict__ img2_ptr = nullptr)
{
#pragma unroll
    for (int jo = -2; jo <= 2; jo++) {
        const int j1 = imgj + jo;
        const float pj = (float)(j1 - imgCenter);
#pragma unroll
        for (int io = -2; io <= 2; io++) {
            const int i1 = imgi + io;
            const float pi = (float)(i1 - imgCenter);
            float r = fminf(fmaxf(ref_pixel_pos(pi, pj, q.nx0, q.ny0, q.vc) - q.vi, -2.0f), 2.0f);
            float w = sker[__float2int_rd(__fmaf_rn(r, q.kerScale, q.kerCenterHalf)) * rep];
            r = fminf(fmaxf(ref_pixel_pos(pi, pj, q.nx1, q.ny1, q.vc) - q.vj, -2.0f), 2.0f);
            w = __fmul_rn(w, sker[__float2int_rd(__fmaf_rn(r, q.kerScale, q.kerCenterHalf)) * rep]);
            r = fminf(fmaxf(ref_pixel_pos(pi, pj, q.nx2, q.ny2, q.vc) - q.vk, -2.0f), 2.0f);
            w = __fmul_rn(w, sker[__float2int_rd(__fmaf_rn(r, q.kerScale, q.kerCenterHalf)) * rep]);
            const int lin = j1 * M + i1;
            if (INSIDE || (lin < M * M && lin >= 0)) {
                // cumSum += img * w, fused as the reference's build fuses it
                cumSum = __fmaf_rn(ONES ? 1.0f : ld_f32(img_ptr + lin), w, cumSum);
                if (DENS) cumW = __fadd_rn(cumW, w);
                if (DW) cumW = __fmaf_rn(__ldg(img2_ptr + lin), w, cumW);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Back projection, reference window rule
// ---------------------------------------------------------------------------
// Only the voxels inside a direction's slab (|f_imgk| <= 2, a few percent of
// the volume) run the 25-pixel window.  A group of 256 threads (8 warps) owns
// a 16x8x(2 BD) brick and each warp an 8x4xBD block of it, BD voxels per lane:
// block voxel l = lane + 32 s (x = l & 7, y = (l >> 3) & 3, z = l >> 5).  Per
// direction a warp tests its 32 BD voxels against the slab, lists the active
// ones in shared memory and runs them 32 at a time, one per lane.  Every voxel
// still receives its directions one by one in order and its window in the
// reference's order, so the per-voxel sums are those of the reference
// kernel's loops, bit for bit.  A CTA holds kBpGroups groups on neighbouring
// bricks, which share one copy of the KB table (below); each group
// synchronises on its own named barrier.
constexpr int kCBX = 16, kCBY = 8; // brick: 2x2x2 warp blocks of 8x4xBD (BD = 6, or 8 on large images)
constexpr int kCThreads = 256;  // threads of a group
constexpr int kBpGroups = 3;    // groups (bricks) per CTA, one CTA per SM
// The adjoint's and the two-stack form's 6-deep kernels run two groups per CTA: with the
// adjoint's 24-wide footprints, or the second stack's footprints, the voxel queue's two
// buffers fit only beside two groups (adjoint of 4,096 directions at 128^3: 67.8 ms with
// three one-buffer groups, 62.0 ms with two queued ones).
template <bool ADJ, bool DW, bool DEEP> constexpr int kGroupsOf = ((ADJ || DW) && !DEEP) ? 2 : kBpGroups;
static_assert(kBpChunk % kCThreads == 0, "the cull gives each thread kBpChunk / kCThreads directions");
// Depth of a warp block: 6 voxels, or 8 (DEEP, reference rule) on CAS images
// of 512^2 and more.  Deeper blocks have more active voxels per direction
// (fewer idle lanes in the last round of 32) and stage a footprint for more
// voxels, which pays most where the images are large (each staging reads from
// L2 or DRAM); on 256^2 images 8-deep blocks measured 20% slower than 4-deep
// ones and 6-deep ones 0.7% faster.  With 6 the footprint still fits 16
// pixels for any orthonormal axes (2 |(3.5, 1.5, 2.5)| + 1.2 < 11), and the
// adjoint's 7x7 windows fit 24.  The adjoint and the two-stack form had 4
// while their 256-thread CTAs held a padded table each; with the shared table
// copies 6-deep blocks measured faster for both (gradient step 89.6 -> 87.4
// ms, CTF-corrected reconstructVol 88.6 -> 84.1 ms).
template <bool ADJ, bool DW, bool DEEP>
struct BpShape {
    static constexpr int BD = DEEP ? 8 : 6;
    static constexpr int WV = 32 * BD;                         // voxels per warp block
    static constexpr int BZ = 2 * BD;                          // brick depth
    static constexpr int FW = ADJ ? 24 : (BD == 8 ? 20 : 16);  // footprint width and height
};

// The fast window.  For a voxel coordinate v and a window pixel whose
// volume-frame position along the same axis is Q, the reference's table
// index is floor(fma(clamp(fl(Q - v), -2, 2), s, h)), s = kerScale,
// h = kerCenter + 1/2 (see kb_weight).  For v >= 4 and |Q - v| <= 2,
// Sterbenz's lemma makes fl(Q - v) = Q - v exact, so that fma and
// fma(Q, s, h - v*s) round the same real number (h - v*s is exact: s and h
// are multiples of 1/4).  Scaled by 1/P, P a power of two >= kerSize - 1,
// y = fma(Q, s/P, (h - v*s)/P) is that rounded value over P exactly, and the
// saturating fma clamps it to [0, 1]: for |Q - v| > 2 it lands at or beyond
// the same end of the table as the reference's clamp, and a table of P + 1
// entries that repeats the last one past kerSize - 1 gives the clamped
// entry.  floor(P y) is the low bits of y + 1.5*2^23/P added with round-down.
// The unscaled index was checked on the CPU against the reference formula for
// every float Q within 4.2 of v (v = 4..40; tables of 501 and 1000 entries);
// the scaled, clamped entry on 1.4e8 values of Q within 4.2 of v (v up to
// 600), both neighbours of every index boundary among them, for tables of
// 501, 1000, 101 and 513 entries: identical entries.
//
// The table is held in `copies` interleaved copies (entry k of copy c at word
// k * copies + c) and lane l reads copy l % copies.  With 32 copies (66 KB
// for P = 512) each lane reads its own bank, so the three data-dependent
// lookups per pixel never conflict; shared by the groups of a CTA, the table
// fits beside their working sets.
//
// The pixels come from a per-warp footprint in shared memory: the pixels any
// window of the warp's block can touch, staged per direction with the
// reference's linear-index rule (a pixel whose index falls outside the image
// reads as zero), so the windows read them at constant offsets.
struct BpTable {
    int copies;          // interleaved copies (32: conflict-free)
    int entries;         // P + 1
    float scale;         // 1 / P
    float magic;         // 1.5 * 2^23 / P
    unsigned magic_bits; // its bits: entry floor(P y) sits at bits(y + magic) - magic_bits
};

// A 2-byte value held in the low 16 bits of u, widened to FP32 exactly.
template <typename T> __device__ __forceinline__ float widen16(unsigned u);
template <> __device__ __forceinline__ float widen16<__nv_bfloat16>(unsigned u) { return __uint_as_float(u << 16); }
template <> __device__ __forceinline__ float widen16<__half>(unsigned u)
{
    return __half2float(__ushort_as_half((unsigned short)u));
}
template <> __device__ __forceinline__ float widen16<float>(unsigned u) { return __uint_as_float(u); }

// Four consecutive values from a 4-element-aligned address, as FP32.
__device__ __forceinline__ void ld_quad(const float *p, float (&v)[4])
{
    const float4 q = __ldg(reinterpret_cast<const float4 *>(p));
    v[0] = q.x;
    v[1] = q.y;
    v[2] = q.z;
    v[3] = q.w;
}
template <typename T>
__device__ __forceinline__ void ld_quad(const T *p, float (&v)[4])
{
    const uint2 w = __ldg(reinterpret_cast<const uint2 *>(p));
    v[0] = widen16<T>(w.x & 0xffffu);
    v[1] = widen16<T>(w.x >> 16);
    v[2] = widen16<T>(w.y & 0xffffu);
    v[3] = widen16<T>(w.y >> 16);
}

__device__ __forceinline__ float lds_f32(unsigned addr)
{
    float v;
    asm("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(addr));
    return v;
}

struct FootWin {
    float nx0, nx1, nx2, ny0, ny1, ny2;
    float vc;         // volume centre
    float s;          // kerScale / P
    float c0, c1, c2; // (h - v*s) / P per axis
    float mg;         // 1.5 * 2^23 / P
    unsigned stride;  // bytes between table entries
};

// fma rounded to nearest, clamped to [0, 1] (a NaN gives 0).
__device__ __forceinline__ float fma_sat(float a, float b, float c)
{
    float d;
    asm("fma.rn.sat.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// One voxel's WI x WJ window from the footprint (fbase = its top-left pixel,
// rows FS apart); table entry floor(P y) is read at
// tab + bits(y + q.mg) * stride.  Sums row by row, as the reference.  TS: the
// stride in bytes when known at compile time (128 for 32 interleaved table
// copies, 4 for one), so the address is a shift-add on the integer pipe
// rather than a multiply on the FMA pipe; 0: q.stride.
template <bool DENS, int WI, int WJ, int FS, bool DW = false, int TS = 0>
__device__ __forceinline__ void foot_window(const FootWin &q, const float *fbase, unsigned tab, float pi0, float pj0,
                                            float &cumSum, float &cumW, const float *fbase2 = nullptr)
{
    const unsigned st = TS ? (unsigned)TS : q.stride;
#pragma unroll
    for (int jo = 0; jo < WJ; jo++) {
        const float pj = pj0 + (float)jo;
        const float py0 = __fmul_rn(pj, q.ny0), py1 = __fmul_rn(pj, q.ny1), py2 = __fmul_rn(pj, q.ny2);
#pragma unroll
        for (int io = 0; io < WI; io++) {
            const float pi = pi0 + (float)io;
            const float q0 = __fadd_rn(__fmaf_rn(pi, q.nx0, py0), q.vc);
            const float q1 = __fadd_rn(__fmaf_rn(pi, q.nx1, py1), q.vc);
            const float q2 = __fadd_rn(__fmaf_rn(pi, q.nx2, py2), q.vc);
            const unsigned b0 = __float_as_uint(__fadd_rd(fma_sat(q0, q.s, q.c0), q.mg));
            const unsigned b1 = __float_as_uint(__fadd_rd(fma_sat(q1, q.s, q.c1), q.mg));
            const unsigned b2 = __float_as_uint(__fadd_rd(fma_sat(q2, q.s, q.c2), q.mg));
            float w = lds_f32(tab + b0 * st);
            w = __fmul_rn(w, lds_f32(tab + b1 * st));
            w = __fmul_rn(w, lds_f32(tab + b2 * st));
            cumSum = __fmaf_rn(fbase[jo * FS + io], w, cumSum);
            if (DENS) cumW = __fadd_rn(cumW, w);
            if (DW) cumW = __fmaf_rn(fbase2[jo * FS + io], w, cumW);
        }
    }
}

// foot_window with adjacent pixels of a row taken in pairs by the packed
// FP32x2 instructions (sm_100+): the pixel positions, the table addresses and
// the weight products of two pixels per instruction (the saturating index fma
// has no packed form).  Each lane of a packed instruction rounds as the scalar
// instruction does, so every weight, and every sum (accumulated one pixel at a
// time in the same order), is bit-identical to foot_window's.
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

template <bool DENS, int WI, int WJ, int FS, bool DW = false, int TS = 0>
__device__ __forceinline__ void foot_window_x2(const FootWin &q, const float *fbase, unsigned tab, float pi0,
                                               float pj0, float &cumSum, float &cumW, const float *fbase2 = nullptr)
{
    const unsigned st = TS ? (unsigned)TS : q.stride;
    const float2 nx0 = f2(q.nx0, q.nx0), nx1 = f2(q.nx1, q.nx1), nx2 = f2(q.nx2, q.nx2);
    const float2 vc = f2(q.vc, q.vc), mg = f2(q.mg, q.mg);
#pragma unroll
    for (int jo = 0; jo < WJ; jo++) {
        const float pj = pj0 + (float)jo;
        const float py0 = __fmul_rn(pj, q.ny0), py1 = __fmul_rn(pj, q.ny1), py2 = __fmul_rn(pj, q.ny2);
        const float2 qy0 = f2(py0, py0), qy1 = f2(py1, py1), qy2 = f2(py2, py2);
#pragma unroll
        for (int io = 0; io + 1 < WI; io += 2) {
            const float2 pi = f2(pi0 + (float)io, pi0 + (float)(io + 1));
            const float2 q0 = __fadd2_rn(__ffma2_rn(pi, nx0, qy0), vc);
            const float2 q1 = __fadd2_rn(__ffma2_rn(pi, nx1, qy1), vc);
            const float2 q2 = __fadd2_rn(__ffma2_rn(pi, nx2, qy2), vc);
            const float2 b0 = __fadd2_rd(f2(fma_sat(q0.x, q.s, q.c0), fma_sat(q0.y, q.s, q.c0)), mg);
            const float2 b1 = __fadd2_rd(f2(fma_sat(q1.x, q.s, q.c1), fma_sat(q1.y, q.s, q.c1)), mg);
            const float2 b2 = __fadd2_rd(f2(fma_sat(q2.x, q.s, q.c2), fma_sat(q2.y, q.s, q.c2)), mg);
            const float2 t0 = f2(lds_f32(tab + __float_as_uint(b0.x) * st),
                                 lds_f32(tab + __float_as_uint(b0.y) * st));
            const float2 t1 = f2(lds_f32(tab + __float_as_uint(b1.x) * st),
                                 lds_f32(tab + __float_as_uint(b1.y) * st));
            const float2 t2 = f2(lds_f32(tab + __float_as_uint(b2.x) * st),
                                 lds_f32(tab + __float_as_uint(b2.y) * st));
            const float2 w = __fmul2_rn(__fmul2_rn(t0, t1), t2);
            cumSum = __fmaf_rn(fbase[jo * FS + io], w.x, cumSum);
            if (DENS) cumW = __fadd_rn(cumW, w.x);
            if (DW) cumW = __fmaf_rn(fbase2[jo * FS + io], w.x, cumW);
            cumSum = __fmaf_rn(fbase[jo * FS + io + 1], w.y, cumSum);
            if (DENS) cumW = __fadd_rn(cumW, w.y);
            if (DW) cumW = __fmaf_rn(fbase2[jo * FS + io + 1], w.y, cumW);
        }
        if (WI & 1) {
            constexpr int io = WI - 1;
            const float pi = pi0 + (float)io;
            const float q0 = __fadd_rn(__fmaf_rn(pi, q.nx0, py0), q.vc);
            const float q1 = __fadd_rn(__fmaf_rn(pi, q.nx1, py1), q.vc);
            const float q2 = __fadd_rn(__fmaf_rn(pi, q.nx2, py2), q.vc);
            const unsigned b0 = __float_as_uint(__fadd_rd(fma_sat(q0, q.s, q.c0), q.mg));
            const unsigned b1 = __float_as_uint(__fadd_rd(fma_sat(q1, q.s, q.c1), q.mg));
            const unsigned b2 = __float_as_uint(__fadd_rd(fma_sat(q2, q.s, q.c2), q.mg));
            float w = lds_f32(tab + b0 * st);
            w = __fmul_rn(w, lds_f32(tab + b1 * st));
            w = __fmul_rn(w, lds_f32(tab + b2 * st));
            cumSum = __fmaf_rn(fbase[jo * FS + io], w, cumSum);
            if (DENS) cumW = __fadd_rn(cumW, w);
            if (DW) cumW = __fmaf_rn(fbase2[jo * FS + io], w, cumW);
        }
    }
}

static int max_dyn_smem()
{
    static std::atomic<int> cache[kAttrCacheDevices];
    return device_attr(cudaDevAttrMaxSharedMemoryPerBlockOptin, cache, 48 * 1024);
}

// The table layout for kerSize entries beside other_bytes of shared memory:
// P = 512 (kerSize <= 513) or the next power of two, and as many copies, 32
// down to 1, as fit.  copies = 0: not even one copy fits.
static BpTable bp_table(int kerSize, size_t other_bytes, int max_copies = 32, size_t limit_bytes = 0)
{
    int P = 512;
    while (P < kerSize - 1) P *= 2;
    BpTable t;
    t.entries = P + 1;
    t.scale = 1.0f / (float)P;
    t.magic = 12582912.0f / (float)P;
    std::memcpy(&t.magic_bits, &t.magic, sizeof(float));
    t.copies = max_copies;
    const size_t limit = limit_bytes ? limit_bytes : (size_t)max_dyn_smem();
    while (t.copies > 0 && (((size_t)t.entries * t.copies + 3) & ~(size_t)3) * sizeof(float) + other_bytes > limit)
        t.copies /= 2;
    return t;
}

// The exact adjoint of fp_kernel<., 4> for one voxel, without the fast
// path's assumptions: every in-mask pixel whose 4^3 forward window contains
// the voxel, with the forward weight.  Such a pixel lies within 2*sqrt(3) of
// the voxel's projection.
template <typename TI>
__device__ float adjoint_window_slow(int vi, int vj, int vk, int volCenter, float nx0, float nx1, float nx2, float ny0,
                                     float ny1, float ny2, const TI *__restrict__ img_ptr, int M, int imgCenter,
                                     int maskR, const float *sker, int rep, float kerScale, float kerCenterHalf,
                                     int kerSize)
{
    const float pi = ((float)vi - volCenter) * nx0 + ((float)vj - volCenter) * nx1 + ((float)vk - volCenter) * nx2;
    const float pj = ((float)vi - volCenter) * ny0 + ((float)vj - volCenter) * ny1 + ((float)vk - volCenter) * ny2;
    const int ilo = (int)ceilf(pi - 3.47f), ihi = (int)floorf(pi + 3.47f);
    const int jlo = (int)ceilf(pj - 3.47f), jhi = (int)floorf(pj + 3.47f);
    const long long R2 = (long long)maskR * maskR;
    float s = 0.0f;
    for (int dj = jlo; dj <= jhi; dj++) {
        for (int di = ilo; di <= ihi; di++) {
            if ((long long)di * di + (long long)dj * dj > R2) continue;
            const int pxi = di + imgCenter, pxj = dj + imgCenter;
            if (pxi < 0 || pxi >= M || pxj < 0 || pxj >= M) continue;
            const float fi = sample_coord(nx0, ny0, di, dj, volCenter);
            const float fj = sample_coord(nx1, ny1, di, dj, volCenter);
            const float fk = sample_coord(nx2, ny2, di, dj, volCenter);
            // membership in the forward window floor(f)-1 .. floor(f)+2
            const int oi = vi - ((int)floorf(fi) - 1), oj = vj - ((int)floorf(fj) - 1), ok = vk - ((int)floorf(fk) - 1);
            if ((unsigned)oi > 3u || (unsigned)oj > 3u || (unsigned)ok > 3u) continue;
            const float w = kb_weight(sker, (float)vi - fi, kerScale, kerCenterHalf, kerSize, rep) *
                            kb_weight(sker, (float)vj - fj, kerScale, kerCenterHalf, kerSize, rep) *
                            kb_weight(sker, (float)vk - fk, kerScale, kerCenterHalf, kerSize, rep);
            s = fmaf(w, ld_f32(img_ptr + (size_t)pxj * M + pxi), s);
        }
    }
    return s;
}

// ADJ: the exact adjoint of fp_kernel<., 4> (gradient of the forward
// projection) instead of the reference rule.  The same pixel positions and
// table indices (sample_coord is the reference's pixel-position expression),
// a 7x7 window around the voxel's projection for voxels within 2*sqrt(3) of
// the plane, pixels outside the image or the mask staged as zero, and the
// index of r = v - Q: floor(fma(Q, -s, h + v*s)).  With a zero-edge table
// every pixel whose forward window misses the voxel gets weight 0, so the
// wider window adds exact zeros (zero_edges; otherwise the slow path checks
// window membership as the forward does).
// DW (reference rule, FP32 images): pd accumulates the back projection of a
// second image stack img2 (the same directions) in the same pass, with the
// same weights and summation order as a separate back projection of img2.
// What a queued voxel's window needs of its direction, copied when the
// direction's footprint is staged.
struct alignas(16) BpDirMeta {
    float nx0, nx1, nx2, ny0, ny1, ny2;
    int fi0, fj0, fh, foot, dir, pad;
};

// A warp's queue of voxel windows: entries (block voxel | footprint buffer
// << 8) in direction order, run 32 at a time, so that rounds are full across
// directions.  NB footprint buffers per warp: 2 where shared memory allows
// (the 6-deep reference-rule form, and the adjoint's with two groups per CTA;
// a direction's footprint is staged while the previous direction's last
// voxels still wait in the queue); else 1, and each direction's active voxels
// run at once from the same array (a plain list, no queue): queue rounds with
// one buffer measured slower (per-lane direction records, spills).
template <bool ADJ, bool DW, bool DEEP>
struct BpQueue {
    static constexpr int NB = !DEEP ? 2 : 1;
    static constexpr int NEED = (NB - 1) * 31 + BpShape<ADJ, DW, DEEP>::WV; // most entries held at once
    static constexpr int CAP = NEED <= 128 ? 128 : (NEED <= 256 ? 256 : 512);
};

// One group's working set in shared memory (after the table).  LEAN (the
// launches that own the GPU): 8-bit queue entries with the footprint buffer
// tracked per warp, 16-bit direction-list entries, and in the two-buffer form
// footprint rows of FW + 4 pixels from fi0 & ~3 (16-byte aligned, written by
// vector stores).  Otherwise (the serving lanes' one-group CTAs): 16-bit
// entries carrying the buffer bit, rows of FW + 1 pixels from fi0.
template <bool DENS, bool ADJ, bool DW, bool DEEP, bool LEAN = true>
struct BpGroupMem {
    using Shape = BpShape<ADJ, DW, DEEP>;
    using Q = BpQueue<ADJ, DW, DEEP>;
    using QEnt = typename std::conditional<LEAN, unsigned char, unsigned short>::type;
    using LEnt = typename std::conditional<LEAN, unsigned short, int>::type;
    static constexpr int NW = kCThreads / 32, WV = Shape::WV,
                         FP = Shape::FW * (Shape::FW + (LEAN && Q::NB == 2 ? 4 : 1));
    BpDirMeta smeta[NW * Q::NB];
    float sax[kBpChunk * 9];
    LEnt slist[kBpChunk];
    int swarp[kBpChunk / 32]; // kept directions per (pass, warp)
    int scount;
    // per-voxel sums [warp][block voxel]; a voxel is updated by at most one
    // lane per direction, directions in order, so no atomics are needed
    float sacc[NW * WV];
    float saccw[DENS || DW ? NW * WV : 1];
    alignas(16) float sfoot[NW * Q::NB * FP];
    float sfoot2[DW ? NW * Q::NB * FP : 1];
    QEnt squeue[NW * Q::CAP];
};

// Bricks of x-width kCBX in row (y brick j, z brick k) that meet the sphere of
// radius reach about the volume centre c (within the +1 margin of the test
// d^2 <= reach^2 + 1, d the distance from the centre to the brick's box):
// x bricks lo .. lo + n - 1.  In doubled coordinates the box's distance per
// axis is max(|2 B i + B - 1 - 2c| - (B - 1), 0) for bricks of size B, all
// integers, so the test is exact; along x the bricks that pass form the
// interval |2 B i + B - 1 - 2c| <= B - 1 + t, t = isqrt(rem).
__device__ __forceinline__ int box_dist2(int i, int B, int c)
{
    return max(abs(2 * B * i + B - 1 - 2 * c) - (B - 1), 0);
}

__device__ __forceinline__ int floor_div(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

__device__ void brick_row(int j, int k, int bricksX, int c, int BZ, int reach, int &lo, int &n)
{
    const long long dy = box_dist2(j, kCBY, c), dz = box_dist2(k, BZ, c);
    const long long rem = 4 * ((long long)reach * reach + 1) - dy * dy - dz * dz;
    lo = 0;
    n = 0;
    if (rem < 0) return;
    long long t = (long long)sqrt((double)rem);
    while (t * t > rem) t--;
    while ((t + 1) * (t + 1) <= rem) t++;
    const int B = kCBX;
    const int ilo = max(-floor_div(-(2 * c - 2 * (B - 1) - (int)t), 2 * B), 0); // ceil
    const int ihi = min(floor_div(2 * c + (int)t, 2 * B), bricksX - 1);
    if (ihi >= ilo) {
        lo = ilo;
        n = ihi - ilo + 1;
    }
}

__device__ __forceinline__ void group_sync(int id)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "n"(kCThreads) : "memory");
}

template <typename TI, bool ONES, bool DENS, bool ADJ, bool DW = false, bool DEEP = false, int G = kBpGroups,
          int TS = 0, bool LEAN = true>
__global__ void __launch_bounds__(kCThreads *G, G == 1 ? 3 : 1)
bp_ref_compact_kernel(float *__restrict__ vol, float *__restrict__ pd, int V, const TI *__restrict__ img, int M,
                      const float *__restrict__ axes, int n, int maskR, const float *__restrict__ ker, int kerSize,
                      float kerHW, int bricksX, int bricksY, BpTable tb, int zeroEdges,
                      const float *__restrict__ d_scale, const float *__restrict__ img2, int vecImg)
{
    static_assert(!DW || (!ONES && !DENS && !ADJ), "the second image stack is a reference-rule option");
    constexpr int W = ADJ ? 7 : 5, HALF = W / 2;
    using Shape = BpShape<ADJ, DW, DEEP>;
    constexpr int BD = Shape::BD, kWarpVox = Shape::WV, kCBZ = Shape::BZ;
    // LEAN two-buffer form: footprint rows hold the pixels from fi0 & ~3 (16-byte aligned rows)
    constexpr bool QALIGN = LEAN && BpQueue<ADJ, DW, DEEP>::NB == 2;
    constexpr int FW = Shape::FW, FH = FW, FS = FW + (QALIGN ? 4 : 1);
    using Mem = BpGroupMem<DENS, ADJ, DW, DEEP, LEAN>;
    using QEnt = typename Mem::QEnt;
    // [table: tb.entries x tb.copies][G x Mem][row starts][row prefix]
    extern __shared__ __align__(16) float bp_smem[];
    const int cp = tb.copies, tabWords = tb.entries * cp;
    Mem *gmem = reinterpret_cast<Mem *>(bp_smem + ((tabWords + 3) & ~3)); // 16-byte aligned
    int *slo = reinterpret_cast<int *>(gmem + G), *spre = slo + bricksY;
    const int volCenter = (int)((float)V) / 2;
    const int imgCenter = (int)((float)M) / 2;

    // The CTA's bricks: those of z-layer blockIdx.y that meet the sphere of
    // radius `reach` (the adjoint reaches voxels up to 2*sqrt(3) beyond the
    // mask), numbered row by row; the CTA takes the run of RUN * G numbers
    // from RUN * G * blockIdx.x (below).  Row (y, z) holds the x interval
    // [slo, slo + n).
    const int reach = ADJ ? maskR + 4 : maskR;
    const int kz = blockIdx.y;
    for (int j = threadIdx.x; j < bricksY; j += blockDim.x) {
        int lo, n;
        brick_row(j, kz, bricksX, volCenter, kCBZ, reach, lo, n);
        slo[j] = lo;
        spre[j] = n;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int j = 0; j < bricksY; j++) {
            const int c = spre[j];
            spre[j] = acc;
            acc += c;
        }
        spre[bricksY] = acc;
    }
    __syncthreads();
    const int total = spre[bricksY];
    if (((DEEP && G > 1) ? 2 : 1) * G * (int)blockIdx.x >= total) return; // the whole CTA
    for (int t = threadIdx.x; t < tabWords; t += blockDim.x) bp_smem[t] = __ldg(ker + min(t / cp, kerSize - 1));
    __syncthreads();

    // Group g runs brick g of the CTA's run of RUN * G bricks, and
    // with 8-deep blocks (RUN = 2) then brick 2 G - 1 - g: along a run
    // the work drifts (about 2/r of the directions reach a voxel at radius r),
    // and the mirrored pairs even it out.  On 512^2 images that measured 2-3%
    // faster; on 256^2 images 8% slower, as the groups drift apart in time and
    // lose the L1 reuse of the neighbouring bricks' footprints.
    constexpr int RUN = (DEEP && G > 1) ? 2 : 1;
    const int grp = threadIdx.x / kCThreads;
    for (int pass = 0; pass < RUN; pass++) {
        const int a = RUN * G * blockIdx.x + (pass == 0 ? grp : RUN * G - 1 - grp);
        if (a >= total) break;
        int row = 0; // the last row whose prefix is <= a (it holds brick a)
        for (int hi = bricksY - 1; row < hi;) {
            const int mid = (row + hi + 1) >> 1;
            if (spre[mid] <= a) row = mid;
            else hi = mid - 1;
        }
        Mem &sm = gmem[grp];
        float *sax = sm.sax;
        typename Mem::LEnt *slist = sm.slist;
        int *swarp = sm.swarp;
        const int tid = threadIdx.x - grp * kCThreads, warp = tid >> 5, lane = tid & 31;
        const int x0 = (slo[row] + a - spre[row]) * kCBX, y0 = row * kCBY, z0 = kz * kCBZ;
        const int bx = x0 + (warp & 1) * 8, by = y0 + ((warp >> 1) & 1) * 4, bz = z0 + (warp >> 2) * BD;
        const float *sker = bp_smem + lane % cp; // entry k at sker[k * cp]
        const unsigned stride = 4u * (unsigned)cp;
        const unsigned tab = (unsigned)__cvta_generic_to_shared(bp_smem) + 4u * (unsigned)(lane % cp) - tb.magic_bits * stride;
        constexpr int NB = BpQueue<ADJ, DW, DEEP>::NB, QM = BpQueue<ADJ, DW, DEEP>::CAP - 1;
        float *const wfoot0 = sm.sfoot + warp * (NB * FH * FS);
        float *const wfoot20 = sm.sfoot2 + (DW ? warp * (NB * FH * FS) : 0);
        BpDirMeta *const wmeta = sm.smeta + warp * NB;
        QEnt *const wq = sm.squeue + warp * (QM + 1);
        float *const wacc = sm.sacc + warp * kWarpVox;
        float *const waccw = sm.saccw + (DENS || DW ? warp * kWarpVox : 0);

        // this lane's voxels: x = lx, y = ly, z = bz + s
        const int lx = bx + (lane & 7), ly = by + (lane >> 3);
        const long long R2 = (long long)maskR * maskR;
        const long long reach2 = ADJ ? (long long)(maskR + 4) * (maskR + 4) : R2;
        unsigned inmask = 0;
#pragma unroll
        for (int s = 0; s < BD; s++) {
            const int lz = bz + s;
            const long long d2 = (long long)(lx - volCenter) * (lx - volCenter) + (long long)(ly - volCenter) * (ly - volCenter) +
                                 (long long)(lz - volCenter) * (lz - volCenter);
            if (lx < V && ly < V && lz < V && d2 <= reach2) inmask |= 1u << s;
            wacc[lane + 32 * s] = 0.0f;
            if (DENS || DW) waccw[lane + 32 * s] = 0.0f;
        }
        const float kerCenter = ((float)kerSize - 1) / 2;
        const float kerScale = kerCenter / kerHW;
        const float kerCenterHalf = kerCenter + 0.5f;
        const float ax0 = (float)lx - volCenter, ay0 = (float)ly - volCenter;
        const float wcx = bx + 3.5f - volCenter, wcy = by + 1.5f - volCenter, wcz = bz + 0.5f * (BD - 1) - volCenter;
        // slab half-thickness: kerHW for the reference rule; for the adjoint, any
        // voxel within the 4^3 window of a sample point (|r| < 2 per axis)
        const float slab = ADJ ? 2.0f * 1.7320508f + kCullEps : kerHW + kCullEps;
        const int MM = M * M;
        // Directions are staged through shared memory in chunks, culled against
        // the brick (compacted in order), then against each warp's 8x4xBD block.
        const float bcx = x0 + 0.5f * (kCBX - 1) - volCenter, bcy = y0 + 0.5f * (kCBY - 1) - volCenter,
                    bcz = z0 + 0.5f * (kCBZ - 1) - volCenter;
        const unsigned lt_mask = (1u << lane) - 1u;
        // the warp's queue (uniform): qsize entries from qhead.  LEAN: the first
        // nfront belong to footprint buffer bfront, the rest to the other
        // buffer; otherwise each entry carries its buffer in bit 8
        int qhead = 0, qsize = 0, nbuf = 0, nfront = 0, bfront = 0;

        // One voxel's window sum for one direction: the fast window from the
        // footprint, or the reference's (or the adjoint's) window from the image.
        auto voxel_window = [&](const int l, const float nx0, const float nx1, const float nx2, const float ny0,
                                const float ny1, const float ny2, const int fi0, const int fj0, const int fh,
                                const bool foot, const TI *img_ptr, const float *img2_ptr, const float *wfoot,
                                const float *wfoot2, float &cs, float &cw) {
            const int vi = bx + (l & 7), vj = by + ((l >> 3) & 3), vk = bz + (l >> 5);
            const float a0 = (float)vi - volCenter, a1 = (float)vj - volCenter, a2 = (float)vk - volCenter;
            const float f_imgi = __fadd_rn(voxel_proj(a0, a1, a2, nx0, nx1, nx2), (float)imgCenter);
            const float f_imgj = __fadd_rn(voxel_proj(a0, a1, a2, ny0, ny1, ny2), (float)imgCenter);
            const int imgi = (int)roundf(f_imgi);
            const int imgj = (int)roundf(f_imgj);
            const bool inside = imgi >= 2 && imgj >= 2 && imgi + 2 < M && imgj + 2 < M;
            const int ri = imgi - HALF - fi0, rj = imgj - HALF - fj0;
            if (foot && (unsigned)ri <= (unsigned)(FW - W) && (unsigned)rj <= (unsigned)(fh - W) && vi >= 4 &&
                vj >= 4 && vk >= 4 && (ADJ || inside || !DENS)) {
                // reference rule: index of r = Q - v; adjoint: of r = v - Q
                const float sg = ADJ ? -kerScale : kerScale;
                // scaled by 1/P (exact): the saturating index form
                const FootWin fwin{nx0, nx1, nx2, ny0, ny1, ny2, (float)volCenter, sg * tb.scale,
                                   (kerCenterHalf - (float)vi * sg) * tb.scale,
                                   (kerCenterHalf - (float)vj * sg) * tb.scale,
                                   (kerCenterHalf - (float)vk * sg) * tb.scale, tb.magic, stride};
                const float *fb = wfoot + rj * FS + ri + (QALIGN ? (fi0 & 3) : 0);
                const float pi0 = (float)(imgi - HALF - imgCenter), pj0 = (float)(imgj - HALF - imgCenter);
                foot_window_x2<DENS, W, W, FS, DW, TS>(fwin, fb, tab, pi0, pj0, cs, cw,
                                                DW ? wfoot2 + rj * FS + ri + (QALIGN ? (fi0 & 3) : 0) : nullptr);
            } else if (ADJ) {
                cs = adjoint_window_slow<TI>(vi, vj, vk, volCenter, nx0, nx1, nx2, ny0, ny1, ny2, img_ptr, M,
                                             imgCenter, maskR, sker, cp, kerScale, kerCenterHalf, kerSize);
            } else {
                const RefWindow rw{nx0, nx1, nx2, ny0, ny1, ny2, (float)vi, (float)vj, (float)vk,
                                   (float)volCenter, kerScale, kerCenterHalf};
                if (inside)
                    ref_window<TI, ONES, DENS, true, DW>(rw, sker, cp, img_ptr, M, imgi, imgj, imgCenter, cs, cw,
                                                         img2_ptr);
                else
                    ref_window<TI, ONES, DENS, false, DW>(rw, sker, cp, img_ptr, M, imgi, imgj, imgCenter, cs, cw,
                                                          img2_ptr);
            }
        };

        // One round of the queue (NB = 2): its first cnt (<= 32) voxels, one per
        // lane.  Each voxel's window sum is added to its total in direction
        // order: the round holds at most one direction per buffer, the older
        // one's first.
        auto run_round = [&](const int cnt) {
            float cs = 0.0f, cw = 0.0f;
            int l = 0, b = 0;
            if (lane < cnt) {
                const unsigned ent = wq[(qhead + lane) & QM];
                l = ent & 0xff;
                b = LEAN ? (lane < nfront ? bfront : (bfront ^ 1)) : (int)(ent >> 8);
                const BpDirMeta m = wmeta[b];
                voxel_window(l, m.nx0, m.nx1, m.nx2, m.ny0, m.ny1, m.ny2, m.fi0, m.fj0, m.fh, m.foot != 0,
                             img + (size_t)m.dir * MM, DW ? img2 + (size_t)m.dir * MM : nullptr, wfoot0 + b * (FH * FS),
                             wfoot20 + (DW ? b * (FH * FS) : 0), cs, cw);
            }
            // cumSumAllAxes += cumSum (gpuBackProject.cu:106), in direction order
            const int bf = LEAN ? bfront : (int)(wq[qhead & QM] >> 8);
            if (lane < cnt && b == bf) {
                wacc[l] = __fadd_rn(wacc[l], cs);
                if (DENS || DW) waccw[l] = __fadd_rn(waccw[l], cw);
            }
            __syncwarp();
            if (lane < cnt && b != bf) {
                wacc[l] = __fadd_rn(wacc[l], cs);
                if (DENS || DW) waccw[l] = __fadd_rn(waccw[l], cw);
            }
            __syncwarp(); // the entries, buffers and sums are free again
            qhead = (qhead + cnt) & QM;
            qsize -= cnt;
            nfront -= cnt;
            if (nfront <= 0) { // the front direction is done: the rest are the other buffer's
                bfront ^= 1;
                nfront = qsize;
            }
        };

        for (int c0 = 0; c0 < n; c0 += kBpChunk) {
            const int cn = min(kBpChunk, n - c0);
            group_sync(grp + 1);
            if (cn == kBpChunk) {
                // a whole chunk: all of a thread's loads in flight before its stores
                constexpr int KA = kBpChunk * 9 / kCThreads;
                float a[KA];
#pragma unroll
                for (int u = 0; u < KA; u++) a[u] = __ldg(axes + (size_t)c0 * 9 + tid + u * kCThreads);
#pragma unroll
                for (int u = 0; u < KA; u++) sax[tid + u * kCThreads] = a[u];
            } else {
                for (int t = tid; t < cn * 9; t += kCThreads) sax[t] = __ldg(axes + (size_t)c0 * 9 + t);
            }
            group_sync(grp + 1);
            // cull: thread tid takes directions tid + p * kCThreads; the kept
            // ones are listed in direction order (pass by pass, warp by warp)
            constexpr int kPasses = kBpChunk / kCThreads;
            unsigned ballots[kPasses];
            bool keeps[kPasses];
            int orthos[kPasses];
#pragma unroll
            for (int pss = 0; pss < kPasses; pss++) {
                const int d = tid + pss * kCThreads;
                bool keep = false;
                int ortho = 0;
                if (d < cn) {
                    const float *ax = sax + d * 9;
                    const float zx = ax[6], zy = ax[7], zz = ax[8];
                    const float dd = bcx * zx + bcy * zy + bcz * zz;
                    const float ext = 0.5f * ((kCBX - 1) * fabsf(zx) + (kCBY - 1) * fabsf(zy) + (kCBZ - 1) * fabsf(zz));
                    keep = fabsf(dd) <= slab + ext;
                    // the fast window needs orthonormal axes (they bound |Q - v|);
                    // NaN or infinite entries fail these tests
                    const float xx = ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2];
                    const float yy = ax[3] * ax[3] + ax[4] * ax[4] + ax[5] * ax[5];
                    const float zz2 = zx * zx + zy * zy + zz * zz;
                    const float xy = ax[0] * ax[3] + ax[1] * ax[4] + ax[2] * ax[5];
                    const float xz = ax[0] * zx + ax[1] * zy + ax[2] * zz;
                    const float yz = ax[3] * zx + ax[4] * zy + ax[5] * zz;
                    ortho = (fabsf(xx - 1.0f) <= 1e-3f && fabsf(yy - 1.0f) <= 1e-3f && fabsf(zz2 - 1.0f) <= 1e-3f &&
                             fabsf(xy) <= 1e-3f && fabsf(xz) <= 1e-3f && fabsf(yz) <= 1e-3f) ? kBpChunk : 0;
                }
                keeps[pss] = keep;
                orthos[pss] = ortho;
                ballots[pss] = __ballot_sync(0xffffffffu, keep);
                if (lane == 0) swarp[pss * (kCThreads / 32) + warp] = __popc(ballots[pss]);
            }
            group_sync(grp + 1);
            {
                int off = 0;
#pragma unroll
                for (int pss = 0; pss < kPasses; pss++) {
                    int o = off;
                    for (int w = 0; w < warp; w++) o += swarp[pss * (kCThreads / 32) + w];
                    if (keeps[pss])
                        slist[o + __popc(ballots[pss] & lt_mask)] = (typename Mem::LEnt)((tid + pss * kCThreads) | orthos[pss]);
                    for (int w = 0; w < kCThreads / 32; w++) off += swarp[pss * (kCThreads / 32) + w];
                }
                if (tid == kCThreads - 1) sm.scount = off;
            }
            group_sync(grp + 1);
            const int count = sm.scount;

            for (int q = 0; q < count; q++) {
                const int e = slist[q];
                const int al = e & (kBpChunk - 1);
                const float *ax = sax + al * 9;
                const float nz0 = ax[6], nz1 = ax[7], nz2 = ax[8];
                // Adjoint, orthonormal axes: a pixel weighs non-zero only if its
                // sample point f lies in the voxel's cube |f - v| < 2 (each axis),
                // which the plane reaches only if |f_k| < 2 |nz|_1: a slab
                // thinner than 2 sqrt(3) for most directions.
                const float slabD = ADJ && (e & kBpChunk)
                                        ? fminf(slab, 2.0f * (fabsf(nz0) + fabsf(nz1) + fabsf(nz2)) + kCullEps)
                                        : slab;
                {   // the warp's 8x4xBD block against the slab (uniform)
                    const float d = wcx * nz0 + wcy * nz1 + wcz * nz2;
                    const float ext = 0.5f * (7.0f * fabsf(nz0) + 3.0f * fabsf(nz1) + (float)(BD - 1) * fabsf(nz2));
                    if (fabsf(d) > slab + ext) continue;
                }
                // the reference's per-voxel slab test (gpuBackProject.cu:64-66), or
                // the adjoint's reach
                unsigned actm = 0;
                int total = 0;
#pragma unroll
                for (int s = 0; s < BD; s++) {
                    const float az = (float)(bz + s) - volCenter;
                    const float fk = voxel_proj(ax0, ay0, az, nz0, nz1, nz2);
                    const bool act = ((inmask >> s) & 1u) && (ADJ ? fabsf(fk) < slabD : fabsf(fk) <= kerHW);
                    actm |= (act ? 1u : 0u) << s;
                    total += __popc(__ballot_sync(0xffffffffu, act));
                }
                if (total == 0) continue;
                int b = 0;
                if (NB > 1) {
                    b = nbuf;
                    nbuf ^= 1;
                    // buffer b's earlier voxels (all at the front of the queue) run first
                    while (qsize > 0 && (LEAN ? bfront : (int)(wq[qhead & QM] >> 8)) == b) run_round(min(qsize, 32));
                }
                float *const wfoot = wfoot0 + b * (FH * FS);
                float *const wfoot2 = wfoot20 + (DW ? b * (FH * FS) : 0);
                const float nx0 = ax[0], nx1 = ax[1], nx2 = ax[2];
                const float ny0 = ax[3], ny1 = ax[4], ny2 = ax[5];
                const TI *img_ptr = img + (size_t)(c0 + al) * MM;
                const float *img2_ptr = DW ? img2 + (size_t)(c0 + al) * MM : nullptr;
                // this warp's footprint (uniform across the warp)
                int fi0 = 0, fj0 = 0, fh = 0;
                bool foot = false;
                if (e & kBpChunk) {
                    const float ic = wcx * nx0 + wcy * nx1 + wcz * nx2 + (float)imgCenter;
                    const float jc = wcx * ny0 + wcy * ny1 + wcz * ny2 + (float)imgCenter;
                    const float hz = 0.5f * (float)(BD - 1);
                    const float hi = 3.5f * fabsf(nx0) + 1.5f * fabsf(nx1) + hz * fabsf(nx2);
                    const float hj = 3.5f * fabsf(ny0) + 1.5f * fabsf(ny1) + hz * fabsf(ny2);
                    fi0 = (int)floorf(ic - hi - 0.6f) - HALF;
                    fj0 = (int)floorf(jc - hj - 0.6f) - HALF;
                    const int fw = (int)floorf(ic + hi + 0.6f) + HALF - fi0 + 1;
                    fh = (int)floorf(jc + hj + 0.6f) + HALF - fj0 + 1;
                    foot = fw <= FW && fh <= FH && fh >= W && (!ADJ || zeroEdges);
                    if (foot && !ADJ && !ONES && vecImg) {
                        // vector loads of aligned pixel quads (rows start at
                        // multiples of 4 elements: 4 divides M, the image stacks
                        // are aligned), the linear-index rule still applied
                        // pixel by pixel
                        constexpr int NQ = FW / 4 + 1; // quads per footprint row
                        const int base = fi0 & ~3, sh = fi0 & 3;
                        if constexpr (DW) {
                            // two image stacks: one quad at a time (both stacks'
                            // quads held at once would spill)
                            for (int t = lane; t < fh * NQ; t += 32) {
                                const int r = t / NQ, qq = t - r * NQ;
                                const int c0 = 4 * qq - sh; // footprint column of the quad's first pixel
                                const int lin0 = (fj0 + r) * M + base + 4 * qq;
                                float v[4] = {0.0f, 0.0f, 0.0f, 0.0f}, v2[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                                if (lin0 >= 0 && lin0 + 3 < MM) {
                                    ld_quad(img_ptr + lin0, v);
                                    ld_quad(img2_ptr + lin0, v2);
                                } else {
#pragma unroll
                                    for (int e = 0; e < 4; e++)
                                        if (lin0 + e >= 0 && lin0 + e < MM) {
                                            v[e] = ld_f32(img_ptr + lin0 + e);
                                            v2[e] = __ldg(img2_ptr + lin0 + e);
                                        }
                                }
                                if (QALIGN) {
                                    *reinterpret_cast<float4 *>(wfoot + r * FS + 4 * qq) = make_float4(v[0], v[1], v[2], v[3]);
                                    *reinterpret_cast<float4 *>(wfoot2 + r * FS + 4 * qq) =
                                        make_float4(v2[0], v2[1], v2[2], v2[3]);
                                } else {
#pragma unroll
                                    for (int e = 0; e < 4; e++)
                                        if (c0 + e >= 0 && c0 + e < FW) {
                                            wfoot[r * FS + c0 + e] = v[e];
                                            wfoot2[r * FS + c0 + e] = v2[e];
                                        }
                                }
                            }
                        } else {
                            // a lane's quads (at most KQ) are all loaded before any is
                            // stored, so their L2 latencies overlap
                            constexpr int KQ = (FH * NQ + 31) / 32;
                            const int nq = fh * NQ;
                            float v[KQ][4];
#pragma unroll
                            for (int u = 0; u < KQ; u++) {
                                const int t = lane + 32 * u;
#pragma unroll
                                for (int e = 0; e < 4; e++) v[u][e] = 0.0f;
                                if (t < nq) {
                                    const int r = t / NQ, qq = t - r * NQ;
                                    const int lin0 = (fj0 + r) * M + base + 4 * qq;
                                    if (lin0 >= 0 && lin0 + 3 < MM) {
                                        ld_quad(img_ptr + lin0, v[u]);
                                    } else {
#pragma unroll
                                        for (int e = 0; e < 4; e++)
                                            if (lin0 + e >= 0 && lin0 + e < MM) v[u][e] = ld_f32(img_ptr + lin0 + e);
                                    }
                                }
                            }
#pragma unroll
                            for (int u = 0; u < KQ; u++) {
                                const int t = lane + 32 * u;
                                if (t < nq) {
                                    const int r = t / NQ, qq = t - r * NQ;
                                    const int c0 = 4 * qq - sh; // footprint column of the quad's first pixel
                                    if (QALIGN) {
                                        *reinterpret_cast<float4 *>(wfoot + r * FS + 4 * qq) =
                                            make_float4(v[u][0], v[u][1], v[u][2], v[u][3]);
                                    } else {
#pragma unroll
                                        for (int e = 0; e < 4; e++)
                                            if (c0 + e >= 0 && c0 + e < FW) wfoot[r * FS + c0 + e] = v[u][e];
                                    }
                                }
                            }
                        }
                    } else if (foot && !ADJ && sizeof(TI) == 2 && !ONES && !(M & 1)) {
                        // the same with 4-byte pixel pairs when only 2 divides M
                        constexpr int NPR = FW / 2 + 1; // pairs per footprint row
                        const int base = fi0 & ~1, odd = fi0 & 1;
                        for (int t = lane; t < fh * NPR; t += 32) {
                            const int r = t / NPR, pp = t - r * NPR;
                            const int c0 = 2 * pp - odd; // footprint column of the pair's first pixel
                            const int lin0 = (fj0 + r) * M + base + 2 * pp;
                            float v0 = 0.0f, v1 = 0.0f;
                            if (lin0 >= 0 && lin0 + 1 < MM) {
                                const unsigned w = __ldg(reinterpret_cast<const unsigned *>(img_ptr + lin0));
                                v0 = widen16<TI>(w & 0xffffu);
                                v1 = widen16<TI>(w >> 16);
                            } else {
                                if (lin0 >= 0 && lin0 < MM) v0 = ld_f32(img_ptr + lin0);
                                if (lin0 + 1 >= 0 && lin0 + 1 < MM) v1 = ld_f32(img_ptr + lin0 + 1);
                            }
                            const int ash = QALIGN ? (fi0 & 3) : 0;
                            if (c0 >= 0 && c0 < FW) wfoot[r * FS + c0 + ash] = v0;
                            if (c0 + 1 < FW) wfoot[r * FS + c0 + 1 + ash] = v1; // c0 + 1 >= 0
                        }
                    } else if (foot && !ADJ) {
                        // the reference's linear-index rule (gpuBackProject.cu:99)
                        for (int t = lane; t < fh * FW; t += 32) {
                            const int r = t / FW, c = t - r * FW;
                            const int lin = (fj0 + r) * M + (fi0 + c);
                            float v = 0.0f, v2 = 0.0f;
                            if (lin >= 0 && lin < MM) {
                                v = ONES ? 1.0f : ld_f32(img_ptr + lin);
                                if (DW) v2 = __ldg(img2_ptr + lin);
                            }
                            wfoot[r * FS + c + (QALIGN ? (fi0 & 3) : 0)] = v;
                            if (DW) wfoot2[r * FS + c + (QALIGN ? (fi0 & 3) : 0)] = v2;
                        }
                    } else if (foot) {
                        // the forward projection's pixels: inside the image and the mask
                        if (vecImg && !ONES) {
                            // aligned pixel quads (4 divides M: a quad lies wholly inside or
                            // outside the image rows), three in flight per lane at a time;
                            // the mask is applied pixel by pixel
                            constexpr int NQ = FW / 4 + 1; // quads per footprint row
                            const int base = fi0 & ~3, sh = fi0 & 3, nq = fh * NQ;
                            for (int t0 = lane; t0 < nq; t0 += 96) {
                                float v[3][4];
#pragma unroll
                                for (int u = 0; u < 3; u++) {
                                    const int t = t0 + 32 * u;
#pragma unroll
                                    for (int e = 0; e < 4; e++) v[u][e] = 0.0f;
                                    const int r = t / NQ, qq = t - r * NQ;
                                    const int pj = fj0 + r, pi = base + 4 * qq;
                                    if (t < nq && pj >= 0 && pj < M && pi >= 0 && pi < M) {
                                        ld_quad(img_ptr + (size_t)pj * M + pi, v[u]);
                                        const long long dj = pj - imgCenter;
#pragma unroll
                                        for (int e = 0; e < 4; e++) {
                                            const long long di = pi + e - imgCenter;
                                            if (di * di + dj * dj > R2) v[u][e] = 0.0f;
                                        }
                                    }
                                }
#pragma unroll
                                for (int u = 0; u < 3; u++) {
                                    const int t = t0 + 32 * u;
                                    if (t < nq) {
                                        const int r = t / NQ, qq = t - r * NQ;
                                        const int c0 = 4 * qq - sh; // footprint column of the quad's first pixel
                                        if (QALIGN) {
                                            *reinterpret_cast<float4 *>(wfoot + r * FS + 4 * qq) =
                                                make_float4(v[u][0], v[u][1], v[u][2], v[u][3]);
                                        } else {
#pragma unroll
                                            for (int e = 0; e < 4; e++)
                                                if (c0 + e >= 0 && c0 + e < FW) wfoot[r * FS + c0 + e] = v[u][e];
                                        }
                                    }
                                }
                            }
                        } else {
                            for (int t = lane; t < fh * FW; t += 32) {
                                const int r = t / FW, c = t - r * FW;
                                const int pi = fi0 + c, pj = fj0 + r, di = pi - imgCenter, dj = pj - imgCenter;
                                float v = 0.0f;
                                if (pi >= 0 && pi < M && pj >= 0 && pj < M && (long long)di * di + (long long)dj * dj <= R2)
                                    v = ld_f32(img_ptr + (size_t)pj * M + pi);
                                wfoot[r * FS + c + (QALIGN ? (fi0 & 3) : 0)] = v;
                            }
                        }
                    }
                }
                if (NB > 1) {
                    if (lane == 0)
                        wmeta[b] = BpDirMeta{nx0, nx1, nx2, ny0, ny1, ny2, fi0, fj0, fh, foot ? 1 : 0, c0 + al, 0};
                    // the active voxels join the queue slot by slot, in lane order
                    int pos = qhead + qsize;
#pragma unroll
                    for (int s = 0; s < BD; s++) {
                        const bool act = (actm >> s) & 1u;
                        const unsigned bal = __ballot_sync(0xffffffffu, act);
                        if (act) wq[(pos + __popc(bal & lt_mask)) & QM] = (QEnt)((lane + 32 * s) | (LEAN ? 0 : b << 8));
                        pos += __popc(bal);
                    }
                    if (qsize == 0) {
                        bfront = b;
                        nfront = total;
                    }
                    qsize += total;
                    __syncwarp(); // the queue entries, the footprint and its record are complete
                    while (qsize >= 32) run_round(32);
                } else {
                    // the active voxels, slot by slot in lane order, run at once
                    int pos = 0;
#pragma unroll
                    for (int s = 0; s < BD; s++) {
                        const bool act = (actm >> s) & 1u;
                        const unsigned bal = __ballot_sync(0xffffffffu, act);
                        if (act) wq[pos + __popc(bal & lt_mask)] = (QEnt)(lane + 32 * s);
                        pos += __popc(bal);
                    }
                    __syncwarp(); // the voxel list and the footprint are complete
                    for (int base = 0; base < total; base += 32) {
                        const int t = base + lane;
                        if (t < total) {
                            float cs = 0.0f, cw = 0.0f;
                            const int l = wq[t];
                            voxel_window(l, nx0, nx1, nx2, ny0, ny1, ny2, fi0, fj0, fh, foot, img_ptr, img2_ptr, wfoot,
                                         wfoot2, cs, cw);
                            // cumSumAllAxes += cumSum (gpuBackProject.cu:106), in direction order
                            wacc[l] = __fadd_rn(wacc[l], cs);
                            if (DENS || DW) waccw[l] = __fadd_rn(waccw[l], cw);
                        }
                    }
                    __syncwarp(); // the next direction rewrites the list, the footprint and these sums
                }
            }
        }
        if (NB > 1)
            while (qsize > 0) run_round(min(qsize, 32));
        __syncwarp();
        const float sc = d_scale ? *d_scale : 1.0f;
#pragma unroll
        for (int s = 0; s < BD; s++) {
            if (!((inmask >> s) & 1u)) continue;
            const size_t o = (size_t)(bz + s) * V * V + (size_t)ly * V + lx;
            vol[o] = vol[o] + wacc[lane + 32 * s] * sc;
            if (DENS || DW) pd[o] = pd[o] + waccw[lane + 32 * s];
        }
    }
}

template <typename TI, bool ONES, bool DENS, bool ADJ, bool DW, bool DEEP, int G>
static cudaError_t launch_bp_compact_g(float *vol, const TI *img, const float *ker, const float *axes, int n,
                                       const Geom &g, const float *scale, cudaStream_t s, float *pd, bool zero_edges,
                                       const float *img2, int max_copies)
{
    constexpr int kCBZ = BpShape<ADJ, DW, DEEP>::BZ;
    const int bx = (g.V + kCBX - 1) / kCBX, by = (g.V + kCBY - 1) / kCBY, bz = (g.V + kCBZ - 1) / kCBZ;
    // one group per CTA (the serving lanes): the non-LEAN layout
    constexpr bool LEAN = G > 1;
    using Mem = BpGroupMem<DENS, ADJ, DW, DEEP, LEAN>;
    const size_t other = G * sizeof(Mem) + (2 * (size_t)by + 1) * sizeof(int);
    // one group per CTA: three CTAs an SM (228 KB, 1 KB reserved per CTA)
    const size_t limit = G == 1 ? (size_t)(228 * 1024 / 3 - 1024) : 0;
    const BpTable tb = bp_table(g.ker_size, other, max_copies, limit);
    if (tb.copies == 0) return cudaErrorInvalidValue; // a KB table too long for shared memory
    const size_t dyn = (((size_t)tb.entries * tb.copies + 3) & ~(size_t)3) * sizeof(float) + other;
    // quad loads of image rows: 4 | M and the stacks aligned to 4 elements
    const size_t qa = 4 * sizeof(TI);
    const int vec = (g.M % 4 == 0) && ((size_t)img % qa == 0) && (!img2 || (size_t)img2 % 16 == 0) ? 1 : 0;
    // CTA (x, z): bricks run x .. of z-layer z that meet the sphere
    const int run = ((DEEP && G > 1) ? 2 : 1) * G;
    const dim3 grid((unsigned)((bx * by + run - 1) / run), (unsigned)bz);
    // the table stride as a compile-time constant where the copy count gives one
    auto go = [&](auto kern) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
        if (e != cudaSuccess) return e;
        kern<<<grid, kCThreads * G, dyn, s>>>(vol, pd, g.V, img, g.M, axes, n, g.mask_radius, ker, g.ker_size,
                                              g.ker_hw, bx, by, tb, zero_edges ? 1 : 0, scale, img2, vec);
        count_launches(1);
        return cudaGetLastError();
    };
    if constexpr (LEAN) {
        if (tb.copies == 32) return go(bp_ref_compact_kernel<TI, ONES, DENS, ADJ, DW, DEEP, G, 128, true>);
    }
    return go(bp_ref_compact_kernel<TI, ONES, DENS, ADJ, DW, DEEP, G, 0, LEAN>);
}

template <typename TI, bool ONES, bool DENS = false, bool ADJ = false, bool DW = false, bool DEEP = false>
static cudaError_t launch_bp_compact_t(float *vol, const TI *img, const float *ker, const float *axes, int n,
                                       const Geom &g, const float *scale, cudaStream_t s, float *pd = nullptr,
                                       bool zero_edges = true, const float *img2 = nullptr, bool shared = false)
{
    if (n <= 0) return cudaSuccess;
    // A GPU shared with concurrent launches (the serving lanes): one group
    // and one table copy per CTA, three CTAs an SM, which the launches of
    // other lanes can fill as they free (serving capacity 172 -> 195 req/s);
    // alone, three groups sharing 32 table copies (batched back projection
    // 78.5 -> 71.7 ms per 10k images).
    if constexpr (std::is_same<TI, float>::value && !ONES && !DENS && !ADJ && !DW) {
        if (shared)
            return launch_bp_compact_g<TI, ONES, DENS, ADJ, DW, DEEP, 1>(vol, img, ker, axes, n, g, scale, s, pd,
                                                                         zero_edges, img2, 1);
    }
    return launch_bp_compact_g<TI, ONES, DENS, ADJ, DW, DEEP, kGroupsOf<ADJ, DW, DEEP>>(vol, img, ker, axes, n, g, scale, s, pd,
                                                                         zero_edges, img2, 32);
}

// Reference-rule launch with the block depth chosen by the image size.
template <typename TI, bool ONES, bool DENS>
static cudaError_t launch_bp_ref_sized(float *vol, const TI *img, const float *ker, const float *axes, int n,
                                       const Geom &g, const float *scale, cudaStream_t s, float *pd = nullptr,
                                       bool shared = false)
{
    if (g.M >= 512)
        return launch_bp_compact_t<TI, ONES, DENS, false, false, true>(vol, img, ker, axes, n, g, scale, s, pd, true,
                                                                        nullptr, shared);
    return launch_bp_compact_t<TI, ONES, DENS>(vol, img, ker, axes, n, g, scale, s, pd, true, nullptr, shared);
}

cudaError_t launch_back_project_ref(float *d_vol, const void *d_img, int iprec, bool ones, const float *d_ker,
                                    const float *d_axes, int n, const Geom &g, const float *scale, cudaStream_t s,
                                    bool shared)
{
    if (ones) return launch_bp_ref_sized<float, true, false>(d_vol, nullptr, d_ker, d_axes, n, g, scale, s);
    if (iprec == kF32)
        return launch_bp_ref_sized<float, false, false>(d_vol, (const float *)d_img, d_ker, d_axes, n, g, scale, s,
                                                        nullptr, shared);
    if (iprec == kF16)
        return launch_bp_ref_sized<__half, false, false>(d_vol, (const __half *)d_img, d_ker, d_axes, n, g, scale, s);
    return launch_bp_ref_sized<__nv_bfloat16, false, false>(d_vol, (const __nv_bfloat16 *)d_img, d_ker, d_axes, n, g,
                                                            scale, s);
}

cudaError_t launch_back_project_ref_density(float *d_vol, float *d_pd, const void *d_img, int iprec, const float *d_ker,
                                            const float *d_axes, int n, const Geom &g, const float *scale, cudaStream_t s)
{
    if (iprec == kF32)
        return launch_bp_ref_sized<float, false, true>(d_vol, (const float *)d_img, d_ker, d_axes, n, g, scale, s, d_pd);
    if (iprec == kF16)
        return launch_bp_ref_sized<__half, false, true>(d_vol, (const __half *)d_img, d_ker, d_axes, n, g, scale, s,
                                                        d_pd);
    return launch_bp_ref_sized<__nv_bfloat16, false, true>(d_vol, (const __nv_bfloat16 *)d_img, d_ker, d_axes, n, g,
                                                           scale, s, d_pd);
}

cudaError_t launch_back_project_ref_pair(float *d_vol, float *d_pd, const float *d_img, const float *d_img2,
                                         const float *d_ker, const float *d_axes, int n, const Geom &g, cudaStream_t s)
{
    return launch_bp_compact_t<float, false, false, false, true>(d_vol, d_img, d_ker, d_axes, n, g, nullptr, s, d_pd,
                                                                  true, d_img2);
}

cudaError_t launch_back_project_adjoint(float *d_vol, const void *d_img, int iprec, const float *d_ker,
                                        const float *d_axes, int n, const Geom &g, const float *scale, bool zero_edges,
                                        cudaStream_t s)
{
    if (iprec == kF32)
        return launch_bp_compact_t<float, false, false, true>(d_vol, (const float *)d_img, d_ker, d_axes, n, g, scale, s,
                                                               nullptr, zero_edges);
    if (iprec == kF16)
        return launch_bp_compact_t<__half, false, false, true>(d_vol, (const __half *)d_img, d_ker, d_axes, n, g, scale,
                                                                s, nullptr, zero_edges);
    return launch_bp_compact_t<__nv_bfloat16, false, false, true>(d_vol, (const __nv_bfloat16 *)d_img, d_ker, d_axes, n,
                                                                   g, scale, s, nullptr, zero_edges);
}

} // namespace gg
