/*
 * CPU oracle for the Kaiser-Bessel Fourier-slice projection path.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, the smoke check in __graft_entry__.py
 * and the CPU-baseline / reference arm of bench.py load it. The product
 * (libgg_gridder.so) never links or calls it.
 *
 * It restates, loop for loop, the two projection kernels of
 * tagarelab/MultiGPUGridder:
 *   - gpuForwardProjectKernel   src/Projection/gpuForwardProject.cu:4-101
 *   - gpuBackProjectKernel      src/Projection/gpuBackProject.cu:4-113
 * in three forms:
 *   *_ref_f32   single precision, same operation order, roundf() index
 *               rounding, int mask radius, linear-index bounds checks, and
 *               the fused multiply-adds the reference's nvcc build forms:
 *               table index roundf(fma(r, kerScale, kerCenter)), sums
 *               acc = fma(x, w, acc), sample coordinates fma(a, x, b*y) + c.
 *               (Identified by replaying the reference kernels' own outputs,
 *               tests/golden/reference_kernels.npz, bit for bit.)  Compiled
 *               with -ffp-contract=off and explicit fmaf(), so it gives the
 *               same bits on x86-64 and aarch64.
 *   *_f64       the same discrete operator evaluated in double precision
 *               (same float KB table, same nearest-index rule), the
 *               "FP64 oracle" the reduced-precision forms are measured against.
 *   bp_adjoint  the exact adjoint of the forward projector (scatter of each
 *               pixel over the 5x5x5 window the forward gather reads), which
 *               the reference does not have; it defines the gradient.
 *
 * Layouts follow the reference (MATLAB column-major): x fastest,
 * vol[k*V*V + j*V + i], img[a*M*M + j*M + i], axes 9 floats per direction
 * (columns x, y, z of the rotation; get_axes_from_n_rot.m:36-37).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>

#ifdef _OPENMP
#include <omp.h>
#endif

static inline int imin(int a, int b) { return a < b ? a : b; }
static inline int imax(int a, int b) { return a > b ? a : b; }
static inline float fclampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

int gg_oracle_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void gg_oracle_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* Forward projection, reference rule, FP32 (gpuForwardProject.cu:4-101).   */
/* img must hold n*M*M floats; pixels outside the mask are left untouched    */
/* (the reference memsets the CAS images to zero first,                      */
/* gpuGridder.cpp:232-236, so callers pass a zeroed buffer).                 */
/* ------------------------------------------------------------------------ */
void gg_oracle_fp_ref_f32(const float *vol, int V, float *img, int M,
                          const float *axes, int n, int mask_radius,
                          const float *ker, int ker_size, float ker_hw)
{
    const int volCenter = V / 2;
    const int imgCenter = M / 2;
    const int convW = (int)roundf(ker_hw);
    const float kerCenter = ((float)ker_size - 1) / 2;
    const float kerScale = kerCenter / ker_hw;
    const float maskR = (float)mask_radius;
    const long long V3 = (long long)V * V * V;

#pragma omp parallel for schedule(dynamic, 1)
    for (int a = 0; a < n; a++) {
        const float *nx = axes + 9 * (size_t)a;
        const float *ny = nx + 3;
        float *img_ptr = img + (size_t)a * M * M;
        for (int j = 0; j < M; j++) {
            for (int i = 0; i < M; i++) {
                float r = sqrtf((float)(i - imgCenter) * (i - imgCenter) +
                                (float)((j - imgCenter) * (j - imgCenter)));
                if (!(r <= maskR)) continue;
                const float x = (float)(i - imgCenter), y = (float)(j - imgCenter);
                float fi = fmaf(nx[0], x, ny[0] * y) + (float)volCenter;
                float fj = fmaf(nx[1], x, ny[1] * y) + (float)volCenter;
                float fk = fmaf(nx[2], x, ny[2] * y) + (float)volCenter;
                int ii = (int)roundf(fi), jj = (int)roundf(fj), kk = (int)roundf(fk);
                float acc = 0.0f;
                for (int i1 = ii - convW; i1 <= ii + convW; i1++) {
                    float ri = fclampf((float)i1 - fi, (float)-convW, (float)convW);
                    int ki = imin(imax((int)roundf(fmaf(ri, kerScale, kerCenter)), 0), ker_size - 1);
                    float wi = ker[ki];
                    for (int j1 = jj - convW; j1 <= jj + convW; j1++) {
                        float rj = fclampf((float)j1 - fj, (float)-convW, (float)convW);
                        int kj = imin(imax((int)roundf(fmaf(rj, kerScale, kerCenter)), 0), ker_size - 1);
                        float wj = ker[kj];
                        for (int k1 = kk - convW; k1 <= kk + convW; k1++) {
                            float rk = fclampf((float)k1 - fk, (float)-convW, (float)convW);
                            int kx = imin(imax((int)roundf(fmaf(rk, kerScale, kerCenter)), 0), ker_size - 1);
                            float wk = ker[kx];
                            float w = wi * wj * wk;
                            long long lin = (long long)k1 * V * V + (long long)j1 * V + i1;
                            /* the reference checks only the upper bound; a
                               lower-bound check is added so a bad input cannot
                               read outside the buffer here */
                            if (lin < V3 && lin >= 0)
                                acc = fmaf(w, vol[lin], acc);
                        }
                    }
                }
                img_ptr[(size_t)j * M + i] = acc;
            }
        }
    }
}

/* Round half away from zero in double, the MATLAB/C round() rule. */
static inline double dround(double x) { return round(x); }

/* Forward projection, same discrete operator in FP64. */
void gg_oracle_fp_f64(const double *vol, int V, double *img, int M,
                      const double *axes, int n, int mask_radius,
                      const float *ker, int ker_size, double ker_hw)
{
    const int volCenter = V / 2;
    const int imgCenter = M / 2;
    const int convW = (int)dround(ker_hw);
    const double kerCenter = ((double)ker_size - 1) / 2;
    const double kerScale = kerCenter / ker_hw;
    const long long V3 = (long long)V * V * V;
    const long long R2 = (long long)mask_radius * mask_radius;

#pragma omp parallel for schedule(dynamic, 1)
    for (int a = 0; a < n; a++) {
        const double *nx = axes + 9 * (size_t)a;
        const double *ny = nx + 3;
        double *img_ptr = img + (size_t)a * M * M;
        for (int j = 0; j < M; j++) {
            for (int i = 0; i < M; i++) {
                long long d2 = (long long)(i - imgCenter) * (i - imgCenter) + (long long)(j - imgCenter) * (j - imgCenter);
                if (d2 > R2) continue;
                double x = i - imgCenter, y = j - imgCenter;
                double fi = nx[0] * x + ny[0] * y + volCenter;
                double fj = nx[1] * x + ny[1] * y + volCenter;
                double fk = nx[2] * x + ny[2] * y + volCenter;
                int ii = (int)dround(fi), jj = (int)dround(fj), kk = (int)dround(fk);
                double acc = 0.0;
                for (int i1 = ii - convW; i1 <= ii + convW; i1++) {
                    double ri = fmin(fmax((double)i1 - fi, -convW), convW);
                    int ki = imin(imax((int)dround(ri * kerScale + kerCenter), 0), ker_size - 1);
                    double wi = ker[ki];
                    for (int j1 = jj - convW; j1 <= jj + convW; j1++) {
                        double rj = fmin(fmax((double)j1 - fj, -convW), convW);
                        int kj = imin(imax((int)dround(rj * kerScale + kerCenter), 0), ker_size - 1);
                        double wj = ker[kj];
                        for (int k1 = kk - convW; k1 <= kk + convW; k1++) {
                            double rk = fmin(fmax((double)k1 - fk, -convW), convW);
                            int kx = imin(imax((int)dround(rk * kerScale + kerCenter), 0), ker_size - 1);
                            double w = wi * wj * (double)ker[kx];
                            long long lin = (long long)k1 * V * V + (long long)j1 * V + i1;
                            if (lin < V3 && lin >= 0) acc += w * vol[lin];
                        }
                    }
                }
                img_ptr[(size_t)j * M + i] = acc;
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Back projection, reference window rule, FP32 (gpuBackProject.cu:4-113).  */
/* vol (V^3) is ACCUMULATED into: the reference adds one per-voxel sum with  */
/* atomicAdd (gpuBackProject.cu:111) onto a volume zeroed at BP start        */
/* (gpuGridder.cpp:332).                                                     */
/* ------------------------------------------------------------------------ */
void gg_oracle_bp_ref_f32(float *vol, int V, const float *img, int M,
                          const float *axes, int n, int mask_radius,
                          const float *ker, int ker_size, float ker_hw)
{
    const int convW = (int)roundf(ker_hw);
    const float kerCenter = ((float)ker_size - 1) / 2;
    const float kerScale = kerCenter / ker_hw;
    const int volCenter = (int)((float)V) / 2;
    const int imgCenter = (int)((float)M) / 2;
    const float maskR = (float)mask_radius;

#pragma omp parallel for collapse(2) schedule(dynamic, 4)
    for (int vk = 0; vk < V; vk++) {
        for (int vj = 0; vj < V; vj++) {
            for (int vi = 0; vi < V; vi++) {
                float r = sqrtf((float)(vi - volCenter) * (vi - volCenter) +
                                (float)((vj - volCenter) * (vj - volCenter)) +
                                (float)((vk - volCenter) * (vk - volCenter)));
                if (!(r <= maskR)) continue;
                float cumSumAllAxes = 0;
                for (int a = 0; a < n; a++) {
                    const float *nx = axes + 9 * (size_t)a;
                    const float *ny = nx + 3;
                    const float *nz = ny + 3;
                    const float a0 = (float)vi - volCenter, a1 = (float)vj - volCenter, a2 = (float)vk - volCenter;
                    float f_imgi = fmaf(a2, nx[2], fmaf(a0, nx[0], a1 * nx[1])) + imgCenter;
                    float f_imgj = fmaf(a2, ny[2], fmaf(a0, ny[0], a1 * ny[1])) + imgCenter;
                    float f_imgk = fmaf(a2, nz[2], fmaf(a0, nz[0], a1 * nz[1]));
                    if (!(fabsf(f_imgk) <= ker_hw)) continue;
                    int imgi = (int)roundf(f_imgi);
                    int imgj = (int)roundf(f_imgj);
                    const float *img_ptr = img + (size_t)a * M * M;
                    float cumSum = 0;
                    for (int j1 = imgj - convW; j1 <= imgj + convW; j1++) {
                        for (int i1 = imgi - convW; i1 <= imgi + convW; i1++) {
                            const float pi = (float)(i1 - imgCenter), pj = (float)(j1 - imgCenter);
                            float p = fmaf(pi, nx[0], pj * ny[0]) + volCenter;
                            float rr = fclampf(p - vi, (float)-convW, (float)convW);
                            int kidx = imin(imax((int)roundf(fmaf(rr, kerScale, kerCenter)), 0), ker_size - 1);
                            float w = ker[kidx];
                            p = fmaf(pi, nx[1], pj * ny[1]) + volCenter;
                            rr = fclampf(p - vj, (float)-convW, (float)convW);
                            kidx = imin(imax((int)roundf(fmaf(rr, kerScale, kerCenter)), 0), ker_size - 1);
                            w = w * ker[kidx];
                            p = fmaf(pi, nx[2], pj * ny[2]) + volCenter;
                            rr = fclampf(p - vk, (float)-convW, (float)convW);
                            kidx = imin(imax((int)roundf(fmaf(rr, kerScale, kerCenter)), 0), ker_size - 1);
                            w = w * ker[kidx];
                            long long lin = (long long)j1 * M + i1;
                            /* linear-index check only: windows that cross a
                               row edge wrap into the neighbouring row, as in
                               gpuBackProject.cu:99 */
                            if (lin < (long long)M * M && lin >= 0)
                                cumSum = fmaf(img_ptr[lin], w, cumSum);
                        }
                    }
                    cumSumAllAxes += cumSum;
                }
                vol[(size_t)vk * V * V + (size_t)vj * V + vi] += cumSumAllAxes;
            }
        }
    }
}

/* Back projection, reference window rule, FP64. */
void gg_oracle_bp_ref_f64(double *vol, int V, const double *img, int M,
                          const double *axes, int n, int mask_radius,
                          const float *ker, int ker_size, double ker_hw)
{
    const int convW = (int)dround(ker_hw);
    const double kerCenter = ((double)ker_size - 1) / 2;
    const double kerScale = kerCenter / ker_hw;
    const int volCenter = V / 2;
    const int imgCenter = M / 2;
    const long long R2 = (long long)mask_radius * mask_radius;

#pragma omp parallel for collapse(2) schedule(dynamic, 4)
    for (int vk = 0; vk < V; vk++) {
        for (int vj = 0; vj < V; vj++) {
            for (int vi = 0; vi < V; vi++) {
                long long d2 = (long long)(vi - volCenter) * (vi - volCenter) + (long long)(vj - volCenter) * (vj - volCenter) +
                               (long long)(vk - volCenter) * (vk - volCenter);
                if (d2 > R2) continue;
                double x = vi - volCenter, y = vj - volCenter, z = vk - volCenter;
                double acc = 0;
                for (int a = 0; a < n; a++) {
                    const double *nx = axes + 9 * (size_t)a;
                    const double *ny = nx + 3;
                    const double *nz = ny + 3;
                    double fi = x * nx[0] + y * nx[1] + z * nx[2] + imgCenter;
                    double fj = x * ny[0] + y * ny[1] + z * ny[2] + imgCenter;
                    double fk = x * nz[0] + y * nz[1] + z * nz[2];
                    if (!(fabs(fk) <= ker_hw)) continue;
                    int imgi = (int)dround(fi), imgj = (int)dround(fj);
                    const double *img_ptr = img + (size_t)a * M * M;
                    for (int j1 = imgj - convW; j1 <= imgj + convW; j1++) {
                        for (int i1 = imgi - convW; i1 <= imgi + convW; i1++) {
                            double w = 1.0;
                            for (int c = 0; c < 3; c++) {
                                double p = (i1 - imgCenter) * nx[c] + (j1 - imgCenter) * ny[c] + volCenter;
                                double v = c == 0 ? vi : (c == 1 ? vj : vk);
                                double rr = fmin(fmax(p - v, -convW), convW);
                                int kidx = imin(imax((int)dround(rr * kerScale + kerCenter), 0), ker_size - 1);
                                w *= ker[kidx];
                            }
                            long long lin = (long long)j1 * M + i1;
                            if (lin < (long long)M * M && lin >= 0) acc += img_ptr[lin] * w;
                        }
                    }
                }
                vol[(size_t)vk * V * V + (size_t)vj * V + vi] += acc;
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Exact adjoint of gg_oracle_fp_f64: every (pixel, voxel) pair the forward  */
/* gather reads, with the same weight, scattered back. FP64, accumulates.    */
/* Parallel over directions into per-thread volumes, then summed.            */
/* ------------------------------------------------------------------------ */
void gg_oracle_bp_adjoint_f64(double *vol, int V, const double *img, int M,
                              const double *axes, int n, int mask_radius,
                              const float *ker, int ker_size, double ker_hw)
{
    const int volCenter = V / 2;
    const int imgCenter = M / 2;
    const int convW = (int)dround(ker_hw);
    const double kerCenter = ((double)ker_size - 1) / 2;
    const double kerScale = kerCenter / ker_hw;
    const long long V3 = (long long)V * V * V;
    const long long R2 = (long long)mask_radius * mask_radius;
    int nt = gg_oracle_num_threads();
    if (nt > n) nt = n > 0 ? n : 1;
    double *part = (double *)calloc((size_t)nt * (size_t)V3, sizeof(double));
    if (!part) return;

#pragma omp parallel num_threads(nt)
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        double *pv = part + (size_t)t * (size_t)V3;
#pragma omp for schedule(dynamic, 1)
        for (int a = 0; a < n; a++) {
            const double *nx = axes + 9 * (size_t)a;
            const double *ny = nx + 3;
            const double *img_ptr = img + (size_t)a * M * M;
            for (int j = 0; j < M; j++) {
                for (int i = 0; i < M; i++) {
                    long long d2 = (long long)(i - imgCenter) * (i - imgCenter) + (long long)(j - imgCenter) * (j - imgCenter);
                    if (d2 > R2) continue;
                    double g = img_ptr[(size_t)j * M + i];
                    if (g == 0.0) continue;
                    double x = i - imgCenter, y = j - imgCenter;
                    double fi = nx[0] * x + ny[0] * y + volCenter;
                    double fj = nx[1] * x + ny[1] * y + volCenter;
                    double fk = nx[2] * x + ny[2] * y + volCenter;
                    int ii = (int)dround(fi), jj = (int)dround(fj), kk = (int)dround(fk);
                    for (int i1 = ii - convW; i1 <= ii + convW; i1++) {
                        double ri = fmin(fmax((double)i1 - fi, -convW), convW);
                        double wi = ker[imin(imax((int)dround(ri * kerScale + kerCenter), 0), ker_size - 1)];
                        for (int j1 = jj - convW; j1 <= jj + convW; j1++) {
                            double rj = fmin(fmax((double)j1 - fj, -convW), convW);
                            double wj = ker[imin(imax((int)dround(rj * kerScale + kerCenter), 0), ker_size - 1)];
                            for (int k1 = kk - convW; k1 <= kk + convW; k1++) {
                                double rk = fmin(fmax((double)k1 - fk, -convW), convW);
                                double wk = ker[imin(imax((int)dround(rk * kerScale + kerCenter), 0), ker_size - 1)];
                                long long lin = (long long)k1 * V * V + (long long)j1 * V + i1;
                                if (lin < V3 && lin >= 0) pv[lin] += g * wi * wj * wk;
                            }
                        }
                    }
                }
            }
        }
    }
    for (int t = 0; t < nt; t++) {
        const double *pv = part + (size_t)t * (size_t)V3;
#pragma omp parallel for schedule(static)
        for (long long q = 0; q < V3; q++) vol[q] += pv[q];
    }
    free(part);
}
