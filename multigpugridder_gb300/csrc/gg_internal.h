// Internal launcher interface shared by the kernel and API translation units.
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>
#include <stddef.h>

namespace gg {

enum Prec { kF32 = 0, kF16 = 1, kBF16 = 2 };

inline size_t prec_bytes(int p) { return p == kF32 ? 4 : 2; }

// Largest KB table accepted (the kernels stage it in shared memory).
constexpr int kMaxKerSizeHost = 1000;

// Geometry of one projection problem.
struct Geom {
    int V;           // CAS volume edge
    int M;           // CAS image edge
    int mask_radius; // int, as RunKernel passes it
    int ker_size;    // KB table length
    float ker_hw;    // KB half-width (2)
};

// ---- projection kernels (gg_project.cu) ----------------------------------
// Forward projection: CAS volume (storage `vprec`) -> CAS images (FP32,
// n*M*M, zero outside the mask).  `five_taps` selects the reference's full
// 5x5x5 window (needed only for KB tables whose edge values are not zero).
// Storage scaling: FP16 storage holds x / scale, with scale a power of two
// kept in device memory (d_scale; NULL means 1) so no host sync is needed.
// The forward projection multiplies every output pixel by *d_scale.
// The volume's rows are `pitch` elements apart (planes pitch*V); the
// reference's dense layout is pitch = V.  fp_pitch(V) rows let the 4-tap
// kernel read each row of taps with aligned vector loads.
// d_vol_y, d_vol_z (optional): copies of the volume, in the same storage and
// pitch, with y and z as the contiguous axis (launch_transpose_volume for
// dense FP32, launch_pitch_volume layouts 1 and 2 for FP16/BF16); each
// direction then reads the copy whose contiguous axis is the most
// perpendicular to it.  d_order (optional, n ints of scratch, used with the
// copies): the directions then run grouped by the copy they read (a stable
// partition computed on the device), so that one copy at a time is hot in
// L2; each image is still written at its direction's slot.
cudaError_t launch_forward_project(const void *d_vol, int vprec, int pitch, float *d_img, const float *d_ker,
                                   const float *d_axes, int n, const Geom &g, bool five_taps,
                                   const float *d_scale, cudaStream_t s, const void *d_vol_y = nullptr,
                                   const void *d_vol_z = nullptr, int *d_order = nullptr);
// FP32 volume V^3 (x fastest) -> the same volume with y (layout 1: [z][x][y])
// or z (layout 2: [y][x][z]) as the contiguous axis.
cudaError_t launch_transpose_volume(const float *d_in, int V, float *d_out, int layout, cudaStream_t s);
inline int fp_pitch(int V) { return (V + 4 + 7) / 8 * 8; }
// FP32 CAS volume V^3 -> the same volume with row pitch P (zero-filled past
// V) in storage `prec` (x / *d_scale for FP16), with x (layout 0: [z][y][x]),
// y (layout 1: [z][x][y]) or z (layout 2: [y][x][z]) as the contiguous axis.
cudaError_t launch_pitch_volume(const float *d_cas, int V, int P, void *d_out, int prec, const float *d_scale,
                                cudaStream_t s, int layout = 0);

// Back projection with the reference window rule, accumulated (+=) into the
// FP32 CAS volume.  d_img holds n*M*M CAS images in storage `iprec`; when
// `ones` is set the images are taken to be all ones (plane density) and
// d_img is not read.
// *d_scale multiplies each voxel's sum before it is added.  shared: the GPU
// runs other launches concurrently (smaller CTAs that share an SM; FP32
// images, the same sums bit for bit).
cudaError_t launch_back_project_ref(float *d_vol, const void *d_img, int iprec, bool ones,
                                    const float *d_ker, const float *d_axes, int n, const Geom &g,
                                    const float *d_scale, cudaStream_t s, bool shared = false);

// Reference-rule back projection of d_img into d_vol and, in the same pass,
// of all-ones images (the plane density) into d_pd; both accumulated.
cudaError_t launch_back_project_ref_density(float *d_vol, float *d_pd, const void *d_img, int iprec,
                                            const float *d_ker, const float *d_axes, int n, const Geom &g,
                                            const float *d_scale, cudaStream_t s);

// Reference-rule back projection of two FP32 image stacks over the same
// directions in one pass: d_img into d_vol and d_img2 into d_pd, both
// accumulated, each equal to its own launch_back_project_ref.
cudaError_t launch_back_project_ref_pair(float *d_vol, float *d_pd, const float *d_img, const float *d_img2,
                                         const float *d_ker, const float *d_axes, int n, const Geom &g, cudaStream_t s);

// Exact adjoint of launch_forward_project (4 taps), accumulated into d_vol.
// zero_edges: the KB table's first and last entries are 0 (the fast path
// relies on it).
cudaError_t launch_back_project_adjoint(float *d_vol, const void *d_img, int iprec, const float *d_ker,
                                        const float *d_axes, int n, const Geom &g, const float *d_scale,
                                        bool zero_edges, cudaStream_t s);

// ---- CAS / FFT stages (gg_cas.cu) ------------------------------------------
// Volume N^3 -> real M^3 FFT input: centred zero-pad, separable precomp
// multiply, fftshift folded into the index map.
cudaError_t launch_vol_to_fft_input(const float *d_vol, int N, int M, const double *d_precomp,
                                    float *d_x, cudaStream_t s);
// R2C half spectrum [M][M][M/2+1] -> CAS volume V^3 (storage `prec`), border zeroed.
cudaError_t launch_spectrum_to_cas_volume(const cufftComplex *d_spec, int M, int V, void *d_cas,
                                          int prec, const float *d_scale, cudaStream_t s);
// CAS volume V^3 (FP32) -> Hermitian half spectrum for C2R: crop the pad,
// FromCAS 3-D, fftshift folded into the index map.
cudaError_t launch_cas_volume_to_spectrum(const float *d_cas, int V, int M, cufftComplex *d_spec,
                                          cudaStream_t s);
// C2R output M^3 -> volume N^3: fftshift, 1/M^3, precomp, centred crop.
cudaError_t launch_fft_output_to_vol(const float *d_y, int M, int N, const double *d_precomp,
                                     float *d_vol, cudaStream_t s);
// CAS images n*M*M -> Hermitian half spectra n*M*(M/2+1) (FromCAS 2-D + shift).
cudaError_t launch_cas_images_to_spectrum(const float *d_cas, int M, int n, cufftComplex *d_spec,
                                          cudaStream_t s);
// C2R outputs n*M*M -> images n*N*N (shift, centred crop, 1/M^2).
cudaError_t launch_fft_output_to_images(const float *d_y, int M, int N, int n, float *d_img,
                                        cudaStream_t s);
// Images n*N*N -> R2C inputs n*M*M (centred zero-pad, shift).
cudaError_t launch_images_to_fft_input(const float *d_img, int N, int M, int n, float *d_x,
                                       cudaStream_t s);
// R2C half spectra n*M*(M/2+1) -> CAS images n*M*M (shift, Re+Im) in storage `prec`.
cudaError_t launch_spectrum_to_cas_images(const cufftComplex *d_spec, int M, int n, void *d_cas,
                                          int prec, const float *d_scale, cudaStream_t s);
// Adjoint of the whole forward operator (volume -> images), by stage:
// R2C half spectra of padded, shifted image gradients -> CAS-image gradients
// (Re+Im, first row/column zero, 1/M^2).
cudaError_t launch_spectrum_to_cas_images_adjoint(const cufftComplex *d_spec, int M, int n, float *d_cas,
                                                  cudaStream_t s);
// CAS-volume gradient V^3 -> R2C input M^3 (inner crop + shift).
cudaError_t launch_cas_volume_adjoint_input(const float *d_g, int V, int M, float *d_x, cudaStream_t s);
// R2C spectrum -> volume gradient N^3 (Re+Im, shift, precomp, crop).
cudaError_t launch_spectrum_to_vol_adjoint(const cufftComplex *d_spec, int M, int N, const double *d_precomp,
                                           float *d_vol, cudaStream_t s);
// d[0..count) = value.
cudaError_t launch_fill(float *d, size_t count, float value, cudaStream_t s);
// a = a / (b + eps) over `count` elements (reconstructVol's plane-density division).
cudaError_t launch_divide_plane_density(float *d_a, const float *d_b, size_t count, float eps,
                                        cudaStream_t s);
// FP32 -> storage conversion (count elements): out = in / *d_scale.
cudaError_t launch_convert(const float *d_in, void *d_out, int prec, size_t count, const float *d_scale,
                           cudaStream_t s);
// *d_scale = smallest power of two >= max|x| / target (at least 1) over
// `count` floats; d_work is one scratch unsigned int.
cudaError_t launch_storage_scale(const float *d_x, size_t count, float target, unsigned int *d_work,
                                 float *d_scale, cudaStream_t s);

// Weak-phase CTF parameters (defocus per image, underfocus positive, Å).
struct CtfParams {
    float voltage_kv, cs_mm, amp_contrast, pixel_size; // pixel_size: real-space Å of the N x N images
};
// Constants of the CTF kernel: alpha, beta as float pairs, 2 pi in three
// parts for the reduction, the sin / cos weights.
struct CtfConsts {
    double alpha; // pi lambda / (M px)^2 (FP64, for the astigmatic terms)
    float a_hi, a_lo, b_hi, b_lo, p1, p2, p3, inv_2pi, w_sin, w_cos;
};
// Over n CAS images of M x M (d_defocus: n defoci in Å; with d_defocus_v and
// d_astig both given, defocus U / V and the astigmatism angle in radians):
// d_mul (optional) *= CTF^mul_power and d_gen (optional) = CTF^gen_power, in
// one pass.
cudaError_t launch_ctf(float *d_mul, int mul_power, float *d_gen, int gen_power, int M, int n, const float *d_defocus,
                       const float *d_defocus_v, const float *d_astig, const CtfParams &c, cudaStream_t s);

// ---- fused 2-D FFT stages (gg_fft2.cu) ----------------------------------------
// True when N, M take the fused kernels: M in {64, 128, 256}, N <= M/2, N a
// multiple of M/16, and the shared memory fits.
bool fft2_fused_ok(int N, int M);
// Images n*N*N -> CAS images n*M*M in storage `prec` (FP32 or BF16; FP16
// needs the spectrum's scale first and is refused), in one launch: the pad,
// shifts, forward 2-D FFT and Re+Im of the path above.  adjoint: the gradient
// form of launch_spectrum_to_cas_images_adjoint (FP32 only).
cudaError_t launch_images_to_cas_fused(const float *d_img, int N, int M, int n, void *d_cas, int prec, bool adjoint,
                                       cudaStream_t s);
// CAS images n*M*M (FP32) -> images n*N*N in one launch: FromCAS, shifts,
// inverse 2-D FFT, crop and 1/M^2.
cudaError_t launch_cas_to_images_fused(const float *d_cas, int M, int N, int n, float *d_img, cudaStream_t s);

// Adds to the process-wide count of kernels launched by this library.
void count_launches(long long n);

// Sets the calling thread's message returned by gg_global_error().
void set_global_error(const char *msg);

// Argument checks shared by the stateless kernel entry points: kerHWidth 2,
// sizes positive, a KB table of 3..kMaxKerSizeHost entries.  Returns GG_OK or
// GG_ERR_INVALID_ARG with the message set for gg_global_error().
int check_kernel_args(float ker_hwidth, int n_axes, int V, int M, int mask_radius, int kb_size);

// ---- a gridder's resident state, for the serving loop (gg_api.cu) ---------
struct GridderView {
    int device, N, M, V;
    Geom g;
    const float *cas; // FP32 CAS volume V^3
    const float *cas_y, *cas_z; // its copies with y / z contiguous (may be null)
    const float *ker; // KB table
    bool five_taps;
    bool fused_fft;   // fft2_fused_ok(N, M)
};

} // namespace gg

struct gg_gridder;

namespace gg {

// Fills `out` from a gridder whose volume is set; false if it has none.
bool gridder_view(gg_gridder *h, GridderView *out);
// Frees the gridder's set-up scratch (the M^3 FFT buffers and plans); the
// CAS volume stays resident.
void gridder_trim(gg_gridder *h);
// Builds the copies of the CAS volume the FP32 forward projection reads
// (synchronous); false on failure.
bool gridder_prepare_forward(gg_gridder *h);

// ---- host math (gg_kb.cpp) --------------------------------------------------
void kb_table_f64(int hw, int size, double *out);
void precomp_f64(int M, int hw, double *out);

} // namespace gg
