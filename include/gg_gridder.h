/*
 * gg_gridder.h - C ABI of the GB300 Kaiser-Bessel Fourier gridder.
 *
 * Drop-in for the setVolume / forwardProject / backProject / getVol /
 * reconstructVol path of tagarelab/MultiGPUGridder.  Every entry point takes
 * plain pointers and sizes and returns an int status (GG_OK = 0); a failing
 * call leaves a message in gg_last_error(handle) (or gg_global_error() for
 * calls without a handle) and never aborts the process.
 *
 * Layouts are the reference's (MATLAB column-major, x fastest):
 *   volume      N*N*N floats,  vol[k*N*N + j*N + i]
 *   CAS volume  V*V*V floats,  V = M + 2*extra_padding, M = N*interp_factor
 *   images      n*N*N floats,  img[a*N*N + j*N + i]
 *   CAS images  n*M*M floats
 *   coordAxes   9 floats per direction: the x, y and z (projection) columns
 *               of the rotation, src/Matlab/utils/get_axes_from_n_rot.m:36-37
 *
 * Host-pointer calls copy through the library; pinned host memory
 * (cudaHostAlloc / cudaHostRegister) is transferred directly, pageable memory
 * is staged through an internal pinned buffer.  *_dev calls take device
 * pointers and a cudaStream_t (passed as void*, NULL = the legacy default
 * stream) and are asynchronous with respect to the host.
 *
 * Calls on one handle are serialised by a mutex.  The library owns its device
 * state and never calls cudaDeviceReset (the reference does, in its
 * constructor and destructor: MultiGPUGridder.h:72, gpuGridder.cpp:758).
 */
#ifndef GG_GRIDDER_H
#define GG_GRIDDER_H

#ifdef __cplusplus
extern "C" {
#endif

#define GG_ABI_VERSION 1

/* status codes */
#define GG_OK 0
#define GG_ERR_INVALID_ARG 1
#define GG_ERR_CUDA 2
#define GG_ERR_OUT_OF_MEMORY 3
#define GG_ERR_STATE 4
#define GG_ERR_NO_DEVICE 5
#define GG_ERR_CUFFT 6
#define GG_ERR_TIMEOUT 7 /* gg_server_wait: the request is not done yet */
#define GG_ERR_BUSY 8    /* gg_server_submit: the backlog bound is reached; retry later */

/* storage precision of the resident CAS volume and of the CAS images the
   projection kernels read (window accumulation is always FP32) */
#define GG_PREC_F32 0
#define GG_PREC_F16 1
#define GG_PREC_BF16 2

/* back-projection rule */
#define GG_BP_REF 0     /* the reference's window rule, gpuBackProject.cu:54-107 */
#define GG_BP_ADJOINT 1 /* exact adjoint of the forward projection (no reference counterpart) */

typedef struct gg_gridder gg_gridder;

/* Library version (GG_ABI_VERSION) and last error of a call without a handle. */
int gg_version(void);
const char *gg_global_error(void);

/* Replaces MultiGPUGridder::MultiGPUGridder(int VolumeSize, int numCoordAxes,
   float interpFactor, int extraPadding, int Num_GPUs, int *GPU_Devices,
   int RunFFTOnDevice, bool verbose)  (src/Gridders/MultiGPUGridder.h:36).
   num_coord_axes sizes the first device batch (it may be 0); gpu_devices may
   be NULL (device 0).  One device per handle: a GB300 machine runs one GPU per
   process, so num_gpus > 1 selects gpu_devices[0] and orientation sharding is
   left to the caller (one handle per GPU).  run_fft_on_device = 0 keeps the
   CAS-image interface of the reference's host-FFT mode. */
int gg_create(int volume_size, int num_coord_axes, float interp_factor, int extra_padding,
              int num_gpus, const int *gpu_devices, int run_fft_on_device, int verbose,
              gg_gridder **out);

/* Replaces MultiGPUGridder::~MultiGPUGridder (MultiGPUGridder.h:101-104)
   without the cudaDeviceReset of gpuGridder::FreeMemory (gpuGridder.cpp:754-764). */
void gg_destroy(gg_gridder *h);
const char *gg_last_error(const gg_gridder *h);

/* Derived sizes: N, M (CAS image edge), V (CAS volume edge), mask radius (int). */
int gg_get_sizes(const gg_gridder *h, int *N, int *M, int *V, int *mask_radius);

/* Setters of AbstractGridder (src/Gridders/AbstractGridder.h:53-89) and
   MultiGPUGridder (MultiGPUGridder.h:107-110). */
int gg_set_kb_table(gg_gridder *h, const float *table, int n);      /* SetKerBesselVector; default: getKernelFiltTable(2,501) computed in FP64 */
int gg_set_mask_radius(gg_gridder *h, float radius);                /* SetMaskRadius (truncated to int like RunKernel) */
int gg_set_max_axes_to_allocate(gg_gridder *h, int max_axes);       /* SetMaxAxesToAllocate: directions per device batch */
int gg_set_num_streams_fp(gg_gridder *h, int n);                    /* SetNumStreamsFP: copy/compute pipeline depth */
int gg_set_num_streams_bp(gg_gridder *h, int n);                    /* SetNumStreamsBP */
int gg_set_precision(gg_gridder *h, int precision);                 /* GG_PREC_*: storage of CAS volume / CAS images */
/* Storage of the CAS images the back projection reads, apart from the CAS
   volume's: GG_PREC_* or -1 (the default) to follow gg_set_precision.
   GG_PREC_F32 under a 2-byte volume keeps the images exact; it costs about
   the same as 2-byte images.  No counterpart in the reference. */
int gg_set_image_precision(gg_gridder *h, int precision);
int gg_set_bp_mode(gg_gridder *h, int mode);                        /* GG_BP_REF (default) or GG_BP_ADJOINT */

/* setVolume + the CAS preparation of forwardProject
   (MultiGPUGridder_Matlab_Class.m:272-275, :226-227; CASFromVol_Gridder.m:25-60),
   done on the device: pad N^3 -> M^3, KB pre-compensation, 3-D FFT, Re+Im,
   pad to V^3.  The CAS volume stays resident. dims = {N, N, N}. */
int gg_set_volume(gg_gridder *h, const float *volume, const int dims[3]);
/* AbstractGridder::SetCASVolume (AbstractGridder.h:71): upload a CAS volume V^3. */
int gg_set_cas_volume(gg_gridder *h, const float *cas_volume, const int dims[3]);
/* gpuGridder::CopyCASVolumeToHost (gpuGridder.cpp:14-17): read the CAS volume V^3. */
int gg_get_cas_volume(gg_gridder *h, float *cas_volume_out);
/* resetVolume (MultiGPUGridder_Matlab_Class.m:277-282): zero the CAS volume. */
int gg_reset_volume(gg_gridder *h);

/* MultiGPUGridder::ForwardProject (MultiGPUGridder.cpp:98-184 ->
   gpuGridder::ForwardProject, gpuGridder.cpp:180-305): n directions ->
   images_out (n*N*N, may be NULL) and/or cas_images_out (n*M*M, may be NULL). */
int gg_forward_project(gg_gridder *h, const float *axes, int n_axes,
                       float *images_out, float *cas_images_out);

/* MultiGPUGridder::BackProject (MultiGPUGridder.cpp:186-269 ->
   gpuGridder::BackProject, gpuGridder.cpp:307-430).  Give images (n*N*N,
   FFT on the device) or cas_images (n*M*M, the host-FFT mode).  accumulate = 0
   zeroes the CAS volume first as the reference does (gpuGridder.cpp:332). */
int gg_back_project(gg_gridder *h, const float *axes, int n_axes,
                    const float *images, const float *cas_images, int accumulate);

/* getVol (MultiGPUGridder_Matlab_Class.m:314-327 ->
   MultiGPUGridder::CASVolumeToVolume, MultiGPUGridder.cpp:271-304, then
   volFromCAS_Gridder.m:26-56) on the device: CAS volume -> volume N^3. */
int gg_get_volume(gg_gridder *h, float *volume_out);

/* reconstructVol (MultiGPUGridder_Matlab_Class.m:284-312): back-project the
   images, back-project all-ones CAS images (plane density), divide
   CAS ./ (PD + 1e-6), then getVol.  Leaves the divided CAS volume resident. */
int gg_reconstruct_volume(gg_gridder *h, const float *axes, int n_axes,
                          const float *images, float *volume_out);

/* Device-pointer forms of the calls above. */
int gg_set_volume_dev(gg_gridder *h, const float *d_volume, void *stream);
int gg_set_cas_volume_dev(gg_gridder *h, const float *d_cas_volume, void *stream);
int gg_get_cas_volume_dev(gg_gridder *h, float *d_cas_volume_out, void *stream);
int gg_forward_project_dev(gg_gridder *h, const float *d_axes, int n_axes,
                           float *d_images_out, float *d_cas_images_out, void *stream);
int gg_back_project_dev(gg_gridder *h, const float *d_axes, int n_axes,
                        const float *d_images, const float *d_cas_images, int accumulate, void *stream);
int gg_get_volume_dev(gg_gridder *h, float *d_volume_out, void *stream);
int gg_reconstruct_volume_dev(gg_gridder *h, const float *d_axes, int n_axes,
                              const float *d_images, float *d_volume_out, void *stream);

/* Sharded reconstructVol, one gridder per GPU (one process per GPU).  The
   reference splits the directions over its GPUs (ceil(n/G) each,
   MultiGPUGridder::PlanCoordinateAxes, MultiGPUGridder.cpp:37-96), each GPU
   back-projects its slice into its own CAS volume (MultiGPUGridder::BackProject,
   MultiGPUGridder.cpp:186-269), the volumes are summed on one GPU by peer
   copies (MultiGPUGridder.cpp:376-411), and reconstructVol divides by the
   plane density (MultiGPUGridder_Matlab_Class.m:293-311).
   gg_back_project_sums_dev: this GPU's slice -> d_sums, 2*V^3 floats written
   (not accumulated): [0, V^3) the CAS volume of the images' back projection,
   [V^3, 2V^3) the plane density (back projection of all-ones CAS images),
   both in one fused pass, un-divided.  The caller sums d_sums over the GPUs
   (one all-reduce or reduce of 2*V^3 floats).
   gg_volume_from_sums_dev: summed d_sums -> CAS volume sums[0] ./ (sums[1] +
   1e-6), left resident, then getVol into d_volume_out (N^3).  With one GPU
   the two calls give gg_reconstruct_volume_dev's result bit for bit. */
int gg_back_project_sums_dev(gg_gridder *h, const float *d_axes, int n_axes, const float *d_images,
                             float *d_sums, void *stream);
int gg_volume_from_sums_dev(gg_gridder *h, const float *d_sums, float *d_volume_out, void *stream);

/* reconstructVol with CTF correction.  The reference carries only the flag
   for it (`ApplyCTFs`, src/Gridders/AbstractGridder.h:118-119) and never
   reads it.  Each image's CAS image is multiplied by its weak-phase CTF
   before the back projection, and the plane density back-projects CTF^2
   images instead of all-ones ones:
     vol = getVol( BP(CTF . CAS(img)) ./ (BP(CTF^2) + 1e-6) ).
   CTF(s) = -(sqrt(1 - A^2) sin chi + A cos chi),
   chi = pi lambda df s^2 - (pi/2) Cs lambda^3 s^4, s the spatial frequency
   (1/Å) of the padded image's pixel, lambda the relativistic electron
   wavelength at voltage_kv.  defocus: n_axes values in Å (underfocus
   positive).  Astigmatism (both NULL for none): defocus_v, n_axes defoci V
   in Å (defocus is then U), and astig_angle, n_axes angles in radians of the
   U axis from the image x axis; df at frequency angle theta is
   (U + V)/2 + (U - V)/2 cos 2(theta - angle).  cs_mm in mm; amp_contrast A
   in [0, 1]; pixel_size: Å per pixel of the N x N images.  With defocus 0,
   Cs 0 and A = 1 the CTF is -1 and the result equals gg_reconstruct_volume's. */
int gg_reconstruct_volume_ctf(gg_gridder *h, const float *axes, int n_axes, const float *images,
                              const float *defocus, const float *defocus_v, const float *astig_angle,
                              float voltage_kv, float cs_mm, float amp_contrast, float pixel_size, float *volume_out);
int gg_reconstruct_volume_ctf_dev(gg_gridder *h, const float *d_axes, int n_axes, const float *d_images,
                                  const float *d_defocus, const float *d_defocus_v, const float *d_astig_angle,
                                  float voltage_kv, float cs_mm, float amp_contrast, float pixel_size,
                                  float *d_volume_out, void *stream);

/* Exact adjoint of the whole forward operator (setVolume's CAS preparation
   followed by forwardProject to images): image gradients n*N*N -> volume
   gradient N^3 (written, not accumulated).  Uses the exact-adjoint back
   projection whatever gg_set_bp_mode says and leaves the resident CAS volume
   untouched.  No counterpart in the reference, which has no gradient. */
int gg_forward_project_adjoint(gg_gridder *h, const float *axes, int n_axes, const float *image_grads,
                               float *volume_grad_out);
int gg_forward_project_adjoint_dev(gg_gridder *h, const float *d_axes, int n_axes, const float *d_image_grads,
                                   float *d_volume_grad_out, void *stream);

/* ---------------------------------------------------------------------------
 * Stateless kernel entry points (device pointers).
 * ------------------------------------------------------------------------- */

/* Replaces gpuForwardProject::RunKernel (src/Projection/gpuForwardProject.cu:103-144):
   CAS volume (V^3) -> CAS images (n*M*M, pixels outside the mask are written 0). */
int gg_forward_project_kernel(const float *d_cas_volume, float *d_cas_images, const float *d_kb_table,
                              const float *d_axes, float ker_hwidth, int n_axes, int cas_vol_size,
                              int cas_img_size, int extra_padding, int mask_radius, int kb_table_size,
                              void *stream);

/* Replaces gpuBackProject::RunKernel (src/Projection/gpuBackProject.cu:115-155):
   CAS images (n*M*M) -> CAS volume (V^3), accumulated into (+=). */
int gg_back_project_kernel(float *d_cas_volume, const float *d_cas_images, const float *d_kb_table,
                           const float *d_axes, float ker_hwidth, int n_axes, int cas_vol_size,
                           int cas_img_size, int mask_radius, int kb_table_size, int extra_padding,
                           void *stream);

/* Exact adjoint of gg_forward_project_kernel (same weights, every pair the
   forward gather reads).  No counterpart in the reference. */
int gg_back_project_adjoint_kernel(float *d_cas_volume, const float *d_cas_images, const float *d_kb_table,
                                   const float *d_axes, float ker_hwidth, int n_axes, int cas_vol_size,
                                   int cas_img_size, int mask_radius, int kb_table_size, void *stream);

/* Plane-density-normalised back projection that allocates no memory: writes
   d_cas_volume_out = BP(d_cas_images) / (BP(all-ones images) + 1e-6), the
   CAS-volume half of reconstructVol (MultiGPUGridder_Matlab_Class.m:293-308),
   both back projections under the reference window rule in one fused pass.
   No counterpart in the reference: its plane density lives in a per-gridder
   buffer; here it lives in a fixed scratch array in the library's device
   memory, so the call makes no cudaMalloc, cudaFree or other allocating call.
   Limit: cas_vol_size^3 <= 4,194,304 (16 MiB of scratch; cas_vol_size <= 161);
   larger sizes return GG_ERR_INVALID_ARG.  The output is overwritten and need
   not start at zero; the scratch must be zero when the back projection
   starts, and the call zeroes it itself on `stream` first.  All calls on one
   device share the scratch: calls that overlap (different streams or threads
   with no ordering between them) race on it.  Every call looks up the
   scratch address in the current context (cudaGetSymbolAddress, no cache:
   a cudaDeviceReset or a second context on the device would leave a cached
   address stale).  The first call in a context may load the library's
   module onto the device, so it should come before any stream capture. */
int gg_back_project_normalized_noalloc(float *d_cas_volume_out, const float *d_cas_images, const float *d_kb_table,
                                       const float *d_axes, float ker_hwidth, int n_axes, int cas_vol_size,
                                       int cas_img_size, int mask_radius, int kb_table_size, void *stream);

/* ---------------------------------------------------------------------------
 * Building blocks: the reference's filters (src/Filters/<name>Filter.cu) on device
 * pointers; `n_slices` = 0 selects the 3-D form where the reference has one.
 * ------------------------------------------------------------------------- */
int gg_filter_complex_to_cas(const float *d_complex, float *d_cas, int size, int n_slices, void *stream);      /* ComplexToCASFilter.cu:3-26 */
int gg_filter_cas_to_complex(const float *d_cas, float *d_complex, int size, int n_slices, void *stream);      /* CASToComplexFilter.cu:3-81 */
int gg_filter_fftshift_2d(float *d_data, int complex_elems, int size, int n_slices, void *stream);           /* FFTShift2DFilter.cu:4-62 (in place, even size) */
int gg_filter_fftshift_3d(float *d_data, int complex_elems, int size, void *stream);                         /* FFTShift3DFilter.cu:4-98 (in place, even size) */
int gg_filter_pad_volume(const float *d_in, float *d_out, int in_x, int in_y, int in_z,
                         int pad_x, int pad_y, int pad_z, void *stream);                                      /* PadVolumeFilter.cu:4-36 (writes the border zeros too) */
int gg_filter_crop_volume(const float *d_in, float *d_out, int in_x, int in_y, int in_z,
                          int crop_x, int crop_y, int crop_z, void *stream);                                  /* CropVolumeFilter.cu:5-39 */
int gg_filter_divide_volumes(float *d_a, const float *d_b, int size, int n_slices, void *stream);             /* DivideVolumeFilter.cu:3-33 (zero guard) */
int gg_filter_multiply_volumes(float *d_a, const float *d_b, int a_complex, int size, int n_slices, void *stream); /* MultiplyVolumeFilter.cu:3-53 */
int gg_filter_add_volumes(float *d_a, const float *d_b, int size, int n_slices, void *stream);                /* AddVolumeFilter.cu:4-27 */
int gg_filter_divide_scalar(float *d_a, float scalar, int size, int n_slices, void *stream);                  /* DivideScalarFilter.cu:3-25 */
int gg_filter_real_to_complex(const float *d_real, float *d_complex, int size, int n_slices, void *stream);   /* RealToComplexFilter.cu:3-26 */
int gg_filter_complex_to_real(const float *d_complex, float *d_real, int size, int n_slices, void *stream);   /* ComplexToRealFilter.cu:3-25 */

/* CTF on CAS images (n_images * size^2, the gridder's CAS-image layout, DC at
   (size/2, size/2)): generate = 0 multiplies them by CTF^power, generate = 1
   overwrites them with CTF^power (power 1 or 2).  Parameters as for
   gg_reconstruct_volume_ctf (d_defocus_v and d_astig_angle both NULL for no
   astigmatism).  No counterpart in the reference. */
int gg_filter_apply_ctf(float *d_cas_images, int size, int n_images, const float *d_defocus,
                        const float *d_defocus_v, const float *d_astig_angle, float voltage_kv, float cs_mm,
                        float amp_contrast, float pixel_size, int power, int generate, void *stream);

/* Host helpers: the KB lookup table (getKernelFiltTable.m:1-22) and the
   pre-compensation vector (getPreComp.m:1-28), computed in FP64. */
int gg_kb_table(int ker_hwidth, int table_size, double *table_out);
int gg_precomp(int M, int ker_hwidth, double *precomp_out);

/* ---------------------------------------------------------------------------
 * Instrumentation.  The reference has none beyond verbose prints and
 * MATLAB tic/toc (src/Examples/TimingTestScript.m:20-38).
 * ------------------------------------------------------------------------- */
#define GG_KERNEL_FORWARD 0   /* forward projection kernel */
#define GG_KERNEL_BACK 1      /* back projection kernel (images) */
#define GG_KERNEL_DENSITY 2   /* back projection of all-ones images (plane density) */

/* L2 read bandwidth of the current device in GB/s, the peak the projection
   kernels' L2 roofline is taken against: a buffer of about 40% of the L2
   read repeatedly with L2-only loads by 4 CTAs per SM, best of `runs`
   event-timed launches.  Allocates and frees its own buffer. */
int gg_measure_l2_read_gbs(int runs, double *gbs_out);

/* Number of kernels this library has launched in the process so far. */
long long gg_kernel_launch_count(void);
/* Per-handle kernel timing with CUDA events recorded around each projection
   kernel launch on its stream; enabling resets the totals. */
int gg_profile_enable(gg_gridder *h, int enable);
/* Total device time (ms) and launch count of one GG_KERNEL_* kernel since
   profiling was enabled (synchronises on the recorded events). */
int gg_profile_read(gg_gridder *h, int kernel, double *total_ms, long long *launches);

#ifdef __cplusplus
/* ---------------------------------------------------------------------------
 * Serving: a persistent request loop on one GPU.  No counterpart in the
 * reference, whose calls run one at a time and end with a device sync
 * (MultiGPUGridder.cpp ForwardProject/BackProject).  A server keeps CAS
 * volumes resident (each prepared once, as setVolume does) and runs forward and
 * back projection requests of any volume size and orientation count on
 * `lanes` lanes (CUDA stream pairs).  Requests run in chunks of directions of
 * about one quantum of estimated device time; a free lane takes the chunk of
 * the request with the least estimated work left (less 0.2 s per second
 * waited); requests of one quantum or less run on high-priority streams and
 * have a quarter of the lanes to themselves.
 * A request starts once its device buffers fit the HBM budget (admission by
 * footprint, in that order), so the work of requests that arrive while others
 * run overlaps on the device.  A request's result does not depend on what
 * else runs (same kernels on the same chunks, in order).  Host buffers should
 * be pinned (cudaHostAlloc) for the copies to overlap; they must stay valid
 * until gg_server_wait returns.
 * ------------------------------------------------------------------------- */
typedef struct gg_server gg_server;

#define GG_OP_FORWARD 0 /* out = forwardProject(volume, axes): n*N*N images */
#define GG_OP_BACK 1    /* out = backProject(images, axes) into a zeroed CAS volume: V^3 floats */

/* hbm_budget_gb <= 0: 90% of the device memory free at creation. */
int gg_server_create(int device, double hbm_budget_gb, int lanes, gg_server **out);
/* Finishes the queued and running requests, then frees everything. */
void gg_server_destroy(gg_server *s);
const char *gg_server_last_error(const gg_server *s);
/* A resident volume (N^3 FP32, host or device pointer), interpolation factor
   interp_factor, extra padding 3 as the reference's default. */
int gg_server_add_volume(gg_server *s, const float *volume, int volume_size, float interp_factor, int on_device,
                         int *volume_id);
int gg_server_remove_volume(gg_server *s, int volume_id);
int gg_server_volume_sizes(gg_server *s, int volume_id, int *N, int *M, int *V);
/* Queues a request; returns at once.  images: n*N*N (GG_OP_BACK only). */
int gg_server_submit(gg_server *s, int volume_id, int op, const float *axes, int n_axes, const float *images,
                     float *out, long long *request_id);
/* Waits for a request (timeout_s < 0: no limit) and returns its status;
   latency_ms (nullable) = completion - submission.  Each request is waited
   for once. */
int gg_server_wait(gg_server *s, long long request_id, double timeout_s, double *latency_ms);
/* Latency percentiles (submission to completion) of the requests completed
   since the last reset, the most requests run at once and the most device
   memory in use (GB, resident volumes included). */
int gg_server_stats(gg_server *s, long long *completed, double *p50_ms, double *p99_ms, double *mean_ms,
                    long long *peak_inflight, double *peak_gb);
int gg_server_reset_stats(gg_server *s);
/* Estimated device time of one chunk (default 8 ms).  Smaller quanta let short
   requests overtake long ones sooner; larger ones cost fewer launches.  It
   applies to requests submitted afterwards, and fixes how they are chunked
   (and so the order of a back projection's sums). */
int gg_server_set_quantum(gg_server *s, double quantum_ms);
/* Bound on the estimated device time of the requests queued and not yet
   started; a submission beyond it fails with GG_ERR_BUSY.  0 (the default):
   no bound. */
int gg_server_set_max_backlog(gg_server *s, double seconds);
/* Requests queued (not started) and admitted (started, not done), the
   estimated seconds of queued work, and the submissions refused with
   GG_ERR_BUSY since the last reset (each pointer nullable). */
int gg_server_load(gg_server *s, long long *queued, long long *active, double *queued_seconds,
                   long long *rejected);

}
#endif
#endif /* GG_GRIDDER_H */
