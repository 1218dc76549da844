// Plane-density-normalised back projection that allocates no memory.
//
// gg_back_project_normalized_noalloc writes
//     cas_out = BP(cas_images) ./ (BP(ones) + 1e-6)
// the CAS-volume half of reconstructVol
// (src/Matlab/MultiGPUGridder_Matlab_Class.m:293-308): the back projection of
// the images, the plane density (the back projection of all-ones CAS images
// over the same directions) and their voxel-wise quotient.  The fused kernel
// of the gridder forms both sums in one pass; here its plane-density buffer is
// a fixed array in the library's device memory instead of a per-gridder
// allocation, so a call makes no cudaMalloc, cudaFree or other allocating call.
//
// The scratch holds the plane density of one call: kNoAllocMaxVoxels floats
// (16 MiB), so cas_vol_size^3 <= 4,194,304 (cas_vol_size <= 161).  Calls that
// overlap on one device share it and race; callers order them (one stream, or
// events between streams).
#include "gg_internal.h"
#include "../../include/gg_gridder.h"

namespace gg {

constexpr size_t kNoAllocMaxVoxels = (size_t)4 << 20; // 16 MiB of FP32

// Plane density of the current call.  Only its first V^3 floats are used;
// they must be zero when the fused kernel starts, and each call zeroes them
// itself on its stream before the back projection.
static __device__ __align__(256) float g_noalloc_plane_density[kNoAllocMaxVoxels];

namespace {

// Device address of the scratch array in the current context.  In host code
// the array's name stands for a host-side shadow, not device memory, so the
// address is looked up with cudaGetSymbolAddress.  The lookup is made on
// every call and not cached: the address belongs to the context the
// library's module is loaded in, and a cudaDeviceReset (a MATLAB
// reset(gpuDevice), say) or another context on the same device makes a
// cached address stale.  The lookup allocates nothing; the first one in a
// context may load the module onto the device.
int noalloc_scratch(float **out)
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_plane_density);
    if (e != cudaSuccess || !p) {
        set_global_error(e != cudaSuccess ? cudaGetErrorString(e)
                                          : "cudaGetSymbolAddress returned no address for the scratch array");
        return GG_ERR_CUDA;
    }
    *out = (float *)p;
    return GG_OK;
}

} // namespace
} // namespace gg

using namespace gg;

extern "C" int gg_back_project_normalized_noalloc(float *d_cas_volume_out, const float *d_cas_images,
                                                  const float *d_kb_table, const float *d_axes, float ker_hwidth,
                                                  int n_axes, int cas_vol_size, int cas_img_size, int mask_radius,
                                                  int kb_table_size, void *stream)
{
    int rc = check_kernel_args(ker_hwidth, n_axes, cas_vol_size, cas_img_size, mask_radius, kb_table_size);
    if (rc != GG_OK) return rc;
    const size_t V3 = (size_t)cas_vol_size * cas_vol_size * cas_vol_size;
    if (V3 > kNoAllocMaxVoxels) {
        set_global_error("gg_back_project_normalized_noalloc: cas_vol_size^3 exceeds the fixed plane-density "
                         "scratch of 4,194,304 voxels (16 MiB; cas_vol_size <= 161)");
        return GG_ERR_INVALID_ARG;
    }
    if (!d_cas_volume_out || !d_cas_images || !d_kb_table || (n_axes > 0 && !d_axes)) {
        set_global_error("null pointer");
        return GG_ERR_INVALID_ARG;
    }
    float *pd = nullptr;
    rc = noalloc_scratch(&pd);
    if (rc != GG_OK) return rc;

    const cudaStream_t s = (cudaStream_t)stream;
    const Geom g{cas_vol_size, cas_img_size, mask_radius, kb_table_size, ker_hwidth};
    cudaError_t e = launch_fill(pd, V3, 0.0f, s);
    if (e == cudaSuccess) e = launch_fill(d_cas_volume_out, V3, 0.0f, s);
    if (e == cudaSuccess && n_axes > 0)
        e = launch_back_project_ref_density(d_cas_volume_out, pd, d_cas_images, kF32, d_kb_table, d_axes, n_axes, g,
                                            nullptr, s);
    // tmpCASVolume ./ (PlaneDensity + 1e-6) (MultiGPUGridder_Matlab_Class.m:308)
    if (e == cudaSuccess) e = launch_divide_plane_density(d_cas_volume_out, pd, V3, 1e-6f, s);
    if (e != cudaSuccess) {
        set_global_error(cudaGetErrorString(e));
        return GG_ERR_CUDA;
    }
    return GG_OK;
}
