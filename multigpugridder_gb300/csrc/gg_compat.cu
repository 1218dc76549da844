// The older C entry points bound by the reference's Python ctypes class
// (src/Python/MultiGPUGridder_Python.py:11-48; declared in include/gg_compat.h),
// over the stateless projection kernels of this library.  Host arrays are
// registered by pointer and read or written at Forward_Project / Back_Project,
// as the reference's AbstractGridder does with its HostMemory wrappers.
#include <cstring>
#include <string>
#include <vector>

#include "gg_internal.h"
#include "../../include/gg_compat.h"
#include "../../include/gg_gridder.h"

namespace {

struct CompatGridder {
    int n_gpus = 1, n_streams = 1;
    float *vol = nullptr;             // registered CAS volume V^3
    int V = 0;
    float *imgs = nullptr;            // registered CAS images n*M*M
    std::vector<float> own_imgs;      // Forward_Project output when none is registered
    float *axes = nullptr;            // registered directions
    int n_axes = 0;
    int M = 0;
    float mask_radius = -1.0f;        // < 0: M/2 - 1 (AbstractGridder.cpp:13)
    float *d_vol = nullptr, *d_imgs = nullptr, *d_axes = nullptr, *d_ker = nullptr;
    size_t cap_vol = 0, cap_imgs = 0, cap_axes = 0;
};

// Records the message for gg_global_error(); the old API has no status.
void *fail(const char *msg)
{
    gg::set_global_error(msg);
    return nullptr;
}

bool ensure(float *&p, size_t &cap, size_t count)
{
    if (count <= cap && p) return true;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    if (cudaMalloc(&p, count * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        fail("out of device memory");
        return false;
    }
    cap = count;
    return true;
}

// Uploads the volume (when `upload_vol`), the directions and the KB table.
bool stage(CompatGridder *g, bool upload_vol)
{
    const char *why = !g->vol || g->V <= 0 ? "SetVolume first"
                      : !g->axes || g->n_axes <= 0 ? "SetAxes first"
                      : g->M <= 0 ? "SetImgSize first" : nullptr;
    if (why) {
        fail(why);
        return false;
    }
    const size_t V3 = (size_t)g->V * g->V * g->V;
    if (!ensure(g->d_vol, g->cap_vol, V3) || !ensure(g->d_axes, g->cap_axes, (size_t)g->n_axes * 9) ||
        !ensure(g->d_imgs, g->cap_imgs, (size_t)g->n_axes * g->M * g->M))
        return false;
    if (!g->d_ker) {
        double t[501];
        gg_kb_table(2, 501, t);
        float tf[501];
        for (int i = 0; i < 501; i++) tf[i] = (float)t[i];
        if (cudaMalloc(&g->d_ker, sizeof(tf)) != cudaSuccess ||
            cudaMemcpy(g->d_ker, tf, sizeof(tf), cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaGetLastError();
            fail("could not stage the KB table");
            return false;
        }
    }
    if ((upload_vol && cudaMemcpy(g->d_vol, g->vol, V3 * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) ||
        cudaMemcpy(g->d_axes, g->axes, (size_t)g->n_axes * 9 * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        fail("host to device copy failed");
        return false;
    }
    return true;
}

int mask_radius(const CompatGridder *g)
{
    // RunKernel passes the mask radius as int (gpuForwardProject.h:57)
    return (int)(g->mask_radius >= 0.0f ? g->mask_radius : (float)g->M / 2.0f - 1.0f);
}

} // namespace

extern "C" void *Gridder_new(void) { return new CompatGridder(); }

extern "C" void Gridder_delete(void *p)
{
    auto *g = static_cast<CompatGridder *>(p);
    if (!g) return;
    cudaFree(g->d_vol);
    cudaFree(g->d_imgs);
    cudaFree(g->d_axes);
    cudaFree(g->d_ker);
    delete g;
}

extern "C" void *SetNumberGPUs(void *p, int n)
{
    if (p) static_cast<CompatGridder *>(p)->n_gpus = n;
    return nullptr;
}

extern "C" void *SetNumberStreams(void *p, int n)
{
    if (p) static_cast<CompatGridder *>(p)->n_streams = n;
    return nullptr;
}

extern "C" void *SetVolume(void *p, float *vol, int *size)
{
    auto *g = static_cast<CompatGridder *>(p);
    if (!g || !vol || !size) return fail("SetVolume: null argument");
    if (size[0] <= 0 || size[1] != size[0] || size[2] != size[0]) return fail("SetVolume: the volume must be a cube");
    g->vol = vol;
    g->V = size[0];
    return nullptr;
}

extern "C" float *GetVolume(void *p) { return p ? static_cast<CompatGridder *>(p)->vol : nullptr; }

extern "C" void *ResetVolume(void *p)
{
    auto *g = static_cast<CompatGridder *>(p);
    if (g && g->vol) std::memset(g->vol, 0, (size_t)g->V * g->V * g->V * sizeof(float));
    return nullptr;
}

extern "C" void *SetImages(void *p, float *imgs)
{
    if (p) static_cast<CompatGridder *>(p)->imgs = imgs;
    return nullptr;
}

extern "C" float *GetImages(void *p)
{
    auto *g = static_cast<CompatGridder *>(p);
    if (!g) return nullptr;
    return g->imgs ? g->imgs : (g->own_imgs.empty() ? nullptr : g->own_imgs.data());
}

extern "C" void *SetAxes(void *p, float *axes, int *size)
{
    auto *g = static_cast<CompatGridder *>(p);
    if (!g || !axes || !size) return fail("SetAxes: null argument");
    if (size[0] <= 0 || size[0] % 9) return fail("SetAxes: axesSize[0] must be 9 x the number of directions");
    g->axes = axes;
    g->n_axes = size[0] / 9;
    return nullptr;
}

extern "C" void *SetImgSize(void *p, int *size)
{
    auto *g = static_cast<CompatGridder *>(p);
    if (!g || !size || size[0] <= 0) return fail("SetImgSize: invalid size");
    g->M = size[0];
    return nullptr;
}

extern "C" void *SetMaskRadius(void *p, float *r)
{
    if (p && r) static_cast<CompatGridder *>(p)->mask_radius = *r;
    return nullptr;
}

extern "C" void *Forward_Project(void *p)
{
    auto *g = static_cast<CompatGridder *>(p);
    if (!g) return fail("null gridder");
    if (!stage(g, true)) return nullptr;
    if (gg_forward_project_kernel(g->d_vol, g->d_imgs, g->d_ker, g->d_axes, 2.0f, g->n_axes, g->V, g->M, 0,
                                  mask_radius(g), 501, nullptr) != GG_OK)
        return nullptr; // the message is in gg_global_error()
    const size_t count = (size_t)g->n_axes * g->M * g->M;
    float *out = g->imgs;
    if (!out) {
        g->own_imgs.resize(count);
        out = g->own_imgs.data();
    }
    if (cudaMemcpy(out, g->d_imgs, count * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        return fail("device to host copy failed");
    }
    return nullptr;
}

extern "C" void *Back_Project(void *p)
{
    auto *g = static_cast<CompatGridder *>(p);
    if (!g) return fail("null gridder");
    const float *imgs = g->imgs ? g->imgs : (g->own_imgs.empty() ? nullptr : g->own_imgs.data());
    if (!imgs) return fail("SetImages first");
    if (!stage(g, false)) return nullptr;
    const size_t V3 = (size_t)g->V * g->V * g->V, count = (size_t)g->n_axes * g->M * g->M;
    // the reference zeroes the CAS volume before each back projection (gpuGridder.cpp:332)
    if (cudaMemcpy(g->d_imgs, imgs, count * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(g->d_vol, 0, V3 * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        return fail("host to device copy failed");
    }
    if (gg_back_project_kernel(g->d_vol, g->d_imgs, g->d_ker, g->d_axes, 2.0f, g->n_axes, g->V, g->M, mask_radius(g),
                               501, 0, nullptr) != GG_OK)
        return nullptr;
    if (cudaMemcpy(g->vol, g->d_vol, V3 * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        return fail("device to host copy failed");
    }
    return nullptr;
}
