// Host engine and C ABI of the GB300 gridder (include/gg_gridder.h).
//
// One handle owns one GPU's state: the resident FP32 CAS volume (plus, with
// FP16/BF16 storage, the copy the forward projection reads: rows padded for
// aligned vector loads), the KB table and pre-compensation vector, batch buffers and
// cached cuFFT plans.  It replaces the reference's MultiGPUGridder /
// gpuGridder / AbstractGridder trio (src/Gridders/) for one device:
//   * the volume is prepared on the device once per setVolume instead of on
//     the host (CASFromVol_Gridder.m) and re-uploaded on every forward
//     projection (gpuGridder.cpp:194);
//   * directions are processed in batches of max_batch (SetMaxAxesToAllocate)
//     by one kernel launch each, with one batched cuFFT transform per batch
//     instead of one cuFFT call per image (gpuGridder.cpp:476-482);
//   * host transfers run on a copy stream, double-buffered against the
//     compute stream;
//   * back projection accumulates into one device volume on one compute
//     stream, so the per-GPU volume sum (MultiGPUGridder.cpp:376-411) is not
//     needed and no atomics are used.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "gg_internal.h"
#include "../../include/gg_gridder.h"

using namespace gg;

namespace {
std::atomic<long long> g_launches{0};
}

void gg::count_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

namespace {

thread_local std::string g_global_err;

struct GGError {
    int code;
    std::string msg;
};

[[noreturn]] void fail(int code, const char *fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    throw GGError{code, buf};
}

#define GG_CK(call)                                                                                         \
    do {                                                                                                    \
        cudaError_t _e = (call);                                                                            \
        if (_e != cudaSuccess)                                                                              \
            fail(_e == cudaErrorMemoryAllocation ? GG_ERR_OUT_OF_MEMORY : GG_ERR_CUDA, "%s failed: %s (%s:%d)", \
                 #call, cudaGetErrorString(_e), __FILE__, __LINE__);                                        \
    } while (0)

#define GG_CKF(call)                                                                              \
    do {                                                                                          \
        cufftResult _r = (call);                                                                  \
        if (_r != CUFFT_SUCCESS) fail(GG_ERR_CUFFT, "%s failed: cufft status %d", #call, (int)_r); \
    } while (0)

template <typename T> struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void ensure(size_t count)
    {
        if (count <= n && p) return;
        release();
        if (count == 0) return;
        void *q = nullptr;
        GG_CK(cudaMalloc(&q, count * sizeof(T)));
        p = (T *)q;
        n = count;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

struct PinBuf {
    float *p = nullptr;
    size_t n = 0;
    void ensure(size_t count)
    {
        if (count <= n && p) return;
        release();
        void *q = nullptr;
        GG_CK(cudaHostAlloc(&q, count * sizeof(float), cudaHostAllocDefault));
        p = (float *)q;
        n = count;
    }
    void release()
    {
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
    }
};

bool host_is_pinned(const void *ptr)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

} // namespace

struct gg_gridder {
    std::mutex mu;
    std::string err;
    int device = 0;
    int N = 0, M = 0, V = 0, pad = 0;
    float interp = 2.0f;
    int mask_radius = 0;
    int run_fft_on_device = 1;
    int verbose = 0;
    int max_batch = 1024;
    bool fused_fft = false;     // fft2_fused_ok(N, M): the 2-D FFT stages run as one kernel each
    int nstreams_fp = 2, nstreams_bp = 2;
    int prec = kF32;            // storage of the resident CAS volume the forward projection reads
    int img_prec_set = -1;      // storage of the CAS images the back projection reads; -1: as prec
    int bp_mode = GG_BP_REF;
    bool five_taps = false;
    int ker_size = 501;
    float ker_hw = 2.0f;

    DevBuf<float> ker;
    DevBuf<double> precomp;
    DevBuf<float> cas;       // FP32 CAS volume V^3 (resident)
    DevBuf<float> cas_fp;    // FP16/BF16 copy the forward projection reads: row pitch
                             // fp_pitch(V) (FP16 scaled by scales[0])
    DevBuf<float> cas_y, cas_z; // FP32: the CAS volume with y / z as the contiguous axis
    bool cas_fp_valid = false;  // cas_fp (FP16/BF16) or cas_y/cas_z (FP32) match cas
    DevBuf<float> pd;        // plane density V^3
    DevBuf<float> adj;       // CAS-volume gradient V^3 (forward-operator adjoint)
    DevBuf<float> axes;
    DevBuf<float> vol_io;    // N^3
    DevBuf<float> x3;        // M^3 real FFT input/output
    DevBuf<cufftComplex> spec3;
    DevBuf<float> scales;    // [0] CAS-volume storage scale, [1] CAS-image storage scale
    DevBuf<unsigned int> work;

    struct Slot {
        DevBuf<float> casimg, real, img;
        DevBuf<cufftComplex> spec;
        DevBuf<uint16_t> casimg_lp;
        DevBuf<int> order; // the forward projection's direction order (grouped by copy)
        PinBuf stage;
        cudaEvent_t ev_ready = nullptr, ev_free = nullptr;
    } slot[2];

    cudaStream_t cs = nullptr, cp = nullptr;
    cudaEvent_t ev_dev = nullptr; // end of the last *_dev call (serialises scratch use across streams)
    bool dev_pending = false;
    std::map<std::pair<int, int>, cufftHandle> plans2d;
    // profiling: events around projection-kernel launches
    struct ProfRec {
        cudaEvent_t a, b;
        int kind;
    };
    bool prof = false;
    std::vector<ProfRec> prof_recs;
    std::vector<cudaEvent_t> prof_pool;
    cufftHandle plan3_r2c = 0, plan3_c2r = 0;
    bool have3_r2c = false, have3_c2r = false;

    Geom geom() const { return Geom{V, M, mask_radius, ker_size, ker_hw}; }
    const float *vol_scale() const { return prec == kF16 ? scales.p : nullptr; }
    int img_prec() const { return img_prec_set < 0 ? prec : img_prec_set; }
    const float *img_scale() const { return img_prec() == kF16 ? scales.p + 1 : nullptr; }
};

namespace {

void set_device(gg_gridder *h) { GG_CK(cudaSetDevice(h->device)); }

cufftHandle plan2d(gg_gridder *h, cufftType type, int batch)
{
    auto key = std::make_pair((int)type, batch);
    auto it = h->plans2d.find(key);
    if (it != h->plans2d.end()) return it->second;
    if (h->plans2d.size() >= 6) { // keep a handful: full batch and remainders
        for (auto &kv : h->plans2d) cufftDestroy(kv.second);
        h->plans2d.clear();
    }
    cufftHandle p;
    int dims[2] = {h->M, h->M};
    GG_CKF(cufftPlanMany(&p, 2, dims, nullptr, 1, 0, nullptr, 1, 0, type, batch));
    h->plans2d[key] = p;
    return p;
}

cufftHandle plan3(gg_gridder *h, bool r2c)
{
    if (r2c) {
        if (!h->have3_r2c) {
            GG_CKF(cufftPlan3d(&h->plan3_r2c, h->M, h->M, h->M, CUFFT_R2C));
            h->have3_r2c = true;
        }
        return h->plan3_r2c;
    }
    if (!h->have3_c2r) {
        GG_CKF(cufftPlan3d(&h->plan3_c2r, h->M, h->M, h->M, CUFFT_C2R));
        h->have3_c2r = true;
    }
    return h->plan3_c2r;
}

void ensure_slot(gg_gridder *h, int s, int b, bool need_img)
{
    auto &sl = h->slot[s];
    const size_t MM = (size_t)h->M * h->M, NN = (size_t)h->N * h->N, H = (size_t)h->M * (h->M / 2 + 1);
    sl.casimg.ensure(MM * b);
    sl.real.ensure(MM * b);
    sl.spec.ensure(H * b);
    if (need_img) sl.img.ensure(NN * b);
    if (h->img_prec() != kF32) sl.casimg_lp.ensure(MM * b);
    sl.order.ensure(b);
    if (!sl.ev_ready) GG_CK(cudaEventCreateWithFlags(&sl.ev_ready, cudaEventDisableTiming));
    if (!sl.ev_free) {
        GG_CK(cudaEventCreateWithFlags(&sl.ev_free, cudaEventDisableTiming));
        GG_CK(cudaEventRecord(sl.ev_free, h->cp));
    }
}

void begin_dev(gg_gridder *h, cudaStream_t s)
{
    // the handle's scratch may still be in use by an earlier call on another stream
    if (h->dev_pending) GG_CK(cudaStreamWaitEvent(s, h->ev_dev, 0));
}

void end_dev(gg_gridder *h, cudaStream_t s)
{
    GG_CK(cudaEventRecord(h->ev_dev, s));
    h->dev_pending = true;
}

void require_volume(gg_gridder *h)
{
    if (!h->cas.p) fail(GG_ERR_STATE, "no volume: call gg_set_volume or gg_set_cas_volume first");
}

cudaEvent_t prof_event(gg_gridder *h)
{
    if (!h->prof_pool.empty()) {
        cudaEvent_t e = h->prof_pool.back();
        h->prof_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    GG_CK(cudaEventCreate(&e));
    return e;
}

// Brackets one projection-kernel launch with events when profiling is on.
struct ProfScope {
    gg_gridder *h;
    cudaStream_t s;
    int kind;
    cudaEvent_t a = nullptr;
    ProfScope(gg_gridder *h_, cudaStream_t s_, int kind_) : h(h_), s(s_), kind(kind_)
    {
        if (h->prof) {
            a = prof_event(h);
            GG_CK(cudaEventRecord(a, s));
        }
    }
    void done()
    {
        if (!a) return;
        cudaEvent_t b = prof_event(h);
        GG_CK(cudaEventRecord(b, s));
        h->prof_recs.push_back({a, b, kind});
        a = nullptr;
    }
};

void check_axes_count(int n)
{
    if (n < 0) fail(GG_ERR_INVALID_ARG, "n_axes must be >= 0 (got %d)", n);
}

// Floats taken by one pitched 2-byte copy of the CAS volume (a multiple of 4,
// so each copy starts 16-byte aligned).
size_t fp_copy_floats(const gg_gridder *h)
{
    return ((size_t)fp_pitch(h->V) * h->V * h->V * prec_bytes(h->prec) + 15) / 16 * 4;
}

// Refresh the copies of the CAS volume read by the forward projection.
void update_fp(gg_gridder *h, cudaStream_t s)
{
    if (h->cas_fp_valid) return;
    if (h->prec == kF32) {
        // FP32 taps are read one by one: the dense volume and its two transposes
        const size_t V3 = (size_t)h->V * h->V * h->V;
        h->cas_y.ensure(V3);
        h->cas_z.ensure(V3);
        GG_CK(launch_transpose_volume(h->cas.p, h->V, h->cas_y.p, 1, s));
        GG_CK(launch_transpose_volume(h->cas.p, h->V, h->cas_z.p, 2, s));
        h->cas_fp_valid = true;
        return;
    }
    // FP16/BF16: three pitched copies with x, y and z contiguous, back to back
    const size_t V3 = (size_t)h->V * h->V * h->V;
    h->cas_fp.ensure(3 * fp_copy_floats(h));
    if (h->prec == kF16) GG_CK(launch_storage_scale(h->cas.p, V3, 8192.0f, h->work.p, h->scales.p, s));
    for (int l = 0; l < 3; l++)
        GG_CK(launch_pitch_volume(h->cas.p, h->V, fp_pitch(h->V), h->cas_fp.p + l * fp_copy_floats(h), h->prec,
                                  h->vol_scale(), s, l));
    h->cas_fp_valid = true;
}

// ---- device-side pipelines (all on stream s) --------------------------------

void do_set_volume(gg_gridder *h, const float *d_vol, cudaStream_t s)
{
    const size_t V3 = (size_t)h->V * h->V * h->V;
    const size_t M3 = (size_t)h->M * h->M * h->M;
    h->cas.ensure(V3);
    h->x3.ensure(M3);
    h->spec3.ensure((size_t)h->M * h->M * (h->M / 2 + 1));
    GG_CK(launch_vol_to_fft_input(d_vol, h->N, h->M, h->precomp.p, h->x3.p, s));
    cufftHandle p = plan3(h, true);
    GG_CKF(cufftSetStream(p, s));
    GG_CKF(cufftExecR2C(p, h->x3.p, h->spec3.p));
    GG_CK(launch_spectrum_to_cas_volume(h->spec3.p, h->M, h->V, h->cas.p, kF32, nullptr, s));
    h->cas_fp_valid = false;
}

void do_get_volume(gg_gridder *h, const float *d_cas, float *d_vol, cudaStream_t s)
{
    const size_t M3 = (size_t)h->M * h->M * h->M;
    h->x3.ensure(M3);
    h->spec3.ensure((size_t)h->M * h->M * (h->M / 2 + 1));
    GG_CK(launch_cas_volume_to_spectrum(d_cas, h->V, h->M, h->spec3.p, s));
    cufftHandle p = plan3(h, false);
    GG_CKF(cufftSetStream(p, s));
    GG_CKF(cufftExecC2R(p, h->spec3.p, h->x3.p));
    GG_CK(launch_fft_output_to_vol(h->x3.p, h->M, h->N, h->precomp.p, d_vol, s));
}

// Forward-project directions [a0, a0+b) of d_axes into slot `sl`:
// CAS images -> cas_out (device, may be the slot buffer), images -> img_out.
void fp_batch(gg_gridder *h, const float *d_axes, int b, float *cas_out, float *img_out, int sl, cudaStream_t s)
{
    auto &S = h->slot[sl];
    ProfScope ps(h, s, GG_KERNEL_FORWARD);
    const bool dense = h->prec == kF32;
    GG_CK(launch_forward_project(dense ? h->cas.p : h->cas_fp.p, h->prec, dense ? h->V : fp_pitch(h->V), cas_out,
                                 h->ker.p, d_axes, b, h->geom(), h->five_taps, h->vol_scale(), s,
                                 dense ? (const void *)h->cas_y.p : (const void *)(h->cas_fp.p + fp_copy_floats(h)),
                                 dense ? (const void *)h->cas_z.p : (const void *)(h->cas_fp.p + 2 * fp_copy_floats(h)),
                                 S.order.p));
    ps.done();
    if (img_out && h->fused_fft) {
        GG_CK(launch_cas_to_images_fused(cas_out, h->M, h->N, b, img_out, s));
    } else if (img_out) {
        GG_CK(launch_cas_images_to_spectrum(cas_out, h->M, b, S.spec.p, s));
        cufftHandle p = plan2d(h, CUFFT_C2R, b);
        GG_CKF(cufftSetStream(p, s));
        GG_CKF(cufftExecC2R(p, S.spec.p, S.real.p));
        GG_CK(launch_fft_output_to_images(S.real.p, h->M, h->N, b, img_out, s));
    }
}

// Back-project b directions: images (device, FFT path) or CAS images (device).
// With `pd`, the plane density of the same directions is accumulated into pd
// as well (fused into the same kernel for the reference rule).
void bp_batch(gg_gridder *h, const float *d_axes, int b, const float *img, const float *casimg, float *target, bool ones,
              int sl, cudaStream_t s, float *pd = nullptr)
{
    auto &S = h->slot[sl];
    const void *src = nullptr;
    const int ip = h->img_prec(); // storage of the CAS images read here
    int iprec = ip;
    const float *scale = nullptr;
    if (!ones) {
        const size_t MM = (size_t)h->M * h->M;
        if (casimg) {
            if (ip == kF32) {
                src = casimg;
            } else {
                if (ip == kF16) GG_CK(launch_storage_scale(casimg, MM * b, 8192.0f, h->work.p, h->scales.p + 1, s));
                GG_CK(launch_convert(casimg, S.casimg_lp.p, ip, MM * b, h->img_scale(), s));
                src = S.casimg_lp.p;
                scale = h->img_scale();
            }
        } else if (h->fused_fft && ip != kF16) {
            void *dst = ip == kF32 ? (void *)S.casimg.p : (void *)S.casimg_lp.p;
            GG_CK(launch_images_to_cas_fused(img, h->N, h->M, b, dst, ip, false, s));
            src = dst;
        } else if (h->fused_fft) {
            // FP16: FP32 CAS images first, then the storage scale from their
            // largest magnitude and the conversion
            GG_CK(launch_images_to_cas_fused(img, h->N, h->M, b, S.casimg.p, kF32, false, s));
            GG_CK(launch_storage_scale(S.casimg.p, MM * b, 8192.0f, h->work.p, h->scales.p + 1, s));
            GG_CK(launch_convert(S.casimg.p, S.casimg_lp.p, ip, MM * b, h->img_scale(), s));
            src = S.casimg_lp.p;
            scale = h->img_scale();
        } else {
            GG_CK(launch_images_to_fft_input(img, h->N, h->M, b, S.real.p, s));
            cufftHandle p = plan2d(h, CUFFT_R2C, b);
            GG_CKF(cufftSetStream(p, s));
            GG_CKF(cufftExecR2C(p, S.real.p, S.spec.p));
            if (ip == kF16)
                // |Re + Im| <= 2 max(|Re|, |Im|)
                GG_CK(launch_storage_scale((const float *)S.spec.p, (size_t)h->M * (h->M / 2 + 1) * 2 * b, 4096.0f,
                                           h->work.p, h->scales.p + 1, s));
            void *dst = ip == kF32 ? (void *)S.casimg.p : (void *)S.casimg_lp.p;
            GG_CK(launch_spectrum_to_cas_images(S.spec.p, h->M, b, dst, ip, h->img_scale(), s));
            src = dst;
            scale = h->img_scale();
        }
    }
    if (ones) iprec = kF32;
    ProfScope ps(h, s, ones ? GG_KERNEL_DENSITY : GG_KERNEL_BACK);
    if (h->bp_mode == GG_BP_ADJOINT && !ones) {
        GG_CK(launch_back_project_adjoint(target, src, iprec, h->ker.p, d_axes, b, h->geom(), scale, !h->five_taps, s));
    } else if (pd && !ones) {
        GG_CK(launch_back_project_ref_density(target, pd, src, iprec, h->ker.p, d_axes, b, h->geom(), scale, s));
        pd = nullptr;
    } else {
        GG_CK(launch_back_project_ref(target, src, iprec, ones, h->ker.p, d_axes, b, h->geom(), scale, s));
    }
    ps.done();
    if (pd) {
        // adjoint rule: the plane density is the adjoint applied to all-ones CAS images
        const size_t MM = (size_t)h->M * h->M;
        ProfScope pd_ps(h, s, GG_KERNEL_DENSITY);
        GG_CK(launch_fill(S.casimg.p, MM * b, 1.0f, s));
        GG_CK(launch_back_project_adjoint(pd, S.casimg.p, kF32, h->ker.p, d_axes, b, h->geom(), nullptr, !h->five_taps, s));
        pd_ps.done();
    }
}

// One batch of the CTF-corrected reconstruction: the images' CAS images times
// the CTF are back-projected into h->cas, and CTF^2 images into h->pd (the
// CTF-weighted plane density), both by the gridder's back-projection rule.
void ctf_batch(gg_gridder *h, const float *d_axes, int b, const float *img, const float *d_defocus,
               const float *d_defocus_v, const float *d_astig, const CtfParams &c, int sl, cudaStream_t s)
{
    auto &S = h->slot[sl];
    if (h->fused_fft) {
        GG_CK(launch_images_to_cas_fused(img, h->N, h->M, b, S.casimg.p, kF32, false, s));
    } else {
        GG_CK(launch_images_to_fft_input(img, h->N, h->M, b, S.real.p, s));
        cufftHandle p = plan2d(h, CUFFT_R2C, b);
        GG_CKF(cufftSetStream(p, s));
        GG_CKF(cufftExecR2C(p, S.real.p, S.spec.p));
        GG_CK(launch_spectrum_to_cas_images(S.spec.p, h->M, b, S.casimg.p, kF32, nullptr, s));
    }
    // CAS images *= CTF, and CTF^2 into S.real (free after the R2C), in one pass
    GG_CK(launch_ctf(S.casimg.p, 1, S.real.p, 2, h->M, b, d_defocus, d_defocus_v, d_astig, c, s));
    if (h->img_prec() == kF32 && h->bp_mode != GG_BP_ADJOINT) {
        // both stacks in one back-projection pass
        ProfScope ps(h, s, GG_KERNEL_BACK);
        GG_CK(launch_back_project_ref_pair(h->cas.p, h->pd.p, S.casimg.p, S.real.p, h->ker.p, d_axes, b, h->geom(), s));
        ps.done();
    } else {
        bp_batch(h, d_axes, b, nullptr, S.casimg.p, h->cas.p, false, sl, s);
        bp_batch(h, d_axes, b, nullptr, S.real.p, h->pd.p, false, sl, s);
    }
}

void check_ctf(const CtfParams &c)
{
    if (!(c.voltage_kv > 0.0f) || !(c.pixel_size > 0.0f) || !(c.amp_contrast >= 0.0f && c.amp_contrast <= 1.0f) ||
        !std::isfinite(c.cs_mm) || !std::isfinite(c.voltage_kv) || !std::isfinite(c.pixel_size))
        fail(GG_ERR_INVALID_ARG, "CTF needs voltage > 0, pixel size > 0, 0 <= amplitude contrast <= 1, finite Cs");
}

// Exact adjoint of (CAS preparation + forward projection + CAS images ->
// images): image gradients (device, n*N*N) -> volume gradient (device, N^3).
void forward_adjoint(gg_gridder *h, const float *d_axes, int n, const float *d_img_grad, float *d_vol_grad, cudaStream_t s)
{
    const size_t V3 = (size_t)h->V * h->V * h->V, NN = (size_t)h->N * h->N;
    h->adj.ensure(V3);
    GG_CK(cudaMemsetAsync(h->adj.p, 0, V3 * sizeof(float), s));
    const int B = h->max_batch;
    for (int a0 = 0; a0 < n; a0 += B) {
        const int b = std::min(B, n - a0);
        ensure_slot(h, 0, B, false);
        auto &S = h->slot[0];
        if (h->fused_fft) {
            GG_CK(launch_images_to_cas_fused(d_img_grad + (size_t)a0 * NN, h->N, h->M, b, S.casimg.p, kF32, true, s));
        } else {
            GG_CK(launch_images_to_fft_input(d_img_grad + (size_t)a0 * NN, h->N, h->M, b, S.real.p, s));
            cufftHandle p = plan2d(h, CUFFT_R2C, b);
            GG_CKF(cufftSetStream(p, s));
            GG_CKF(cufftExecR2C(p, S.real.p, S.spec.p));
            GG_CK(launch_spectrum_to_cas_images_adjoint(S.spec.p, h->M, b, S.casimg.p, s));
        }
        ProfScope ps(h, s, GG_KERNEL_BACK);
        GG_CK(launch_back_project_adjoint(h->adj.p, S.casimg.p, kF32, h->ker.p, d_axes + (size_t)a0 * 9, b, h->geom(),
                                          nullptr, !h->five_taps, s));
        ps.done();
    }
    const size_t M3 = (size_t)h->M * h->M * h->M;
    h->x3.ensure(M3);
    h->spec3.ensure((size_t)h->M * h->M * (h->M / 2 + 1));
    GG_CK(launch_cas_volume_adjoint_input(h->adj.p, h->V, h->M, h->x3.p, s));
    cufftHandle p = plan3(h, true);
    GG_CKF(cufftSetStream(p, s));
    GG_CKF(cufftExecR2C(p, h->x3.p, h->spec3.p));
    GG_CK(launch_spectrum_to_vol_adjoint(h->spec3.p, h->M, h->N, h->precomp.p, d_vol_grad, s));
}

void upload_axes(gg_gridder *h, const float *axes, int n, cudaStream_t s)
{
    h->axes.ensure((size_t)(n > 0 ? n : 1) * 9);
    if (n > 0) GG_CK(cudaMemcpyAsync(h->axes.p, axes, (size_t)n * 9 * sizeof(float), cudaMemcpyHostToDevice, s));
}

// ---- host pipelines -----------------------------------------------------------

// Forward projection with host outputs, double-buffered: batch c computes in
// slot c&1 on the compute stream while batch c-1 is copied out on the copy
// stream (through pinned staging when the destination is pageable).
void fp_host(gg_gridder *h, const float *axes, int n, float *images_out, float *cas_out)
{
    cudaStream_t cs = h->cs, cp = h->cp;
    upload_axes(h, axes, n, cs);
    update_fp(h, cs);
    const int B = h->max_batch;
    const size_t MM = (size_t)h->M * h->M, NN = (size_t)h->N * h->N;
    const bool pin_img = images_out && host_is_pinned(images_out);
    const bool pin_cas = cas_out && host_is_pinned(cas_out);
    const int nb = (n + B - 1) / B;
    struct Pending {
        int a0 = 0, b = 0;
        bool live = false;
    } pend[2];
    auto drain = [&](int sl) {
        Pending &p = pend[sl];
        if (!p.live) return;
        auto &S = h->slot[sl];
        GG_CK(cudaEventSynchronize(S.ev_free));
        size_t off = 0;
        if (cas_out && !pin_cas) {
            memcpy(cas_out + (size_t)p.a0 * MM, S.stage.p, (size_t)p.b * MM * sizeof(float));
            off = (size_t)p.b * MM;
        }
        if (images_out && !pin_img) memcpy(images_out + (size_t)p.a0 * NN, S.stage.p + off, (size_t)p.b * NN * sizeof(float));
        p.live = false;
    };
    for (int c = 0; c < nb; c++) {
        const int sl = c & 1, a0 = c * B, b = std::min(B, n - a0);
        auto &S = h->slot[sl];
        ensure_slot(h, sl, B, images_out != nullptr);
        drain(sl); // host copy-out of batch c-2 from this slot's staging
        GG_CK(cudaStreamWaitEvent(cs, S.ev_free, 0));
        fp_batch(h, h->axes.p + (size_t)a0 * 9, b, S.casimg.p, images_out ? S.img.p : nullptr, sl, cs);
        GG_CK(cudaEventRecord(S.ev_ready, cs));
        GG_CK(cudaStreamWaitEvent(cp, S.ev_ready, 0));
        size_t stage_need = 0;
        if (cas_out && !pin_cas) stage_need += (size_t)b * MM;
        if (images_out && !pin_img) stage_need += (size_t)b * NN;
        if (stage_need) S.stage.ensure(stage_need);
        size_t off = 0;
        if (cas_out) {
            float *dst = pin_cas ? cas_out + (size_t)a0 * MM : S.stage.p;
            GG_CK(cudaMemcpyAsync(dst, S.casimg.p, (size_t)b * MM * sizeof(float), cudaMemcpyDeviceToHost, cp));
            if (!pin_cas) off = (size_t)b * MM;
        }
        if (images_out) {
            float *dst = pin_img ? images_out + (size_t)a0 * NN : S.stage.p + off;
            GG_CK(cudaMemcpyAsync(dst, S.img.p, (size_t)b * NN * sizeof(float), cudaMemcpyDeviceToHost, cp));
        }
        GG_CK(cudaEventRecord(S.ev_free, cp));
        pend[sl] = Pending{a0, b, stage_need > 0};
    }
    drain(0);
    drain(1);
    GG_CK(cudaStreamSynchronize(cp));
    GG_CK(cudaStreamSynchronize(cs));
}

// Back projection with host inputs: batch c is copied in on the copy stream
// (staged when pageable) while batch c-1 is transformed and back-projected.
// Host input pipeline, double-buffered: batch c's inputs (b * per floats from
// `src`) are copied into slot c&1 on the copy stream (through pinned staging
// when `src` is pageable) while batch c-1 computes; compute(a0, b, sl, dbuf)
// then enqueues the batch's work on the compute stream.  src = NULL uploads
// nothing.  casimg_slot: the inputs land in the slot's CAS-image buffer
// instead of its image buffer.
template <typename F>
void host_batches(gg_gridder *h, int n, const float *src, size_t per, bool casimg_slot, F compute)
{
    cudaStream_t cs = h->cs, cp = h->cp;
    const int B = h->max_batch;
    const bool pinned = src && host_is_pinned(src);
    const int nb = (n + B - 1) / B;
    for (int c = 0; c < nb; c++) {
        const int sl = c & 1, a0 = c * B, b = std::min(B, n - a0);
        auto &S = h->slot[sl];
        ensure_slot(h, sl, B, true);
        float *dbuf = casimg_slot ? S.casimg.p : S.img.p;
        if (src) {
            // the slot's buffers are free once its previous batch finished computing
            GG_CK(cudaStreamWaitEvent(cp, S.ev_ready, 0));
            const float *hsrc = src + (size_t)a0 * per;
            if (!pinned) {
                S.stage.ensure((size_t)b * per);
                GG_CK(cudaEventSynchronize(S.ev_free)); // staging no longer read by an earlier copy
                memcpy(S.stage.p, hsrc, (size_t)b * per * sizeof(float));
                hsrc = S.stage.p;
            }
            GG_CK(cudaMemcpyAsync(dbuf, hsrc, (size_t)b * per * sizeof(float), cudaMemcpyHostToDevice, cp));
            GG_CK(cudaEventRecord(S.ev_free, cp));
            GG_CK(cudaStreamWaitEvent(cs, S.ev_free, 0));
        }
        compute(a0, b, sl, dbuf);
        GG_CK(cudaEventRecord(S.ev_ready, cs));
    }
    GG_CK(cudaStreamSynchronize(cs));
    GG_CK(cudaStreamSynchronize(cp));
}

void bp_host(gg_gridder *h, const float *axes, int n, const float *images, const float *casimgs, float *target,
             bool ones, float *pd = nullptr)
{
    upload_axes(h, axes, n, h->cs);
    const size_t MM = (size_t)h->M * h->M, NN = (size_t)h->N * h->N;
    const float *src = ones ? nullptr : (casimgs ? casimgs : images);
    host_batches(h, n, src, casimgs ? MM : NN, casimgs != nullptr, [&](int a0, int b, int sl, float *dbuf) {
        bp_batch(h, h->axes.p + (size_t)a0 * 9, b, casimgs ? nullptr : dbuf, casimgs ? dbuf : nullptr, target, ones,
                 sl, h->cs, pd);
    });
}

void init_handle(gg_gridder *h)
{
    set_device(h);
    GG_CK(cudaStreamCreateWithFlags(&h->cs, cudaStreamNonBlocking));
    GG_CK(cudaStreamCreateWithFlags(&h->cp, cudaStreamNonBlocking));
    GG_CK(cudaEventCreateWithFlags(&h->ev_dev, cudaEventDisableTiming));
    std::vector<double> t(h->ker_size), pc(h->M);
    kb_table_f64((int)h->ker_hw, h->ker_size, t.data());
    std::vector<float> tf(h->ker_size);
    for (int i = 0; i < h->ker_size; i++) tf[i] = (float)t[i];
    h->ker.ensure(h->ker_size);
    GG_CK(cudaMemcpy(h->ker.p, tf.data(), tf.size() * sizeof(float), cudaMemcpyHostToDevice));
    h->five_taps = !(tf[0] == 0.0f && tf[h->ker_size - 1] == 0.0f);
    precomp_f64(h->M, (int)h->ker_hw, pc.data());
    h->precomp.ensure(h->M);
    GG_CK(cudaMemcpy(h->precomp.p, pc.data(), pc.size() * sizeof(double), cudaMemcpyHostToDevice));
    h->scales.ensure(2);
    const float ones[2] = {1.0f, 1.0f};
    GG_CK(cudaMemcpy(h->scales.p, ones, sizeof(ones), cudaMemcpyHostToDevice));
    h->work.ensure(1);
    GG_CK(cudaMemset(h->work.p, 0, sizeof(unsigned int)));
    h->fused_fft = fft2_fused_ok(h->N, h->M);
}

void destroy_handle(gg_gridder *h)
{
    cudaSetDevice(h->device);
    if (h->cs) cudaStreamSynchronize(h->cs);
    if (h->cp) cudaStreamSynchronize(h->cp);
    for (auto &kv : h->plans2d) cufftDestroy(kv.second);
    if (h->have3_r2c) cufftDestroy(h->plan3_r2c);
    if (h->have3_c2r) cufftDestroy(h->plan3_c2r);
    for (auto &S : h->slot) {
        S.casimg.release();
        S.real.release();
        S.img.release();
        S.spec.release();
        S.casimg_lp.release();
        S.stage.release();
        if (S.ev_ready) cudaEventDestroy(S.ev_ready);
        if (S.ev_free) cudaEventDestroy(S.ev_free);
    }
    h->ker.release();
    h->precomp.release();
    h->cas.release();
    h->cas_fp.release();
    h->cas_y.release();
    h->cas_z.release();
    h->pd.release();
    h->adj.release();
    h->axes.release();
    h->vol_io.release();
    h->x3.release();
    h->spec3.release();
    h->scales.release();
    h->work.release();
    for (auto &r : h->prof_recs) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    for (auto e : h->prof_pool) cudaEventDestroy(e);
    if (h->ev_dev) cudaEventDestroy(h->ev_dev);
    if (h->cs) cudaStreamDestroy(h->cs);
    if (h->cp) cudaStreamDestroy(h->cp);
}

template <typename F> int guarded(gg_gridder *h, F &&f)
{
    if (!h) {
        g_global_err = "null gridder handle";
        return GG_ERR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lk(h->mu);
    try {
        set_device(h);
        f();
        h->err.clear();
        return GG_OK;
    } catch (const GGError &e) {
        h->err = e.msg;
        if (h->verbose) fprintf(stderr, "gg_gridder: %s\n", e.msg.c_str());
        return e.code;
    } catch (const std::bad_alloc &) {
        h->err = "host allocation failed";
        return GG_ERR_OUT_OF_MEMORY;
    }
}

template <typename F> int guarded_global(F &&f)
{
    try {
        f();
        return GG_OK;
    } catch (const GGError &e) {
        g_global_err = e.msg;
        return e.code;
    }
}

void check_cube(const int *dims, int want, const char *what)
{
    if (!dims) fail(GG_ERR_INVALID_ARG, "%s dims is NULL", what);
    if (dims[0] != want || dims[1] != want || dims[2] != want)
        fail(GG_ERR_INVALID_ARG, "%s must be %d^3 (got %dx%dx%d)", what, want, dims[0], dims[1], dims[2]);
}

} // namespace

// =============================================================================
// C ABI
// =============================================================================

extern "C" int gg_version(void) { return GG_ABI_VERSION; }

extern "C" const char *gg_global_error(void) { return g_global_err.c_str(); }

void gg::set_global_error(const char *msg) { g_global_err = msg; }

extern "C" const char *gg_last_error(const gg_gridder *h) { return h ? h->err.c_str() : "null gridder handle"; }

extern "C" int gg_create(int volume_size, int num_coord_axes, float interp_factor, int extra_padding, int num_gpus,
                         const int *gpu_devices, int run_fft_on_device, int verbose, gg_gridder **out)
{
    if (!out) {
        g_global_err = "out is NULL";
        return GG_ERR_INVALID_ARG;
    }
    *out = nullptr;
    gg_gridder *h = nullptr;
    int rc = guarded_global([&] {
        if (volume_size <= 0 || (volume_size & 1)) fail(GG_ERR_INVALID_ARG, "VolumeSize must be a positive even number (got %d)", volume_size);
        if (!(interp_factor > 0.0f)) fail(GG_ERR_INVALID_ARG, "interpFactor must be positive (got %g)", (double)interp_factor);
        if (extra_padding < 0) fail(GG_ERR_INVALID_ARG, "extraPadding must be >= 0 (got %d)", extra_padding);
        if (num_coord_axes < 0) fail(GG_ERR_INVALID_ARG, "numCoordAxes must be >= 0 (got %d)", num_coord_axes);
        int ndev = 0;
        cudaError_t e = cudaGetDeviceCount(&ndev);
        if (e != cudaSuccess || ndev <= 0) {
            cudaGetLastError();
            fail(GG_ERR_NO_DEVICE, "no CUDA device available");
        }
        if (num_gpus <= 0 || num_gpus > ndev)
            fail(GG_ERR_INVALID_ARG, "Num_GPUs must be between 1 and %d (got %d)", ndev, num_gpus);
        const int dev = gpu_devices ? gpu_devices[0] : 0;
        if (dev < 0 || dev >= ndev) fail(GG_ERR_INVALID_ARG, "GPU device %d out of range [0, %d)", dev, ndev);
        // interp*N must be an even integer (MATLAB computes interpSize = N*interpFactor)
        const double Md = (double)volume_size * (double)interp_factor;
        const int M = (int)(Md + 0.5);
        if (std::fabs(Md - M) > 1e-3 * Md || M < volume_size || (M & 1))
            fail(GG_ERR_INVALID_ARG, "VolumeSize*interpFactor must be an even integer >= VolumeSize (got %g)", Md);
        h = new gg_gridder();
        h->device = dev;
        h->N = volume_size;
        h->M = M;
        h->pad = extra_padding;
        h->V = M + 2 * extra_padding;
        h->interp = interp_factor;
        // maskRadius = VolumeSize*interpFactor/2 - 1 (AbstractGridder.cpp:13), int at RunKernel
        h->mask_radius = (int)(((float)volume_size * interp_factor) / 2.0f - 1.0f);
        h->run_fft_on_device = run_fft_on_device;
        h->verbose = verbose;
        if (num_coord_axes > 0 && num_coord_axes < h->max_batch) h->max_batch = std::max(1, num_coord_axes);
        try {
            init_handle(h);
        } catch (...) {
            destroy_handle(h);
            delete h;
            h = nullptr;
            throw;
        }
    });
    if (rc == GG_OK) *out = h;
    return rc;
}

extern "C" void gg_destroy(gg_gridder *h)
{
    if (!h) return;
    {
        std::lock_guard<std::mutex> lk(h->mu);
        destroy_handle(h);
    }
    delete h;
}

extern "C" int gg_get_sizes(const gg_gridder *h, int *N, int *M, int *V, int *mask_radius)
{
    if (!h) return GG_ERR_INVALID_ARG;
    if (N) *N = h->N;
    if (M) *M = h->M;
    if (V) *V = h->V;
    if (mask_radius) *mask_radius = h->mask_radius;
    return GG_OK;
}

extern "C" int gg_set_kb_table(gg_gridder *h, const float *table, int n)
{
    return guarded(h, [&] {
        if (!table || n < 3 || n > kMaxKerSizeHost) fail(GG_ERR_INVALID_ARG, "KB table length must be in [3, %d] (got %d)", kMaxKerSizeHost, n);
        GG_CK(cudaStreamSynchronize(h->cs));
        h->ker.release();
        h->ker.ensure(n);
        GG_CK(cudaMemcpy(h->ker.p, table, (size_t)n * sizeof(float), cudaMemcpyHostToDevice));
        h->ker_size = n;
        h->five_taps = !(table[0] == 0.0f && table[n - 1] == 0.0f);
    });
}

extern "C" int gg_set_mask_radius(gg_gridder *h, float radius)
{
    return guarded(h, [&] {
        const int r = (int)radius;
        // radii past M/2 - 1 sample the padding; the kernels bound every read
        if (r < 0 || r > h->M) fail(GG_ERR_INVALID_ARG, "mask radius must be in [0, %d] (got %g)", h->M, (double)radius);
        h->mask_radius = r;
    });
}

extern "C" int gg_set_max_axes_to_allocate(gg_gridder *h, int max_axes)
{
    return guarded(h, [&] {
        if (max_axes <= 0) fail(GG_ERR_INVALID_ARG, "MaxAxesToAllocate must be positive (got %d)", max_axes);
        h->max_batch = max_axes;
    });
}

extern "C" int gg_set_num_streams_fp(gg_gridder *h, int n)
{
    return guarded(h, [&] {
        if (n <= 0) fail(GG_ERR_INVALID_ARG, "number of streams must be positive (got %d)", n);
        h->nstreams_fp = n;
    });
}

extern "C" int gg_set_num_streams_bp(gg_gridder *h, int n)
{
    return guarded(h, [&] {
        if (n <= 0) fail(GG_ERR_INVALID_ARG, "number of streams must be positive (got %d)", n);
        h->nstreams_bp = n;
    });
}

extern "C" int gg_set_precision(gg_gridder *h, int precision)
{
    return guarded(h, [&] {
        if (precision != GG_PREC_F32 && precision != GG_PREC_F16 && precision != GG_PREC_BF16)
            fail(GG_ERR_INVALID_ARG, "unknown precision %d", precision);
        if (precision != h->prec) {
            GG_CK(cudaStreamSynchronize(h->cs));
            h->prec = precision;
            h->cas_fp_valid = false;
            for (auto &S : h->slot) S.casimg_lp.release();
        }
    });
}

extern "C" int gg_set_image_precision(gg_gridder *h, int precision)
{
    return guarded(h, [&] {
        if (precision != -1 && precision != GG_PREC_F32 && precision != GG_PREC_F16 && precision != GG_PREC_BF16)
            fail(GG_ERR_INVALID_ARG, "unknown image precision %d", precision);
        if (precision != h->img_prec_set) {
            GG_CK(cudaStreamSynchronize(h->cs));
            h->img_prec_set = precision;
            for (auto &S : h->slot) S.casimg_lp.release();
        }
    });
}

extern "C" int gg_set_bp_mode(gg_gridder *h, int mode)
{
    return guarded(h, [&] {
        if (mode != GG_BP_REF && mode != GG_BP_ADJOINT) fail(GG_ERR_INVALID_ARG, "unknown back-projection mode %d", mode);
        if (mode == GG_BP_ADJOINT && h->five_taps)
            fail(GG_ERR_STATE, "the adjoint back projection needs a KB table with zero edge values");
        h->bp_mode = mode;
    });
}

extern "C" int gg_set_volume(gg_gridder *h, const float *volume, const int dims[3])
{
    return guarded(h, [&] {
        if (!volume) fail(GG_ERR_INVALID_ARG, "volume is NULL");
        check_cube(dims, h->N, "volume");
        const size_t N3 = (size_t)h->N * h->N * h->N;
        h->vol_io.ensure(N3);
        GG_CK(cudaMemcpyAsync(h->vol_io.p, volume, N3 * sizeof(float), cudaMemcpyHostToDevice, h->cs));
        do_set_volume(h, h->vol_io.p, h->cs);
        GG_CK(cudaStreamSynchronize(h->cs));
    });
}

extern "C" int gg_set_cas_volume(gg_gridder *h, const float *cas_volume, const int dims[3])
{
    return guarded(h, [&] {
        if (!cas_volume) fail(GG_ERR_INVALID_ARG, "cas_volume is NULL");
        check_cube(dims, h->V, "CAS volume");
        const size_t V3 = (size_t)h->V * h->V * h->V;
        h->cas.ensure(V3);
        GG_CK(cudaMemcpyAsync(h->cas.p, cas_volume, V3 * sizeof(float), cudaMemcpyHostToDevice, h->cs));
        GG_CK(cudaStreamSynchronize(h->cs));
        h->cas_fp_valid = false;
    });
}

extern "C" int gg_get_cas_volume(gg_gridder *h, float *out)
{
    return guarded(h, [&] {
        if (!out) fail(GG_ERR_INVALID_ARG, "output is NULL");
        require_volume(h);
        const size_t V3 = (size_t)h->V * h->V * h->V;
        GG_CK(cudaMemcpyAsync(out, h->cas.p, V3 * sizeof(float), cudaMemcpyDeviceToHost, h->cs));
        GG_CK(cudaStreamSynchronize(h->cs));
    });
}

extern "C" int gg_reset_volume(gg_gridder *h)
{
    return guarded(h, [&] {
        const size_t V3 = (size_t)h->V * h->V * h->V;
        h->cas.ensure(V3);
        GG_CK(cudaMemsetAsync(h->cas.p, 0, V3 * sizeof(float), h->cs));
        GG_CK(cudaStreamSynchronize(h->cs));
        h->cas_fp_valid = false;
    });
}

extern "C" int gg_forward_project(gg_gridder *h, const float *axes, int n_axes, float *images_out, float *cas_images_out)
{
    return guarded(h, [&] {
        check_axes_count(n_axes);
        if (n_axes > 0 && !axes) fail(GG_ERR_INVALID_ARG, "axes is NULL");
        if (!images_out && !cas_images_out) fail(GG_ERR_INVALID_ARG, "no output requested");
        require_volume(h);
        if (n_axes == 0) return;
        fp_host(h, axes, n_axes, images_out, cas_images_out);
    });
}

extern "C" int gg_back_project(gg_gridder *h, const float *axes, int n_axes, const float *images, const float *cas_images,
                               int accumulate)
{
    return guarded(h, [&] {
        check_axes_count(n_axes);
        if (n_axes > 0 && !axes) fail(GG_ERR_INVALID_ARG, "axes is NULL");
        if (!images && !cas_images) fail(GG_ERR_INVALID_ARG, "give images or cas_images");
        const size_t V3 = (size_t)h->V * h->V * h->V;
        h->cas.ensure(V3);
        if (!accumulate) GG_CK(cudaMemsetAsync(h->cas.p, 0, V3 * sizeof(float), h->cs));
        if (n_axes > 0) bp_host(h, axes, n_axes, images, cas_images, h->cas.p, false);
        GG_CK(cudaStreamSynchronize(h->cs));
        h->cas_fp_valid = false;
    });
}

extern "C" int gg_get_volume(gg_gridder *h, float *volume_out)
{
    return guarded(h, [&] {
        if (!volume_out) fail(GG_ERR_INVALID_ARG, "output is NULL");
        require_volume(h);
        const size_t N3 = (size_t)h->N * h->N * h->N;
        h->vol_io.ensure(N3);
        do_get_volume(h, h->cas.p, h->vol_io.p, h->cs);
        GG_CK(cudaMemcpyAsync(volume_out, h->vol_io.p, N3 * sizeof(float), cudaMemcpyDeviceToHost, h->cs));
        GG_CK(cudaStreamSynchronize(h->cs));
    });
}

extern "C" int gg_reconstruct_volume(gg_gridder *h, const float *axes, int n_axes, const float *images, float *volume_out)
{
    return guarded(h, [&] {
        check_axes_count(n_axes);
        if (n_axes > 0 && (!axes || !images)) fail(GG_ERR_INVALID_ARG, "axes and images are required");
        if (!volume_out) fail(GG_ERR_INVALID_ARG, "output is NULL");
        const size_t V3 = (size_t)h->V * h->V * h->V, N3 = (size_t)h->N * h->N * h->N;
        h->cas.ensure(V3);
        h->pd.ensure(V3);
        GG_CK(cudaMemsetAsync(h->cas.p, 0, V3 * sizeof(float), h->cs));
        GG_CK(cudaMemsetAsync(h->pd.p, 0, V3 * sizeof(float), h->cs));
        // back projection of the images and, in the same pass, the plane
        // density (the same directions with all-ones CAS images)
        if (n_axes > 0) bp_host(h, axes, n_axes, images, nullptr, h->cas.p, false, h->pd.p);
        GG_CK(launch_divide_plane_density(h->cas.p, h->pd.p, V3, 1e-6f, h->cs));
        h->vol_io.ensure(N3);
        do_get_volume(h, h->cas.p, h->vol_io.p, h->cs);
        GG_CK(cudaMemcpyAsync(volume_out, h->vol_io.p, N3 * sizeof(float), cudaMemcpyDeviceToHost, h->cs));
        GG_CK(cudaStreamSynchronize(h->cs));
        h->cas_fp_valid = false;
    });
}

// ---- device-pointer forms ---------------------------------------------------

extern "C" int gg_set_volume_dev(gg_gridder *h, const float *d_volume, void *stream)
{
    return guarded(h, [&] {
        if (!d_volume) fail(GG_ERR_INVALID_ARG, "volume is NULL");
        cudaStream_t s = (cudaStream_t)stream;
        begin_dev(h, s);
        do_set_volume(h, d_volume, s);
        end_dev(h, s);
    });
}

extern "C" int gg_set_cas_volume_dev(gg_gridder *h, const float *d_cas_volume, void *stream)
{
    return guarded(h, [&] {
        if (!d_cas_volume) fail(GG_ERR_INVALID_ARG, "cas_volume is NULL");
        cudaStream_t s = (cudaStream_t)stream;
        begin_dev(h, s);
        const size_t V3 = (size_t)h->V * h->V * h->V;
        h->cas.ensure(V3);
        GG_CK(cudaMemcpyAsync(h->cas.p, d_cas_volume, V3 * sizeof(float), cudaMemcpyDeviceToDevice, s));
        h->cas_fp_valid = false;
        end_dev(h, s);
    });
}

extern "C" int gg_get_cas_volume_dev(gg_gridder *h, float *d_out, void *stream)
{
    return guarded(h, [&] {
        if (!d_out) fail(GG_ERR_INVALID_ARG, "output is NULL");
        require_volume(h);
        cudaStream_t s = (cudaStream_t)stream;
        begin_dev(h, s);
        const size_t V3 = (size_t)h->V * h->V * h->V;
        GG_CK(cudaMemcpyAsync(d_out, h->cas.p, V3 * sizeof(float), cudaMemcpyDeviceToDevice, s));
        end_dev(h, s);
    });
}

extern "C" int gg_forward_project_dev(gg_gridder *h, const float *d_axes, int n_axes, float *d_images_out,
                                      float *d_cas_images_out, void *stream)
{
    return guarded(h, [&] {
        check_axes_count(n_axes);
        if (n_axes > 0 && !d_axes) fail(GG_ERR_INVALID_ARG, "axes is NULL");
        if (!d_images_out && !d_cas_images_out) fail(GG_ERR_INVALID_ARG, "no output requested");
        require_volume(h);
        if (n_axes == 0) return;
        cudaStream_t s = (cudaStream_t)stream;
        begin_dev(h, s);
        update_fp(h, s);
        const int B = h->max_batch;
        const size_t MM = (size_t)h->M * h->M, NN = (size_t)h->N * h->N;
        for (int a0 = 0; a0 < n_axes; a0 += B) {
            const int b = std::min(B, n_axes - a0);
            ensure_slot(h, 0, B, false);
            float *cas_out = d_cas_images_out ? d_cas_images_out + (size_t)a0 * MM : h->slot[0].casimg.p;
            fp_batch(h, d_axes + (size_t)a0 * 9, b, cas_out, d_images_out ? d_images_out + (size_t)a0 * NN : nullptr, 0, s);
        }
        end_dev(h, s);
    });
}

extern "C" int gg_back_project_dev(gg_gridder *h, const float *d_axes, int n_axes, const float *d_images,
                                   const float *d_cas_images, int accumulate, void *stream)
{
    return guarded(h, [&] {
        check_axes_count(n_axes);
        if (n_axes > 0 && !d_axes) fail(GG_ERR_INVALID_ARG, "axes is NULL");
        if (!d_images && !d_cas_images) fail(GG_ERR_INVALID_ARG, "give images or cas_images");
        cudaStream_t s = (cudaStream_t)stream;
        begin_dev(h, s);
        const size_t V3 = (size_t)h->V * h->V * h->V;
        h->cas.ensure(V3);
        if (!accumulate) GG_CK(cudaMemsetAsync(h->cas.p, 0, V3 * sizeof(float), s));
        const int B = h->max_batch;
        const size_t MM = (size_t)h->M * h->M, NN = (size_t)h->N * h->N;
        for (int a0 = 0; a0 < n_axes; a0 += B) {
            const int b = std::min(B, n_axes - a0);
            ensure_slot(h, 0, B, false);
            bp_batch(h, d_axes + (size_t)a0 * 9, b, d_images ? d_images + (size_t)a0 * NN : nullptr,
                     d_cas_images ? d_cas_images + (size_t)a0 * MM : nullptr, h->cas.p, false, 0, s);
        }
        h->cas_fp_valid = false;
        end_dev(h, s);
    });
}

extern "C" int gg_get_volume_dev(gg_gridder *h, float *d_volume_out, void *stream)
{
    return guarded(h, [&] {
        if (!d_volume_out) fail(GG_ERR_INVALID_ARG, "output is NULL");
        require_volume(h);
        cudaStream_t s = (cudaStream_t)stream;
        begin_dev(h, s);
        do_get_volume(h, h->cas.p, d_volume_out, s);
        end_dev(h, s);
    });
}

extern "C" int gg_reconstruct_volume_dev(gg_gridder *h, const float *d_axes, int n_axes, const float *d_images,
                                         float *d_volume_out, void *stream)
{
    return guarded(h, [&] {
        check_axes_count(n_axes);
        if (n_axes > 0 && (!d_axes || !d_images)) fail(GG_ERR_INVALID_ARG, "axes and images are required");
        if (!d_volume_out) fail(GG_ERR_INVALID_ARG, "output is NULL");
        cudaStream_t s = (cudaStream_t)stream;
        begin_dev(h, s);
        const size_t V3 = (size_t)h->V * h->V * h->V, NN = (size_t)h->N * h->N;
        h->cas.ensure(V3);
        h->pd.ensure(V3);
        GG_CK(cudaMemsetAsync(h->cas.p, 0, V3 * sizeof(float), s));
        GG_CK(cudaMemsetAsync(h->pd.p, 0, V3 * sizeof(float), s));
        const int B = h->max_batch;
        for (int a0 = 0; a0 < n_axes; a0 += B) {
            const int b = std::min(B, n_axes - a0);
            ensure_slot(h, 0, B, false);
            bp_batch(h, d_axes + (size_t)a0 * 9, b, d_images + (size_t)a0 * NN, nullptr, h->cas.p, false, 0, s, h->pd.p);
        }
        GG_CK(launch_divide_plane_density(h->cas.p, h->pd.p, V3, 1e-6f, s));
        do_get_volume(h, h->cas.p, d_volume_out, s);
        h->cas_fp_valid = false;
        end_dev(h, s);
    });
}

extern "C" int gg_back_project_sums_dev(gg_gridder *h, const float *d_axes, int n_axes, const float *d_images,
                                        float *d_sums, void *stream)
{
    return guarded(h, [&] {
        check_axes_count(n_axes);
        if (n_axes > 0 && (!d_axes || !d_images)) fail(GG_ERR_INVALID_ARG, "axes and images are required");
        if (!d_sums) fail(GG_ERR_INVALID_ARG, "sums buffer is NULL");
        cudaStream_t s = (cudaStream_t)stream;
        begin_dev(h, s);
        const size_t V3 = (size_t)h->V * h->V * h->V, NN = (size_t)h->N * h->N;
        GG_CK(cudaMemsetAsync(d_sums, 0, 2 * V3 * sizeof(float), s));
        const int B = h->max_batch;
        for (int a0 = 0; a0 < n_axes; a0 += B) {
            const int b = std::min(B, n_axes - a0);
            ensure_slot(h, 0, B, false);
            bp_batch(h, d_axes + (size_t)a0 * 9, b, d_images + (size_t)a0 * NN, nullptr, d_sums, false, 0, s,
                     d_sums + V3);
        }
        end_dev(h, s);
    });
}

extern "C" int gg_volume_from_sums_dev(gg_gridder *h, const float *d_sums, float *d_volume_out, void *stream)
{
    return guarded(h, [&] {
        if (!d_sums || !d_volume_out) fail(GG_ERR_INVALID_ARG, "sums and output are required");
        cudaStream_t s = (cudaStream_t)stream;
        begin_dev(h, s);
        const size_t V3 = (size_t)h->V * h->V * h->V;
        h->cas.ensure(V3);
        GG_CK(cudaMemcpyAsync(h->cas.p, d_sums, V3 * sizeof(float), cudaMemcpyDeviceToDevice, s));
        // tmpCASVolume ./ (PlaneDensity + 1e-6) (MultiGPUGridder_Matlab_Class.m:308)
        GG_CK(launch_divide_plane_density(h->cas.p, d_sums + V3, V3, 1e-6f, s));
        do_get_volume(h, h->cas.p, d_volume_out, s);
        h->cas_fp_valid = false;
        end_dev(h, s);
    });
}

extern "C" int gg_reconstruct_volume_ctf_dev(gg_gridder *h, const float *d_axes, int n_axes, const float *d_images,
                                             const float *d_defocus, const float *d_defocus_v,
                                             const float *d_astig_angle, float voltage_kv, float cs_mm,
                                             float amp_contrast, float pixel_size, float *d_volume_out, void *stream)
{
    return guarded(h, [&] {
        check_axes_count(n_axes);
        if (n_axes > 0 && (!d_axes || !d_images || !d_defocus))
            fail(GG_ERR_INVALID_ARG, "axes, images and defocus are required");
        if ((d_defocus_v == nullptr) != (d_astig_angle == nullptr))
            fail(GG_ERR_INVALID_ARG, "defocus_v and astig_angle are given together or not at all");
        if (!d_volume_out) fail(GG_ERR_INVALID_ARG, "output is NULL");
        const CtfParams c{voltage_kv, cs_mm, amp_contrast, pixel_size};
        check_ctf(c);
        cudaStream_t s = (cudaStream_t)stream;
        begin_dev(h, s);
        const size_t V3 = (size_t)h->V * h->V * h->V, NN = (size_t)h->N * h->N;
        h->cas.ensure(V3);
        h->pd.ensure(V3);
        GG_CK(cudaMemsetAsync(h->cas.p, 0, V3 * sizeof(float), s));
        GG_CK(cudaMemsetAsync(h->pd.p, 0, V3 * sizeof(float), s));
        const int B = h->max_batch;
        for (int a0 = 0; a0 < n_axes; a0 += B) {
            const int b = std::min(B, n_axes - a0);
            ensure_slot(h, 0, B, false);
            ctf_batch(h, d_axes + (size_t)a0 * 9, b, d_images + (size_t)a0 * NN, d_defocus + a0,
                      d_defocus_v ? d_defocus_v + a0 : nullptr, d_astig_angle ? d_astig_angle + a0 : nullptr, c, 0,
                      s);
        }
        GG_CK(launch_divide_plane_density(h->cas.p, h->pd.p, V3, 1e-6f, s));
        do_get_volume(h, h->cas.p, d_volume_out, s);
        h->cas_fp_valid = false;
        end_dev(h, s);
    });
}

extern "C" int gg_reconstruct_volume_ctf(gg_gridder *h, const float *axes, int n_axes, const float *images,
                                         const float *defocus, const float *defocus_v, const float *astig_angle,
                                         float voltage_kv, float cs_mm, float amp_contrast, float pixel_size,
                                         float *volume_out)
{
    return guarded(h, [&] {
        check_axes_count(n_axes);
        if (n_axes > 0 && (!axes || !images || !defocus))
            fail(GG_ERR_INVALID_ARG, "axes, images and defocus are required");
        if ((defocus_v == nullptr) != (astig_angle == nullptr))
            fail(GG_ERR_INVALID_ARG, "defocus_v and astig_angle are given together or not at all");
        if (!volume_out) fail(GG_ERR_INVALID_ARG, "output is NULL");
        const CtfParams c{voltage_kv, cs_mm, amp_contrast, pixel_size};
        check_ctf(c);
        cudaStream_t s = h->cs;
        const size_t V3 = (size_t)h->V * h->V * h->V, NN = (size_t)h->N * h->N, N3 = NN * h->N;
        upload_axes(h, axes, n_axes, s);
        // per-image CTF parameters: defocus U, then (astigmatic) defocus V and angle
        const bool astig = defocus_v != nullptr;
        const size_t nn = (size_t)std::max(1, n_axes);
        DevBuf<float> df;
        df.ensure(astig ? 3 * nn : nn);
        if (n_axes > 0) {
            GG_CK(cudaMemcpyAsync(df.p, defocus, (size_t)n_axes * sizeof(float), cudaMemcpyHostToDevice, s));
            if (astig) {
                GG_CK(cudaMemcpyAsync(df.p + nn, defocus_v, (size_t)n_axes * sizeof(float), cudaMemcpyHostToDevice, s));
                GG_CK(cudaMemcpyAsync(df.p + 2 * nn, astig_angle, (size_t)n_axes * sizeof(float),
                                      cudaMemcpyHostToDevice, s));
            }
        }
        h->cas.ensure(V3);
        h->pd.ensure(V3);
        GG_CK(cudaMemsetAsync(h->cas.p, 0, V3 * sizeof(float), s));
        GG_CK(cudaMemsetAsync(h->pd.p, 0, V3 * sizeof(float), s));
        if (n_axes > 0)
            host_batches(h, n_axes, images, NN, false, [&](int a0, int b, int sl, float *dbuf) {
                ctf_batch(h, h->axes.p + (size_t)a0 * 9, b, dbuf, df.p + a0, astig ? df.p + nn + a0 : nullptr,
                          astig ? df.p + 2 * nn + a0 : nullptr, c, sl, s);
            });
        GG_CK(launch_divide_plane_density(h->cas.p, h->pd.p, V3, 1e-6f, s));
        h->vol_io.ensure(N3);
        do_get_volume(h, h->cas.p, h->vol_io.p, s);
        GG_CK(cudaMemcpyAsync(volume_out, h->vol_io.p, N3 * sizeof(float), cudaMemcpyDeviceToHost, s));
        GG_CK(cudaStreamSynchronize(s));
        df.release();
        h->cas_fp_valid = false;
    });
}

extern "C" int gg_forward_project_adjoint_dev(gg_gridder *h, const float *d_axes, int n_axes, const float *d_image_grads,
                                              float *d_volume_grad_out, void *stream)
{
    return guarded(h, [&] {
        check_axes_count(n_axes);
        if (n_axes > 0 && (!d_axes || !d_image_grads)) fail(GG_ERR_INVALID_ARG, "axes and image gradients are required");
        if (!d_volume_grad_out) fail(GG_ERR_INVALID_ARG, "output is NULL");
        if (h->five_taps) fail(GG_ERR_STATE, "the adjoint needs a KB table with zero edge values");
        cudaStream_t s = (cudaStream_t)stream;
        begin_dev(h, s);
        forward_adjoint(h, d_axes, n_axes, d_image_grads, d_volume_grad_out, s);
        end_dev(h, s);
    });
}

extern "C" int gg_forward_project_adjoint(gg_gridder *h, const float *axes, int n_axes, const float *image_grads,
                                          float *volume_grad_out)
{
    return guarded(h, [&] {
        check_axes_count(n_axes);
        if (n_axes > 0 && (!axes || !image_grads)) fail(GG_ERR_INVALID_ARG, "axes and image gradients are required");
        if (!volume_grad_out) fail(GG_ERR_INVALID_ARG, "output is NULL");
        if (h->five_taps) fail(GG_ERR_STATE, "the adjoint needs a KB table with zero edge values");
        const size_t NN = (size_t)h->N * h->N, N3 = NN * h->N;
        upload_axes(h, axes, n_axes, h->cs);
        DevBuf<float> g;
        g.ensure(std::max<size_t>(1, NN * (size_t)n_axes));
        if (n_axes > 0)
            GG_CK(cudaMemcpyAsync(g.p, image_grads, NN * (size_t)n_axes * sizeof(float), cudaMemcpyHostToDevice, h->cs));
        h->vol_io.ensure(N3);
        forward_adjoint(h, h->axes.p, n_axes, g.p, h->vol_io.p, h->cs);
        GG_CK(cudaMemcpyAsync(volume_grad_out, h->vol_io.p, N3 * sizeof(float), cudaMemcpyDeviceToHost, h->cs));
        GG_CK(cudaStreamSynchronize(h->cs));
        g.release();
    });
}

// ---- stateless kernel entry points ------------------------------------------

int gg::check_kernel_args(float ker_hwidth, int n_axes, int V, int M, int mask_radius, int kb_size)
{
    if ((int)roundf(ker_hwidth) != 2 || ker_hwidth != 2.0f) {
        g_global_err = "only kerHWidth = 2 is supported (the reference fixes it, AbstractGridder.cpp:10)";
        return GG_ERR_INVALID_ARG;
    }
    if (n_axes < 0 || V <= 0 || M <= 0 || mask_radius < 0 || kb_size < 3 || kb_size > kMaxKerSizeHost) {
        g_global_err = "invalid sizes";
        return GG_ERR_INVALID_ARG;
    }
    return GG_OK;
}

static bool table_has_zero_edges(const float *d_ker, int n)
{
    float e[2] = {1.f, 1.f};
    if (cudaMemcpy(&e[0], d_ker, sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(&e[1], d_ker + n - 1, sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return e[0] == 0.0f && e[1] == 0.0f;
}

extern "C" int gg_forward_project_kernel(const float *d_cas_volume, float *d_cas_images, const float *d_kb_table,
                                         const float *d_axes, float ker_hwidth, int n_axes, int cas_vol_size,
                                         int cas_img_size, int extra_padding, int mask_radius, int kb_table_size,
                                         void *stream)
{
    (void)extra_padding;
    int rc = check_kernel_args(ker_hwidth, n_axes, cas_vol_size, cas_img_size, mask_radius, kb_table_size);
    if (rc != GG_OK) return rc;
    if (!d_cas_volume || !d_cas_images || !d_kb_table || (n_axes > 0 && !d_axes)) {
        g_global_err = "null pointer";
        return GG_ERR_INVALID_ARG;
    }
    const bool five = !table_has_zero_edges(d_kb_table, kb_table_size);
    Geom g{cas_vol_size, cas_img_size, mask_radius, kb_table_size, ker_hwidth};
    cudaError_t e = launch_forward_project(d_cas_volume, kF32, cas_vol_size, d_cas_images, d_kb_table, d_axes, n_axes, g, five, nullptr,
                                           (cudaStream_t)stream);
    if (e != cudaSuccess) {
        g_global_err = cudaGetErrorString(e);
        return GG_ERR_CUDA;
    }
    return GG_OK;
}

extern "C" int gg_back_project_kernel(float *d_cas_volume, const float *d_cas_images, const float *d_kb_table,
                                      const float *d_axes, float ker_hwidth, int n_axes, int cas_vol_size, int cas_img_size,
                                      int mask_radius, int kb_table_size, int extra_padding, void *stream)
{
    (void)extra_padding;
    int rc = check_kernel_args(ker_hwidth, n_axes, cas_vol_size, cas_img_size, mask_radius, kb_table_size);
    if (rc != GG_OK) return rc;
    if (!d_cas_volume || !d_cas_images || !d_kb_table || (n_axes > 0 && !d_axes)) {
        g_global_err = "null pointer";
        return GG_ERR_INVALID_ARG;
    }
    Geom g{cas_vol_size, cas_img_size, mask_radius, kb_table_size, ker_hwidth};
    cudaError_t e = launch_back_project_ref(d_cas_volume, d_cas_images, kF32, false, d_kb_table, d_axes, n_axes, g, nullptr,
                                            (cudaStream_t)stream);
    if (e != cudaSuccess) {
        g_global_err = cudaGetErrorString(e);
        return GG_ERR_CUDA;
    }
    return GG_OK;
}

extern "C" int gg_back_project_adjoint_kernel(float *d_cas_volume, const float *d_cas_images, const float *d_kb_table,
                                              const float *d_axes, float ker_hwidth, int n_axes, int cas_vol_size,
                                              int cas_img_size, int mask_radius, int kb_table_size, void *stream)
{
    int rc = check_kernel_args(ker_hwidth, n_axes, cas_vol_size, cas_img_size, mask_radius, kb_table_size);
    if (rc != GG_OK) return rc;
    if (!d_cas_volume || !d_cas_images || !d_kb_table || (n_axes > 0 && !d_axes)) {
        g_global_err = "null pointer";
        return GG_ERR_INVALID_ARG;
    }
    if (!table_has_zero_edges(d_kb_table, kb_table_size)) {
        g_global_err = "the adjoint back projection needs a KB table with zero edge values";
        return GG_ERR_INVALID_ARG;
    }
    Geom g{cas_vol_size, cas_img_size, mask_radius, kb_table_size, ker_hwidth};
    // zero table edges were checked above
    cudaError_t e = launch_back_project_adjoint(d_cas_volume, d_cas_images, kF32, d_kb_table, d_axes, n_axes, g, nullptr,
                                                true, (cudaStream_t)stream);
    if (e != cudaSuccess) {
        g_global_err = cudaGetErrorString(e);
        return GG_ERR_CUDA;
    }
    return GG_OK;
}

// ---- host helpers -----------------------------------------------------------

extern "C" int gg_kb_table(int ker_hwidth, int table_size, double *table_out)
{
    if (ker_hwidth < 1 || ker_hwidth > 5 || table_size < 3 || !table_out) return GG_ERR_INVALID_ARG;
    kb_table_f64(ker_hwidth, table_size, table_out);
    return GG_OK;
}

extern "C" int gg_precomp(int M, int ker_hwidth, double *precomp_out)
{
    if (M <= 0 || (M & 1) || ker_hwidth < 1 || ker_hwidth > 5 || !precomp_out) return GG_ERR_INVALID_ARG;
    precomp_f64(M, ker_hwidth, precomp_out);
    return GG_OK;
}

// ---- instrumentation ----------------------------------------------------------

extern "C" long long gg_kernel_launch_count(void) { return g_launches.load(); }

bool gg::gridder_view(gg_gridder *h, GridderView *out)
{
    if (!h || !h->cas.p) return false;
    std::lock_guard<std::mutex> lock(h->mu);
    const bool t = h->prec == kF32 && h->cas_fp_valid;
    *out = GridderView{h->device, h->N, h->M, h->V, h->geom(), h->cas.p, t ? h->cas_y.p : nullptr,
                       t ? h->cas_z.p : nullptr, h->ker.p, h->five_taps, h->fused_fft};
    return true;
}

bool gg::gridder_prepare_forward(gg_gridder *h)
{
    return guarded(h, [&] {
        set_device(h);
        require_volume(h);
        update_fp(h, h->cs);
        GG_CK(cudaStreamSynchronize(h->cs));
    }) == GG_OK;
}

void gg::gridder_trim(gg_gridder *h)
{
    std::lock_guard<std::mutex> lock(h->mu);
    cudaSetDevice(h->device);
    cudaStreamSynchronize(h->cs);
    h->x3.release();
    h->spec3.release();
    h->vol_io.release();
    if (h->have3_r2c) cufftDestroy(h->plan3_r2c);
    if (h->have3_c2r) cufftDestroy(h->plan3_c2r);
    h->have3_r2c = h->have3_c2r = false;
}

extern "C" int gg_profile_enable(gg_gridder *h, int enable)
{
    return guarded(h, [&] {
        for (auto &r : h->prof_recs) {
            cudaEventSynchronize(r.b);
            h->prof_pool.push_back(r.a);
            h->prof_pool.push_back(r.b);
        }
        h->prof_recs.clear();
        h->prof = enable != 0;
    });
}

extern "C" int gg_profile_read(gg_gridder *h, int kernel, double *total_ms, long long *launches)
{
    return guarded(h, [&] {
        double tot = 0.0;
        long long cnt = 0;
        for (auto &r : h->prof_recs) {
            if (r.kind != kernel) continue;
            GG_CK(cudaEventSynchronize(r.b));
            float ms = 0.f;
            GG_CK(cudaEventElapsedTime(&ms, r.a, r.b));
            tot += ms;
            cnt++;
        }
        if (total_ms) *total_ms = tot;
        if (launches) *launches = cnt;
    });
}
