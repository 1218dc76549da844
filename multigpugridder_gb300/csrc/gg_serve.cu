// Serving: a persistent request loop on one GPU.
//
// The reference runs one synchronous call at a time (MultiGPUGridder.cpp's
// ForwardProject / BackProject end with a device sync).  Here a server keeps
// any number of CAS volumes resident (one gridder each, prepared once) and a
// worker thread runs forward and back projection requests of any size and
// orientation count:
//
//   * continuous batching: a request is admitted as soon as a lane (a CUDA
//     stream with its own cuFFT plans) is free and its device memory fits the
//     HBM budget, whatever else is running; the requests on different lanes
//     overlap on the device;
//   * admission by HBM footprint: every request's buffers (directions,
//     per-chunk images / spectra / CAS images, and for a back projection a
//     CAS volume) are counted before it starts, in FIFO order;
//   * each request's work is the same stream-ordered sequence of the same
//     kernels whatever else runs, so its result does not depend on the mix.
//
// A forward request writes n*N*N images (forwardProject); a back request
// writes the V^3 CAS volume of its images back-projected into zeros
// (backProject's CASVolume, gpuGridder.cpp:332 zeroes it per call).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "gg_internal.h"
#include "../../include/gg_gridder.h"

using namespace gg;

namespace {

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct ServeError {
    int code;
    std::string msg;
};

[[noreturn]] void sfail(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    throw ServeError{code, buf};
}

#define GS_CK(call)                                                                                          \
    do {                                                                                                     \
        cudaError_t _e = (call);                                                                             \
        if (_e != cudaSuccess)                                                                               \
            sfail(_e == cudaErrorMemoryAllocation ? GG_ERR_OUT_OF_MEMORY : GG_ERR_CUDA, "%s: %s", #call,     \
                  cudaGetErrorString(_e));                                                                   \
    } while (0)

#define GS_CKF(call)                                                                               \
    do {                                                                                           \
        cufftResult _r = (call);                                                                   \
        if (_r != CUFFT_SUCCESS) sfail(GG_ERR_CUFFT, "%s failed: cufft status %d", #call, (int)_r); \
    } while (0)

int pow2ceil(int x)
{
    int p = 16;
    while (p < x) p <<= 1;
    return p;
}

// Directions per chunk for CAS images of edge M: about 64 M floats of CAS
// images per chunk, a power of two between 16 and 1024.
int chunk_for(int M)
{
    int c = 1024;
    while (c > 16 && (size_t)c * M * M > ((size_t)64 << 20)) c >>= 1;
    return c;
}

struct Volume {
    int id;
    gg_gridder *h = nullptr;
    GridderView view{};
    int refs = 0; // queued or running requests
};

struct Request {
    long long id;
    int vol_id, op, n;
    const float *axes;
    const float *in;
    float *out;
    GridderView view{};
    size_t footprint = 0;
    int chunk = 0;
    int lane = -1;
    int status = GG_OK;
    std::string err;
    double t_submit = 0, t_start = 0, t_done = 0;
    cudaError_t cuda_status = cudaSuccess; // from the stream callback
    bool gpu_done = false;                 // set by the stream callback
    bool done = false;                     // retired by the worker
};

struct Lane {
    cudaStream_t s = nullptr;
    bool busy = false;
    std::map<std::tuple<int, int, int>, cufftHandle> plans; // (type, M, batch)
    void *work = nullptr;                                   // shared cuFFT work area
    size_t work_bytes = 0;
};

} // namespace

struct gg_server {
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::thread worker;
    bool stop = false;
    int paused = 0; // admission held while lanes are being set up
    int device = 0;
    size_t budget = 0, used = 0, resident = 0, peak_used = 0;
    long long peak_inflight = 0;
    cudaMemPool_t pool = nullptr;
    std::vector<Lane> lanes;
    std::map<int, Volume> volumes;
    int next_vol = 1;
    long long next_req = 1;
    std::deque<std::shared_ptr<Request>> queue;
    std::vector<std::shared_ptr<Request>> running;
    std::map<long long, std::shared_ptr<Request>> reqs;
    std::vector<double> latencies; // seconds, completed requests since the last reset
    std::string err;
};

namespace {

// Footprint and chunking of a request (bytes held on the device while it runs).
void plan_request(Request &r)
{
    const GridderView &v = r.view;
    const size_t MM = (size_t)v.M * v.M, NN = (size_t)v.N * v.N, H = (size_t)v.M * (v.M / 2 + 1);
    r.chunk = std::min(chunk_for(v.M), pow2ceil(std::max(r.n, 1)));
    const size_t b = (size_t)r.chunk;
    size_t bytes = (size_t)std::max(r.n, 1) * 9 * sizeof(float);
    bytes += b * (MM * sizeof(float) + H * sizeof(cufftComplex) + MM * sizeof(float) + NN * sizeof(float) +
                  sizeof(int));
    if (r.op == GG_OP_BACK) bytes += (size_t)v.V * v.V * v.V * sizeof(float);
    r.footprint = bytes;
}

cufftHandle lane_plan(Lane &L, cufftType type, int M, int batch)
{
    auto key = std::make_tuple((int)type, M, batch);
    auto it = L.plans.find(key);
    if (it != L.plans.end()) return it->second;
    cufftHandle p;
    GS_CKF(cufftCreate(&p));
    GS_CKF(cufftSetAutoAllocation(p, 0));
    int dims[2] = {M, M};
    size_t ws = 0;
    GS_CKF(cufftMakePlanMany(p, 2, dims, nullptr, 1, 0, nullptr, 1, 0, type, batch, &ws));
    if (ws > L.work_bytes) {
        // the lane is idle here (plans are made before work is enqueued)
        GS_CK(cudaStreamSynchronize(L.s));
        if (L.work) GS_CK(cudaFree(L.work));
        L.work = nullptr;
        GS_CK(cudaMalloc(&L.work, ws));
        L.work_bytes = ws;
        for (auto &kv : L.plans) GS_CKF(cufftSetWorkArea(kv.second, L.work));
    }
    GS_CKF(cufftSetWorkArea(p, L.work));
    GS_CKF(cufftSetStream(p, L.s));
    L.plans[key] = p;
    return p;
}

// Plans for every batch size a request on CAS images of edge M can use.
void warm_plans(gg_server *S, int M)
{
    for (auto &L : S->lanes)
        for (int b = 16; b <= chunk_for(M); b <<= 1) {
            lane_plan(L, CUFFT_C2R, M, b);
            lane_plan(L, CUFFT_R2C, M, b);
        }
}

void CUDART_CB on_done(cudaStream_t, cudaError_t status, void *p)
{
    // runs on a CUDA callback thread after the request's stream work: no CUDA
    // calls here; `status` carries any error of that work
    auto *pair = static_cast<std::pair<gg_server *, Request *> *>(p);
    gg_server *S = pair->first;
    Request *r = pair->second;
    delete pair;
    {
        std::lock_guard<std::mutex> lock(S->mu);
        r->t_done = now_s();
        r->cuda_status = status;
        r->gpu_done = true;
    }
    S->cv_work.notify_all();
}

template <typename T> T *pool_alloc(gg_server *S, size_t count, cudaStream_t s)
{
    void *p = nullptr;
    GS_CK(cudaMallocFromPoolAsync(&p, count * sizeof(T), S->pool, s));
    return (T *)p;
}

// Enqueues a request's whole pipeline on its lane's stream.
void enqueue(gg_server *S, Request &r)
{
    Lane &L = S->lanes[r.lane];
    const cudaStream_t s = L.s;
    const GridderView &v = r.view;
    const size_t MM = (size_t)v.M * v.M, NN = (size_t)v.N * v.N, H = (size_t)v.M * (v.M / 2 + 1);
    const int B = r.chunk;
    // plans first: making one may synchronise the (idle) lane
    for (int b = 16; b <= B; b <<= 1) lane_plan(L, r.op == GG_OP_FORWARD ? CUFFT_C2R : CUFFT_R2C, v.M, b);

    float *d_axes = pool_alloc<float>(S, (size_t)std::max(r.n, 1) * 9, s);
    float *d_cas = pool_alloc<float>(S, MM * B, s);
    cufftComplex *d_spec = pool_alloc<cufftComplex>(S, H * B, s);
    float *d_real = pool_alloc<float>(S, MM * B, s);
    float *d_img = pool_alloc<float>(S, NN * B, s);
    int *d_order = r.op == GG_OP_FORWARD ? pool_alloc<int>(S, B, s) : nullptr;
    float *d_acc = nullptr;
    const size_t V3 = (size_t)v.V * v.V * v.V;
    if (r.n > 0) GS_CK(cudaMemcpyAsync(d_axes, r.axes, (size_t)r.n * 9 * sizeof(float), cudaMemcpyHostToDevice, s));
    if (r.op == GG_OP_BACK) {
        d_acc = pool_alloc<float>(S, V3, s);
        GS_CK(cudaMemsetAsync(d_acc, 0, V3 * sizeof(float), s));
    }
    for (int c0 = 0; c0 < r.n; c0 += B) {
        const int b = std::min(B, r.n - c0);
        const cufftHandle p =
            v.fused_fft ? 0 : lane_plan(L, r.op == GG_OP_FORWARD ? CUFFT_C2R : CUFFT_R2C, v.M, pow2ceil(b));
        if (r.op == GG_OP_FORWARD) {
            GS_CK(launch_forward_project(v.cas, kF32, v.V, d_cas, v.ker, d_axes + (size_t)c0 * 9, b, v.g, v.five_taps,
                                         nullptr, s, v.cas_y, v.cas_z, d_order));
            if (v.fused_fft) {
                GS_CK(launch_cas_to_images_fused(d_cas, v.M, v.N, b, d_img, s));
            } else {
                GS_CK(launch_cas_images_to_spectrum(d_cas, v.M, b, d_spec, s));
                GS_CKF(cufftExecC2R(p, d_spec, d_real));
                GS_CK(launch_fft_output_to_images(d_real, v.M, v.N, b, d_img, s));
            }
            GS_CK(cudaMemcpyAsync(r.out + (size_t)c0 * NN, d_img, (size_t)b * NN * sizeof(float),
                                  cudaMemcpyDeviceToHost, s));
        } else {
            GS_CK(cudaMemcpyAsync(d_img, r.in + (size_t)c0 * NN, (size_t)b * NN * sizeof(float),
                                  cudaMemcpyHostToDevice, s));
            if (v.fused_fft) {
                GS_CK(launch_images_to_cas_fused(d_img, v.N, v.M, b, d_cas, kF32, false, s));
            } else {
                GS_CK(launch_images_to_fft_input(d_img, v.N, v.M, b, d_real, s));
                GS_CKF(cufftExecR2C(p, d_real, d_spec));
                GS_CK(launch_spectrum_to_cas_images(d_spec, v.M, b, d_cas, kF32, nullptr, s));
            }
            GS_CK(launch_back_project_ref(d_acc, d_cas, kF32, false, v.ker, d_axes + (size_t)c0 * 9, b, v.g, nullptr,
                                          s, true));
        }
    }
    if (r.op == GG_OP_BACK) {
        GS_CK(cudaMemcpyAsync(r.out, d_acc, V3 * sizeof(float), cudaMemcpyDeviceToHost, s));
        GS_CK(cudaFreeAsync(d_acc, s));
    }
    if (d_order) GS_CK(cudaFreeAsync(d_order, s));
    GS_CK(cudaFreeAsync(d_img, s));
    GS_CK(cudaFreeAsync(d_real, s));
    GS_CK(cudaFreeAsync(d_spec, s));
    GS_CK(cudaFreeAsync(d_cas, s));
    GS_CK(cudaFreeAsync(d_axes, s));
    auto *arg = new std::pair<gg_server *, Request *>(S, &r);
    cudaError_t e = cudaStreamAddCallback(s, on_done, arg, 0);
    if (e != cudaSuccess) {
        delete arg;
        sfail(GG_ERR_CUDA, "cudaStreamAddCallback: %s", cudaGetErrorString(e));
    }
}

// Marks a finished request done and returns its resources (lock held).
void retire(gg_server *S, Request &r)
{
    if (r.cuda_status != cudaSuccess && r.status == GG_OK) {
        r.status = GG_ERR_CUDA;
        r.err = cudaGetErrorString(r.cuda_status);
    }
    r.done = true;
    S->lanes[r.lane].busy = false;
    S->used -= r.footprint;
    auto vit = S->volumes.find(r.vol_id);
    if (vit != S->volumes.end()) vit->second.refs--;
    if (r.status == GG_OK) S->latencies.push_back(r.t_done - r.t_submit);
}

void worker_main(gg_server *S)
{
    cudaSetDevice(S->device);
    std::unique_lock<std::mutex> lk(S->mu);
    for (;;) {
        bool progress = false;
        // retire requests whose stream work has finished
        for (size_t i = 0; i < S->running.size();) {
            Request &r = *S->running[i];
            if (!r.gpu_done) {
                i++;
                continue;
            }
            retire(S, r);
            S->running.erase(S->running.begin() + i);
            progress = true;
        }
        if (progress) S->cv_done.notify_all();
        // admit in arrival order while a lane is free and the footprint fits
        while (!S->queue.empty() && !S->paused) {
            auto r = S->queue.front();
            int lane = -1;
            for (size_t i = 0; i < S->lanes.size(); i++)
                if (!S->lanes[i].busy) {
                    lane = (int)i;
                    break;
                }
            if (lane < 0) break;
            if (S->resident + r->footprint > S->budget) {
                S->queue.pop_front();
                r->status = GG_ERR_OUT_OF_MEMORY;
                r->err = "request footprint exceeds the server's HBM budget";
                r->done = true;
                r->t_done = now_s();
                auto vit = S->volumes.find(r->vol_id);
                if (vit != S->volumes.end()) vit->second.refs--;
                S->cv_done.notify_all();
                continue;
            }
            if (S->resident + S->used + r->footprint > S->budget) break;
            S->queue.pop_front();
            r->lane = lane;
            S->lanes[lane].busy = true;
            S->used += r->footprint;
            S->peak_used = std::max(S->peak_used, S->resident + S->used);
            r->t_start = now_s();
            S->running.push_back(r);
            S->peak_inflight = std::max<long long>(S->peak_inflight, (long long)S->running.size());
            lk.unlock();
            try {
                enqueue(S, *r);
            } catch (const ServeError &e) {
                lk.lock();
                r->status = e.code;
                r->err = e.msg;
                // what was enqueued still runs; the request retires when the lane drains
                lk.unlock();
                cudaStreamSynchronize(S->lanes[lane].s);
                lk.lock();
                r->t_done = now_s();
                r->gpu_done = true;
                lk.unlock();
            }
            lk.lock();
            progress = true;
        }
        if (S->stop && S->queue.empty() && S->running.empty()) break;
        if (!progress) S->cv_work.wait(lk);
    }
}

template <typename F> int sguard(gg_server *S, F &&f)
{
    if (!S) {
        set_global_error("null server handle");
        return GG_ERR_INVALID_ARG;
    }
    try {
        f();
        return GG_OK;
    } catch (const ServeError &e) {
        std::lock_guard<std::mutex> lock(S->mu);
        S->err = e.msg;
        return e.code;
    }
}

} // namespace

extern "C" int gg_server_create(int device, double hbm_budget_gb, int lanes, gg_server **out)
{
    if (!out) {
        set_global_error("out is NULL");
        return GG_ERR_INVALID_ARG;
    }
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        set_global_error("no CUDA device available");
        return GG_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= ndev || lanes < 1 || lanes > 64) {
        set_global_error("invalid device or lane count (1..64)");
        return GG_ERR_INVALID_ARG;
    }
    auto *S = new gg_server();
    S->device = device;
    try {
        GS_CK(cudaSetDevice(device));
        size_t free_b = 0, total_b = 0;
        GS_CK(cudaMemGetInfo(&free_b, &total_b));
        S->budget = hbm_budget_gb > 0 ? (size_t)(hbm_budget_gb * (1 << 30)) : (size_t)(0.9 * (double)free_b);
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        GS_CK(cudaMemPoolCreate(&S->pool, &props));
        uint64_t keep = UINT64_MAX; // keep freed blocks for reuse
        GS_CK(cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrReleaseThreshold, &keep));
        S->lanes.resize(lanes);
        for (auto &L : S->lanes) GS_CK(cudaStreamCreateWithFlags(&L.s, cudaStreamNonBlocking));
    } catch (const ServeError &e) {
        set_global_error(e.msg.c_str());
        gg_server_destroy(S);
        return e.code;
    }
    S->worker = std::thread(worker_main, S);
    *out = S;
    return GG_OK;
}

extern "C" void gg_server_destroy(gg_server *S)
{
    if (!S) return;
    if (S->worker.joinable()) {
        {
            std::lock_guard<std::mutex> lock(S->mu);
            S->stop = true;
        }
        S->cv_work.notify_all();
        S->worker.join();
    }
    cudaSetDevice(S->device);
    for (auto &L : S->lanes) {
        if (L.s) cudaStreamSynchronize(L.s);
        for (auto &kv : L.plans) cufftDestroy(kv.second);
        if (L.work) cudaFree(L.work);
        if (L.s) cudaStreamDestroy(L.s);
    }
    for (auto &kv : S->volumes) gg_destroy(kv.second.h);
    if (S->pool) cudaMemPoolDestroy(S->pool);
    delete S;
}

extern "C" const char *gg_server_last_error(const gg_server *S) { return S ? S->err.c_str() : "null server handle"; }

extern "C" int gg_server_add_volume(gg_server *S, const float *volume, int volume_size, float interp_factor,
                                    int on_device, int *volume_id)
{
    return sguard(S, [&] {
        if (!volume || !volume_id) sfail(GG_ERR_INVALID_ARG, "volume and volume_id are required");
        gg_gridder *h = nullptr;
        int dev = S->device;
        int rc = gg_create(volume_size, 0, interp_factor, 3, 1, &dev, 1, 0, &h);
        if (rc != GG_OK) sfail(rc, "gg_create: %s", gg_global_error());
        const int dims[3] = {volume_size, volume_size, volume_size};
        rc = on_device ? gg_set_volume_dev(h, volume, nullptr) : gg_set_volume(h, volume, dims);
        if (rc == GG_OK && on_device) rc = cudaDeviceSynchronize() == cudaSuccess ? GG_OK : GG_ERR_CUDA;
        if (rc != GG_OK) {
            std::string m = gg_last_error(h);
            gg_destroy(h);
            sfail(rc, "setting the volume: %s", m.c_str());
        }
        gridder_trim(h);
        if (!gridder_prepare_forward(h)) {
            std::string m = gg_last_error(h);
            gg_destroy(h);
            sfail(GG_ERR_CUDA, "preparing the volume copies: %s", m.c_str());
        }
        Volume v;
        if (!gridder_view(h, &v.view)) {
            gg_destroy(h);
            sfail(GG_ERR_STATE, "volume not resident");
        }
        v.h = h;
        {   // hold admission and let the lanes drain: plans are made on idle lanes
            std::unique_lock<std::mutex> lk(S->mu);
            S->paused++;
            S->cv_done.wait(lk, [&] { return S->running.empty(); });
        }
        try {
            warm_plans(S, v.view.M);
        } catch (...) {
            {
                std::lock_guard<std::mutex> lock(S->mu);
                S->paused--;
            }
            S->cv_work.notify_all();
            gg_destroy(h);
            throw;
        }
        std::lock_guard<std::mutex> lock(S->mu);
        S->paused--;
        S->cv_work.notify_all();
        v.id = S->next_vol++;
        S->resident += (size_t)v.view.V * v.view.V * v.view.V * sizeof(float);
        S->volumes[v.id] = v;
        *volume_id = v.id;
    });
}

extern "C" int gg_server_remove_volume(gg_server *S, int volume_id)
{
    return sguard(S, [&] {
        gg_gridder *h = nullptr;
        {
            std::lock_guard<std::mutex> lock(S->mu);
            auto it = S->volumes.find(volume_id);
            if (it == S->volumes.end()) sfail(GG_ERR_INVALID_ARG, "unknown volume id %d", volume_id);
            if (it->second.refs > 0) sfail(GG_ERR_STATE, "volume %d has requests queued or running", volume_id);
            h = it->second.h;
            S->resident -= (size_t)it->second.view.V * it->second.view.V * it->second.view.V * sizeof(float);
            S->volumes.erase(it);
        }
        gg_destroy(h);
    });
}

extern "C" int gg_server_volume_sizes(gg_server *S, int volume_id, int *N, int *M, int *V)
{
    return sguard(S, [&] {
        std::lock_guard<std::mutex> lock(S->mu);
        auto it = S->volumes.find(volume_id);
        if (it == S->volumes.end()) sfail(GG_ERR_INVALID_ARG, "unknown volume id %d", volume_id);
        if (N) *N = it->second.view.N;
        if (M) *M = it->second.view.M;
        if (V) *V = it->second.view.V;
    });
}

extern "C" int gg_server_submit(gg_server *S, int volume_id, int op, const float *axes, int n_axes,
                                const float *images, float *out, long long *request_id)
{
    return sguard(S, [&] {
        if (op != GG_OP_FORWARD && op != GG_OP_BACK) sfail(GG_ERR_INVALID_ARG, "unknown op %d", op);
        if (n_axes < 0) sfail(GG_ERR_INVALID_ARG, "n_axes must be >= 0");
        if ((n_axes > 0 && !axes) || !out || !request_id) sfail(GG_ERR_INVALID_ARG, "axes, out and request_id are required");
        if (op == GG_OP_BACK && n_axes > 0 && !images) sfail(GG_ERR_INVALID_ARG, "a back projection needs images");
        auto r = std::make_shared<Request>();
        r->vol_id = volume_id;
        r->op = op;
        r->n = n_axes;
        r->axes = axes;
        r->in = images;
        r->out = out;
        {
            std::lock_guard<std::mutex> lock(S->mu);
            auto it = S->volumes.find(volume_id);
            if (it == S->volumes.end()) sfail(GG_ERR_INVALID_ARG, "unknown volume id %d", volume_id);
            r->view = it->second.view;
            plan_request(*r);
            it->second.refs++;
            r->id = S->next_req++;
            r->t_submit = now_s();
            S->reqs[r->id] = r;
            S->queue.push_back(r);
            *request_id = r->id;
        }
        S->cv_work.notify_all();
    });
}

extern "C" int gg_server_wait(gg_server *S, long long request_id, double timeout_s, double *latency_ms)
{
    if (!S) {
        set_global_error("null server handle");
        return GG_ERR_INVALID_ARG;
    }
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->reqs.find(request_id);
    if (it == S->reqs.end()) {
        S->err = "unknown request id (already waited for?)";
        return GG_ERR_INVALID_ARG;
    }
    auto r = it->second;
    auto pred = [&] { return r->done; };
    if (timeout_s < 0) {
        S->cv_done.wait(lk, pred);
    } else if (!S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) {
        S->err = "timed out waiting for the request";
        return GG_ERR_TIMEOUT;
    }
    if (latency_ms) *latency_ms = (r->t_done - r->t_submit) * 1e3;
    S->reqs.erase(it);
    if (r->status != GG_OK) S->err = r->err;
    return r->status;
}

extern "C" int gg_server_stats(gg_server *S, long long *completed, double *p50_ms, double *p99_ms, double *mean_ms,
                               long long *peak_inflight, double *peak_gb)
{
    return sguard(S, [&] {
        std::lock_guard<std::mutex> lock(S->mu);
        std::vector<double> l = S->latencies;
        std::sort(l.begin(), l.end());
        auto pct = [&](double q) {
            if (l.empty()) return 0.0;
            const size_t i = std::min(l.size() - 1, (size_t)(q * (double)(l.size() - 1) + 0.5));
            return l[i] * 1e3;
        };
        double sum = 0;
        for (double x : l) sum += x;
        if (completed) *completed = (long long)l.size();
        if (p50_ms) *p50_ms = pct(0.50);
        if (p99_ms) *p99_ms = pct(0.99);
        if (mean_ms) *mean_ms = l.empty() ? 0.0 : sum / (double)l.size() * 1e3;
        if (peak_inflight) *peak_inflight = S->peak_inflight;
        if (peak_gb) *peak_gb = (double)S->peak_used / (double)(1 << 30);
    });
}

extern "C" int gg_server_reset_stats(gg_server *S)
{
    return sguard(S, [&] {
        std::lock_guard<std::mutex> lock(S->mu);
        S->latencies.clear();
        S->peak_inflight = (long long)S->running.size();
        S->peak_used = S->resident + S->used;
    });
}
