// Serving: a persistent request loop on one GPU.
//
// The reference runs one synchronous call at a time (MultiGPUGridder.cpp's
// ForwardProject / BackProject end with a device sync).  Here a server keeps
// any number of CAS volumes resident (one gridder each, prepared once) and a
// worker thread runs forward and back projection requests of any size and
// orientation count:
//
//   * continuous batching: a request is split into chunks of directions of
//     about one quantum of estimated device time (8 ms by default); a lane (a
//     pair of CUDA streams with its own cuFFT plans) runs one chunk at a time,
//     and the chunks of different requests on different lanes overlap on the
//     device.  Requests that arrive while others run start on the next lane
//     that frees, so a 4,096-direction request on a 256^3 volume holds a
//     lane for one chunk, not for its whole run;
//   * scheduling by remaining work: a free lane takes the chunk of the
//     request with the least estimated work left, less 0.2 s per second it
//     has waited (so no request waits for ever); requests of one quantum or
//     less ("short") run on the lanes' high-priority streams, whose blocks
//     the GPU starts before those of the long requests, and long requests
//     hold at most all lanes but a quarter, which stay free for short ones;
//   * admission by HBM footprint: every request's buffers (directions, one
//     chunk of images / spectra / CAS images, and for a back projection a
//     CAS volume) are counted before its first chunk, in scheduling order; a
//     request that does not fit waits, and none behind it is admitted first;
//   * an optional bound on the queued work (gg_server_set_max_backlog):
//     beyond it a submission is refused with GG_ERR_BUSY, as an overloaded
//     server sheds load instead of growing its queue without limit;
//   * each request's work is the same sequence of the same kernels on the
//     same chunks whatever else runs, one chunk after the other, so its
//     result does not depend on the mix.
//
// A forward request writes n*N*N images (forwardProject); a back request
// writes the V^3 CAS volume of its images back-projected into zeros
// (backProject's CASVolume, gpuGridder.cpp:332 zeroes it per call).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <map>
#include <memory>
#include <mutex>
#include <set>
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

// Directions per chunk that fit the chunk buffers for CAS images of edge M:
// about 64 M floats of CAS images, a power of two between 16 and 1024.
int chunk_cap(int M)
{
    int c = 1024;
    while (c > 16 && (size_t)c * M * M > ((size_t)64 << 20)) c >>= 1;
    return c;
}

// Estimated device seconds of one direction, for ranking requests and bounding
// the backlog: one GB300 runs the forward projection with its 2-D stage in
// about 34 ps and the serving back projection in about 120 ps per CAS-image
// pixel (2.2 and 7.9 ms per 1,000 directions at M = 256).
double dir_seconds(int op, int M)
{
    return (double)M * M * (op == GG_OP_FORWARD ? 3.4e-11 : 1.2e-10);
}
constexpr double kChunkSeconds = 2e-5;  // launches and copies of one chunk
constexpr double kAging = 0.2;          // seconds of work a request gains per second it waits
constexpr int kActivePerLane = 4;       // admitted requests at most, per lane
constexpr int kReserveDiv = 4;          // lanes / kReserveDiv lanes are kept for short requests

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
    size_t footprint = 0; // device bytes held from admission to completion
    int chunk = 0;        // directions per chunk
    int next = 0;         // first direction of the next chunk
    double est = 0;       // estimated device seconds of the whole request
    double key = 0;       // scheduling key: smaller runs first
    bool admitted = false, started = false, high = false;
    int lane = -1;        // lane of the chunk in flight
    // device buffers, allocated by the first chunk and freed by the last
    float *d_axes = nullptr, *d_cas = nullptr, *d_real = nullptr, *d_img = nullptr, *d_acc = nullptr;
    cufftComplex *d_spec = nullptr;
    int *d_order = nullptr;
    int status = GG_OK;
    std::string err;
    double t_submit = 0, t_start = 0, t_done = 0;
    cudaError_t cuda_status = cudaSuccess; // of the chunk in flight, from the stream callback
    bool gpu_done = false;                 // the chunk in flight has finished (stream callback)
    bool done = false;                     // retired by the worker
};

struct KeyLess {
    bool operator()(const Request *a, const Request *b) const
    {
        return a->key != b->key ? a->key < b->key : a->id < b->id;
    }
};

struct Lane {
    cudaStream_t lo = nullptr, hi = nullptr; // low and high stream priority
    bool busy = false;
    bool long_chunk = false; // the chunk in flight belongs to a long request
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
    double quantum = 8e-3;     // estimated seconds of one chunk
    double max_backlog = 0;    // estimated seconds of queued work; 0: unbounded
    double queued_work = 0;    // estimated seconds of the queued (not admitted) requests
    long long rejected = 0;
    int active = 0;            // admitted, not yet retired
    cudaMemPool_t pool = nullptr;
    std::vector<Lane> lanes;
    std::map<int, Volume> volumes;
    int next_vol = 1;
    long long next_req = 1;
    // by class (index 1: short requests, of one quantum or less; 0: long ones)
    std::set<Request *, KeyLess> queued[2]; // submitted, not admitted
    std::set<Request *, KeyLess> ready[2];  // admitted, no chunk in flight
    int long_busy = 0;                      // lanes running a chunk of a long request
    std::vector<Request *> inflight;     // a chunk on a lane
    std::map<long long, std::shared_ptr<Request>> reqs; // until waited for
    std::map<long long, std::shared_ptr<Request>> live; // until retired
    std::vector<double> latencies; // seconds, completed requests since the last reset
    std::string err;
};

namespace {

// Remaining estimated device seconds of a request.
double remaining(const Request &r)
{
    const int left = std::max(r.n - r.next, 0);
    double t = left * dir_seconds(r.op, r.view.M) + ((left + r.chunk - 1) / r.chunk) * kChunkSeconds;
    if (r.op == GG_OP_BACK) t += (double)r.view.V * r.view.V * r.view.V * 4 * 2e-11; // zeroing and read-back
    return t;
}

// Footprint, chunking and cost of a request.  A chunk is the largest power
// of two of directions (16 at least) whose estimated time fits the quantum,
// capped by the chunk buffers and the request's size.
void plan_request(Request &r, double quantum)
{
    const GridderView &v = r.view;
    const size_t MM = (size_t)v.M * v.M, NN = (size_t)v.N * v.N, H = (size_t)v.M * (v.M / 2 + 1);
    int c = 16;
    while (c < chunk_cap(v.M) && 2 * c * dir_seconds(r.op, v.M) <= quantum) c <<= 1;
    r.chunk = std::min(c, pow2ceil(std::max(r.n, 1)));
    const size_t b = (size_t)r.chunk;
    size_t bytes = (size_t)std::max(r.n, 1) * 9 * sizeof(float);
    bytes += b * (MM * sizeof(float) + NN * sizeof(float) + sizeof(int));
    if (!v.fused_fft) bytes += b * (H * sizeof(cufftComplex) + MM * sizeof(float));
    if (r.op == GG_OP_BACK) bytes += (size_t)v.V * v.V * v.V * sizeof(float);
    r.footprint = bytes;
    r.est = remaining(r);
    r.high = r.est <= quantum;
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
        GS_CK(cudaStreamSynchronize(L.lo));
        GS_CK(cudaStreamSynchronize(L.hi));
        if (L.work) GS_CK(cudaFree(L.work));
        L.work = nullptr;
        GS_CK(cudaMalloc(&L.work, ws));
        L.work_bytes = ws;
        for (auto &kv : L.plans) GS_CKF(cufftSetWorkArea(kv.second, L.work));
    }
    GS_CKF(cufftSetWorkArea(p, L.work));
    L.plans[key] = p;
    return p;
}

// Plans for every batch size a request on CAS images of edge M can use.
void warm_plans(gg_server *S, int M)
{
    for (auto &L : S->lanes)
        for (int b = 16; b <= chunk_cap(M); b <<= 1) {
            lane_plan(L, CUFFT_C2R, M, b);
            lane_plan(L, CUFFT_R2C, M, b);
        }
}

void CUDART_CB on_done(cudaStream_t, cudaError_t status, void *p)
{
    // runs on a CUDA callback thread after the chunk's stream work: no CUDA
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

// Hands the request's device buffers to `out` (to be freed with
// cudaFreeAsync) and clears them.
void take_buffers(Request &r, std::vector<void *> &out)
{
    void *bufs[] = {r.d_acc, r.d_order, r.d_img, r.d_real, r.d_spec, r.d_cas, r.d_axes};
    for (void *p : bufs)
        if (p) out.push_back(p);
    r.d_acc = r.d_cas = r.d_real = r.d_img = r.d_axes = nullptr;
    r.d_spec = nullptr;
    r.d_order = nullptr;
}

void free_buffers(Request &r, cudaStream_t s)
{
    std::vector<void *> bufs;
    take_buffers(r, bufs);
    for (void *p : bufs) cudaFreeAsync(p, s);
}

// Enqueues the request's next chunk on its lane: the first chunk also
// allocates the buffers, uploads the directions and zeroes the accumulator;
// the last one also reads the accumulator back and frees the buffers.  The
// chunks of a request run one after another (each starts once the previous
// one has finished), whichever lanes they land on.
void enqueue_chunk(gg_server *S, Request &r)
{
    Lane &L = S->lanes[r.lane];
    const cudaStream_t s = r.high ? L.hi : L.lo;
    const GridderView &v = r.view;
    const size_t MM = (size_t)v.M * v.M, NN = (size_t)v.N * v.N, H = (size_t)v.M * (v.M / 2 + 1);
    const int B = r.chunk;
    const size_t V3 = (size_t)v.V * v.V * v.V;
    if (!r.started) {
        r.started = true;
        r.d_axes = pool_alloc<float>(S, (size_t)std::max(r.n, 1) * 9, s);
        r.d_cas = pool_alloc<float>(S, MM * B, s);
        r.d_img = pool_alloc<float>(S, NN * B, s);
        if (!v.fused_fft) {
            r.d_spec = pool_alloc<cufftComplex>(S, H * B, s);
            r.d_real = pool_alloc<float>(S, MM * B, s);
        }
        if (r.op == GG_OP_FORWARD) r.d_order = pool_alloc<int>(S, B, s);
        if (r.n > 0)
            GS_CK(cudaMemcpyAsync(r.d_axes, r.axes, (size_t)r.n * 9 * sizeof(float), cudaMemcpyHostToDevice, s));
        if (r.op == GG_OP_BACK) {
            r.d_acc = pool_alloc<float>(S, V3, s);
            GS_CK(cudaMemsetAsync(r.d_acc, 0, V3 * sizeof(float), s));
        }
    }
    const int c0 = r.next;
    const int b = std::min(B, r.n - c0);
    if (b > 0) {
        cufftHandle p = 0;
        if (!v.fused_fft) {
            p = lane_plan(L, r.op == GG_OP_FORWARD ? CUFFT_C2R : CUFFT_R2C, v.M, pow2ceil(b));
            GS_CKF(cufftSetStream(p, s));
        }
        const float *axes = r.d_axes + (size_t)c0 * 9;
        if (r.op == GG_OP_FORWARD) {
            GS_CK(launch_forward_project(v.cas, kF32, v.V, r.d_cas, v.ker, axes, b, v.g, v.five_taps, nullptr, s,
                                         v.cas_y, v.cas_z, r.d_order));
            if (v.fused_fft) {
                GS_CK(launch_cas_to_images_fused(r.d_cas, v.M, v.N, b, r.d_img, s));
            } else {
                GS_CK(launch_cas_images_to_spectrum(r.d_cas, v.M, b, r.d_spec, s));
                GS_CKF(cufftExecC2R(p, r.d_spec, r.d_real));
                GS_CK(launch_fft_output_to_images(r.d_real, v.M, v.N, b, r.d_img, s));
            }
            GS_CK(cudaMemcpyAsync(r.out + (size_t)c0 * NN, r.d_img, (size_t)b * NN * sizeof(float),
                                  cudaMemcpyDeviceToHost, s));
        } else {
            GS_CK(cudaMemcpyAsync(r.d_img, r.in + (size_t)c0 * NN, (size_t)b * NN * sizeof(float),
                                  cudaMemcpyHostToDevice, s));
            if (v.fused_fft) {
                GS_CK(launch_images_to_cas_fused(r.d_img, v.N, v.M, b, r.d_cas, kF32, false, s));
            } else {
                GS_CK(launch_images_to_fft_input(r.d_img, v.N, v.M, b, r.d_real, s));
                GS_CKF(cufftExecR2C(p, r.d_real, r.d_spec));
                GS_CK(launch_spectrum_to_cas_images(r.d_spec, v.M, b, r.d_cas, kF32, nullptr, s));
            }
            GS_CK(launch_back_project_ref(r.d_acc, r.d_cas, kF32, false, v.ker, axes, b, v.g, nullptr, s, true));
        }
    }
    r.next = c0 + std::max(b, 0);
    if (r.next >= r.n) {
        if (r.op == GG_OP_BACK) GS_CK(cudaMemcpyAsync(r.out, r.d_acc, V3 * sizeof(float), cudaMemcpyDeviceToHost, s));
        free_buffers(r, s);
    }
    auto *arg = new std::pair<gg_server *, Request *>(S, &r);
    cudaError_t e = cudaStreamAddCallback(s, on_done, arg, 0);
    if (e != cudaSuccess) {
        delete arg;
        sfail(GG_ERR_CUDA, "cudaStreamAddCallback: %s", cudaGetErrorString(e));
    }
}

// Marks a request done and returns its resources (lock held).  A failed
// request may still hold device buffers (its lane has drained): they go to
// `frees`, for cudaFreeAsync once the lock is released.
void retire(gg_server *S, Request *r, std::vector<std::pair<void *, cudaStream_t>> &frees)
{
    if (r->lane >= 0) {
        std::vector<void *> bufs;
        take_buffers(*r, bufs);
        for (void *p : bufs) frees.emplace_back(p, S->lanes[r->lane].lo);
    }
    if (r->admitted) {
        S->used -= r->footprint;
        S->active--;
    }
    r->done = true;
    auto vit = S->volumes.find(r->vol_id);
    if (vit != S->volumes.end()) vit->second.refs--;
    if (r->status == GG_OK) S->latencies.push_back(r->t_done - r->t_submit);
    S->live.erase(r->id);
}

void worker_main(gg_server *S)
{
    cudaSetDevice(S->device);
    std::unique_lock<std::mutex> lk(S->mu);
    std::vector<std::pair<void *, cudaStream_t>> frees;
    for (;;) {
        bool progress = false;
        // chunks whose stream work has finished
        for (size_t i = 0; i < S->inflight.size();) {
            Request *r = S->inflight[i];
            if (!r->gpu_done) {
                i++;
                continue;
            }
            S->inflight.erase(S->inflight.begin() + i);
            Lane &L = S->lanes[r->lane];
            L.busy = false;
            if (L.long_chunk) S->long_busy--;
            L.long_chunk = false;
            r->gpu_done = false;
            if (r->cuda_status != cudaSuccess && r->status == GG_OK) {
                r->status = GG_ERR_CUDA;
                r->err = cudaGetErrorString(r->cuda_status);
            }
            if (r->status != GG_OK || r->next >= r->n) {
                retire(S, r, frees);
            } else {
                r->key = remaining(*r) + kAging * r->t_submit;
                S->ready[r->high].insert(r);
            }
            progress = true;
        }
        if (progress) S->cv_done.notify_all();
        if (!frees.empty()) {
            lk.unlock();
            for (auto &f : frees) cudaFreeAsync(f.first, f.second);
            lk.lock();
            frees.clear();
        }
        // a free lane runs the chunk of the request with the least remaining
        // work (less kAging per second it has waited), admitted or not; long
        // requests fill at most all lanes but lanes / kReserveDiv, which stay
        // free for short ones.  A request whose footprint does not fit waits
        // for memory, and no request with a larger key is admitted before it.
        while (!S->paused) {
            int lane = -1;
            for (size_t i = 0; i < S->lanes.size(); i++)
                if (!S->lanes[i].busy) {
                    lane = (int)i;
                    break;
                }
            if (lane < 0) break;
            for (auto &qs : S->queued)
                while (!qs.empty() && S->resident + (*qs.begin())->footprint > S->budget) {
                    Request *x = *qs.begin();
                    qs.erase(qs.begin());
                    S->queued_work -= x->est;
                    x->status = GG_ERR_OUT_OF_MEMORY;
                    x->err = "request footprint exceeds the server's HBM budget";
                    x->t_done = now_s();
                    retire(S, x, frees);
                    S->cv_done.notify_all();
                }
            const int nl = (int)S->lanes.size();
            const bool long_ok = S->long_busy < nl - nl / kReserveDiv;
            auto best = [&](std::set<Request *, KeyLess> *sets) {
                Request *x = sets[1].empty() ? nullptr : *sets[1].begin();
                if (long_ok && !sets[0].empty() && (!x || KeyLess()(*sets[0].begin(), x))) x = *sets[0].begin();
                return x;
            };
            Request *q = best(S->queued), *a = best(S->ready);
            const bool admit = q && (!a || KeyLess()(q, a)) &&
                               S->resident + S->used + q->footprint <= S->budget &&
                               S->active < kActivePerLane * nl;
            Request *r = admit ? q : a;
            if (!r) break;
            if (admit) {
                S->queued[r->high].erase(r);
                S->queued_work -= r->est;
                if (S->queued[0].empty() && S->queued[1].empty()) S->queued_work = 0; // no rounding drift
                r->admitted = true;
                S->used += r->footprint;
                S->active++;
                S->peak_used = std::max(S->peak_used, S->resident + S->used);
                S->peak_inflight = std::max<long long>(S->peak_inflight, S->active);
                r->t_start = now_s();
            } else {
                S->ready[r->high].erase(r);
            }
            if (!r->high) {
                S->lanes[lane].long_chunk = true;
                S->long_busy++;
            }
            r->lane = lane;
            S->lanes[lane].busy = true;
            S->inflight.push_back(r);
            lk.unlock();
            try {
                enqueue_chunk(S, *r);
            } catch (const ServeError &e) {
                // what was enqueued still runs; the request retires once its lane drains
                cudaStreamSynchronize(S->lanes[lane].lo);
                cudaStreamSynchronize(S->lanes[lane].hi);
                lk.lock();
                r->status = e.code;
                r->err = e.msg;
                r->t_done = now_s();
                r->gpu_done = true;
                lk.unlock();
            }
            lk.lock();
            progress = true;
        }
        if (S->stop && S->queued[0].empty() && S->queued[1].empty() && S->active == 0 && S->inflight.empty()) break;
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
        int least = 0, greatest = 0;
        GS_CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        S->lanes.resize(lanes);
        for (auto &L : S->lanes) {
            GS_CK(cudaStreamCreateWithPriority(&L.lo, cudaStreamNonBlocking, least));
            GS_CK(cudaStreamCreateWithPriority(&L.hi, cudaStreamNonBlocking, greatest));
        }
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
        if (L.lo) cudaStreamSynchronize(L.lo);
        if (L.hi) cudaStreamSynchronize(L.hi);
        for (auto &kv : L.plans) cufftDestroy(kv.second);
        if (L.work) cudaFree(L.work);
        if (L.lo) cudaStreamDestroy(L.lo);
        if (L.hi) cudaStreamDestroy(L.hi);
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
            S->cv_done.wait(lk, [&] { return S->inflight.empty(); });
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
            plan_request(*r, S->quantum);
            if (S->max_backlog > 0 && S->queued_work >= S->max_backlog) {
                S->rejected++;
                sfail(GG_ERR_BUSY, "the server's backlog is full (%.3f s of queued work); retry later",
                      S->queued_work);
            }
            it->second.refs++;
            r->id = S->next_req++;
            r->t_submit = now_s();
            r->key = r->est + kAging * r->t_submit;
            S->reqs[r->id] = r;
            S->live[r->id] = r;
            S->queued[r->high].insert(r.get());
            S->queued_work += r->est;
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
        S->peak_inflight = S->active;
        S->peak_used = S->resident + S->used;
        S->rejected = 0;
    });
}

extern "C" int gg_server_set_quantum(gg_server *S, double quantum_ms)
{
    return sguard(S, [&] {
        if (!(quantum_ms > 0)) sfail(GG_ERR_INVALID_ARG, "quantum_ms must be > 0");
        std::lock_guard<std::mutex> lock(S->mu);
        S->quantum = quantum_ms * 1e-3;
    });
}

extern "C" int gg_server_set_max_backlog(gg_server *S, double seconds)
{
    return sguard(S, [&] {
        if (!(seconds >= 0)) sfail(GG_ERR_INVALID_ARG, "the backlog bound must be >= 0 seconds");
        std::lock_guard<std::mutex> lock(S->mu);
        S->max_backlog = seconds;
    });
}

extern "C" int gg_server_load(gg_server *S, long long *queued, long long *active, double *queued_seconds,
                              long long *rejected)
{
    return sguard(S, [&] {
        std::lock_guard<std::mutex> lock(S->mu);
        if (queued) *queued = (long long)(S->queued[0].size() + S->queued[1].size());
        if (active) *active = S->active;
        if (queued_seconds) *queued_seconds = S->queued_work;
        if (rejected) *rejected = S->rejected;
    });
}
