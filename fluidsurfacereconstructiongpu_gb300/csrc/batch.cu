// Batches of frames in one CUDA graph launch (include/fsr.h, fsr_batch_*).
//
// Each frame slot owns an fsr_handle (its pooled buffers and counters), so
// every frame's intermediates and mesh stay resident after the batch.  A
// plan runs every frame once on its own (frame_plan / frame_buffers /
// frame_enqueue / frame_finish, exactly the single-frame path) to size its
// buffers and to measure its cost; frames are then assigned to L lanes by
// longest-processing-time first, and the graph is captured: a fork event on
// the origin stream, each lane waits on it and queues its frames' kernels
// back to back, the origin joins every lane.  The autotuner captures and
// times each (lanes, grid_div) candidate on the real frames, then the best
// one again with 128-thread blocks for the per-item and warp-staged kernels
// (the block shape), and keeps the fastest executable graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/fsr.h"
#include "fsr_internal.h"

using namespace fsr;

struct fsr_batch {
    int device = 0;
    fsr_params params[4]{};
    std::string last_error;

    std::vector<fsr_handle*> slots;  // one handle per frame
    std::vector<FramePlan> plans;
    std::vector<uint32_t> method;
    std::vector<float> cost_ms;      // single-frame time of each frame (plan pass)
    std::vector<uint8_t> shape;      // bytes of the planned frame set
    std::vector<uint32_t> lane_of;

    cudaStream_t origin = nullptr;
    std::vector<cudaStream_t> lanes;
    std::vector<cudaEvent_t> lane_done;
    cudaEvent_t fork = nullptr, t0 = nullptr, t1 = nullptr;
    cudaGraphExec_t exec = nullptr;
    fsr_batch_tuning tuning{};

    ~fsr_batch()
    {
        int prev = -1;
        cudaGetDevice(&prev);
        if (prev != device) cudaSetDevice(device);
        if (exec) cudaGraphExecDestroy(exec);
        for (auto s : lanes) cudaStreamDestroy(s);
        for (auto e : lane_done) cudaEventDestroy(e);
        if (origin) cudaStreamDestroy(origin);
        if (fork) cudaEventDestroy(fork);
        if (t0) cudaEventDestroy(t0);
        if (t1) cudaEventDestroy(t1);
        for (auto h : slots) fsr_destroy(h);
        if (prev >= 0 && prev != device) cudaSetDevice(prev);
    }
};

namespace {

fsr_status bfail(fsr_batch* b, fsr_status s, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    b->last_error = buf;
    return s;
}

#define BK(call)                                                                                          \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess)                                                                            \
            return bfail(b, e_ == cudaErrorMemoryAllocation ? FSR_ERR_OUT_OF_MEMORY : FSR_ERR_CUDA,       \
                         "%s: %s", #call, cudaGetErrorString(e_));                                        \
    } while (0)

#define FK(b, i, expr)                                                                                    \
    do {                                                                                                  \
        fsr_status s_ = (expr);                                                                           \
        if (s_ != FSR_OK)                                                                                 \
            return bfail(b, s_, "frame %u: %s", (unsigned)(i), b->slots[i]->last_error.c_str());         \
    } while (0)

struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(int dev)
    {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceScope()
    {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

// Longest processing time first onto the least loaded lane.
std::vector<uint32_t> assign_lanes(const std::vector<float>& cost, uint32_t lanes)
{
    std::vector<uint32_t> order(cost.size()), lane(cost.size(), 0);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t c) { return cost[a] > cost[c]; });
    std::vector<double> load(lanes, 0.0);
    for (uint32_t i : order) {
        const uint32_t l = (uint32_t)(std::min_element(load.begin(), load.end()) - load.begin());
        lane[i] = l;
        load[l] += cost[i];
    }
    return lane;
}

fsr_status ensure_lanes(fsr_batch* b, uint32_t lanes)
{
    while (b->lanes.size() < lanes) {
        cudaStream_t s = nullptr;
        cudaEvent_t e = nullptr;
        BK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        BK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        b->lanes.push_back(s);
        b->lane_done.push_back(e);
    }
    return FSR_OK;
}

// Captures the batch with the given lane assignment and instantiates it.
fsr_status capture(fsr_batch* b, uint32_t lanes, const std::vector<uint32_t>& lane_of, cudaGraphExec_t* out,
                   uint32_t* kernels)
{
    fsr_status s = ensure_lanes(b, lanes);
    if (s != FSR_OK) return s;
    const uint32_t count = (uint32_t)b->plans.size();
    BK(cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeThreadLocal));
    fsr_status err = FSR_OK;
    uint64_t k = 0;
    cudaError_t ce = cudaEventRecord(b->fork, b->origin);
    for (uint32_t l = 0; l < lanes && ce == cudaSuccess; ++l) ce = cudaStreamWaitEvent(b->lanes[l], b->fork, 0);
    for (uint32_t l = 0; l < lanes && ce == cudaSuccess && err == FSR_OK; ++l) {
        for (uint32_t i = 0; i < count && err == FSR_OK; ++i) {
            if (lane_of[i] != l) continue;
            fsr_handle* h = b->slots[i];
            err = frame_enqueue(h, b->plans[i], (const float*)h->in_xyz.ptr, (const float*)h->in_den.ptr,
                                b->lanes[l], false);
            if (err != FSR_OK) b->last_error = "frame " + std::to_string(i) + ": " + h->last_error;
            k += h->launches_frame;
        }
        if (err == FSR_OK) ce = cudaEventRecord(b->lane_done[l], b->lanes[l]);
        if (ce == cudaSuccess) ce = cudaStreamWaitEvent(b->origin, b->lane_done[l], 0);
    }
    cudaGraph_t g = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(b->origin, &g);
    if (err != FSR_OK) {
        if (g) cudaGraphDestroy(g);
        return err;
    }
    if (ce != cudaSuccess || ee != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return bfail(b, FSR_ERR_CUDA, "graph capture: %s",
                     cudaGetErrorString(ce != cudaSuccess ? ce : ee));
    }
    const cudaError_t ie = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return bfail(b, FSR_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ie));
    *kernels = (uint32_t)k;
    return FSR_OK;
}

fsr_status time_exec(fsr_batch* b, cudaGraphExec_t ex, cudaStream_t st, int reps, float* ms)
{
    BK(cudaGraphLaunch(ex, st));  // warm
    BK(cudaEventRecord(b->t0, st));
    for (int r = 0; r < reps; ++r) BK(cudaGraphLaunch(ex, st));
    BK(cudaEventRecord(b->t1, st));
    BK(cudaEventSynchronize(b->t1));
    float t = 0.f;
    BK(cudaEventElapsedTime(&t, b->t0, b->t1));
    *ms = t / reps;
    return FSR_OK;
}

// Runs every frame once on its own: sizes its buffers (capacity growth
// included) and measures it.
fsr_status size_frames(fsr_batch* b, cudaStream_t st)
{
    const uint32_t count = (uint32_t)b->plans.size();
    b->cost_ms.assign(count, 0.f);
    double total = 0.0;
    for (uint32_t i = 0; i < count; ++i) {
        fsr_handle* h = b->slots[i];
        h->grid_div = 1;
        h->block = 256;
        bool retry = true;
        for (int attempt = 0; attempt < 4 && retry; ++attempt) {
            FK(b, i, frame_buffers(h, b->plans[i]));
            BK(cudaEventRecord(b->t0, st));
            FK(b, i, frame_enqueue(h, b->plans[i], (const float*)h->in_xyz.ptr, (const float*)h->in_den.ptr, st,
                                   false));
            BK(cudaEventRecord(b->t1, st));
            BK(cudaStreamSynchronize(st));
            FK(b, i, frame_finish(h, b->plans[i], false, &retry));
        }
        if (retry) return bfail(b, FSR_ERR_OUT_OF_MEMORY, "frame %u: capacity growth did not converge", i);
        float t = 0.f;
        BK(cudaEventElapsedTime(&t, b->t0, b->t1));
        b->cost_ms[i] = t;
        total += t;
    }
    b->tuning.frames_ms = (float)total;
    return FSR_OK;
}

fsr_status plan(fsr_batch* b, uint32_t flags, cudaStream_t st)
{
    fsr_status s = size_frames(b, st);
    if (s != FSR_OK) return s;
    const uint32_t count = (uint32_t)b->plans.size();
    // candidates: (lanes, grid_div, block) -- the block shape is tried for
    // the best (lanes, grid_div) after those have been timed at 256 threads
    struct Cand {
        uint32_t lanes, grid_div, block;
    };
    std::vector<Cand> cand;
    if (flags & FSR_BATCH_NO_AUTOTUNE) {
        cand.push_back({std::min<uint32_t>(count, 8), 1, 256});
    } else {
        for (uint32_t L : {1u, 2u, 4u, 8u, 16u, 32u}) {
            if (L > count && L != 1) continue;
            for (uint32_t gd : {1u, 4u}) cand.push_back({L, gd, 256});
        }
    }
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    float best = 3.4e38f;
    uint32_t best_k = 0;
    uint32_t n_timed = 0;
    auto try_cand = [&](const Cand& c) -> fsr_status {
        for (auto h : b->slots) {
            h->grid_div = (int)c.grid_div;
            h->block = (int)c.block;
        }
        const std::vector<uint32_t> lane_of = assign_lanes(b->cost_ms, c.lanes);
        cudaGraphExec_t ex = nullptr;
        uint32_t k = 0;
        fsr_status cs = capture(b, c.lanes, lane_of, &ex, &k);
        if (cs != FSR_OK) return cs;
        float ms = 0.f;
        ++n_timed;
        if (cand.size() > 1) {
            cs = time_exec(b, ex, st, 2, &ms);
            if (cs != FSR_OK) {
                cudaGraphExecDestroy(ex);
                return cs;
            }
        }
        if (ms < best) {
            if (b->exec) cudaGraphExecDestroy(b->exec);
            b->exec = ex;
            best = ms;
            best_k = k;
            b->lane_of = lane_of;
            b->tuning.lanes = c.lanes;
            b->tuning.grid_div = c.grid_div;
            b->tuning.block_threads = c.block;
        } else {
            cudaGraphExecDestroy(ex);
        }
        return FSR_OK;
    };
    for (const auto& c : cand)
        if ((s = try_cand(c)) != FSR_OK) return s;
    if (cand.size() > 1) {
        const Cand c{b->tuning.lanes, b->tuning.grid_div, 128};
        if ((s = try_cand(c)) != FSR_OK) return s;
    }
    for (auto h : b->slots) {
        h->grid_div = (int)b->tuning.grid_div;
        h->block = (int)b->tuning.block_threads;
    }
    b->tuning.n_candidates = n_timed;
    b->tuning.kernels_per_launch = best_k;
    b->tuning.graph_ms = cand.size() > 1 ? best : 0.f;
    return FSR_OK;
}

std::vector<uint8_t> shape_of(const fsr_batch_frame* f, uint32_t count)
{
    std::vector<uint8_t> v;
    v.reserve(count * (sizeof(fsr_frame_header) + 16));
    auto put = [&](const void* p, size_t n) {
        const uint8_t* c = (const uint8_t*)p;
        v.insert(v.end(), c, c + n);
    };
    for (uint32_t i = 0; i < count; ++i) {
        put(&f[i].header, sizeof(fsr_frame_header));
        put(&f[i].method, 4);
        put(&f[i].n_particles, 8);
    }
    return v;
}

}  // namespace

extern "C" {

fsr_status fsr_batch_create(const fsr_params* params, int device, fsr_batch** out)
{
    if (!out) return FSR_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return FSR_ERR_CUDA;
    }
    fsr_batch* b = new (std::nothrow) fsr_batch();
    if (!b) return FSR_ERR_OUT_OF_MEMORY;
    b->device = device;
    for (uint32_t m = 0; m < 4; ++m) {
        if (params) {
            b->params[m] = params[m];
            if (b->params[m].method != m) {
                delete b;
                return FSR_ERR_INVALID_ARGUMENT;
            }
        } else {
            fsr_default_params(m, &b->params[m]);
        }
        b->params[m].flags &= FSR_FLAG_SMALL_POOLS;
    }
    DeviceScope g(device);
    if (cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&b->t0) != cudaSuccess || cudaEventCreate(&b->t1) != cudaSuccess) {
        cudaGetLastError();
        delete b;
        return FSR_ERR_CUDA;
    }
    *out = b;
    return FSR_OK;
}

void fsr_batch_destroy(fsr_batch* b) { delete b; }

const char* fsr_batch_last_error(const fsr_batch* b) { return b ? b->last_error.c_str() : "null batch"; }

fsr_status fsr_reconstruct_batch(fsr_batch* b, const fsr_batch_frame* frames, uint32_t count, uint32_t flags,
                                 void* stream)
{
    if (!b || (!frames && count)) return FSR_ERR_INVALID_ARGUMENT;
    if (count == 0) return bfail(b, FSR_ERR_INVALID_ARGUMENT, "empty batch");
    for (uint32_t i = 0; i < count; ++i) {
        if (frames[i].method > FSR_METHOD_AKINCI12)
            return bfail(b, FSR_ERR_INVALID_ARGUMENT, "frame %u: unknown method %u", i, frames[i].method);
        if (frames[i].n_particles && (!frames[i].xyz || !frames[i].density))
            return bfail(b, FSR_ERR_INVALID_ARGUMENT, "frame %u: null particle arrays", i);
    }
    DeviceScope g(b->device);
    cudaStream_t st = (cudaStream_t)stream;

    // frame slots and their parameters
    while (b->slots.size() < count) {
        fsr_handle* h = nullptr;
        const fsr_status s = fsr_create(&b->params[frames[b->slots.size()].method], b->device, &h);
        if (s != FSR_OK) return bfail(b, s, "frame slot %zu: fsr_create failed", b->slots.size());
        b->slots.push_back(h);
    }
    std::vector<uint8_t> shape = shape_of(frames, count);
    const bool replan = !b->exec || (flags & FSR_BATCH_RETUNE) || shape != b->shape;
    if (replan) {
        b->plans.assign(count, FramePlan{});
        b->method.assign(count, 0);
        for (uint32_t i = 0; i < count; ++i) {
            fsr_handle* h = b->slots[i];
            if (h->params.method != frames[i].method) {
                h->params = b->params[frames[i].method];
                h->cap_band = h->cap_valid = h->cap_mesh = 0;
            }
            h->frame_ready = false;
            b->method[i] = frames[i].method;
            FK(b, i, frame_plan(h, frames[i].header, frames[i].n_particles, b->plans[i]));
        }
    }
    // particles into the batch's buffers (one copy per array)
    for (uint32_t i = 0; i < count; ++i) {
        fsr_handle* h = b->slots[i];
        const uint64_t n = frames[i].n_particles, nn = std::max<uint64_t>(n, 1);
        if (h->in_xyz.bytes < 12ull * nn || h->in_den.bytes < 4ull * nn) {
            BK(cudaStreamSynchronize(st));
            BK(h->in_xyz.ensure(12ull * nn));
            BK(h->in_den.ensure(4ull * nn));
            if (b->exec) {  // the graph read the old buffers
                cudaGraphExecDestroy(b->exec);
                b->exec = nullptr;
            }
        }
        if (n) {
            BK(cudaMemcpyAsync(h->in_xyz.ptr, frames[i].xyz, 12ull * n, cudaMemcpyDefault, st));
            BK(cudaMemcpyAsync(h->in_den.ptr, frames[i].density, 4ull * n, cudaMemcpyDefault, st));
        }
    }
    if (replan || !b->exec) {
        b->shape.clear();
        const fsr_status s = plan(b, flags, st);
        if (s != FSR_OK) return s;
        b->shape = shape;
    }
    for (int attempt = 0; attempt < 4; ++attempt) {
        BK(cudaGraphLaunch(b->exec, st));
        BK(cudaStreamSynchronize(st));
        bool any = false;
        for (uint32_t i = 0; i < count; ++i) {
            bool retry = false;
            FK(b, i, frame_finish(b->slots[i], b->plans[i], false, &retry));
            if (retry) {
                FK(b, i, frame_buffers(b->slots[i], b->plans[i]));
                any = true;
            }
        }
        if (!any) return FSR_OK;
        // some frame outgrew its buffers: capture again over the grown ones
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
        uint32_t k = 0;
        const fsr_status s = capture(b, b->tuning.lanes, b->lane_of, &b->exec, &k);
        if (s != FSR_OK) return s;
        b->tuning.kernels_per_launch = k;
    }
    return bfail(b, FSR_ERR_OUT_OF_MEMORY, "capacity growth did not converge");
}

fsr_status fsr_batch_get_tuning(const fsr_batch* b, fsr_batch_tuning* out)
{
    if (!b || !out) return FSR_ERR_INVALID_ARGUMENT;
    if (!b->exec) return FSR_ERR_NOT_READY;
    *out = b->tuning;
    return FSR_OK;
}

fsr_status fsr_batch_frame_stats(const fsr_batch* b, uint32_t frame, fsr_stats* out)
{
    if (!b || !out) return FSR_ERR_INVALID_ARGUMENT;
    if (frame >= b->plans.size() || !b->exec) return FSR_ERR_NOT_READY;
    return fsr_get_stats(b->slots[frame], out);
}

fsr_status fsr_batch_mesh_device(const fsr_batch* b, uint32_t frame, const float** d_pos, const float** d_nrm,
                                 uint64_t* n_vertices)
{
    if (!b) return FSR_ERR_INVALID_ARGUMENT;
    if (frame >= b->plans.size() || !b->exec) return FSR_ERR_NOT_READY;
    return fsr_mesh_device(b->slots[frame], d_pos, d_nrm, n_vertices);
}

fsr_status fsr_batch_copy_mesh(const fsr_batch* b, uint32_t frame, float* pos, float* nrm, uint64_t capacity,
                               uint64_t* n_vertices)
{
    if (!b) return FSR_ERR_INVALID_ARGUMENT;
    if (frame >= b->plans.size() || !b->exec || !n_vertices) return FSR_ERR_NOT_READY;
    const fsr_handle* h = b->slots[frame];
    if (!h->frame_ready) return FSR_ERR_NOT_READY;
    const uint64_t nv = h->stats.n_mesh_vertices;
    *n_vertices = nv;
    if (nv > capacity) return FSR_ERR_CAPACITY;
    if (nv == 0) return FSR_OK;
    if (!pos || !nrm) return FSR_ERR_INVALID_ARGUMENT;
    DeviceScope g(b->device);
    if (cudaMemcpy(pos, h->mesh_pos.ptr, 12ull * nv, cudaMemcpyDefault) != cudaSuccess ||
        cudaMemcpy(nrm, h->mesh_nrm.ptr, 12ull * nv, cudaMemcpyDefault) != cudaSuccess) {
        cudaGetLastError();
        return FSR_ERR_CUDA;
    }
    return FSR_OK;
}

}  // extern "C"
