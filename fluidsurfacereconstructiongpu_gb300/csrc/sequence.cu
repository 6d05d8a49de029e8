// A sequence of frames from host memory to host memory with the copies
// overlapped (fsr_reconstruct_host_frames, include/fsr.h).
//
// Frame i is reconstructed on the caller's stream while frame i + 1's
// particles go up on one copy stream and frame i - 1's triangle soup comes
// down on another.  Two input buffers, two mesh buffers and two pinned
// counter blocks alternate between consecutive frames; every other buffer of
// the handle is used by one frame at a time, in stream order.  The host loop
// per frame i:
//   enqueue i     (waits for its upload and for the download of frame i - 2,
//                  which used the same mesh buffer)
//   finish i - 1  (waits for its kernels, reads its counters; a capacity
//                  overflow re-runs it here, on its input buffer, which is
//                  still intact) and queue its download
//   upload i + 1  (into the input buffer frame i - 1 has released)
// so each frame's copies overlap its neighbours' kernels and the host's wait
// for frame i - 1 overlaps frame i's kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <utility>
#include <vector>

#include "../../include/fsr.h"
#include "fsr_internal.h"

using namespace fsr;

namespace {

fsr_status sfail(fsr_handle* h, fsr_status s, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    h->last_error = buf;
    return s;
}

#define SCK(call)                                                                                         \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess)                                                                            \
            return sfail(h, e_ == cudaErrorMemoryAllocation ? FSR_ERR_OUT_OF_MEMORY : FSR_ERR_CUDA, "%s: %s", \
                         #call, cudaGetErrorString(e_));                                                  \
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

// The handle's alternating buffers.  Slot s of the mesh and counters is in
// the handle's primary members (mesh_pos, mesh_nrm, pinned_ctr: what
// frame_buffers, frame_enqueue and frame_finish use) when cur == s, else in
// the _b members; select(s) swaps them into place.
struct Slots {
    fsr_handle* h;
    int cur = 0;
    void select(int s)
    {
        if (cur == s) return;
        std::swap(h->mesh_pos, h->mesh_pos_b);
        std::swap(h->mesh_nrm, h->mesh_nrm_b);
        std::swap(h->pinned_ctr, h->pinned_ctr_b);
        cur = s;
    }
    const DevBuf& pos(int s) const { return cur == s ? h->mesh_pos : h->mesh_pos_b; }
    const DevBuf& nrm(int s) const { return cur == s ? h->mesh_nrm : h->mesh_nrm_b; }
    DevBuf& in_xyz(int s) { return s == 0 ? h->in_xyz : h->in_xyz_b; }
    DevBuf& in_den(int s) { return s == 0 ? h->in_den : h->in_den_b; }
};

fsr_status setup(fsr_handle* h)
{
    if (!h->pinned_ctr) SCK(cudaMallocHost(&h->pinned_ctr, sizeof(Counters)));
    if (!h->pinned_ctr_b) SCK(cudaMallocHost(&h->pinned_ctr_b, sizeof(Counters)));
    if (!h->up) SCK(cudaStreamCreateWithFlags(&h->up, cudaStreamNonBlocking));
    if (!h->down) SCK(cudaStreamCreateWithFlags(&h->down, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k) {
        if (!h->ev_up[k]) SCK(cudaEventCreateWithFlags(&h->ev_up[k], cudaEventDisableTiming));
        if (!h->ev_done[k]) SCK(cudaEventCreateWithFlags(&h->ev_done[k], cudaEventDisableTiming));
        if (!h->ev_down[k]) SCK(cudaEventCreateWithFlags(&h->ev_down[k], cudaEventDisableTiming));
    }
    return FSR_OK;
}

}  // namespace

extern "C" fsr_status fsr_reconstruct_host_frames(fsr_handle* h, fsr_host_frame* f, uint32_t count, void* stream)
{
    if (!h || (count > 0 && !f)) return FSR_ERR_INVALID_ARGUMENT;
    const bool own_density = (h->params.flags & FSR_FLAG_COMPUTE_DENSITY) != 0;
    for (uint32_t i = 0; i < count; ++i) {
        f[i].status = FSR_ERR_NOT_READY;
        f[i].n_vertices = 0;
    }
    for (uint32_t i = 0; i < count; ++i)
        if (f[i].n > 0 && (!f[i].xyz || (!f[i].density && !own_density)))
            return sfail(h, f[i].status = FSR_ERR_INVALID_ARGUMENT, "frame %u: null particle arrays", i);
    if (count == 0) return FSR_OK;
    DeviceScope guard(h->device);
    fsr_status s = setup(h);
    if (s != FSR_OK) return s;
    cudaStream_t st = (cudaStream_t)stream;
    h->frame_ready = false;
    Slots sl{h, 0};
    std::vector<FramePlan> plan(count);
    fsr_status first = FSR_OK;
    auto note = [&](uint32_t i, fsr_status e) {
        f[i].status = e;
        if (first == FSR_OK) first = e;
    };

    auto upload = [&](uint32_t i) -> fsr_status {
        const int b = (int)(i & 1u);
        const uint64_t nn = std::max<uint64_t>(f[i].n, 1);
        SCK(sl.in_xyz(b).ensure(12ull * nn));
        SCK(sl.in_den(b).ensure(4ull * nn));
        if (f[i].n) {
            SCK(cudaMemcpyAsync(sl.in_xyz(b).ptr, f[i].xyz, 12ull * f[i].n, cudaMemcpyHostToDevice, h->up));
            if (!own_density)
                SCK(cudaMemcpyAsync(sl.in_den(b).ptr, f[i].density, 4ull * f[i].n, cudaMemcpyHostToDevice, h->up));
        }
        SCK(cudaEventRecord(h->ev_up[b], h->up));
        return FSR_OK;
    };
    // queues frame i's kernels on st (its input is up and its mesh buffer is free)
    auto enqueue = [&](uint32_t i) -> fsr_status {
        const int b = (int)(i & 1u);
        fsr_status e = frame_plan(h, f[i].header, f[i].n, plan[i]);
        if (e != FSR_OK) return e;
        sl.select(b);
        if ((e = frame_buffers(h, plan[i])) != FSR_OK) return e;
        SCK(cudaStreamWaitEvent(st, h->ev_up[b], 0));
        SCK(cudaStreamWaitEvent(st, h->ev_down[b], 0));
        if ((e = frame_enqueue(h, plan[i], (const float*)sl.in_xyz(b).ptr, (const float*)sl.in_den(b).ptr, st,
                               false)) != FSR_OK)
            return e;
        SCK(cudaEventRecord(h->ev_done[b], st));
        return FSR_OK;
    };
    uint32_t last_enqueued = 0;
    // waits for frame i, reads its counters (re-running it on a capacity
    // overflow) and queues the download of its mesh
    auto finish = [&](uint32_t i) -> fsr_status {
        const int b = (int)(i & 1u);
        SCK(cudaEventSynchronize(h->ev_done[b]));
        sl.select(b);
        bool retry = false;
        fsr_status e = frame_finish(h, plan[i], false, &retry);
        for (int attempt = 0; e == FSR_OK && retry; ++attempt) {
            if (attempt == 4) return sfail(h, FSR_ERR_OUT_OF_MEMORY, "capacity growth did not converge");
            // the next frame may still run on st: let it finish first (it is
            // re-run at its own finish if it overflowed too)
            SCK(cudaStreamSynchronize(st));
            if ((e = enqueue(i)) != FSR_OK) return e;
            last_enqueued = i;
            SCK(cudaStreamSynchronize(st));
            sl.select(b);
            e = frame_finish(h, plan[i], false, &retry);
        }
        if (e != FSR_OK) return e;
        const uint64_t nv = h->stats.n_mesh_vertices;
        f[i].n_vertices = nv;
        if (nv > f[i].capacity) {
            note(i, sfail(h, FSR_ERR_CAPACITY, "frame %u: mesh has %llu vertices, buffer holds %llu", i,
                          (unsigned long long)nv, (unsigned long long)f[i].capacity));
            return FSR_OK;
        }
        if (nv && (!f[i].out_pos || !f[i].out_nrm)) {
            note(i, sfail(h, FSR_ERR_INVALID_ARGUMENT, "frame %u: null mesh output", i));
            return FSR_OK;
        }
        SCK(cudaStreamWaitEvent(h->down, h->ev_done[b], 0));
        if (nv) {
            SCK(cudaMemcpyAsync(f[i].out_pos, sl.pos(b).ptr, 12ull * nv, cudaMemcpyDeviceToHost, h->down));
            SCK(cudaMemcpyAsync(f[i].out_nrm, sl.nrm(b).ptr, 12ull * nv, cudaMemcpyDeviceToHost, h->down));
        }
        SCK(cudaEventRecord(h->ev_down[b], h->down));
        f[i].status = FSR_OK;
        return FSR_OK;
    };
    auto drain = [&]() {
        cudaStreamSynchronize(st);
        cudaStreamSynchronize(h->up);
        cudaStreamSynchronize(h->down);
    };

    // the events of the previous call (if any) have completed; record fresh
    // ones so that the first waits are satisfied
    for (int k = 0; k < 2; ++k) {
        SCK(cudaEventRecord(h->ev_down[k], h->down));
        SCK(cudaEventRecord(h->ev_up[k], h->up));
    }
    if ((s = upload(0)) != FSR_OK) {
        drain();
        note(0, s);
        return first;
    }
    for (uint32_t i = 0; i < count; ++i) {
        if ((s = enqueue(i)) != FSR_OK) {
            drain();
            note(i, s);
            return first;
        }
        last_enqueued = i;
        if (i > 0 && (s = finish(i - 1)) != FSR_OK) {
            drain();
            note(i - 1, s);
            return first;
        }
        if (i + 1 < count && (s = upload(i + 1)) != FSR_OK) {
            drain();
            note(i + 1, s);
            return first;
        }
    }
    if ((s = finish(count - 1)) != FSR_OK) {
        drain();
        note(count - 1, s);
        return first;
    }
    // a re-run of an earlier frame after the last one was queued left its own
    // intermediates in the handle: run the last frame again so that the
    // handle holds it
    if (last_enqueued != count - 1) {
        SCK(cudaStreamSynchronize(h->down));
        const int b = (int)((count - 1) & 1u);
        if ((s = enqueue(count - 1)) == FSR_OK) {
            SCK(cudaStreamSynchronize(st));
            sl.select(b);
            bool retry = false;
            s = frame_finish(h, plan[count - 1], false, &retry);
        }
        if (s != FSR_OK) {
            drain();
            note(count - 1, s);
            return first;
        }
    }
    SCK(cudaStreamSynchronize(h->down));
    sl.select((int)((count - 1) & 1u));
    return first;
}
