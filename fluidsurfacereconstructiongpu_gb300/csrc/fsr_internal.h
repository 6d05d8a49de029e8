// The reconstructor handle: parameters, pooled device buffers and the last
// frame's bookkeeping.  Buffers only grow; they are released by
// fsr_destroy.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/fsr.h"
#include "fsr_common.cuh"

namespace fsr {

struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t want);  // contents are not preserved on growth; growth waits for the device
    void release();
};

bool derive_grids(const fsr_frame_header& hdr, const fsr_params& p, Grid& sp, Grid& sc, float* sp_max,
                  uint64_t& C, uint64_t& V);
float band_threshold(float h);
uint32_t bits_for(uint64_t c);
fsr_status run_frame(fsr_handle* h, const fsr_frame_header& hdr, const float* d_xyz, const float* d_den,
                     uint64_t n, cudaStream_t st);

// One frame in four steps, so that a batch can queue (and capture) the device
// work of many frames before it synchronises:
//   frame_plan     host checks, grids, first capacities
//   frame_buffers  grows the pooled buffers to the current capacities
//   frame_enqueue  queues every kernel of the frame on `st` and, last, the
//                  copy of the Counters block into pinned host memory; it
//                  never synchronises and allocates nothing
//   frame_finish   after the stream has been synchronised: reads the
//                  counters, sets the stats, or grows the capacities and
//                  asks for a re-run (*retry)
struct FramePlan {
    fsr_frame_header hdr{};
    Grid sp{}, sc{};
    uint64_t C = 0, V = 0;
    uint32_t n = 0, nwords = 0;
};
fsr_status frame_plan(fsr_handle* h, const fsr_frame_header& hdr, uint64_t n, FramePlan& fp);
fsr_status frame_buffers(fsr_handle* h, const FramePlan& fp);
fsr_status frame_enqueue(fsr_handle* h, const FramePlan& fp, const float* d_xyz, const float* d_den,
                         cudaStream_t st, bool timing);
fsr_status frame_finish(fsr_handle* h, const FramePlan& fp, bool timing, bool* retry);

}  // namespace fsr

struct fsr_handle {
    fsr_params params{};
    int device = 0;
    int num_sms = 1;
    std::string last_error;

    // particle-sized
    fsr::DevBuf in_xyz, in_den;          // staging for host input
    fsr::DevBuf keys0, vals0, keys1, vals1, radix_tmp;
    fsr::DevBuf sorted;                  // float4 x,y,z,density in cell order
    fsr::DevBuf psurf;                   // Akinci12 per-particle surface flags
    fsr::DevBuf mean, mean32, smoothed, grec, qrec;  // Yu13 (mean: compensated; mean32: the reference's FP32 mean)
    fsr::DevBuf covrec;                  // Yu13: normalised covariance, weight sum, neighbour-count flag
    fsr::DevBuf pflags;                  // u32 surface flags (debug)
    fsr::DevBuf rho;                     // computed densities, sorted order (FSR_FLAG_COMPUTE_DENSITY)
    // cell-sized
    fsr::DevBuf ranges, occ, surf, invol, cell_rmax;
    // vertex-sized
    fsr::DevBuf bits, prefix, scan_tmp;
    fsr::DevBuf gflag, glist;            // window groups holding band vertices: flags, list
    // band-sized
    fsr::DevBuf sv, phi, mc, vofs, valid;
    // mesh
    fsr::DevBuf mesh_pos, mesh_nrm;
    // vertex welding (FSR_FLAG_WELD)
    fsr::DevBuf wkey, wslot, wrank, widx, wpos, wnrm, wtable_keys, wtable_first;
    fsr::DevBuf ctr;
    // backward pass
    fsr::DevBuf mv;                      // ZB05/Akinci12: per band vertex (mean - v, weight sum)
    fsr::DevBuf gphi, gkey, gklist, gsmooth, gG, gmean, gx, gscalar, tri;  // gklist: keys with gradient vertices

    uint32_t cap_band = 0, cap_valid = 0, cap_mesh = 0;
    int grid_div = 1;                    // grid-stride kernels use num_sms * per_sm / grid_div blocks
    int block = 256;                     // threads per block of the per-item and warp-staged kernels
    uint64_t launches_mark = 0;
    uint32_t launches_frame = 0;
    fsr::Counters* pinned_ctr = nullptr;
    // fsr_reconstruct_host_frames: the second input and mesh buffers and
    // counters, the copy streams and their events (created on first use)
    fsr::DevBuf in_xyz_b, in_den_b, mesh_pos_b, mesh_nrm_b;
    fsr::Counters* pinned_ctr_b = nullptr;
    cudaStream_t up = nullptr, down = nullptr;
    cudaEvent_t ev_up[2] = {}, ev_done[2] = {}, ev_down[2] = {};
    cudaEvent_t ev_start = nullptr;
    cudaEvent_t ev[FSR_NUM_STAGES] = {};

    // last frame
    bool frame_ready = false;
    fsr_stats stats{};
    fsr::Grid grid_sp{}, grid_sc{};
    uint64_t n_last = 0, C_last = 0, V_last = 0;
    fsr_frame_header hdr_last{};
    const uint32_t* perm_ptr = nullptr;
    const uint32_t* skeys_ptr = nullptr;

    ~fsr_handle();
    std::vector<fsr::DevBuf*> all_buffers();
};
