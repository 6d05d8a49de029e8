// Launch wrappers of the per-frame kernels.  All are asynchronous on the
// given stream; sizes that are only known on the device (band vertices,
// valid cubes, mesh vertices) are read from Counters inside the kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "fsr_common.cuh"
#include "../../include/fsr.h"

namespace fsr {

enum class Field : int { kZB05 = 0, kTC01 = 1, kAniso = 2 };

struct KernelCtx {
    cudaStream_t stream;
    int num_sms;
    int grid_div = 1;  // grid-stride kernels launch num_sms * per_sm / grid_div blocks (batches run frames side by side)
    int block = 256;   // threads per block of the per-item and warp-staged kernels: 128 or 256 (batch autotuner)
};

// spatial hashing: keys[i] = cell id, vals[i] = i.
void launch_hash(const KernelCtx& c, const float* xyz, uint32_t n, const Grid& sp, uint32_t* keys,
                 uint32_t* vals, Counters* ctr);

// cell ranges, occupancy, sorted float4 (x,y,z,density) gather.
void launch_ranges_gather(const KernelCtx& c, const uint32_t* skeys, const uint32_t* perm, uint32_t n,
                          const float* xyz, const float* dens, float4* sorted, uint2* ranges,
                          uint8_t* occ);

// SPH (poly6) density of each sorted particle into sorted[].w (rho: n
// floats of scratch); for frames without densities (FSR_FLAG_COMPUTE_DENSITY).
void launch_density(const KernelCtx& c, float4* sorted, uint32_t n, const uint2* ranges, const Grid& sp, float h,
                    float mass, float* rho);

void launch_surface_cells(const KernelCtx& c, const Grid& sp, const uint8_t* occ, uint8_t* surf);
void launch_involved_cells(const KernelCtx& c, const Grid& sp, const uint8_t* occ, const uint8_t* surf,
                           uint8_t* invol);

// Akinci12 colour-field surface flags per sorted particle (u8).
void launch_colorfield(const KernelCtx& c, const float4* sorted, uint32_t n, const uint2* ranges,
                       const uint32_t* skeys, const Grid& sp, float h, float h2, float mass, uint8_t* psurf);

// Band stamp around surface particles.  Surface particles are those with
// psurf[i] != 0 when psurf is given, else those whose cell has surf != 0.
void launch_band_stamp(const KernelCtx& c, const float4* sorted, const uint32_t* skeys,
                       const uint8_t* surf, const uint8_t* psurf, uint32_t n, const Grid& sc,
                       float thr, uint32_t* bits, Counters* ctr);

// The band list, and the list of the window groups (spatial cells of the
// (res + 1)^3 grid the grouped field kernels walk) that hold band vertices:
// glist[0 .. ctr->n_groups), in no particular order; gflag (one word per
// group) must start at zero.
struct GroupMark {
    Grid sp, sc;
    uint32_t* gflag;
    uint32_t* glist;
};
void launch_band_list(const KernelCtx& c, const uint32_t* bits, const uint32_t* prefix, uint32_t nwords,
                      uint32_t* sv, uint32_t cap, const GroupMark& gm, Counters* ctr);

struct IsoFieldArgs {
    Grid sp, sc;
    const float4* sorted;
    const uint32_t* skeys;  // cell of each sorted particle
    const uint2* ranges;
    const uint32_t* sv;
    float* phi;
    float4* mv;  // optional (ZB05): per band vertex (mean - v, weight sum), kept for the backward pass
    const uint32_t* glist;  // groups holding band vertices (ctr->n_groups of them)
    float h, h2, inv_h2, rp;
    uint32_t cap;
};
// updateScalarFieldValueZB05 / TC01 (cu:178-289), grouped by window like the
// anisotropic field (field_aniso.cu).
void launch_field_iso_grouped(const KernelCtx& c, bool tc01, const IsoFieldArgs& a, const BandView& band,
                              uint32_t ratio, Counters* ctr);

// Yu13 smoothing: the compensated mean (w: weight sum), the reference's FP32
// mean (mean32, w: its weight sum) and the smoothed position with m/rho in w.
void launch_smooth(const KernelCtx& c, const float4* sorted, uint32_t n, const uint2* ranges, const Grid& sp,
                   float R, float lambda, float mass, float4* mean, float4* mean32, float4* smoothed);

// Smallest float x whose correctly rounded square root is >= R (> R when
// strict): sqrt_rn(d2) < R <=> d2 < sqrt_threshold(R, false) and
// sqrt_rn(d2) <= R <=> d2 < sqrt_threshold(R, true).
float sqrt_threshold(float R, bool strict);

struct CovArgs {
    Grid sp;
    const float4* sorted;
    const float4* mean;      // compensated mean (the covariance's centre), w = weight sum
    const float4* mean32;    // the reference's FP32 mean (the neighbour-count decision)
    const float4* smoothed;  // x,y,z smoothed, w = m / rho
    const uint2* ranges;
    const uint32_t* skeys;
    const uint8_t* invol;
    float4* grec;  // 4 float4 per particle: (x,y,z smoothed, r2max) (G rows, coef in row 0's w)
    float4* qrec;  // 3 float4 per particle for the field: (x~, r2max) (M00, 2M01, 2M02, coef) (M11, 2M12, M22, 0), M = G^T G
    float4* crec;  // 2 float4 per particle: (C00 C01 C02 C11) (C12 C22 W, 1 if C was used else 0)
    float* cell_rmax;  // per cell: largest support radius + smoothing shift of its particles (zeroed per frame)
    uint32_t n;
    float R, h, h2, h_inv, mass, sigma;
    uint32_t min_neighbors;
    float R_lt2, R_le2;  // squared-distance thresholds of d < R and d <= R (set by launch_cov)
    float R_rcp;         // RN(1 / R), for div_exact (set by launch_cov)
    int coop_ok;         // compact warps may walk the union of their windows (set by launch_cov)
};
void launch_cov(const KernelCtx& c, const CovArgs& a, Counters* ctr);

struct AnisoFieldArgs {
    Grid sp, sc;
    const float4* smoothed;
    const float4* grec;
    const float4* qrec;
    const uint2* ranges;
    const uint8_t* invol;
    const uint8_t* occ;
    const float* cell_rmax;
    const uint32_t* sv;
    float* phi;
    const uint32_t* glist;  // groups holding band vertices (ctr->n_groups of them)
    float sigma;
    uint32_t cap;
};
// computationOfScalarFieldGrid (cu:830-906), grouped by window (field_aniso.cu).
void launch_field_aniso_grouped(const KernelCtx& c, const AnisoFieldArgs& a, const BandView& band, uint32_t ratio,
                                Counters* ctr);

// Adjoint of the anisotropic field, grouped like the forward pass: adds
// (dL/dx~, sum dL/dphi (1 - q2)^3) to gsmooth and dL/dG rows (without the
// det(G) term) to gG; both must start at zero.  Returns false (nothing
// launched) when the grid ratio makes a group too large.
struct AnisoBwdArgs {
    Grid sp, sc;
    BandView band;
    const float4* smoothed;
    const float4* grec;
    const float4* qrec;
    const uint2* ranges;
    const uint8_t* invol;
    const float* cell_rmax;
    const float* gphi;
    uint32_t* glist;  // the keys holding gradient vertices and the work counter (BwdArgs::glist)
    float4* gsmooth;
    float4* gG;
    float sigma;
    uint32_t cap;
};
bool launch_field_aniso_backward_grouped(const KernelCtx& c, const AnisoBwdArgs& a, uint32_t ratio,
                                         const Counters* ctr);

struct McArgs {
    Grid sc;
    BandView band;
    const uint32_t* sv;
    uint32_t* mc;          // per band vertex: nverts | case << 8
    uint32_t* vofs;        // exclusive scan of nverts
    uint32_t* valid;       // valid cube list (positions in sv)
    float* out_pos;
    float* out_nrm;
    uint64_t* out_key;     // may be null: per mesh vertex, its grid edge (3 x lower end point + axis)
    float iso, fill;
    int host_mc;           // Akinci12: the host marching cubes' normal/lerp rules
    uint32_t cap_band, cap_valid, cap_mesh;
};
void launch_mc_classify(const KernelCtx& c, const McArgs& a, Counters* ctr);
// vofs, the valid cube list and the vertex / cube counts from the classify
// words (3 launches); scratch: mc_offsets_scratch_words(cap_band) words
size_t mc_offsets_scratch_words(uint32_t cap_band);
void launch_mc_offsets(const KernelCtx& c, const McArgs& a, Counters* ctr, uint32_t* scratch);
void launch_mc_generate(const KernelCtx& c, const McArgs& a, Counters* ctr);

// per-sorted-particle u32 surface flags (parity output)
void launch_particle_flags(const KernelCtx& c, const uint32_t* skeys, const uint8_t* surf,
                           const uint8_t* psurf, uint32_t n, uint32_t* out);

void upload_mc_tables(cudaStream_t s);

// Vertex welding of the triangle soup (weld.cu).
struct WeldArgs {
    const uint64_t* keys;  // per soup vertex: its grid edge (McArgs::out_key)
    const float* pos;      // soup positions and normals, 3 floats per vertex
    const float* nrm;
    uint32_t cap;          // soup capacity (the mesh pool)
    uint64_t* table_keys;  // hash table: table_size keys and first occurrences
    uint32_t* table_first;
    uint32_t table_size;   // power of two, >= 2 cap (weld_table_size)
    uint32_t shift;        // set by launch_weld
    uint32_t* slot;        // per soup vertex: its table slot
    uint32_t* rank;        // per soup vertex: first-occurrence flag, then its number
    uint32_t* index;       // out: per soup vertex, its welded vertex
    float* out_pos;        // out: welded positions and normals (first occurrences)
    float* out_nrm;
};
uint32_t weld_table_size(uint32_t cap);
// Queues the weld; the welded vertex count lands in ctr->n_weld.
cudaError_t launch_weld(const KernelCtx& c, WeldArgs a, Counters* ctr, uint32_t* scan_scratch);

// Number of kernels launched by this thread through the wrappers (the
// frame's gpu_launches figure).
extern thread_local uint64_t g_launches;

}  // namespace fsr
