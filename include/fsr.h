/*
 * fsr.h - C ABI of the GB300 particle-to-mesh surface reconstruction library
 * (libfsr_gb300.so).  Plain C types only; every call returns an fsr_status
 * and never exits the process.
 *
 * The frame-level calls replace the reference's per-frame reconstruct path:
 *   ReconstructorGPU::reconstruct / beginFrame / frameMove / endFrame
 *     (FluidSurfaceReconstruction/GPU/ReconstructorGPU.cpp:25-148)
 *   and the stage sequences of onFrameMove in
 *     ReconstructorGPUOursZB05.cpp:22-78, ReconstructorGPUOursYu13.cpp:24-63,
 *     ReconstructorGPUAkinci12.cpp:34-84.
 * The kernel-level entry points the reference's host classes bind
 * (ReconstructionCUDA.cuh:17-248) are declared in fsr_compat.h.
 *
 * Threading: a handle is used by one host thread at a time.  Work is queued
 * on the stream passed in (NULL = the legacy default stream); calls that
 * return host-visible results synchronise that stream.
 */
#ifndef FSR_GB300_H
#define FSR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FSR_ABI_VERSION 1

typedef enum fsr_status {
    FSR_OK = 0,
    FSR_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad size or parameter */
    FSR_ERR_OUT_OF_GRID = 2,      /* a particle lies outside the expanded bounding box */
    FSR_ERR_CUDA = 3,             /* a CUDA runtime call failed; see fsr_last_error */
    FSR_ERR_OUT_OF_MEMORY = 4,    /* device or host allocation failed */
    FSR_ERR_IO = 5,               /* .xyz / .obj file could not be read or written */
    FSR_ERR_FORMAT = 6,           /* malformed .xyz file */
    FSR_ERR_CAPACITY = 7,         /* a caller-provided output buffer is too small */
    FSR_ERR_TOO_LARGE = 8,        /* grid or particle count beyond the 32-bit index space */
    FSR_ERR_NOT_READY = 9         /* no frame has been reconstructed on this handle yet */
} fsr_status;

/* Field / reconstructor families of the reference. */
typedef enum fsr_method {
    FSR_METHOD_ZB05 = 0,     /* ReconstructorGPUOursZB05: flag-grid surface + ZB05 field */
    FSR_METHOD_TC01 = 1,     /* same pipeline with the TC01 field (cu:178-227) */
    FSR_METHOD_YU13 = 2,     /* ReconstructorGPUOursYu13: anisotropic field */
    FSR_METHOD_AKINCI12 = 3  /* ReconstructorGPUAkinci12: colour-field surface + ZB05 */
} fsr_method;

/* Reconstructor settings.  fsr_default_params fills the values each
 * reference reconstructor sets in onInitialization (ZB05.cpp:85-97,
 * Yu13.cpp:78-99 and :21, Akinci12.cpp:93-106). */
typedef struct fsr_params {
    uint32_t method;             /* fsr_method */
    float iso_value;             /* SimParam.isoValue */
    uint32_t grid_ratio;         /* SimParam.scSpGridResRatio: spatial cell / scalar cell (1..1000) */
    float cell_size_scale;       /* SimParam.spatialCellSizeScale: spatial cell / h */
    float smoothing_lambda;      /* SimParam.lambdaForSmoothed (Yu13) */
    float aniso_radius_over_h;   /* SimParam.anisotropicRadius / h (Yu13: 2) */
    uint32_t min_neighbors;      /* SimParam.minNumNeighbors (Yu13: 25) */
    uint32_t flags;              /* FSR_FLAG_* */
} fsr_params;

/* Keep per-stage intermediates for fsr_debug_fetch (parity tests). */
#define FSR_FLAG_KEEP_INTERMEDIATES 0x1u
/* Record per-stage CUDA event times (fsr_stats.stage_ms). */
#define FSR_FLAG_STAGE_TIMING 0x2u
/* Start the band, valid-cube and mesh pools at a few thousand entries
 * instead of 2^20 (they grow on demand, re-running the frame once): for
 * memory-tight callers and batches of many small frames. */
#define FSR_FLAG_SMALL_POOLS 0x4u
/* Weld the triangle soup into an indexed mesh at the end of every frame
 * (fsr_copy_indexed_mesh).  The soup's vertices sit on scalar-grid edges
 * (generateTriangles, ReconstructionCUDA.cu:383-463, three unshared vertices
 * per triangle); the copies of one edge's vertex become one mesh vertex,
 * numbered in order of first use, with the position and normal of that first
 * copy.  The soup itself is unchanged. */
#define FSR_FLAG_WELD 0x8u
/* Compute each particle's density on the GPU instead of reading it (the
 * density argument may be NULL): an SPH sum with the poly6 kernel over the
 * particles within h, rho_i = m (315 / (64 pi h^3)) sum_j (1 - r_ij^2 / h^2)^3,
 * the normalisation of the reference's field kernel (anisotropicW,
 * ReconstructionCUDA.cuh:294-310).  The reference reads densities from the
 * .xyz file and computes none.  fsr_backward is not available for such
 * frames (the densities would depend on the positions). */
#define FSR_FLAG_COMPUTE_DENSITY 0x10u

/* The .xyz header (data_format.txt:1-15; ReconstructorGPU.cpp:215-251). */
typedef struct fsr_frame_header {
    float bbox_min[3];
    float bbox_max[3];
    float kernel_radius;     /* h */
    float particle_radius;
    float particle_mass;
} fsr_frame_header;

#define FSR_NUM_STAGES 12

typedef struct fsr_stats {
    uint64_t n_particles;
    uint64_t n_cells;              /* spatial cells C */
    uint64_t n_grid_vertices;      /* scalar-grid vertices V */
    uint64_t n_surface_particles;
    uint64_t n_involved_particles; /* Yu13: particles that receive a G matrix */
    uint64_t n_band_vertices;      /* B */
    uint64_t n_valid_cubes;        /* Q */
    uint64_t n_mesh_vertices;      /* 3 x triangles */
    uint32_t spatial_res[3];
    uint32_t scalar_res[3];
    uint32_t n_fp64_fallbacks;     /* Yu13: eigen-solves redone in FP64 */
    uint32_t n_retries;            /* frame re-runs after a capacity grow */
    uint32_t n_kernel_launches;    /* kernels launched by the last frame (its final attempt) */
    uint32_t n_backward_launches;  /* kernels launched by the last fsr_backward call */
    float stage_ms[FSR_NUM_STAGES];/* with FSR_FLAG_STAGE_TIMING */
    float total_ms;
    uint64_t device_bytes;         /* device memory held by the handle's pools */
    uint64_t n_weld_vertices;      /* with FSR_FLAG_WELD: vertices of the indexed mesh */
} fsr_stats;

typedef struct fsr_handle fsr_handle;

/* Library identity: ABI version and the compiled GPU architecture. */
uint32_t fsr_abi_version(void);
const char* fsr_build_info(void);

fsr_status fsr_default_params(uint32_t method, fsr_params* out);

/* Creates a reconstructor bound to CUDA device `device`.  Device memory is
 * pooled inside the handle and grows on demand; it is released by
 * fsr_destroy. */
fsr_status fsr_create(const fsr_params* params, int device, fsr_handle** out);
void fsr_destroy(fsr_handle* h);
fsr_status fsr_set_params(fsr_handle* h, const fsr_params* params);
const char* fsr_last_error(const fsr_handle* h);

/* One frame, inputs on the device: xyz = N x 3 float (x,y,z per particle,
 * the reference's ParticlePosition array), density = N floats.  The inputs
 * are read only.  The mesh stays on the device until the next frame:
 * fsr_mesh_device / fsr_copy_mesh return it.  Synchronises `stream` once at
 * the end to read the frame's sizes. */
fsr_status fsr_reconstruct(fsr_handle* h, const fsr_frame_header* hdr, const float* d_xyz,
                           const float* d_density, uint64_t n, void* stream);

/* One frame end to end from host memory: copies the particles to the
 * device, reconstructs, copies the triangle soup back (positions and
 * normals, 3 floats per mesh vertex, 3 mesh vertices per triangle, in the
 * reference's order).  *n_vertices receives the mesh vertex count; if it
 * exceeds `capacity` nothing is copied and FSR_ERR_CAPACITY is returned. */
fsr_status fsr_reconstruct_host(fsr_handle* h, const fsr_frame_header* hdr, const float* xyz,
                                const float* density, uint64_t n, float* out_pos, float* out_nrm,
                                uint64_t capacity, uint64_t* n_vertices, void* stream);

/* A sequence of frames from host memory to host memory (the reference's
 * frame loop, ReconstructorGPU.cpp:25-79: per frame beginFrame uploads the
 * particles, frameMove reconstructs, endFrame downloads the mesh, each
 * stage followed by a device synchronisation).  Frame i + 1's particles are
 * uploaded and frame i - 1's triangle soup is read back on two copy streams
 * while frame i is reconstructed on `stream`, through a second input and a
 * second mesh buffer of the handle.  Every frame gives exactly the results
 * of fsr_reconstruct_host on the same particles; on return the handle holds
 * the last frame (stats, mesh, intermediates for fsr_backward).  Stage
 * timing (FSR_FLAG_STAGE_TIMING) is not recorded.  Each frame's status and
 * vertex count are set; a frame whose mesh exceeds its capacity gets
 * FSR_ERR_CAPACITY and the others still run.  Returns FSR_OK, or the first
 * failing frame's status (an error other than FSR_ERR_CAPACITY stops the
 * sequence; the frames after it keep FSR_ERR_NOT_READY).  Pinned host
 * buffers let the copies overlap the reconstruction. */
typedef struct fsr_host_frame {
    fsr_frame_header header;
    const float* xyz;      /* n x 3 */
    const float* density;  /* n (not read with FSR_FLAG_COMPUTE_DENSITY) */
    uint64_t n;
    float* out_pos;        /* capacity x 3 */
    float* out_nrm;        /* capacity x 3 */
    uint64_t capacity;     /* mesh vertices the outputs hold */
    uint64_t n_vertices;   /* out: mesh vertices of the frame */
    fsr_status status;     /* out */
} fsr_host_frame;

fsr_status fsr_reconstruct_host_frames(fsr_handle* h, fsr_host_frame* frames, uint32_t count, void* stream);

/* Device pointers to the last frame's mesh (valid until the next frame). */
fsr_status fsr_mesh_device(fsr_handle* h, const float** d_pos, const float** d_nrm,
                           uint64_t* n_vertices);
fsr_status fsr_copy_mesh(fsr_handle* h, float* out_pos, float* out_nrm, uint64_t capacity,
                         uint64_t* n_vertices);

/* The last frame's welded mesh (FSR_FLAG_WELD): n_vertices positions and
 * normals (3 floats each) and one index per soup vertex (n_indices = 3 x
 * triangles, the soup's triangle order).  Host or device buffers.  If either
 * count exceeds its capacity nothing is copied and FSR_ERR_CAPACITY is
 * returned with both counts set. */
fsr_status fsr_copy_indexed_mesh(fsr_handle* h, float* pos, float* nrm, uint64_t vertex_capacity,
                                 uint32_t* indices, uint64_t index_capacity, uint64_t* n_vertices,
                                 uint64_t* n_indices);

/* Device-to-device copy of the last frame's mesh into caller buffers
 * (either pointer may be NULL); queued on `stream`. */
fsr_status fsr_copy_mesh_device(fsr_handle* h, float* d_pos, float* d_nrm, uint64_t capacity,
                                uint64_t* n_vertices, void* stream);

/* Backward pass of the last frame (no counterpart in the reference, which
 * has no gradients).  Given dL/d(mesh vertex positions) of a scalar loss L
 * (device, 3 floats per mesh vertex, the frame's triangle soup order), writes
 * dL/d(particle positions) (device, N x 3 floats, the frame's input order) and,
 * when grad_particle_radius is not NULL, dL/d(particle radius) (host scalar;
 * ZB05 and Akinci12, 0 for the other fields).  The frame's discrete structure
 * is held fixed: sorted order, band, valid cubes and cases, neighbourhoods and
 * isolated-particle decisions; normals are not differentiated.  Neighbour
 * sets are recomputed, not stored.  Queued on `stream`; synchronises it only
 * to return the radius gradient. */
fsr_status fsr_backward(fsr_handle* h, const float* d_grad_mesh_pos, float* d_grad_xyz,
                        float* grad_particle_radius, void* stream);

fsr_status fsr_get_stats(const fsr_handle* h, fsr_stats* out);
/* The last reconstructed frame's header (as read from its .xyz file on the
 * file-driven path). */
fsr_status fsr_get_frame_header(const fsr_handle* h, fsr_frame_header* out);

/* Intermediates of the last frame (requires FSR_FLAG_KEEP_INTERMEDIATES for
 * the arrays marked *).  With dst == NULL only *bytes_needed is set. */
typedef enum fsr_debug_array {
    FSR_DBG_SORT_PERM = 0,       /* u32[N]  input index of each sorted particle */
    FSR_DBG_SORTED_XYZ = 1,      /* f32[N*3] sorted positions */
    FSR_DBG_CELL_RANGES = 2,     /* u32[C*2] {start,end}, 0xFFFFFFFF = empty */
    FSR_DBG_SURFACE_FLAGS = 3,   /* u32[N]  surface particle flags (sorted order) */
    FSR_DBG_INVOLVED_COUNTS = 4, /* u32[C]  Yu13 involved counts per cell */
    FSR_DBG_BAND_VERTICES = 5,   /* u32[B]  band vertex ids, ascending */
    FSR_DBG_FIELD = 6,           /* f32[B]  field at the band vertices */
    FSR_DBG_MC_INFO = 7,         /* u32[B]  case | nverts << 8 | valid << 16 */
    FSR_DBG_VALID_CUBES = 8,     /* u32[Q]  positions in the band list of valid cubes */
    FSR_DBG_MEAN = 9,            /* f32[N*3] Yu13 weighted means, the reference's FP32 sums (sorted order) */
    FSR_DBG_SMOOTHED = 10,       /* f32[N*3] Yu13 smoothed positions */
    FSR_DBG_G = 11,              /* f32[N*9] Yu13 G matrices, row-major, sorted order (*) */
    FSR_DBG_WELD_KEYS = 12,      /* u64[3T] grid edge of each soup vertex, 3 x lower end point + axis
                                    (with FSR_FLAG_WELD) */
    FSR_DBG_DENSITY = 13         /* f32[N]  densities the frame used (sorted order) */
} fsr_debug_array;

fsr_status fsr_debug_fetch(fsr_handle* h, uint32_t which, void* dst, uint64_t dst_bytes,
                           uint64_t* bytes_needed);

/* Pair counts of the last frame's neighbour-sum stages, for throughput
 * accounting (a diagnostic; the reference has none).  For each stage: the
 * candidate pairs the reference's loops visit, i.e. every particle of the
 * unit's cell window (calculationOfMeanAndSmoothParticles,
 * ReconstructionCUDA.cu:598-658, and calculationOfTransformMatricesFor-
 * Particles, cu:689-827: +-2 cells per particle; computationOfScalarFieldGrid,
 * cu:830-906: +-2 cells per band vertex; updateScalarFieldValueZB05 / TC01,
 * cu:178-289, and extractionOfSurfaceParticlesUsingColorField, cu:909-971:
 * +-1 cells), and of those the pairs inside the kernel's support, whose
 * terms are non-zero.  Counted by separate brute-force kernels over the
 * frame's buffers (the frame's own kernels skip most non-contributing
 * candidates); synchronises `stream`.  Stages the method does not run are 0. */
typedef struct fsr_pair_counts {
    uint64_t smooth_candidates, smooth_contributing;  /* Yu13 smoothing: d < R */
    uint64_t cov_candidates, cov_contributing;        /* Yu13 covariance, involved particles: |x - mean| < R */
    uint64_t field_candidates, field_contributing;    /* field: |G (x~ - v)| < 1 (Yu13), d < h (ZB05, TC01) */
    uint64_t color_candidates, color_contributing;    /* Akinci12 colour field: 0 < d < h */
} fsr_pair_counts;

fsr_status fsr_count_pairs(fsr_handle* h, fsr_pair_counts* out, void* stream);

/* ---- spatial hashing without allocation ------------------------------
 *
 * No counterpart in the reference (its launchSpatialGridBuilding,
 * ReconstructionCUDA.cu:1437-1481, cudaMallocs a key array on every call).
 *
 * For callers that must not allocate device memory: an application whose
 * memory is owned by its own pool or arena, a simulation step that runs
 * where a cudaMalloc (and the device-wide synchronisation it can cause) is
 * not allowed, or a host that has reserved the device memory up front.
 * The call hashes the particles into the spatial grid of `hdr` (cell size
 * kernel_radius * cell_size_scale over the bounding box grown by one cell,
 * as fsr_reconstruct does), sorts them stably by cell and writes:
 *   d_sorted_xyz     N x 3 floats, particles in cell order
 *   d_sorted_density N floats in the same order
 *   d_cell_ranges    {start, end} per cell, 0xFFFFFFFF for empty cells;
 *                    cell_capacity is the number of cells the buffer holds
 *   d_perm           (optional) input index of each sorted particle
 *   d_out_of_grid    (optional) device word: number of particles outside the
 *                    grid (their results are meaningless when it is non-zero)
 *   *n_cells         number of cells of the grid (host)
 * Its scratch lives in a static device array sized for
 * FSR_NOALLOC_MAX_PARTICLES particles (about 4.3 MB), which every process
 * that loads the library holds on each device it uses until it exits; larger
 * n is rejected with FSR_ERR_TOO_LARGE before any GPU work.  The first call
 * on a device looks up that array's device address (cudaGetSymbolAddress);
 * make that first call before any stream capture.  The address is kept for
 * the life of the process, so a device reset (cudaDeviceReset) between calls
 * is not supported.  All calls on a device share the array: calls whose GPU
 * work overlaps (two streams, two host threads) race and corrupt each
 * other's results.  A CUDA error already pending on the calling thread makes
 * the call return FSR_ERR_CUDA at once, leaving that error pending.  It calls
 * no cudaMalloc or cudaFree; the work is queued on `stream` and nothing is
 * synchronised. */
#define FSR_NOALLOC_MAX_PARTICLES (1u << 18)

fsr_status fsr_spatial_hash_noalloc(const fsr_frame_header* hdr, float cell_size_scale,
                                    const float* d_xyz, const float* d_density, uint32_t n,
                                    float* d_sorted_xyz, float* d_sorted_density,
                                    uint32_t* d_cell_ranges, uint64_t cell_capacity, uint32_t* d_perm,
                                    uint32_t* d_out_of_grid, uint64_t* n_cells, void* stream);

/* ---- batches of frames ---------------------------------------------- */

/* Many independent frames (uneven particle counts, mixed methods) in one
 * CUDA graph launch.  The reference reconstructs one frame per call
 * (ReconstructorGPU.cpp:25-79: beginFrame / frameMove / endFrame, each
 * stage followed by a device synchronisation); a batch queues every frame's
 * kernels without host round trips, spreads the frames over `lanes`
 * concurrent streams inside the graph (size-balanced: longest frame first
 * onto the least loaded lane) and synchronises once for the whole batch.
 * Every frame gives exactly the results of fsr_reconstruct on the same
 * particles with the same parameters: batching changes no arithmetic.
 *
 * The first call with a new frame set (count, particle counts, methods,
 * headers) plans the batch: each frame runs once on its own to size its
 * buffers, then the autotuner times candidate lane counts and grid sizes
 * (grid-stride kernels launch num_sms * k / grid_div blocks) on the real
 * frames and keeps the fastest graph.  Later calls with the same shape copy
 * the new particles into the batch's buffers and replay that graph.  The
 * spatial cell size and the band width are parameters of the reconstruction
 * (they change the mesh), so the autotuner leaves them alone. */
typedef struct fsr_batch fsr_batch;

typedef struct fsr_batch_frame {
    fsr_frame_header header;
    uint32_t method;          /* fsr_method; the batch's parameters for it */
    uint32_t reserved;        /* 0 */
    uint64_t n_particles;
    const float* xyz;         /* n x 3, device or host (unified addressing) */
    const float* density;     /* n */
} fsr_batch_frame;

typedef struct fsr_batch_tuning {
    uint32_t lanes;               /* concurrent streams inside the graph */
    uint32_t grid_div;            /* grid-stride kernels: num_sms * k / grid_div blocks */
    uint32_t n_candidates;        /* configurations the autotuner timed */
    uint32_t kernels_per_launch;  /* kernel nodes in one graph launch */
    float graph_ms;               /* one graph launch (the autotuner's best) */
    float frames_ms;              /* the same frames one after another, one
                                     synchronised fsr_reconstruct-style run each */
    uint32_t block_threads;       /* threads per block of the per-item and
                                     warp-staged kernels (128 or 256) */
} fsr_batch_tuning;

/* params: four fsr_params indexed by fsr_method (NULL: fsr_default_params
 * for each); of their flags only FSR_FLAG_SMALL_POOLS is kept (no stage
 * timing or intermediates inside graphs). */
fsr_status fsr_batch_create(const fsr_params* params, int device, fsr_batch** out);
void fsr_batch_destroy(fsr_batch* b);
const char* fsr_batch_last_error(const fsr_batch* b);

#define FSR_BATCH_RETUNE 0x1u      /* plan and autotune again even if the shape is unchanged */
#define FSR_BATCH_NO_AUTOTUNE 0x2u /* plan with lanes = min(count, 8), grid_div = 1 */

/* Reconstructs frames[0 .. count).  The particles are copied (one
 * cudaMemcpyAsync per array, on `stream`) into buffers the batch owns, the
 * graph is launched on `stream`, and the call returns after that stream has
 * been synchronised once.  A frame whose band or mesh outgrew its planned
 * capacity is re-sized and the batch re-run (counted in each frame's
 * fsr_stats.n_retries).  The first failing frame's status is returned;
 * fsr_batch_last_error names it. */
fsr_status fsr_reconstruct_batch(fsr_batch* b, const fsr_batch_frame* frames, uint32_t count, uint32_t flags,
                                 void* stream);
fsr_status fsr_batch_get_tuning(const fsr_batch* b, fsr_batch_tuning* out);
fsr_status fsr_batch_frame_stats(const fsr_batch* b, uint32_t frame, fsr_stats* out);
/* Device pointers to frame `frame`'s triangle soup; valid until the next
 * fsr_reconstruct_batch or fsr_batch_destroy. */
fsr_status fsr_batch_mesh_device(const fsr_batch* b, uint32_t frame, const float** d_pos, const float** d_nrm,
                                 uint64_t* n_vertices);
/* Copies frame `frame`'s mesh to host or device memory (synchronous). */
fsr_status fsr_batch_copy_mesh(const fsr_batch* b, uint32_t frame, float* pos, float* nrm, uint64_t capacity,
                               uint64_t* n_vertices);

/* Self-check of the exact division the smoothing and covariance kernels use
 * for d / R (an FMA refinement of d x RN(1/R), Markstein's theorem): runs it
 * and __fdiv_rn on the current device for every float d in [0, 1.01 R] and
 * counts the results that differ (0 expected). */
fsr_status fsr_check_division(float R, uint64_t* n_checked, uint64_t* n_mismatch);

/* Self-check of the FP32 form of the colour field's gradient float(k x x)
 * (evaluated in double by the reference; k < 0, |k| in [1e-20, 1e30]): runs
 * it and the double expression for every float x in (0, 1] and counts the
 * results that differ (0 expected). */
fsr_status fsr_check_spiky_grad(double k, uint64_t* n_checked, uint64_t* n_mismatch);

/* Measured FP32 FMA rate of `device` in TFLOP/s (2 flops per FMA; a kernel of
 * independent FMA chains on every warp slot, best of three timed launches):
 * the denominator of the pair kernels' FP32-pipe fractions.  No counterpart
 * in the reference. */
fsr_status fsr_measure_fp32_rate(int device, double* tflops);

/* ---- file formats -------------------------------------------------- */

/* Parses an .xyz file (data_format.txt; ReconstructorGPU.cpp:200-290).
 * *xyz and *density are allocated with malloc; release them with
 * fsr_free_host. */
fsr_status fsr_read_xyz(const char* path, fsr_frame_header* hdr, float** xyz, float** density,
                        uint64_t* n);
void fsr_free_host(void* p);

/* Writes a triangle soup as .obj: v lines, vn lines, then
 * "f i//i i+1//i+1 i+2//i+2" per triangle (ReconstructorGPUOurs.cpp:58-99),
 * numbers as std::ostream prints them (%g, 6 significant digits).  Lines are
 * formatted by all I/O threads; the bytes do not depend on their number. */
fsr_status fsr_write_obj(const char* path, const float* pos, const float* nrm,
                         uint64_t n_vertices);

/* Writes an indexed mesh as .obj: one v and one vn line per vertex, then
 * "f a//a b//b c//c " per triangle with 1-based indices (the layout of
 * fsr_write_obj with shared vertices). */
fsr_status fsr_write_obj_indexed(const char* path, const float* pos, const float* nrm, uint64_t n_vertices,
                                 const uint32_t* indices, uint64_t n_indices);

/* Writes the last frame's intermediates as a .vis file, the debug dump the
 * reference's viewer reads (saveMiddleDataToVisFile:
 * ReconstructorGPUOursZB05.cpp:104-230, ReconstructorGPUOursYu13.cpp:285-420,
 * ReconstructorGPUAkinci12.cpp:290-420), same layout and number format:
 * both grids (min, max, resolution, cell size), the particle radius, the
 * particles in cell order, the occupied cells, the smoothed particles (Yu13;
 * 0 otherwise), the band vertices, the surface particles, the involved
 * particles (Yu13; 0 otherwise), the valid cubes (positions in the band
 * list), `mesh_name` and the kernel radius h. */
fsr_status fsr_write_vis(fsr_handle* h, const char* path, const char* mesh_name);

/* Host threads of fsr_read_xyz and fsr_write_obj (0, the default: one per
 * core, at most 64). */
void fsr_io_set_threads(uint32_t n);

/* .xyzb, the binary sidecar of an .xyz file: an 80-byte header (magic
 * "FSRXYZB1", u64 particle count, u64 size and i64 modification time in ns of
 * the .xyz it was made from, 9 header floats: bbox min, bbox max, h,
 * particle radius, particle mass, 12 bytes of padding), then n x 3 float
 * positions and n float densities, little-endian.  The same numbers as the
 * .xyz, read without parsing text.  Buffers as for fsr_read_xyz. */
fsr_status fsr_write_xyz_binary(const char* path, const fsr_frame_header* hdr, const float* xyz,
                                const float* density, uint64_t n);
fsr_status fsr_read_xyz_binary(const char* path, fsr_frame_header* hdr, float** xyz, float** density,
                               uint64_t* n);

/* File-driven frame loop of ReconstructorGPU::reconstruct (ReconstructorGPU.cpp:
 * 25-79): frames [from, to) of directory + printf(pattern, frame) + ".xyz",
 * each written to the same stem + ".obj" when write_obj != 0.  Per-frame
 * milliseconds (hashing to mesh, the reference's timer scope) are stored in
 * frame_ms[0 .. to-from) when frame_ms is not NULL. */
fsr_status fsr_reconstruct_files(fsr_handle* h, const char* directory, const char* pattern,
                                 uint32_t from, uint32_t to, int write_obj, double* frame_ms);

/* Flags of fsr_reconstruct_files_ex. */
#define FSR_FILES_WRITE_OBJ 0x1u /* write stem.obj per frame */
/* Read stem.xyzb instead of parsing stem.xyz when the sidecar was made from
 * the .xyz as it is now (same size and modification time); after parsing an
 * .xyz, write its sidecar (best effort). */
#define FSR_FILES_SIDECAR 0x2u
/* Write the welded mesh (fsr_write_obj_indexed) instead of the soup; the
 * handle must have FSR_FLAG_WELD. */
#define FSR_FILES_INDEXED_OBJ 0x4u
/* Write stem.vis per frame (fsr_write_vis; setOutputVisualizeFile). */
#define FSR_FILES_WRITE_VIS 0x8u

/* Host milliseconds of a file-driven run, summed over its frames.  Reading
 * and writing overlap the GPU work (frame k + 1 is read and frame k - 1's
 * .obj written while frame k runs), so wall_ms is less than the sum. */
typedef struct fsr_files_timing {
    double read_ms;        /* .xyz parse or .xyzb read */
    double upload_ms;      /* host -> device copies */
    double reconstruct_ms; /* the reference's timer scope, hashing to mesh */
    double write_ms;       /* .obj formatting and writing */
    double wall_ms;        /* the whole call */
} fsr_files_timing;

/* fsr_reconstruct_files with FSR_FILES_* flags and host timings (timing may be
 * NULL). */
fsr_status fsr_reconstruct_files_ex(fsr_handle* h, const char* directory, const char* pattern,
                                    uint32_t from, uint32_t to, uint32_t flags, double* frame_ms,
                                    fsr_files_timing* timing);

#ifdef __cplusplus
}
#endif
#endif
