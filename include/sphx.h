/* sphx -- C ABI of the GB300 (sm_103a) SPH step.
 *
 * This is the boundary behind which the reference's SPHEngine::step runs on the GPU.
 * The reference has no FFI of its own for this path: its C++ SPHEngine calls the phases
 * directly (src/sph_engine.cpp:93-144) and its pybind11 module binds SPHEngine methods
 * (python/bindings.cpp:83-139).  Each entry point below names the reference interface it
 * stands in for.  Plain pointers and sizes only; no C++ or framework types cross it.
 *
 * Conventions
 *  - Every function returns SPHX_OK (0) or a negative SPHX_ERR_* code; no exception ever
 *    crosses the ABI.  sphx_strerror() turns a code into text.
 *  - One context per host thread.  A context owns all of its device memory and one CUDA
 *    stream (or uses the caller's, see sphx_set_stream).  Calls are stream-ordered:
 *    sphx_step() only enqueues work; the download/stats/time calls synchronise.
 *    Errors detected on the device are reported by the next synchronising call.
 *  - Vectors are 3 floats per particle; all host-side arrays are in insertion order
 *    (particle i is the i-th particle uploaded), like the reference's ParticleSystem.
 *  - Arithmetic is IEEE FP32 with the reference's own operation order.  In
 *    SPHX_MODE_EXACT every field of a step (neighbour lists and their order, density,
 *    pressure, acceleration, position, velocity, time) is bit-identical to the reference
 *    core built with IEEE float semantics (no FMA contraction, no fast-math).
 */
#ifndef SPHX_H
#define SPHX_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPHX_ABI_VERSION 3

/* status codes */
#define SPHX_OK 0
#define SPHX_ERR_INVALID_ARG (-1)  /* null pointer, bad size, bad parameter */
#define SPHX_ERR_OOM (-2)          /* device or pinned-host allocation failed */
#define SPHX_ERR_CUDA (-3)         /* a CUDA runtime call failed (no device, launch error) */
#define SPHX_ERR_TIMEOUT (-4)      /* a bounded device-side wait gave up */
#define SPHX_ERR_CAPACITY (-5)     /* more particles than the context's capacity */
#define SPHX_ERR_NOT_READY (-6)    /* no parameters or no particles yet */
#define SPHX_ERR_DOMAIN (-7)       /* cell grid cannot be laid out (reserved) */
#define SPHX_ERR_OVERFLOW (-8)     /* caller's output buffer too small */

/* SPHParameters (src/sph_engine.h:14-34), same fields, same order, same meaning. */
typedef struct sphx_params {
    float rest_density;
    float gas_constant;
    float viscosity;
    float smoothing_length;
    float particle_mass;
    float timestep;
    float gravity;
    float damping;
    float cfl_factor;
    float xmin, xmax, ymin, ymax, zmin, zmax;
    float neighbor_search_radius;
} sphx_params;

/* mode */
#define SPHX_MODE_EXACT 0 /* reference operation order and IEEE ops: bit-identical step */
/* Precision mode: positions stored as an integer cell (of size neighbor_search_radius)
 * plus an FP32 in-cell offset, pair distances formed from cell differences (no bits lost
 * far from the origin), Neumaier-compensated density and force sums, CFL timestep and
 * current time in FP64.  Results are judged against an FP64 evaluation, not bit for bit
 * against the reference. */
#define SPHX_MODE_PRECISE 1
#define SPHX_MODE_PRECISE_FP16 2 /* as PRECISE, offsets rounded to binary16 at every write */

/* Smoothing kernels, numbered as sph::KernelType (src/kernels.h:94-98). */
#define SPHX_KERNEL_CUBIC_SPLINE 0 /* CubicSplineKernel, the reference engine's choice */
#define SPHX_KERNEL_WENDLAND_C2 1  /* WendlandC2Kernel (src/kernels.cpp:166-200) */
#define SPHX_KERNEL_GAUSSIAN 2     /* GaussianKernel (src/kernels.cpp:203-225) */

typedef struct sphx_tuning {
    int mode;              /* SPHX_MODE_* (default EXACT) */
    int warps_per_block;   /* neighbour-pass CTA size in warps; 0 = default (4) */
    int blocks_per_sm;     /* persistent CTAs per SM for the neighbour passes; 0 = auto */
    int64_t max_grid_cells;/* cap on the dense cell grid (cells), >= 125; a larger box of
                              occupied cells is folded per axis; 0 = default */
    int profile;           /* 1 = time each phase with CUDA events (read back lazily) */
    int graph;             /* 1 = run steps as a captured CUDA graph (recaptured when n,
                              dt, parameters or scenes change) */
    int tile_particles;    /* particles of one cell per warp work item (tile), 1..32;
                              0 = default (32) */
    int bulk_copy;         /* 1 = the force pass stages candidate chunks with cp.async.bulk
                              copies into double buffers (exact mode); 0 = the lanes' own
                              loads (default) */
} sphx_tuning;

/* PerformanceStats (src/sph_engine.h:51-59) plus GPU-side diagnostics. */
typedef struct sphx_stats {
    double total_time;               /* seconds, accumulated like the reference (the
                                        time fields are filled when tuning.profile = 1) */
    double neighbor_search_time;     /* grid build: bbox, keys, sort, reorder, cells */
    double density_computation_time; /* density + pressure pass */
    double force_computation_time;   /* force pass (integration is fused into it) */
    double integration_time;         /* 0: fused into the force pass */
    uint64_t max_neighbors;          /* max |N(i)| including self, since last reset */
    uint64_t total_neighbor_queries; /* particles queried, since last reset */
    uint64_t steps;                  /* steps taken by this context */
    float current_time;              /* sum of dt (float, like SPHEngine::current_time_) */
    float last_dt;                   /* dt used by the last step */
    uint32_t occupied_cells;         /* last step: occupied search cells */
    uint32_t max_cell_occupancy;     /* last step: particles in the fullest cell */
    uint32_t nonfinite_particles;    /* last step: particles with a NaN/inf coordinate */
    uint32_t grid_cells;             /* last step: cells in the dense grid */
    /* FP64 reductions over the current state (after a step: the state it produced),
       computed by this call, not by the steps; sum_density over the densities of the
       last density pass on the current particle set (0 before one) */
    double sum_mass;
    double momentum[3];
    double kinetic_energy;           /* sum 0.5 m |v|^2 */
    double potential_energy;         /* sum -m g y (gravity acts along y) */
    double sum_density;              /* sum rho_i, FP64 (get_total_mass = sum * h^3) */
    uint64_t kernel_launches;        /* GPU kernels launched by steps/evals of this context */
    uint32_t tiles;                  /* last step: warp work items (particle tiles) */
    uint32_t spread_tiles;           /* last step, precision mode: tiles swept in their
                                        particles' own cell frames (only a folded grid
                                        yields them) */
} sphx_stats;

typedef struct sphx_ctx sphx_ctx;

/* Library ABI version (SPHX_ABI_VERSION). */
int sphx_version(void);
const char* sphx_strerror(int code);

/* Creates a context able to hold `capacity` particles on the current CUDA device.
 * Stands in for SPHEngine(size_t max_particles) (src/sph_engine.h:91, cpp:13-18).
 * tuning may be NULL (defaults). */
int sphx_create(sphx_ctx** out, size_t capacity, const sphx_tuning* tuning);
void sphx_destroy(sphx_ctx* ctx);

/* Launch on the caller's CUDA stream (a cudaStream_t passed as void*); NULL restores the
 * context's own stream. */
int sphx_set_stream(sphx_ctx* ctx, void* cuda_stream);

/* SPHEngine::initialize / set_parameters (src/sph_engine.cpp:20-33, 152-156): the step
 * uses params exactly as given (search radius = neighbor_search_radius; the 2h rule of
 * set_smoothing_length is the host engine's business). */
int sphx_set_params(sphx_ctx* ctx, const sphx_params* params);

/* Smoothing kernel of the density and force passes: the kernel create_kernel(kernel, h)
 * returns (src/kernels.cpp:226-236), evaluated per pair through the equations:: formulas
 * (src/sph_engine.cpp:370-432).  The reference engine itself always uses the cubic spline
 * (src/sph_engine.cpp:17, 23, 162); the other two are reachable there only through
 * create_kernel + equations::*, and this call is how the drop-in reaches them.  Unknown
 * kernel -> SPHX_ERR_INVALID_ARG (create_kernel throws std::invalid_argument,
 * kernels.cpp:233-234).  Cubic spline and Wendland C2 results are bit-identical to the
 * reference's; the Gaussian's exp is CUDA's expf (max 2 ulp) where the reference calls
 * the C library's expf, so its terms may differ in the last bits. */
int sphx_set_kernel(sphx_ctx* ctx, int kernel);
int sphx_get_kernel(sphx_ctx* ctx, int* kernel);

/* Replaces the particle set with n particles from host memory (the device side of
 * SPHEngine::add_particles / clear_particles, src/sph_engine.cpp:83-91).  vel may be NULL
 * (zero).  n > capacity -> SPHX_ERR_CAPACITY (the host engine applies the reference's
 * drop-with-warning rule before calling).  The acceleration used by the CFL rule for
 * particle 0 persists across uploads, as the reference's accelerations_ buffer does.
 * Pinned host buffers (cudaHostAlloc / cudaHostRegister) are read in place by the GPU,
 * over the coherent CPU-GPU link, when the stream reaches the call: keep them unchanged
 * until then.  Pageable buffers are copied before the call returns. */
int sphx_upload(sphx_ctx* ctx, size_t n, const float* pos_xyz, const float* vel_xyz,
                const float* mass);

/* SPHEngine::step(float dt) (src/sph_engine.cpp:93-144): dt <= 0 selects the CFL
 * timestep (compute_cfl_timestep, cpp:312-333), computed on the device.  A no-op when no
 * particles are loaded (cpp:94).  Asynchronous. */
int sphx_step(sphx_ctx* ctx, float dt);

/* Runs the neighbour search, density, pressure and force phases of a step on the current
 * state without integrating (positions and velocities unchanged): the state the
 * reference's compute_densities / compute_pressures / compute_forces produce
 * (src/sph_engine.cpp:203-244).  Read the result with sphx_download. */
int sphx_eval(sphx_ctx* ctx);

/* Copies fields of the current state to host memory in insertion order; synchronises.
 * SPHEngine::get_positions / get_velocities / get_densities / get_pressures
 * (src/sph_engine.h:133-136).  Any pointer may be NULL.  rho/p/acc are those of the last
 * step or eval (acc is the reference's accelerations_ buffer).  Returns the step's device
 * status (SPHX_OK, or the error a kernel recorded). */
int sphx_download(sphx_ctx* ctx, float* pos_xyz, float* vel_xyz, float* rho, float* pressure,
                  float* acc_xyz);

/* Replaces the particle set from FP64 positions (host memory).  In the precision modes
 * the cell + offset split is taken in FP64, so positions keep their bits far from the
 * origin; in SPHX_MODE_EXACT positions are rounded to float.  Parameters must be set
 * first (the cell size is the search radius). */
int sphx_upload_f64(sphx_ctx* ctx, size_t n, const double* pos_xyz, const float* vel_xyz,
                    const float* mass);
/* Current positions in FP64 (cell * cell_size + offset in the precision modes). */
int sphx_download_f64(sphx_ctx* ctx, double* pos_xyz);
/* current_time_ and the last dt in FP64 (the FP64 accumulators of the precision modes). */
int sphx_get_time_f64(sphx_ctx* ctx, double* current_time, double* last_dt);

/* ---- batched scenes --------------------------------------------------------------------
 * Splits the loaded particles into nscenes independent scenes -- contiguous ranges
 * [scene_start[s], scene_start[s+1]) of the insertion order, scene_start[0] = 0 and
 * scene_start[nscenes] = n -- each with its own parameters.  sphx_step then advances every
 * scene in one launch sequence: each scene exactly as SPHEngine::step would advance it
 * alone (its own walls, dt/CFL from its own particles and its own first particle's
 * acceleration, its own time), bit for bit; no particle meets another scene's.  The cell
 * boxes of all scenes together must fit max_grid_cells (else SPHX_ERR_DOMAIN).  Exact mode
 * only.  sphx_upload resets to a single scene; nscenes = 0 does too.  No counterpart in
 * the reference, which runs one scene per SPHEngine. */
int sphx_set_scenes(sphx_ctx* ctx, uint32_t nscenes, const uint64_t* scene_start,
                    const sphx_params* params);

typedef struct sphx_scene_stats {
    uint64_t start, count;
    float current_time;
    float last_dt;
    uint32_t grid_cells;
    uint32_t pad;
    double sum_mass;
    double momentum[3];
    double kinetic_energy;
    double potential_energy;
} sphx_scene_stats;
/* Time, dt and FP64 conservation sums of one scene after the last step (synchronises; the
 * sums are computed by this call over the current state, like sphx_get_stats'). */
int sphx_get_scene_stats(sphx_ctx* ctx, uint32_t scene, sphx_scene_stats* out);

/* Picks the neighbour passes' launch shape for the loaded workload: times two steps of
 * dt for each candidate -- warps per CTA x resident CTAs per SM, then the tile size
 * (particles per warp work item) and the force pass's staging (lane loads or bulk copies)
 * at the best of those -- restores the particles, times
 * and scene records after every trial, and keeps the fastest in the context.  Returns
 * the launch choice and its time per step (sphx_get_tuning gives all of it).
 * Synchronises.  No counterpart in the reference (its loops are OpenMP over particles). */
int sphx_autotune(sphx_ctx* ctx, float dt, int* warps_per_block, int* blocks_per_sm,
                  float* best_ms);
/* The context's current tuning (after sphx_create or sphx_autotune). */
int sphx_get_tuning(sphx_ctx* ctx, sphx_tuning* out);

/* Page-locked host memory for a caller's transfer buffers: sphx_upload reads such buffers in
 * place over the CPU-GPU link and sphx_download fills them with the copy engines at full
 * speed (pageable buffers go through staging copies).  The drop-in SPHEngine keeps its
 * host mirror's transfer buffers here.  *out = NULL and SPHX_ERR_OOM when the allocation
 * fails.  No counterpart in the reference (its particle set never leaves the host). */
int sphx_alloc_host(void** out, size_t bytes);
void sphx_free_host(void* ptr);

/* Number of particles currently loaded. */
int sphx_size(sphx_ctx* ctx, size_t* n);

/* current_time_ and the last dt (synchronises). */
int sphx_get_time(sphx_ctx* ctx, float* current_time, float* last_dt);
/* Sets current_time_ (SPHEngine::clear_particles resets it to 0, cpp:87-91). */
int sphx_set_time(sphx_ctx* ctx, float current_time);

/* get_performance_stats / reset_performance_stats (src/sph_engine.h:124-125), plus the
 * FP64 conservation sums (synchronises). */
int sphx_get_stats(sphx_ctx* ctx, sphx_stats* out);
int sphx_reset_stats(sphx_ctx* ctx);

/* Device-side copy of the current positions/velocities, and its restore: lets a caller
 * re-run steps from one state without host traffic (fresh-state benchmarking). */
int sphx_snapshot(sphx_ctx* ctx);
int sphx_restore(sphx_ctx* ctx);

/* Neighbour lists of the current state, as SpatialHash::query_squared returns them for
 * SPHEngine::update_neighbor_lists (src/spatial_hash.cpp:31-57, src/sph_engine.cpp:335-353):
 * counts[i] = |N(i)| (self included); when idx != NULL and *total_inout >= the number of
 * pairs, idx receives the concatenated lists (insertion indices) in the reference's
 * order.  On return *total_inout holds the number of pairs (SPHX_ERR_OVERFLOW when idx
 * was too small).  Test hook; synchronises.  It rebuilds the cell grid, so the
 * rho/pressure/acc fields of the previous step are no longer downloadable afterwards
 * (sphx_download returns zeros for them until the next step or eval). */
int sphx_debug_pairs(sphx_ctx* ctx, int64_t* counts, int64_t* idx, size_t* total_inout);

/* sphx_debug_pairs for the particles sel[0 .. nsel) (insertion indices, in [0, n)) only:
 * counts[q] = |N(sel[q])| and, when idx != NULL and *total_inout is large enough, their
 * lists concatenated in sel's order, each in the reference's order (the lists
 * SpatialHash::query_squared gives update_neighbor_lists, src/sph_engine.cpp:335-353).  The
 * same walk as sphx_debug_pairs; for checking samples of states too large for every list
 * at once.  Test hook; synchronises; rebuilds the cell grid like sphx_debug_pairs. */
int sphx_debug_pairs_subset(sphx_ctx* ctx, size_t nsel, const int64_t* sel, int64_t* counts,
                            int64_t* idx, size_t* total_inout);

/* ---- standalone spatial hash (SpatialHash, src/spatial_hash.h:12-88) --------------------
 * A cell grid of arbitrary positions on the GPU with the reference's query semantics:
 * sphx_grid_query returns, for every query point p, the indices j with
 * dot(p - x_j, p - x_j) <= radius_squared in the reference's order (stencil cells
 * (dx,dy,dz) in [-cr,cr]^3 lexicographically, cr = ceil(sqrt(r2) * inv_cell) + 1, then
 * insertion order), like SpatialHash::query_squared (src/spatial_hash.cpp:31-57). */
typedef struct sphx_grid sphx_grid;
int sphx_grid_create(sphx_grid** out, size_t capacity);
void sphx_grid_destroy(sphx_grid* grid);
/* SpatialHash::build (src/spatial_hash.cpp:15-25) with cells of cell_size; synchronises. */
int sphx_grid_build(sphx_grid* grid, size_t n, const float* pos_xyz, float cell_size);
/* Batched SpatialHash::query_squared: counts[nq]; idx (optional) receives the concatenated
 * lists when *total_inout is large enough (else SPHX_ERR_OVERFLOW); *total_inout returns
 * the number of entries. */
int sphx_grid_query(sphx_grid* grid, size_t nq, const float* query_xyz, float radius_squared,
                    int64_t* counts, int64_t* idx, size_t* total_inout);
/* get_total_cells / get_max_particles_per_cell (src/spatial_hash.h:58-59). */
int sphx_grid_info(sphx_grid* grid, size_t* occupied_cells, size_t* max_per_cell);
/* get_cell_particles (src/spatial_hash.cpp:59-63): insertion indices of cell (x, y, z). */
int sphx_grid_cell(sphx_grid* grid, int x, int y, int z, int64_t* idx, size_t* count_inout);

/* ---- density evaluation that allocates nothing ----------------------------------------
 * No counterpart in the reference (its step always allocates: SPHEngine resizes its
 * buffers and builds fresh neighbour vectors every step).  For callers that must not
 * allocate device memory -- an application that owns the whole device-memory budget and
 * hands libraries pointers into it, or a per-frame loop that cannot afford the device
 * synchronisation a cudaMalloc/cudaFree brings.
 *
 * Computes rho and P (compute_densities / compute_pressures, src/sph_engine.cpp:203-224)
 * of n particles, bit-identical to sphx_eval + sphx_download on a context with the default
 * (cubic-spline) kernel in exact mode.  pos_xyz (3n floats), mass
 * (n), rho (n) and pressure (n) are DEVICE pointers owned by the caller, in insertion
 * order; rho or pressure may be NULL.  Enqueued on cuda_stream (NULL: the default
 * stream) and asynchronous: results are ready when that stream reaches the call.
 * Working memory is one fixed file-scope device array inside the library (about 8 MiB,
 * held by every GPU that loads the library until exit); the function itself calls no
 * allocator.  Rules:
 *  - n > SPHX_NOALLOC_MAX_PARTICLES -> SPHX_ERR_CAPACITY, nothing launched;
 *  - occupied-cell boxes larger than SPHX_NOALLOC_MAX_CELLS cells are folded (results
 *    unchanged);
 *  - every call shares the one array: calls that overlap on the GPU (several streams or
 *    host threads at once) race and must be serialised by the caller;
 *  - the first call on a device looks up the array's device address with that device
 *    current; make that first call before any stream capture begins.  The address is
 *    kept until the process exits: calls after a cudaDeviceReset on that device are not
 *    supported;
 *  - the smoothing kernel is always the cubic spline (the reference engine's kernel);
 *  - the call does not synchronise, so an error a kernel records on the device is not
 *    returned; rho and pressure are then left as they were. */
#define SPHX_NOALLOC_MAX_PARTICLES 65536
#define SPHX_NOALLOC_MAX_CELLS 262144
int sphx_density_noalloc(const sphx_params* params, size_t n, const float* pos_xyz,
                         const float* mass, float* rho, float* pressure, void* cuda_stream);

/* ---- initial conditions generated on the device ---------------------------------------
 * Replaces the particle set (like sphx_upload) with particles generated on the GPU, shape
 * after shape in the given order, each shape's particles in its generator's order: the
 * same positions, bit for bit, as the host generators (the reference's, or the project's
 * benchmark generators), without host generation or host-to-device copies. */
#define SPHX_SHAPE_BLOCK 0   /* create_fluid_block (src/particle.cpp:166-187) */
#define SPHX_SHAPE_BOX 1     /* create_boundary_box (src/particle.cpp:189-226) */
#define SPHX_SHAPE_SPHERE 2  /* create_fluid_drop_setup's ball (src/sph_engine.cpp:492-515) */
#define SPHX_SHAPE_LATTICE 3 /* jittered lattice float32(i)*spacing + (2u-1)*jitter (+origin),
                                u = splitmix64 uniform of (seed, index, axis) */
#define SPHX_SHAPE_BALL 4    /* lattice points c + k*spacing (k integer vector, |k_a| <=
                                int(R/spacing) + 1) with |k*spacing|^2 <= R^2, in FP64 */

typedef struct {
    int kind;             /* SPHX_SHAPE_* */
    float center[3];      /* BLOCK / BOX / SPHERE centre; LATTICE origin */
    float size[3];        /* BLOCK / BOX extents; SPHERE: size[0] = radius */
    float spacing;        /* BLOCK / BOX / SPHERE / LATTICE */
    float mass;           /* every particle's mass */
    float velocity[3];    /* every particle's velocity */
    int counts[3];        /* LATTICE: nx, ny, nz (i along x outermost, k along z innermost) */
    float jitter;         /* LATTICE: 0 for none */
    uint64_t seed;        /* LATTICE */
    double ball_center[3];  /* BALL */
    double ball_radius;     /* BALL */
    double ball_spacing;    /* BALL */
} sphx_shape;

/* Total > capacity -> SPHX_ERR_CAPACITY and the particle set is left as it was.
 * n_out (may be NULL) receives the number of particles. */
int sphx_generate(sphx_ctx* ctx, size_t nshapes, const sphx_shape* shapes, size_t* n_out);

/* The reference's three scenes (SPHEngine::initialize_dam_break / _fluid_drop /
 * _granular_flow, src/sph_engine.cpp:35-71, with their arguments), particle mass given. */
#define SPHX_SCENE_DAM_BREAK 0
#define SPHX_SCENE_FLUID_DROP 1
#define SPHX_SCENE_GRANULAR_FLOW 2
int sphx_generate_scene(sphx_ctx* ctx, int scene, float particle_mass, size_t* n_out);

/* ---- headless rendering ---------------------------------------------------------------
 * The reference draws the particles with OpenGL as instanced camera-facing quads
 * (Renderer::render_particles_instanced, src/renderer.cpp:314-333) shaded by
 * shaders/particle.vert:20-40 and shaders/particle.frag:15-104.  These calls run the same
 * vertex and fragment arithmetic as CUDA kernels on the context's particle state (insertion
 * order) and write device buffers instead of a GL framebuffer.  No window, context or
 * graphics API is involved. */
#define SPHX_COLOR_VELOCITY 0 /* RenderParameters::ColorMode (src/renderer.h:43-48) */
#define SPHX_COLOR_DENSITY 1  /* the shader's placeholder: 1000 + 200 * height */
#define SPHX_COLOR_PRESSURE 2 /* the shader's placeholder: 5000 * |v| */
#define SPHX_COLOR_TYPE 3     /* the particle's own colour */

typedef struct {
    float view[16];        /* column-major (GLM / GL layout) */
    float projection[16];
    float model[16];       /* the reference passes the identity (renderer.cpp:325) */
    float particle_size;   /* RenderParameters::particle_size (default 0.01) */
    int color_mode;        /* SPHX_COLOR_* */
    int width, height;     /* image size (the viewport) */
    float background[3];   /* RenderParameters::background_color */
} sphx_render_params;

/* Camera::update_vectors + get_view_matrix + get_projection_matrix
 * (src/renderer.cpp:12-29): front from yaw / pitch (degrees), right = front x (0, 1, 0),
 * up = right x front, a right-handed look-at view and an OpenGL perspective with fov
 * (degrees), near 0.1, far 100.  Both matrices column-major. */
void sphx_camera_matrices(const float position[3], float yaw_deg, float pitch_deg,
                          float fov_deg, float aspect, float view[16], float projection[16]);

/* Per particle (insertion order), 20 floats: the 4 billboard corners in clip space (x, y,
 * z, w each; corner order (-,-), (+,-), (+,+), (-,+) as the reference's quad VBO,
 * renderer.cpp:118-123) and the fragment colour RGBA.  colors: 3 floats per particle
 * (Particle::color) or NULL for the default (0, 0.5, 1).  Host pointers; the _device form
 * takes device pointers and is asynchronous on the context's stream. */
int sphx_render_instances(sphx_ctx* ctx, const sphx_render_params* params,
                          const float* colors, float* instances);
int sphx_render_instances_device(sphx_ctx* ctx, const sphx_render_params* params,
                                 const float* colors_dev, float* instances_dev);

/* Rasterises the instances into a width x height RGBA8 image (rows bottom-up, as GL reads
 * them back): depth test GL_LESS against the cleared 1.0 (renderer.cpp:51, 275-277),
 * alpha 1 (so the enabled blending keeps the fragment colour), background where no quad
 * covers a pixel centre.  Host pointers; _device as above (rgba_dev: width*height*4
 * bytes). */
int sphx_render_image(sphx_ctx* ctx, const sphx_render_params* params, const float* colors,
                      unsigned char* rgba);
int sphx_render_image_device(sphx_ctx* ctx, const sphx_render_params* params,
                             const float* colors_dev, unsigned char* rgba_dev);

#ifdef __cplusplus
}
#endif
#endif /* SPHX_H */
