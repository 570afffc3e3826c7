/*
 * fluid_gb300.h -- C ABI of libfluidgb, a GB300 (sm_103a) implementation of the
 * Position Based Fluids step and the marching-cubes surface extraction of libfluid.
 *
 * Every entry point returns an int status (FGB_OK == 0); the message of the last
 * failure on the calling thread is returned by fgb_last_error().  No C++ or torch
 * type crosses this boundary: plain pointers, sizes and POD structs only.
 *
 * Reference interface being replaced (tom91136/libfluid):
 *   include/fluid/fluid.hpp:222-232   fluid::SphSolver<T,N>::advance (pure virtual)
 *   include/fluid/oclsph.hpp:170-189  ocl::SphSolver(h, kernelPath, device)
 *   include/fluid/oclsph.hpp:661-936  ocl::SphSolver::advance (predict, grid, solve, MC)
 *   include/fluid/oclsph_type.h:6-56  ClSphConfig / ClMcConfig / ClSphTraiangle PODs
 */
#ifndef FLUID_GB300_H
#define FLUID_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FGB_VERSION 1

/* status codes */
#define FGB_OK              0
#define FGB_ERR_INVALID     1  /* bad argument or configuration */
#define FGB_ERR_CUDA        2  /* a CUDA runtime call failed */
#define FGB_ERR_OOM         3  /* device or host allocation failed */
#define FGB_ERR_CAPACITY    4  /* a size is beyond a documented maximum */
#define FGB_ERR_TIMEOUT     5  /* a bounded device-side wait gave up (error flag set) */
#define FGB_ERR_UNSUPPORTED 6
#define FGB_ERR_BUDGET      7  /* serving: request larger than the HBM budget */

/* physics profiles */
#define FGB_PROFILE_REF      0 /* reference constants and formulas (oclsph_kernel.h:20-35) */
#define FGB_PROFILE_BASELINE 1 /* textbook PBF with s_corr, XSPH and vorticity confinement */

/* particle types (fluid.hpp:18-20) */
#define FGB_TYPE_FLUID    0
#define FGB_TYPE_OBSTACLE 1

#define FGB_MAX_WELLS 16

/* Solver constants, fixed per solver like the reference's -DSPH_H build flag
 * (oclsph.hpp:178) and its compile-time constants (oclsph_kernel.h:20-35). */
typedef struct fgb_params {
    float h;                     /* smoothing length == grid cell size (solver units) */
    int32_t profile;             /* FGB_PROFILE_* */
    float rho0;                  /* rest density (ref 6378, baseline 1000) */
    float cfm_epsilon;           /* lambda relaxation (ref 600, baseline 100) */
    float corr_k;                /* s_corr k (ref 1e-4, baseline 0.1) */
    float corr_n;                /* s_corr exponent n (4) */
    float corr_delta_q;          /* s_corr delta q as a fraction of h (ref 0.3, baseline 0.2) */
    float xsph_c;                /* XSPH viscosity c (baseline 0.01; unused by ref) */
    float vorticity_epsilon;     /* vorticity confinement epsilon (baseline 5e-4; unused by ref) */
    float velocity_damping;      /* ref finalise factor VD (0.49); unused by baseline */
    float mc_particle_size;      /* ref metaball size (oclsph.hpp:672, 25) */
    float mc_particle_influence; /* ref metaball exponent (oclsph.hpp:673, 0.5) */
} fgb_params;

/* A well pulls fluid particles within 75 world units (oclsph.hpp:306-317; fluid.hpp:137-144). */
typedef struct fgb_well {
    float centre[3];
    float force;
} fgb_well;

/* Per-call configuration; mirrors fluid::Config (fluid.hpp:172-209) minus the
 * host-side vectors (sources, drains and queries stay in the C++ adapter). */
typedef struct fgb_config {
    float dt;
    float scale;
    float resolution;            /* MC samples per h (sampleResolution, oclsph.hpp:671) */
    float isolevel;
    uint32_t iterations;         /* solver iterations per step */
    uint32_t surface;            /* 1: fgb_advance also runs marching cubes */
    float constant_force[3];
    float min_bound[3];
    float max_bound[3];
    int32_t sphere_enabled;      /* analytic static sphere collider (world units) */
    float sphere[4];             /* centre xyz, radius */
    uint32_t n_wells;
    fgb_well wells[FGB_MAX_WELLS];
} fgb_config;

/* Host particle view, structure of arrays (the adapter copies fluid::Particle
 * field by field, so the ABI never depends on a GLM vector layout). */
typedef struct fgb_particles {
    size_t n;
    uint64_t *id;
    int32_t *type;
    float *mass;
    float *position;   /* 3n, xyz interleaved */
    float *velocity;   /* 3n */
    uint32_t *colour;  /* ARGB */
} fgb_particles;

/* Collider triangle (ClSphTraiangle, oclsph_type.h:47-51). */
typedef struct fgb_triangle {
    float a[3], b[3], c[3];
} fgb_triangle;

/* Surface triangle; same field order as geometry::MeshTriangle<float> (geometry.hpp:40-44). */
typedef struct fgb_mesh_triangle {
    float v[9];        /* v0, v1, v2 */
    float n[9];        /* n0, n1, n2 */
    uint32_t c[3];     /* per-vertex ARGB colour */
} fgb_mesh_triangle;

typedef struct fgb_mesh {
    fgb_mesh_triangle *triangles; /* owned by the library; release with fgb_mesh_free */
    size_t n;
    size_t capacity;
} fgb_mesh;

/* A query point and its result (fluid::Query, fluid::QueryResult: fluid.hpp:21-49). */
typedef struct fgb_query {
    uint64_t id;
    float point[3];     /* world units */
} fgb_query;
typedef struct fgb_query_result {
    uint64_t id;
    float point[3];
    uint64_t neighbours;      /* fluid particles in the point's grid cell */
    uint32_t average_colour;  /* their mean ARGB colour, each channel truncated */
} fgb_query_result;

/* The caller's array of particle records, e.g. std::vector<fluid::Particle<size_t,
 * float>> (fluid.hpp:52-62), read and written in place: field f of record i lies at
 * base + i * stride + f.  Offsets are bytes within a record (multiples of 4); id and
 * colour may be -1 (absent: the index, and 0xffffffff).  type holds FGB_TYPE_* as a
 * 4-byte integer (the fluid::Type enum); position and velocity are three floats. */
typedef struct fgb_records {
    void *base;
    size_t n;
    uint32_t stride;      /* bytes from one record to the next: a multiple of 4, at most 128 */
    uint32_t id_bytes;    /* 8 (size_t ids) or 4 */
    int32_t id, type, mass, position, velocity, colour;
} fgb_records;

typedef struct fgb_solver fgb_solver;
typedef struct fgb_batch fgb_batch;
typedef struct fgb_server fgb_server;

/* ---- library ---------------------------------------------------------- */
int fgb_version(void);
/* Message of the last failure on this thread ("" when none). */
const char *fgb_last_error(void);
/* sizeof of the ABI structs in this order: fgb_params, fgb_config, fgb_particles,
 * fgb_triangle, fgb_mesh_triangle, fgb_mesh, fgb_grid_info, fgb_well,
 * fgb_serve_options, fgb_serve_result, fgb_serve_stats, fgb_tune_result, fgb_source,
 * fgb_drain, fgb_query, fgb_query_result, fgb_records; writes at most
 * n values and returns how many exist.  Replaces the reference's check_size kernel
 * and host assert of struct layouts (oclsph_kernel.h:276-278, oclsph.hpp:217-243). */
int fgb_struct_sizes(uint64_t *out, int n);
/* Fills constants of a profile; the ref profile replaces oclsph_kernel.h:20-35. */
void fgb_params_default(fgb_params *p, int32_t profile, float h);
/* Fills a config with the reference demo's defaults (samples/main.cpp:398-411) or,
 * for the baseline profile, the dam-break workload parameters. */
void fgb_config_default(fgb_config *c, int32_t profile);

/* ---- solver: replaces ocl::SphSolver (oclsph.hpp:150-189) --------------- */
int fgb_create(const fgb_params *params, fgb_solver **out);
int fgb_destroy(fgb_solver *s);
/* Launch all work of this solver on a caller-owned cudaStream_t (NULL: the
 * library's own stream). */
int fgb_set_stream(fgb_solver *s, void *cuda_stream);
/* One frame, with the reference's contract (oclsph.hpp:661-936): xs is read,
 * advanced and written back REORDERED into Morton order; obstacles keep their
 * state; if cfg->surface, marching cubes runs and mesh_out receives triangles
 * (mesh_out may be NULL).  Host buffers in, host buffers out. */
int fgb_advance(fgb_solver *s, const fgb_config *cfg, fgb_particles *xs,
                const fgb_triangle *colliders, size_t n_colliders, fgb_mesh *mesh_out);
void fgb_mesh_free(fgb_mesh *m);
/* The reference's advance in full (oclsph.hpp:661-936) on the caller's array of
 * records, read and written in place (reordered into Morton order like fgb_advance),
 * with the frame's cell queries (oclsph.hpp:770-791): each query point's cell in the
 * step's grid (of the predicted positions), the fluid particles in it and their mean
 * colour before the step's colour diffusion; results only for points whose cell holds
 * fluid, in query order, *n_results of them (results must hold n_queries).  A point
 * outside the grid has no result.  Records are written back whole: every byte of a
 * record outside the described fields (padding) becomes zero.  Where the device
 * addresses the records directly (a coherent link) kernels read and write them;
 * elsewhere the host threads pack them.  mesh_out as in fgb_advance. */
int fgb_advance_records(fgb_solver *s, const fgb_config *cfg, fgb_records *xs,
                        const fgb_triangle *colliders, size_t n_colliders,
                        const fgb_query *queries, size_t n_queries,
                        fgb_query_result *results, size_t *n_results, fgb_mesh *mesh_out);
/* Give every page of the host range [p, p + bytes) that is not resident a frame
 * before kernels address it over a coherent link (what fgb_advance and the direct
 * downloads do to the caller's arrays): a GPU store into a page the host never wrote
 * faults to the host once per page.  keep_contents = 1 reads a byte of each such page
 * and writes the same value back (for arrays that are also inputs: swapped-out
 * memory, evicted file mappings); 0 stores a zero (outputs that a kernel overwrites
 * completely).  *touched (may be NULL) receives the number of pages touched.  Host
 * only; no counterpart in the reference, which copies through OpenCL buffers. */
int fgb_host_ready_pages(void *p, size_t bytes, int keep_contents, uint64_t *touched);

/* ---- resident scenes (a batch of one is the single-scene path) ---------- */
/* Scenes keep particles, grid and sort scratch on the device between steps.
 * All scenes of a batch share the solver constants and the iteration count. */
int fgb_batch_create(fgb_solver *s, uint32_t n_scenes, const uint64_t *counts,
                     const fgb_config *configs, fgb_batch **out);
int fgb_batch_destroy(fgb_batch *b);
int fgb_batch_upload(fgb_batch *b, uint32_t scene, const fgb_particles *xs);
/* How uploads and downloads reach the caller's arrays: 1 where kernels read and
 * write them directly (a device that addresses pageable memory through the host's
 * page tables, e.g. over Grace's coherent link), 0 where the host packs pinned
 * staging buffers (elsewhere, or with FGB_HOST_IO=staged at batch creation).
 * Both give the same bytes; uploads return once the caller's arrays are free. */
int fgb_batch_host_io(const fgb_batch *b, int *direct);
int fgb_batch_set_colliders(fgb_batch *b, uint32_t scene, const fgb_triangle *tris, size_t n);
/* Advance every scene of the batch by `steps` steps: one launch per stage for
 * all scenes, replayed from a CUDA graph. Asynchronous on the solver stream. */
int fgb_batch_step(fgb_batch *b, uint32_t steps);
/* Upload the scene table and capture, instantiate and upload the step graphs now
 * instead of in the next fgb_batch_step, so that the first step of a new batch (or
 * the first after a change of colliders, timing or launch shape) costs a plain
 * step.  Synchronous; changes no result. */
int fgb_batch_prepare(fgb_batch *b);
int fgb_batch_download(fgb_batch *b, uint32_t scene, fgb_particles *xs);
/* Marching cubes of one scene's current state; synchronous. */
int fgb_batch_surface(fgb_batch *b, uint32_t scene, fgb_mesh *mesh_out);
/* Marching cubes of every scene in one launch per stage; triangle counts only
 * (counts[n_scenes]); triangles of scene k via fgb_batch_surface_fetch. */
int fgb_batch_surface_all(fgb_batch *b, uint64_t *counts);
int fgb_batch_surface_fetch(fgb_batch *b, uint32_t scene, fgb_mesh *mesh_out);
int fgb_batch_sync(fgb_batch *b);
/* Device error flags raised by bounded waits since the last call (0: none). */
int fgb_batch_error_flags(fgb_batch *b, uint32_t *flags);
/* With FGB_ROW_STATS=1 in the environment when the batch is created, counters of the
 * checked neighbour passes (the later lambda passes and the vorticity pass) summed
 * over the steps since the last call, which clears them: [0] warps that ran on their
 * near rows, [1] warps that filtered their candidates instead, and among the particles
 * of later lambda passes that filtered, [2] those whose Verlet list held and [3] those
 * that walked their 27 cells.  Writes min(n, 4) values, zeros without FGB_ROW_STATS.
 * Synchronous. */
int fgb_batch_row_stats(fgb_batch *b, uint32_t *stats, uint32_t n);
/* Number of kernels this batch launched since creation (for accounting). */
uint64_t fgb_batch_launch_count(const fgb_batch *b);
/* Stage timing (replaces the reference's DEBUG-only clutil::Stopwatch phases,
 * oclsph.hpp:666-934): when on, every step records CUDA events between its stages
 * (predict, sort, reorder, lambda/delta per iteration, vorticity, vorticity apply);
 * fgb_batch_stage_times returns the last step's per-stage milliseconds. */
int fgb_batch_set_timing(fgb_batch *b, int on);
/* Autotuner: runs the batch's next steps under each candidate launch shape (gather
 * CTA size 64, 128, 256 at the current Verlet skin, then skins 0.1-0.3 h at the best
 * size, then persistent tile queues of 1 and 2 particles per thread, then near rows
 * with and without Verlet lists in turn (five trials); steps_per_trial steps each, the
 * first untimed), keeps the fastest, and caches
 * it in the solver for every later batch of the same physics profile and size
 * bucket (floor(log2(particles))).  The trial steps are ordinary steps: no knob
 * changes a result, so a tuned batch computes the same bits as an untuned one.
 * No counterpart in the reference (work-group sizes are left to the OpenCL
 * runtime, oclsph.hpp:597). */
typedef struct fgb_tune_result {
    uint32_t block;      /* threads per CTA of the gather kernels */
    float skin;          /* Verlet skin, in units of h */
    float ms_per_step;   /* of the chosen shape */
    uint32_t trials, steps;
    uint32_t persistent; /* 1: the gathers run as persistent grids over a tile queue */
    uint32_t particles_per_thread;  /* of a persistent grid's tiles (1 otherwise) */
    uint32_t verlet;     /* 1: steps build Verlet lists beside the near rows; 0: near rows only */
} fgb_tune_result;
int fgb_batch_autotune(fgb_batch *b, uint32_t steps_per_trial, fgb_tune_result *out);
int fgb_batch_stage_times(fgb_batch *b, float *ms, uint32_t max, uint32_t *count);

/* Parity probes: copy an internal array of the last step to host memory.
 * what: FGB_PROBE_* ; bytes must equal the array size. */
#define FGB_PROBE_KEYS        1 /* u32 sorted keys (scene << morton_bits | morton) */
#define FGB_PROBE_ORDER       2 /* u32 slot of each sorted particle (its index at upload) */
#define FGB_PROBE_CELLS       3 /* u32 pairs {start,end} per Morton key, all scenes' tables */
#define FGB_PROBE_LAMBDA      4 /* f32 lambda of the last solver iteration */
#define FGB_PROBE_DENSITY     5 /* f32 density of the last solver iteration */
#define FGB_PROBE_LATTICE     6 /* f32x4 MC lattice (value, normal) of the last surface call */
#define FGB_PROBE_CUBE_CASES  7 /* u8 MC case index per cube of the last surface call */
#define FGB_PROBE_LIST_COUNT  8 /* u16 neighbour-list length per particle (0xffff: overflow) */
#define FGB_PROBE_LIST_VALID  9 /* u8 per particle: 1 if its list served the last vorticity pass */
#define FGB_PROBE_DISPLACEMENT 10 /* f32 distance moved since the grid was built (last delta) */
#define FGB_PROBE_NEAR_ROW    11 /* u8 per particle: 1 if the last lambda pass ran over the build pass's near row */
int fgb_batch_probe_size(fgb_batch *b, uint32_t what, uint64_t *bytes);
int fgb_batch_probe(fgb_batch *b, uint32_t what, void *host_out, uint64_t bytes);
/* Grid geometry of a scene: minimum extent (solver units), cell extent,
 * table offset/size and Morton bits of the batch. */
typedef struct fgb_grid_info {
    float min_extent[3];
    uint32_t extent[3];
    uint64_t table_offset;
    uint64_t table_size;
    uint32_t morton_bits;
    uint32_t scene_bits;
    uint32_t lattice[3];      /* MC lattice samples per axis */
    float lattice_origin[3];  /* solver units */
    float lattice_step;       /* solver units */
} fgb_grid_info;
int fgb_batch_grid_info(fgb_batch *b, uint32_t scene, fgb_grid_info *out);
/* Cell queries of a resident scene against the grid of the batch's last
 * fgb_batch_step, as fgb_advance_records answers them; FGB_ERR_INVALID when an upload,
 * an edit or a surface since the step replaced that grid. */
int fgb_batch_query(fgb_batch *b, uint32_t scene, const fgb_query *queries, size_t n,
                    fgb_query_result *results, size_t *n_results);
/* Copy resident scene src_scene of src into dst_scene of dst on the device (same
 * particle count, same solver).  The particle order is kept, so the scene's later
 * steps are bit-identical to what src would have computed. */
int fgb_batch_copy_scene(fgb_batch *dst, uint32_t dst_scene, fgb_batch *src, uint32_t src_scene);

/* Sources and drains of a resident scene, applied where the particles are: the
 * reference's per-frame CPU pass over the particle vector (oclsph.hpp:675-708).
 * Each source appends floor(sqrt(rate)) x ceil(sqrt(rate)) fluid particles of mass
 * 1 on a lattice of spacing h*scale/2 in the xz plane centred on `centre`, with the
 * source's velocity, colour and tag as id; then every fluid particle (the new ones
 * included) closer than `width` to a drain's centre is removed.  Survivors keep
 * their order, the new particles follow the scene's survivors, and later scenes
 * follow as before.  Only the emitted particles cross the bus; the arrays grow on
 * the device when the batch needs more room.  *count receives the scene's new
 * particle count.  (fluid.hpp:147-169: Source, Drain.) */
typedef struct fgb_source {
    float centre[3];
    float velocity[3];
    uint64_t rate, tag;
    uint32_t colour;
} fgb_source;
typedef struct fgb_drain {
    float centre[3];
    float width, depth;  /* a particle is drained when closer than width; depth is unused, as in the reference */
} fgb_drain;
int fgb_batch_sources_drains(fgb_batch *b, uint32_t scene, const fgb_source *sources, uint32_t n_sources,
                             const fgb_drain *drains, uint32_t n_drains, uint64_t *count);
/* Device bytes one scene of n particles occupies in a batch (with its surface
 * buffers when want_mesh); used for admission against an HBM budget. */
int fgb_scene_footprint(const fgb_solver *s, const fgb_config *cfg, uint64_t n, int want_mesh, uint64_t *bytes);

/* ---- serving: a resident request loop with continuous batching ---------- */
/* A worker thread admits requests in arrival order while the sum of their device
 * footprints (fgb_scene_footprint) stays within half the budget (a membership
 * change briefly holds two batches) and keeps admitted scenes resident.  Resident
 * scenes are packed into groups of at most tick_particles particles; a tick
 * advances one group by one batched step, the groups taken round robin.  Finished
 * scenes optionally get a surface; their final state waits on the host for
 * fgb_serve_fetch.  Every request of one server must use the same iteration count.
 * While a server runs, its solver must not be used for other calls. */
#define FGB_SERVE_WAITING 0
#define FGB_SERVE_ACTIVE  1
#define FGB_SERVE_DONE    2 /* negative status: the FGB_ERR_* that failed the request */

typedef struct fgb_serve_options {
    uint64_t budget_bytes;   /* HBM budget (0: 150 GiB) */
    uint32_t max_active;     /* most resident scenes (0: 256) */
    uint32_t one_at_a_time;  /* 1: no batching, one scene at a time (the comparison loop) */
    uint64_t tick_particles; /* most particles stepped in one tick (0: 2 097 152); a
                                larger scene is stepped alone */
    uint32_t max_steps_per_tick; /* a group below half of tick_particles is advanced
                                    several steps in one tick, so that every tick does
                                    about a full group's work: at most this many (0: 16;
                                    1: one step per tick); one_at_a_time takes one */
} fgb_serve_options;

typedef struct fgb_serve_result {
    uint64_t ticket;
    uint64_t n;
    uint32_t steps;
    int32_t status;          /* FGB_SERVE_* or -FGB_ERR_* */
    uint64_t triangles;
    double t_submit, t_admit, t_done;  /* seconds since the server started */
} fgb_serve_result;

typedef struct fgb_serve_stats {
    uint64_t ticks, particle_steps, completed, rejected, failed, active, waiting;
    uint64_t used_bytes, budget_bytes, rebuilds;
    double busy_seconds, rebuild_seconds, elapsed_seconds;
} fgb_serve_stats;

int fgb_serve_create(fgb_solver *s, const fgb_serve_options *opt, fgb_server **out);
/* Copies the particles; returns a ticket. */
int fgb_serve_submit(fgb_server *sv, const fgb_config *cfg, const fgb_particles *xs, uint32_t steps,
                     int want_mesh, uint64_t *ticket);
int fgb_serve_poll(fgb_server *sv, uint64_t ticket, fgb_serve_result *out);
/* Final particles (Morton order) and mesh of a finished request; releases it. */
int fgb_serve_fetch(fgb_server *sv, uint64_t ticket, fgb_particles *xs, fgb_mesh *mesh);
int fgb_serve_get_stats(fgb_server *sv, fgb_serve_stats *out);
/* Wall time of every tick (one batched step), in seconds. */
int fgb_serve_step_latencies(fgb_server *sv, double *out, uint64_t max, uint64_t *count);
/* Particles stepped by every tick, in the order of fgb_serve_step_latencies. */
int fgb_serve_tick_particles(fgb_server *sv, uint64_t *out, uint64_t max, uint64_t *count);
/* Requests stepped by every tick, in the same order: each of them saw a step of that
 * tick's latency (the latency a request sees per step is the tick's, weighted by
 * these counts). */
int fgb_serve_tick_scenes(fgb_server *sv, uint32_t *out, uint64_t max, uint64_t *count);
/* Steps every tick advanced its group by, in the same order. */
int fgb_serve_tick_steps(fgb_server *sv, uint32_t *out, uint64_t max, uint64_t *count);
/* Start of every tick in seconds since fgb_serve_create, in the same order. */
int fgb_serve_tick_starts(fgb_server *sv, double *out, uint64_t max, uint64_t *count);
int fgb_serve_drain(fgb_server *sv, double timeout_seconds);
int fgb_serve_destroy(fgb_server *sv);

/* ---- device building blocks (device pointers, caller-provided scratch) --- */
/* Stable LSD radix sort of (key, value) u32 pairs on the low key_bits bits. */
uint64_t fgb_radix_sort_scratch_bytes(uint64_t n);
int fgb_radix_sort_pairs_u32(const uint32_t *d_keys_in, const uint32_t *d_vals_in,
                             uint32_t *d_keys_out, uint32_t *d_vals_out, uint64_t n,
                             uint32_t key_bits, void *d_scratch, uint64_t scratch_bytes,
                             void *cuda_stream);
/* Device error flags of the last fgb_radix_sort_pairs_u32 call that used this scratch
 * for n keys (0: none; bit 0: a look-back wait gave up, and the output is wrong).
 * Waits for the stream, then clears the flag. */
int fgb_radix_sort_error(const void *d_scratch, uint64_t n, void *cuda_stream, uint32_t *flags);
/* Single-pass exclusive prefix sum of u32 (decoupled look-back); writes the
 * total to d_total (device) when not NULL. */
uint64_t fgb_scan_scratch_bytes(uint64_t n);
int fgb_exclusive_scan_u32(const uint32_t *d_in, uint32_t *d_out, uint32_t *d_total, uint64_t n,
                           void *d_scratch, uint64_t scratch_bytes, void *cuda_stream);
/* Device error flags of the last fgb_exclusive_scan_u32 call that used this scratch
 * for n items (0: none; bit 1: a look-back wait gave up, and the offsets are wrong).
 * Waits for the stream, then clears the flag. */
int fgb_scan_error(const void *d_scratch, uint64_t n, void *cuda_stream, uint32_t *flags);

/* The same scan for callers that cannot allocate device memory (a host whose
 * memory manager owns every device allocation, a plugin host that forbids its
 * plugins to allocate, or a real-time loop where an allocation could block or
 * fail).  It calls no
 * cudaMalloc, cudaFree or allocating library routine: its scratch is a fixed
 * device array inside this library (about 33 KB, held by every GPU that loads the
 * library until exit), so n must not exceed FGB_SCAN_NOALLOC_MAX_N (larger n
 * returns FGB_ERR_CAPACITY).  The first call on a device looks up the array's
 * device address; make that first call before any stream capture.  All calls
 * share the array: calls that overlap on the GPU (other streams, other threads)
 * race and must be serialised by the caller.  It has no counterpart in the
 * reference, whose triangle-count reduction allocates a buffer per call. */
#define FGB_SCAN_NOALLOC_MAX_N 16777216ull
int fgb_exclusive_scan_u32_noalloc(const uint32_t *d_in, uint32_t *d_out, uint32_t *d_total, uint64_t n,
                                   void *cuda_stream);
/* Device error flags raised by fgb_exclusive_scan_u32_noalloc calls since the last
 * query (0: none; bit 1: a look-back wait gave up, and that call's offsets are
 * wrong).  Waits for the stream, then clears the flag.  Allocates nothing. */
int fgb_scan_noalloc_error(void *cuda_stream, uint32_t *flags);

/* Test hook for the bounded look-back waits of the radix sort and the scans (no
 * counterpart in the reference, which has no device-side waits).  With skip_tile !=
 * 0xffffffff, tile skip_tile of every later sort pass and scan launch never publishes
 * its status and every look-back wait gives up after spin_limit polls: the tile after
 * it raises its error flag (fgb_*_error, fgb_batch_error_flags, FGB_ERR_TIMEOUT from
 * the step calls) and returns with wrong but in-bounds output.  Nothing hangs or
 * faults.  Step graphs keep the setting they were captured with, so a batch created
 * while the hook is set keeps it.  fgb_test_lookback_fault(0xffffffff, 0) restores
 * the defaults.  Process-wide; not for production use. */
int fgb_test_lookback_fault(uint32_t skip_tile, uint32_t spin_limit);

/* ---- packed record streams (the reference demo's memory-mapped result files) --
 * Replaces strucures::writeParticles / writeTriangles (samples/structures.hpp:
 * 403-424) over mmf::writer::writePacked (include/fluid/mmf.hpp): a stream is a
 * header {int64 timestamp_ms, uint64 entries, uint64 written} followed by `entries`
 * records, every field in declaration order with no padding, little-endian:
 *   particle (44 B): u64 id, i32 type, f32 mass, u32 colour, f32 position[3],
 *                    f32 velocity[3]                  (structures.hpp particleDef)
 *   triangle (84 B): f32 v0..v2[3], f32 n0..n2[3], u32 c[3]  (meshTriangleDef)
 *   query    (32 B): u64 id, f32 point[3], u64 neighbours, u32 averageColour
 * The header is written with written = 0, then the records, then written =
 * entries, so a reader polling the mapped file sees a complete stream once written
 * equals entries.  dst == NULL asks for the size only (*bytes); a capacity below it
 * returns FGB_ERR_INVALID.  dst may be any host memory: a mapped file, a pinned
 * buffer (fastest) or pageable memory. */
#define FGB_WIRE_HEADER_BYTES 24
#define FGB_WIRE_PARTICLE_BYTES 44
#define FGB_WIRE_TRIANGLE_BYTES 84
#define FGB_WIRE_QUERY_BYTES 32
/* host arrays (e.g. what fgb_advance wrote back / returned) */
int fgb_wire_particles(const fgb_particles *xs, int64_t timestamp_ms, void *dst, uint64_t capacity,
                       uint64_t *bytes);
int fgb_wire_triangles(const fgb_mesh *mesh, int64_t timestamp_ms, void *dst, uint64_t capacity,
                       uint64_t *bytes);
/* a resident scene, packed on the device and copied to dst in one transfer; the
 * surface form streams the scene's triangles of the last fgb_batch_surface_all */
int fgb_batch_wire_particles(fgb_batch *b, uint32_t scene, int64_t timestamp_ms, void *dst, uint64_t capacity,
                             uint64_t *bytes);
int fgb_batch_wire_surface(fgb_batch *b, uint32_t scene, int64_t timestamp_ms, void *dst, uint64_t capacity,
                           uint64_t *bytes);

/* ---- vertex welding: an index buffer for a triangle soup -------------------
 * geometry::indexVBO2 (include/fluid/geometry.hpp:152-166): the vertices v0, v1,
 * v2 of each triangle in order; a position byte-identical to an earlier one reuses
 * its index, otherwise it is appended.  Output: indices[3 n] (32-bit; the
 * reference's unsigned short wraps after 65 535 vertices) and the distinct
 * positions in order of first appearance, vertices[3 * *n_vertices] (room for 9 n
 * floats must be given).  Computed on the device; the result is the sequential
 * one exactly.  The batch form welds the scene's triangles of the last
 * fgb_batch_surface_all where they lie. */
int fgb_weld_mesh(const fgb_mesh *mesh, uint32_t *indices, float *vertices, uint64_t *n_vertices);
int fgb_batch_weld_surface(fgb_batch *b, uint32_t scene, uint32_t *indices, float *vertices, uint64_t *n_vertices);

#ifdef __cplusplus
}
#endif

#endif /* FLUID_GB300_H */
