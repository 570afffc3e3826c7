// fgb_internal.h -- host-side declarations shared by the library's translation units.
#pragma once

#include <cstdint>
#include <functional>
#include <cuda_runtime.h>

#include "../../include/fluid_gb300.h"
#include "fgb_device.cuh"

namespace fgb {

// Thread-local last-error message behind fgb_last_error(); both return `code`.
int fail(int code, const char *msg);
int fail_cuda(cudaError_t e, const char *where);

// Morton key bits of one scene's grid under a solver's h (runtime.cu).
uint32_t scene_morton_bits(const fgb_solver *s, const fgb_config *cfg);

// radix sort (sort.cu)
uint64_t radix_scratch_bytes(uint64_t n);
int radix_passes(uint32_t key_bits);
cudaError_t radix_sort_pairs(const uint32_t *keys_in, const uint32_t *vals_in, uint32_t *keys_out,
                             uint32_t *vals_out, uint64_t n, uint32_t key_bits, void *scratch,
                             uint64_t scratch_bytes, cudaStream_t stream, uint32_t *err, uint64_t *launches);

// Copy a device error-flag word to *flags and clear it, after the work queued on
// stream (synchronises the stream; allocates nothing).
int read_clear_flag(void *d_flag, cudaStream_t stream, uint32_t *flags, const char *where);

// prefix scan of a u32 array (scan.cu)
uint64_t scan_u32_scratch_bytes(uint64_t n);
cudaError_t scan_u32(const uint32_t *in, uint32_t *out, uint32_t *total, uint64_t n, void *scratch,
                     uint64_t scratch_bytes, cudaStream_t stream, uint32_t *err, uint64_t *launches);

// PBF stages (pbf.cu).  Arrays are indexed by particle over the whole batch.
struct HostParticlesOut;

struct StepView {
    const SceneDev *scenes;
    const WellDev *wells;
    const TriDev *tris;
    uint32_t n;
    uint32_t mbits;
    Phys ph;
    // state at step start (current order)
    const float4 *x0, *v0;
    const int32_t *type0;
    const uint32_t *col0, *slot0;
    // state in sorted order
    float4 *x1, *v1;
    int32_t *type1;
    uint32_t *col1, *slot1;
    // step temporaries
    uint32_t *keys_prev;   // sorted keys of the previous step (scene id in the high bits)
    uint32_t *keys_in, *vals_in, *keys_sorted, *vals_sorted;
    uint2 *cells;
    uint64_t cells_n;
    float4 *ps_a, *ps_b;
    float *lambda, *density;
    // the lambda pass's p* with lambda in w (the delta pass's neighbour reads; null: off)
    float4 *plam;
    // the vorticity pass's p* with |omega| in w (the apply pass's neighbour reads; null: off)
    float4 *pom;
    // {smallest mass, ~largest mass} as float bits, set by the grid build of each step
    uint32_t *mass_range;
    float4 *omega, *vx;
    uint32_t *err;
    int block;             // threads per CTA of the gather kernels
    // persistent gathers (null: flat grids): one zeroed tile counter per gather launch
    // of the step (slots_of_step), ppt particles per thread of a tile
    uint32_t *queue;
    uint32_t ppt;
    uint32_t verlet_off;  // build near rows but no Verlet lists
    // {1 while steps build Verlet lists, movers of the step} (null: lists every step)
    uint32_t *list_policy;
    uint32_t list_min_use;  // percent of a pass's particles that keeps lists on
    uint32_t n_scenes;
    uint32_t iterations;
    int sm_count;
    // per-step neighbour lists (Verlet lists with a skin), particle-major rows of cap
    // entries (cap a multiple of 4): list[a * cap + j]
    uint32_t *nlist;       // n * cap candidate indices, in 27-cell walk order
    uint16_t *ncount;      // entries per particle (kListOverflow: walk the cells)
    uint32_t cap;          // list capacity per particle (0: lists disabled)
    float list_r2;         // (h + skin)^2: candidates kept at build time
    float skin;            // a list stays exact while disp_a + max disp_b <= skin
    float4 *ps_grid;       // p* at grid build (displacements are measured from it)
    float *disp;           // |p - p_grid| per particle after the last delta pass
    uint32_t *cellmax;     // max displacement (float bits) per cell, same index as cells
    uint8_t *valid;        // per particle: 1 if its list is exact for the current positions
    // per-pass hit lists: the candidates of one pass that lie within h (and not on top
    // of the particle), in walk order; written by a lambda / vorticity pass, read by the
    // delta / vorticity-apply pass over the same positions.  Rows like nlist.
    uint32_t *hlist;       // n * hcap
    uint16_t *hcount;      // entries per particle (kListOverflow: use nlist / the cells)
    uint32_t hcap;
    // near rows: the build pass's hit row keeps every candidate within h + near_skin;
    // near[a] = 1 while particle a's row is that row (null: near rows off)
    uint8_t *near;
    float near_r2;         // (h + near_skin)^2, rounded up
    float near_skin;
    // the step's last kernel also stores each particle's final position and velocity
    // into these host arrays (device-resident pointers, null: no host stores)
    const HostParticlesOut *hout;
    // the build pass counts the Verlet rows [0] and hit rows [1] that overflowed
    uint32_t *over;
    // null, or [0] warps of the checked passes that ran on their near rows and [1]
    // warps that filtered their candidates instead (accumulated until read)
    uint32_t *near_stats;
};


constexpr uint16_t kListOverflow = 0xffffu;
// k_list_policy's words per scene: [0] 1 while steps build the scene's Verlet lists and
// near rows; counts of the current step: [1] fluid particles that its last delta pass
// moved more than half the skin, [2] all fluid particles of that pass, [3] particles of
// its second lambda pass that ran on a near row or a list that held, [4] those that
// walked; [5] steps since the lists were turned off.
constexpr uint32_t kPolicyWords = 6;

void launch_fill_u32(uint32_t *p, uint64_t n, uint32_t value, cudaStream_t st);
void launch_iota_u32(uint32_t *p, uint64_t n, cudaStream_t st);  // p[i] = i
void launch_predict_keys(const StepView &s, cudaStream_t st);
void launch_reorder_cells(const StepView &s, cudaStream_t st);
void launch_lambda(const StepView &s, const float4 *ps, int iteration, cudaStream_t st);
// at the end of a step: whether the next one builds Verlet lists
void launch_list_policy(const StepView &s, cudaStream_t st);
// tile counters a step's gather launches use (persistent gathers)
uint32_t slots_of_step(uint32_t iterations);
void launch_delta(const StepView &s, const float4 *ps_in, float4 *ps_out, int iteration, bool last,
                  cudaStream_t st);
// ref-profile colour diffusion of the sorted colours (col1, in place); agg and count
// are n-entry scratch arrays
void launch_diffuse(const StepView &s, uint4 *agg, uint32_t *count, cudaStream_t st);
// `between` runs after the first of the two kernels (stage timing hook)
void launch_velocity_terms(const StepView &s, const float4 *ps, cudaStream_t st,
                           const std::function<void()> &between = nullptr);
// keys of the current positions (marching-cubes grid); ps_a receives solver-unit
// positions in sorted order, cells the table
void launch_position_keys(const StepView &s, const float4 *x, cudaStream_t st);
void launch_gather_positions(const StepView &s, const float4 *x, const int32_t *type, const uint32_t *col,
                             float4 *xs_sorted, int32_t *type_sorted, uint32_t *col_sorted, cudaStream_t st);

// Device arrays of one resident scene (current state, sorted order; the scene is
// [first, first + n) of each array) and the triangles of its last fgb_batch_surface_all
// (tris == nullptr before one).  Used by the record packers of wire.cu.
struct ResidentScene {
    uint64_t first, n;
    const float4 *x, *v;
    const int32_t *type;
    const uint32_t *col, *slot;
    const uint64_t *ids;  // by upload slot, indexed first + slot
    cudaStream_t stream;
    const fgb_mesh_triangle *tris;
    uint64_t tri_count;
};
int batch_resident(fgb_batch *b, uint32_t scene, ResidentScene *out);
void *batch_wire_scratch(fgb_batch *b, uint64_t bytes);  // device staging, grown on demand

// sources and drains of a resident scene (edit.cu)
struct SceneMove {
    uint64_t first_old, first_new;  // a scene's first particle before and after the edit
};
void launch_drain_flags(uint64_t n, uint32_t mbits, uint32_t scene, const uint32_t *keys, const float4 *x,
                        const int32_t *type, const fgb_drain *drains, uint32_t n_drains, uint32_t *keep,
                        cudaStream_t st);
void launch_edit_scatter(uint64_t n, uint32_t mbits, uint32_t scene, uint64_t emitted, const uint32_t *keys,
                         const uint32_t *keep, const uint32_t *rank, const SceneMove *moves, const float4 *x0,
                         const float4 *v0, const int32_t *t0, const uint32_t *c0, const uint32_t *s0,
                         const uint64_t *ids0, float4 *x1, float4 *v1, int32_t *t1, uint32_t *c1, uint32_t *s1,
                         uint64_t *ids1, cudaStream_t st);

// particles between the caller's host arrays and a scene segment, read and written
// by kernels directly (hostio.cu); only where the device addresses pageable memory
struct HostParticlesIn {
    const float *position, *velocity, *mass;  // position/velocity: 3 floats a particle
    const int32_t *type;
    const uint32_t *colour;  // may be null: 0xffffffff
    const uint64_t *id;      // may be null: the index
};
struct HostParticlesOut {  // any may be null: not written
    float *position, *velocity, *mass;
    int32_t *type;
    uint32_t *colour;
    uint64_t *id;
    // 0: the arrays above are packed (structure of arrays).  Otherwise they address
    // the fields of record 0 of the caller's array of records, record i's fields sit
    // i * stride bytes further, and the id field is id_bytes (4 or 8) wide
    uint32_t stride = 0, id_bytes = 8;
};
// The caller's array of records (e.g. fluid::Particle): field f of record i at
// base + i * stride + off_f; a negative offset marks an absent field (colour: all
// ones, id: the index).  stride and every offset are multiples of 4.
struct HostRecords {
    char *base;
    uint32_t stride, id_bytes;
    int32_t off_id, off_type, off_mass, off_position, off_velocity, off_colour;
};
constexpr uint32_t kMaxRecordStride = 128;  // bytes; the upload stages a tile of records in shared memory
void launch_pack_records(const HostRecords &in, uint64_t n, float4 *x, float4 *v, int32_t *type, uint32_t *col,
                         uint32_t *slot, uint64_t *ids, uint32_t *obstacles, cudaStream_t st);
// the step's final sorted state into whole records (every byte not in a described
// field zero)
void launch_unpack_records(const HostRecords &out, uint64_t n, const float4 *x, const float4 *v, const int32_t *type,
                           const uint32_t *col, const uint32_t *slot, const uint64_t *ids, cudaStream_t st);
// the HostParticlesOut of a HostRecords (stride set)
HostParticlesOut record_fields(const HostRecords &r, bool motion, bool fixed);

// Cell queries against the grid of a batch's last step (query.cu): for each point,
// the fluid particles in its grid cell and their mean ARGB colour, before the
// step's colour diffusion (include/fluid/oclsph.hpp:770-791).
void launch_queries(const SceneDev *scenes, uint32_t scene, float h, const uint2 *cells, const int32_t *type_sorted,
                    const uint32_t *order, const uint32_t *colour_prev, const fgb_query *q, uint32_t nq,
                    uint32_t *count, uint32_t *argb, cudaStream_t st);
void launch_pack_from_host(const HostParticlesIn &in, uint64_t n, float4 *x, float4 *v, int32_t *type, uint32_t *col,
                           uint32_t *slot, uint64_t *ids, uint32_t *obstacles, cudaStream_t st);
void launch_unpack_to_host(const HostParticlesOut &out, uint64_t n, const float4 *x, const float4 *v,
                           const int32_t *type, const uint32_t *col, const uint32_t *slot, const uint64_t *ids,
                           cudaStream_t st);
// an upload in two parts: what the prediction and the sort read (positions,
// velocities, masses, types; obstacles counted into *obstacles) and what only the
// reorder reads (colours, ids, upload slots)
void launch_pack_motion(const HostParticlesIn &in, uint64_t n, float4 *x, float4 *v, int32_t *type,
                        uint32_t *obstacles, cudaStream_t st);
void launch_pack_static(const HostParticlesIn &in, uint64_t n, uint32_t *col, uint32_t *slot, uint64_t *ids,
                        cudaStream_t st);
// type, colour, id and mass (from p*.w) only: final once a step's grid is built
void launch_unpack_static(const HostParticlesOut &out, uint64_t n, const float4 *ps_grid, const int32_t *type,
                          const uint32_t *col, const uint32_t *slot, const uint64_t *ids, cudaStream_t st);

// vertex welding of device-resident triangles (weld.cu)
int weld_device(const fgb_mesh_triangle *d_tris, uint64_t n_tris, uint32_t *d_index, float *d_vertices,
                uint64_t *n_vertices, cudaStream_t st);

// marching cubes (mc.cu)
struct SurfaceView {
    const SceneDev *scenes;   // device
    const SceneDev *h_scenes; // host copy
    uint32_t scene_begin, scene_end;
    uint32_t mbits;
    Phys ph;
    const uint32_t *keys_sorted;
    const uint2 *cells;
    const float4 *xs;        // sorted, solver units, w = mass
    const int32_t *type;
    const uint32_t *col;
    float4 *lattice;
    uint32_t *lattice_col;
    uint8_t *cases;
    uint32_t *offsets;
    uint32_t *total;         // device, one u32
    uint64_t lat_begin, lat_end, cube_begin, cube_end, brick_begin, brick_end;
    void *scan_scratch;
    uint64_t scan_scratch_bytes;
    uint32_t *err;
};
cudaError_t launch_surface_count(const SurfaceView &v, cudaStream_t st, uint64_t *launches);
cudaError_t launch_surface_emit(const SurfaceView &v, fgb_mesh_triangle *out, uint64_t cap, cudaStream_t st,
                                uint64_t *launches);
void mc_tables_upload();

}  // namespace fgb
