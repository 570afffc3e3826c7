/*
 * pbf_oracle.h -- CPU oracle for the PBF step and marching cubes.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load this library, and only as the checker or the timed CPU
 * baseline; the product (libfluidgb) never links or calls it.
 *
 * Parity status:
 *   - Morton keys and the marching-cubes tables are PINNED: tests compare them with
 *     the reference's own curves.h / mctable.hpp / mc.h compiled from the reference
 *     tree (oracle/ref_shim.cpp) and with committed golden vectors (tests/golden).
 *   - The floating-point PBF and MC arithmetic of the ref profile is PINNED to the
 *     reference's own OpenCL kernel bodies (sph_diffuse, sph_lambda, sph_delta with
 *     the triangle collider, sph_finalise, mc_lattice, mc_size, mc_eval) compiled as
 *     C++ (oracle/ref_kernels.cpp): tests/test_oracle_ref_kernels.py compares them
 *     on the same predicted state at the stated tolerances, live and against
 *     committed vectors (tests/golden/reference_kernels.npz).  Not pinned by
 *     reference code: the host-side prediction (GLM host code) and the baseline
 *     profile's XSPH, vorticity and density field, which have no reference code.
 */
#ifndef PBF_ORACLE_H
#define PBF_ORACLE_H

#include <stddef.h>
#include <stdint.h>
#include "../include/fluid_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_grid {
    float min_ext[3];   /* solver units */
    uint32_t ext[3];    /* cell extent; cells are clamped to [0, ext] */
    uint32_t table_n;   /* morton(ext) + 1 */
} orc_grid;

typedef struct orc_lattice {
    uint32_t size[3];   /* samples per axis */
    float origin[3];    /* solver units */
    float step;         /* solver units */
} orc_lattice;

/* Optional outputs of orc_step (NULL members are skipped). */
typedef struct orc_probe {
    uint32_t *keys;     /* n, sorted */
    uint32_t *order;    /* n, input index of each sorted particle */
    uint32_t *cells;    /* 2 * table_n, {start, end} per key (0,0 when empty) */
    float *lambda;      /* n, last iteration */
    float *density;     /* n, last iteration */
    float *pstar;       /* 3n, predicted p* in sorted order, before the solver iterations */
    float *omega;       /* 4n, vorticity (xyz, |omega|) in sorted order (baseline profile) */
} orc_probe;

uint32_t orc_morton(uint32_t x, uint32_t y, uint32_t z);
uint32_t orc_morton_decode(uint32_t key, int axis);
void orc_mc_tables(uint16_t *edge_mask, uint8_t *num_verts, uint8_t *tri);
float orc_poly6(const fgb_params *p, float r);
float orc_spiky_scale(const fgb_params *p, float r); /* scalar s with grad = s * (x - y) */

void orc_grid_geometry(const fgb_params *p, const fgb_config *c, orc_grid *g);
void orc_lattice_geometry(const fgb_params *p, const fgb_config *c, const orc_grid *g,
                          orc_lattice *l);

/* Key of a position in solver units (clamped to the grid). */
uint32_t orc_key(const orc_grid *g, float h, float x, float y, float z);

/* One PBF step on n particles given in caller order.  All arrays are updated in
 * place and come back permuted into Morton order, like the reference's write-back
 * (oclsph.hpp:875-891).  Returns 0 on success. */
int orc_step(const fgb_params *p, const fgb_config *c, size_t n, uint64_t *id, int32_t *type,
             float *mass, float *pos, float *vel, uint32_t *colour, const fgb_triangle *tris,
             size_t n_tris, orc_probe *probe);

/* Marching cubes of the current particle state (any order).  lattice (4 floats per
 * sample), colours (1 u32 per sample) and cases (1 byte per cube) are optional.
 * Triangles are written to tris (capacity cap) in cube-major order; the return
 * value is the total triangle count (which may exceed cap). */
size_t orc_surface(const fgb_params *p, const fgb_config *c, size_t n, const int32_t *type,
                   const float *mass, const float *pos, const uint32_t *colour, float *lattice,
                   uint32_t *lattice_colour, uint8_t *cases, fgb_mesh_triangle *tris, size_t cap);

/* Marching cubes of a given lattice only (for stage-wise parity). */
size_t orc_march(const fgb_params *p, const fgb_config *c, const orc_lattice *l,
                 const float *lattice, const uint32_t *lattice_colour, uint8_t *cases,
                 fgb_mesh_triangle *tris, size_t cap);

/* Vertex welding (geometry::indexVBO2, geometry.hpp:152-166): the vertices of the
 * triangles in order; a position byte-identical to an earlier one takes its index,
 * otherwise it is appended.  indices: 3 n; vertices: room for 9 n floats.  Returns
 * the number of distinct vertices. */
size_t orc_weld(const fgb_mesh_triangle *tris, size_t n, uint32_t *indices, float *vertices);

int orc_num_threads(void);
void orc_set_threads(int n);

#ifdef __cplusplus
}
#endif

#endif /* PBF_ORACLE_H */
