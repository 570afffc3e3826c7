/*
 * pbf_oracle.c -- CPU oracle for the PBF step and marching cubes (TEST INFRASTRUCTURE).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this
 * library; the product never does.  See pbf_oracle.h for the parity status
 * (integer parts pinned against the reference's own headers; float parts pinned
 * against the reference's own kernel bodies compiled as C++, ref_kernels.cpp).
 *
 * The algorithm follows tom91136/libfluid:
 *   predict ............ include/fluid/oclsph.hpp:289-325 (advectAndCopy)
 *   grid + keys ........ include/fluid/oclsph.hpp:327-387, include/fluid/curves.h:56-72
 *   sort + cell ranges . include/fluid/oclsph.hpp:733-767 (stable here: key, then index)
 *   kernels ............ include/fluid/oclsph_kernel.h:50-71 (poly6, spiky gradient)
 *   neighbour walk ..... include/fluid/oclsph_kernel.h:150-192 (27 cells, x fastest)
 *   lambda ............. include/fluid/oclsph_kernel.h:305-332
 *   delta p + collide .. include/fluid/oclsph_kernel.h:335-384, oclsph_collision.h:7-58
 *                        (Jacobi: reads the old p*, writes a new array; the reference
 *                        updates p* in place, a data race with no defined result)
 *   finalise ........... include/fluid/oclsph_kernel.h:404-416
 *   MC field ........... include/fluid/oclsph_kernel.h:421-530 (ref: metaball)
 *   MC count ........... include/fluid/oclsph_kernel.h:545-596
 *   MC emit ............ include/fluid/surface.hpp:47-53,185-266 (cube-major order,
 *                        the CPU marchSingle lerp with its 1e-5 snapping)
 * The baseline profile replaces the reference constants and adds the PBF paper's
 * terms (Macklin & Mueller 2013): textbook lambda denominator, s_corr, XSPH
 * viscosity and vorticity confinement; poly6-density surface field.
 *
 * Every float operation has a fixed order and no implicit fusion (-ffp-contract=off,
 * explicit fmaf where fused), mirroring the CUDA kernels.
 */
#include "pbf_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

#include "../libfluid_gb300/csrc/mc_tables.h"

#define PI_F 3.14159265358979323846f
#define KERNEL_EPSILON 0.00000001f /* oclsph_kernel.h:24 */
#define WELL_RANGE 75.f            /* oclsph.hpp:310 */
#define WELL_CLAMP 10.f            /* oclsph.hpp:312-314 */
#define TRIANGLE_SNAP 40.f         /* oclsph_collision.h:44 */

/* ------------------------------------------------------------------ Morton */

static uint32_t SPREAD[1024];
static int SPREAD_READY = 0;

static void spread_init(void) {
    if (SPREAD_READY) return;
    for (uint32_t v = 0; v < 1024; ++v) {
        uint32_t s = 0;
        for (int b = 0; b < 10; ++b) s |= ((v >> b) & 1u) << (3 * b);
        SPREAD[v] = s;
    }
    SPREAD_READY = 1;
}

uint32_t orc_morton(uint32_t x, uint32_t y, uint32_t z) {
    spread_init();
    return SPREAD[x & 1023u] | (SPREAD[y & 1023u] << 1) | (SPREAD[z & 1023u] << 2);
}

uint32_t orc_morton_decode(uint32_t key, int axis) {
    uint32_t v = 0;
    for (int b = 0; b < 10; ++b) v |= ((key >> (3 * b + axis)) & 1u) << b;
    return v;
}

void orc_mc_tables(uint16_t *edge_mask, uint8_t *num_verts, uint8_t *tri) {
    fgb_mc_tables t;
    fgb_mc_tables_build(&t);
    memcpy(edge_mask, t.edge_mask, sizeof t.edge_mask);
    memcpy(num_verts, t.num_verts, sizeof t.num_verts);
    memcpy(tri, t.tri, sizeof t.tri);
}

int orc_num_threads(void) { return omp_get_max_threads(); }
void orc_set_threads(int n) {
    if (n > 0) omp_set_num_threads(n);
}

/* --------------------------------------------------------------- constants */

typedef struct kc {
    float h, hh, hhh;
    float poly6f;   /* 315 / (64 pi h^9)       oclsph_kernel.h:50 */
    float spikyf;   /* -45 / (pi h^6)          oclsph_kernel.h:51 */
    float rho0, inv_rho0;
    float corr_ref; /* ref: poly6(dq)            oclsph_kernel.h:350 */
    float corr_wdq; /* baseline: (h^2 - dq^2)^3  (poly6 without its factor) */
    float inv_corr_wdq; /* 1 / corr_wdq: s_corr's ratio is a product, no division per pair */
    float corr_k;   /* baseline: k * h^2 (s_corr carried in lambda's units, length^2) */
} kc;

static void consts(const fgb_params *p, kc *k) {
    k->h = p->h;
    k->hh = p->h * p->h;
    k->hhh = p->h * p->h * p->h;
    k->poly6f = 315.f / (64.f * PI_F * (k->hhh * k->hhh * k->hhh));
    k->spikyf = -(45.f / (PI_F * k->hhh * k->hhh));
    k->rho0 = p->rho0;
    k->inv_rho0 = 1.f / p->rho0;
    float dq = p->corr_delta_q * p->h;
    float t = k->hh - dq * dq;
    k->corr_wdq = t * t * t;
    k->inv_corr_wdq = k->corr_wdq != 0.f ? 1.f / k->corr_wdq : 0.f;
    k->corr_ref = orc_poly6(p, dq);
    /* The PBF paper's s_corr = -k (W/W(dq))^n is dimensionless only in units where
     * h = 1; added to lambda (length^2) it is scaled by h^2 here. */
    k->corr_k = p->corr_k * k->hh;
}

float orc_poly6(const fgb_params *p, float r) {
    float h = p->h, hh = h * h, hhh = h * h * h;
    float f = 315.f / (64.f * PI_F * (hhh * hhh * hhh));
    if (!(r <= h)) return 0.f;
    float t = hh - r * r;
    return f * (t * t * t);
}

float orc_spiky_scale(const fgb_params *p, float r) {
    float h = p->h, hhh = h * h * h;
    float f = -(45.f / (PI_F * hhh * hhh));
    if (!(r >= KERNEL_EPSILON && r <= h)) return 0.f;
    float q = h - r;
    return f * ((q * q) / r);
}

/* s_corr ratio^n: n == 4 is evaluated as two squarings on CPU and GPU alike. */
/* Squared distance in the baseline profile: two fused multiply-adds (the GPU's
 * __fmaf_rn gives the same bits). */
static inline float dist2(float dx, float dy, float dz) { return fmaf(dx, dx, fmaf(dy, dy, dz * dz)); }

static inline float corr_pow(float ratio, float n) {
    if (n == 4.f) {
        float r2 = ratio * ratio;
        return r2 * r2;
    }
    return powf(ratio, n);
}

/* -------------------------------------------------------------------- grid */

void orc_grid_geometry(const fgb_params *p, const fgb_config *c, orc_grid *g) {
    spread_init();
    const float pad = p->h * 2.f; /* oclsph.hpp:340 */
    for (int a = 0; a < 3; ++a) {
        float mn = (c->min_bound[a] / c->scale) - pad; /* oclsph.hpp:359 */
        float mx = (c->max_bound[a] / c->scale) + pad; /* oclsph.hpp:360 */
        g->min_ext[a] = mn;
        float e = (mx - mn) / p->h;                    /* oclsph.hpp:386 */
        uint32_t ei = e > 0.f ? (uint32_t)e : 0u;
        if (ei > 1023u) ei = 1023u;
        g->ext[a] = ei;
    }
    g->table_n = orc_morton(g->ext[0], g->ext[1], g->ext[2]) + 1u;
}

static inline uint32_t quantise(float v, float mn, float h, uint32_t ext) {
    float q = (v - mn) / h;          /* oclsph.hpp:327-332, 367-371 */
    if (!(q > 0.f)) return 0u;       /* negative or NaN: the reference's cast is undefined */
    if (q >= (float)ext) return ext; /* clamp into the grid (ext <= 1023 < 2^10) */
    return (uint32_t)q;
}

uint32_t orc_key(const orc_grid *g, float h, float x, float y, float z) {
    return orc_morton(quantise(x, g->min_ext[0], h, g->ext[0]),
                      quantise(y, g->min_ext[1], h, g->ext[1]),
                      quantise(z, g->min_ext[2], h, g->ext[2]));
}

void orc_lattice_geometry(const fgb_params *p, const fgb_config *c, const orc_grid *g,
                          orc_lattice *l) {
    l->step = p->h / c->resolution; /* oclsph_kernel.h:440 */
    for (int a = 0; a < 3; ++a) {
        if (p->profile == FGB_PROFILE_REF) {
            /* oclsph.hpp:817-819: floor(extent * resolution) + 1, origin minExtent */
            l->origin[a] = g->min_ext[a];
            l->size[a] = (uint32_t)floorf((float)g->ext[a] * c->resolution) + 1u;
        } else {
            /* baseline: a box-aligned lattice from min_bound to max_bound */
            float lo = c->min_bound[a] / c->scale, hi = c->max_bound[a] / c->scale;
            l->origin[a] = lo;
            l->size[a] = (uint32_t)floorf((hi - lo) / l->step + 0.5f) + 1u;
        }
    }
}

static int cmp_u64(const void *a, const void *b) {
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return (x > y) - (x < y);
}

/* Stable argsort by key (ties keep input order). */
static void argsort_keys(size_t n, const uint32_t *key, uint32_t *order) {
    uint64_t *kv = (uint64_t *)malloc(n * sizeof(uint64_t));
    for (size_t i = 0; i < n; ++i) kv[i] = ((uint64_t)key[i] << 32) | (uint64_t)i;
    qsort(kv, n, sizeof(uint64_t), cmp_u64);
    for (size_t i = 0; i < n; ++i) order[i] = (uint32_t)(kv[i] & 0xffffffffu);
    free(kv);
}

static void build_cells(size_t n, const uint32_t *skey, uint32_t table_n, uint32_t *cells) {
    memset(cells, 0, (size_t)table_n * 2 * sizeof(uint32_t));
    for (size_t i = 0; i < n; ++i) {
        uint32_t k = skey[i];
        if (i == 0 || skey[i - 1] != k) cells[2 * (size_t)k] = (uint32_t)i;
        if (i + 1 == n || skey[i + 1] != k) cells[2 * (size_t)k + 1] = (uint32_t)(i + 1);
    }
}

/* The 27 neighbour cells of a cell in the order dz, dy, dx (x fastest), as in
 * oclsph_kernel.h:155-183; cells outside [0, ext] hold no particle and are skipped. */
typedef struct ranges {
    int n;
    uint32_t r[27][2];
} ranges;

static void neighbour_ranges(const orc_grid *g, const uint32_t *cells, uint32_t cx, uint32_t cy,
                             uint32_t cz, ranges *out) {
    out->n = 0;
    for (int dz = -1; dz <= 1; ++dz) {
        int z = (int)cz + dz;
        if (z < 0 || z > (int)g->ext[2]) continue;
        for (int dy = -1; dy <= 1; ++dy) {
            int y = (int)cy + dy;
            if (y < 0 || y > (int)g->ext[1]) continue;
            for (int dx = -1; dx <= 1; ++dx) {
                int x = (int)cx + dx;
                if (x < 0 || x > (int)g->ext[0]) continue;
                uint32_t k = orc_morton((uint32_t)x, (uint32_t)y, (uint32_t)z);
                uint32_t s = cells[2 * (size_t)k], e = cells[2 * (size_t)k + 1];
                if (s < e) {
                    out->r[out->n][0] = s;
                    out->r[out->n][1] = e;
                    out->n++;
                }
            }
        }
    }
}

/* ----------------------------------------------------------------- predict */

static void predict_one(const fgb_params *p, const fgb_config *c, int32_t type, float mass,
                        const float *x, float *v, float *ps, float *vkeep) {
    for (int a = 0; a < 3; ++a) {
        ps[a] = x[a] / c->scale; /* oclsph.hpp:301 */
        vkeep[a] = v[a];         /* the copied particle keeps the pre-force velocity */
    }
    if (type == FGB_TYPE_OBSTACLE) return;
    float f[3];
    const int ref = p->profile == FGB_PROFILE_REF;
    for (int a = 0; a < 3; ++a) f[a] = ref ? mass * c->constant_force[a] : c->constant_force[a];
    for (uint32_t w = 0; w < c->n_wells && w < FGB_MAX_WELLS; ++w) {
        const fgb_well *wl = &c->wells[w];
        float d[3] = {x[0] - wl->centre[0], x[1] - wl->centre[1], x[2] - wl->centre[2]};
        float dist = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        if (dist < WELL_RANGE) {
            float u[3] = {wl->centre[0] - x[0], wl->centre[1] - x[1], wl->centre[2] - x[2]};
            float ul = sqrtf(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
            for (int a = 0; a < 3; ++a) {
                float rhat = u[a] / ul;
                float fw = ref ? ((rhat * wl->force) * mass) / (dist * dist)
                               : (rhat * wl->force) / (dist * dist);
                if (fw < -WELL_CLAMP) fw = -WELL_CLAMP;
                if (fw > WELL_CLAMP) fw = WELL_CLAMP;
                f[a] = f[a] + fw;
            }
        }
    }
    for (int a = 0; a < 3; ++a) {
        v[a] = f[a] * c->dt + v[a];         /* oclsph.hpp:319 */
        ps[a] = v[a] * c->dt + x[a] / c->scale; /* oclsph.hpp:320-321 */
    }
}

/* -------------------------------------------------------------- collisions */

static inline float dot3(const float *a, const float *b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

/* oclsph_collision.h:7-22 */
static int in_triangle(const fgb_triangle *t, const float *P) {
    float v0[3], v1[3], v2[3];
    for (int a = 0; a < 3; ++a) {
        v0[a] = t->c[a] - t->a[a];
        v1[a] = t->b[a] - t->a[a];
        v2[a] = P[a] - t->a[a];
    }
    float d00 = dot3(v0, v0), d01 = dot3(v0, v1), d02 = dot3(v0, v2);
    float d11 = dot3(v1, v1), d12 = dot3(v1, v2);
    float inv = 1.f / (d00 * d11 - d01 * d01);
    float u = (d11 * d02 - d01 * d12) * inv;
    float w = (d00 * d12 - d01 * d02) * inv;
    return (u >= 0.f) && (w >= 0.f) && (u + w < 1.f);
}

/* oclsph_collision.h:25-58: snap onto the plane of the first triangle whose
 * projection contains the point (within 40 world units), reflect the velocity. */
static void collide_triangles(const fgb_triangle *tris, size_t n, float *pos, float *vel) {
    for (size_t i = 0; i < n; ++i) {
        const fgb_triangle *t = &tris[i];
        float e1[3], e2[3], nrm[3];
        for (int a = 0; a < 3; ++a) {
            e1[a] = t->b[a] - t->a[a];
            e2[a] = t->c[a] - t->a[a];
        }
        nrm[0] = e1[1] * e2[2] - e1[2] * e2[1];
        nrm[1] = e1[2] * e2[0] - e1[0] * e2[2];
        nrm[2] = e1[0] * e2[1] - e1[1] * e2[0];
        float len = sqrtf(dot3(nrm, nrm));
        float nn[3] = {nrm[0] / len, nrm[1] / len, nrm[2] / len};
        float dist = dot3(nn, t->a) - dot3(nn, pos);
        if (-TRIANGLE_SNAP <= dist && dist <= TRIANGLE_SNAP) {
            float p0[3] = {pos[0] + nn[0] * dist, pos[1] + nn[1] * dist, pos[2] + nn[2] * dist};
            if (in_triangle(t, p0)) {
                float vn = dot3(vel, nn);
                for (int a = 0; a < 3; ++a) {
                    vel[a] = vel[a] - (nn[a] * 2.f) * vn;
                    pos[a] = p0[a];
                }
                return;
            }
        }
    }
}

/* Static sphere (baseline workloads): project points inside onto the surface. */
static void collide_sphere(const fgb_config *c, float *pos) {
    if (!c->sphere_enabled) return;
    float d[3] = {pos[0] - c->sphere[0], pos[1] - c->sphere[1], pos[2] - c->sphere[2]};
    float r = c->sphere[3];
    float d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    if (!(d2 < r * r)) return;
    float dist = sqrtf(d2);
    if (dist > 0.f) {
        float s = r / dist;
        for (int a = 0; a < 3; ++a) pos[a] = c->sphere[a] + d[a] * s;
    } else {
        pos[0] = c->sphere[0];
        pos[1] = c->sphere[1] + r;
        pos[2] = c->sphere[2];
    }
}

/* ------------------------------------------------------------------ passes */

typedef struct state {
    size_t n;
    const fgb_params *p;
    const fgb_config *c;
    kc k;
    orc_grid g;
    const uint32_t *cells;
    const uint32_t *cxyz;  /* 3n cell coordinates of each sorted particle */
    const int32_t *type;
    const float *mass;
} state;

/* oclsph_kernel.h:281-303 (ref profile only): every fluid particle averages the
 * colours of all fluid candidates of its 27 cells (no distance test, itself
 * included) and moves toward 1.33x the mean by dt/750 per 8-bit channel:
 * OpenCL mix(x, y, t) = x + (y - x) t, clamp to [8, 255], convert_uchar rounds to
 * zero.  Channel sums are integers below 2^24, exact in float, so summing them as
 * integers gives the reference's float4 accumulation in any order. */
static void diffuse_colours(const state *s, uint32_t *colour) {
    const size_t n = s->n;
    uint32_t *out = (uint32_t *)malloc(n * sizeof(uint32_t));
    const float t = s->c->dt / 750.f;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)n; ++i) {
        out[i] = colour[i];
        if (s->type[i] == FGB_TYPE_OBSTACLE) continue;
        ranges rg;
        neighbour_ranges(&s->g, s->cells, s->cxyz[3 * i], s->cxyz[3 * i + 1], s->cxyz[3 * i + 2], &rg);
        uint32_t sum[4] = {0, 0, 0, 0}, cnt = 0;
        for (int r = 0; r < rg.n; ++r)
            for (uint32_t b = rg.r[r][0]; b < rg.r[r][1]; ++b) {
                if (s->type[b] == FGB_TYPE_OBSTACLE) continue;
                for (int ch = 0; ch < 4; ++ch) sum[ch] += (colour[b] >> (8 * ch)) & 0xffu;
                ++cnt;
            }
        uint32_t v = 0;
        for (int ch = 0; ch < 4; ++ch) {
            const float x = (float)((colour[i] >> (8 * ch)) & 0xffu);
            const float y = ((float)sum[ch] / (float)cnt) * 1.33f;
            float o = x + (y - x) * t;
            o = fminf(fmaxf(o, 8.f), 255.f);
            v |= (uint32_t)o << (8 * ch);
        }
        out[i] = v;
    }
    memcpy(colour, out, n * sizeof(uint32_t));
    free(out);
}

/* oclsph_kernel.h:305-332 (ref) / PBF paper eq. 8-11 (baseline). */
static void lambda_pass(const state *s, const float *ps, float *lam, float *rho_out) {
    const kc *k = &s->k;
    const int ref = s->p->profile == FGB_PROFILE_REF;
#pragma omp parallel for schedule(static)
    for (long ia = 0; ia < (long)s->n; ++ia) {
        size_t a = (size_t)ia;
        if (s->type[a] == FGB_TYPE_OBSTACLE) {
            lam[a] = 0.f;
            rho_out[a] = 0.f;
            continue;
        }
        ranges R;
        neighbour_ranges(&s->g, s->cells, s->cxyz[3 * a], s->cxyz[3 * a + 1], s->cxyz[3 * a + 2], &R);
        const float ax = ps[3 * a], ay = ps[3 * a + 1], az = ps[3 * a + 2];
        float rho = 0.f, gx = 0.f, gy = 0.f, gz = 0.f, g2 = 0.f;
        for (int q = 0; q < R.n; ++q) {
            for (uint32_t b = R.r[q][0]; b < R.r[q][1]; ++b) {
                float dx = ax - ps[3 * b], dy = ay - ps[3 * b + 1], dz = az - ps[3 * b + 2];
                /* the ref profile sums three products as the reference does; the
                 * baseline takes two fused multiply-adds */
                float r2 = ref ? dx * dx + dy * dy + dz * dz : dist2(dx, dy, dz);
                if (ref) {
                    float r = sqrtf(r2);
                    if (r <= k->h) {
                        float t = k->hh - r * r;
                        rho = fmaf(s->mass[a], k->poly6f * (t * t * t), rho);
                        if (r >= KERNEL_EPSILON) {
                            float hr = k->h - r;
                            float sc = k->spikyf * ((hr * hr) / r);
                            gx = fmaf(dx * sc, k->inv_rho0, gx);
                            gy = fmaf(dy * sc, k->inv_rho0, gy);
                            gz = fmaf(dz * sc, k->inv_rho0, gz);
                        }
                    }
                } else {
                    if (r2 <= k->hh) {
                        float t = k->hh - r2;
                        float mb = s->mass[b];
                        rho = fmaf(mb, t * t * t, rho);
                        float r = sqrtf(r2);
                        if (r >= KERNEL_EPSILON) {
                            float hr = k->h - r;
                            float sc = mb * ((hr * hr) / r);
                            gx = fmaf(sc, dx, gx);
                            gy = fmaf(sc, dy, gy);
                            gz = fmaf(sc, dz, gz);
                            g2 = fmaf(sc * sc, r2, g2);
                        }
                    }
                }
            }
        }
        float density, lambda;
        if (ref) {
            density = rho;
            float norm2 = gx * gx + gy * gy + gz * gz;
            float C = density / k->rho0 - 1.f;
            lambda = -C / (norm2 + s->p->cfm_epsilon);
        } else {
            density = rho * k->poly6f;
            float gs = k->spikyf * k->inv_rho0;
            float sx = gx * gs, sy = gy * gs, sz = gz * gs;
            float denom = (sx * sx + sy * sy + sz * sz) + g2 * (gs * gs);
            float C = density * k->inv_rho0 - 1.f;
            lambda = -C / (denom + s->p->cfm_epsilon);
        }
        lam[a] = lambda;
        rho_out[a] = density;
    }
}

/* oclsph_kernel.h:335-384 (ref) / PBF paper eq. 12-14 (baseline); Jacobi update. */
static void delta_pass(const state *s, const float *ps, const float *lam, float *ps_out,
                       float *vel, const fgb_triangle *tris, size_t n_tris) {
    const kc *k = &s->k;
    const fgb_config *c = s->c;
    const int ref = s->p->profile == FGB_PROFILE_REF;
    const float ck = s->p->corr_k, cn = s->p->corr_n;
#pragma omp parallel for schedule(static)
    for (long ia = 0; ia < (long)s->n; ++ia) {
        size_t a = (size_t)ia;
        if (s->type[a] == FGB_TYPE_OBSTACLE) {
            ps_out[3 * a] = ps[3 * a];
            ps_out[3 * a + 1] = ps[3 * a + 1];
            ps_out[3 * a + 2] = ps[3 * a + 2];
            continue;
        }
        ranges R;
        neighbour_ranges(&s->g, s->cells, s->cxyz[3 * a], s->cxyz[3 * a + 1], s->cxyz[3 * a + 2], &R);
        const float ax = ps[3 * a], ay = ps[3 * a + 1], az = ps[3 * a + 2];
        const float la = lam[a];
        float px = 0.f, py = 0.f, pz = 0.f;
        for (int q = 0; q < R.n; ++q) {
            for (uint32_t b = R.r[q][0]; b < R.r[q][1]; ++b) {
                float dx = ax - ps[3 * b], dy = ay - ps[3 * b + 1], dz = az - ps[3 * b + 2];
                float r2 = ref ? dx * dx + dy * dy + dz * dz : dist2(dx, dy, dz);
                if (ref) {
                    float r = sqrtf(r2);
                    float w = 0.f;
                    if (r <= k->h) {
                        float t = k->hh - r * r;
                        w = k->poly6f * (t * t * t);
                    }
                    float corr = -ck * corr_pow(w / k->corr_ref, cn);
                    float factor = (la + lam[b] + corr) / k->rho0;
                    if (r >= KERNEL_EPSILON && r <= k->h) {
                        float hr = k->h - r;
                        float sc = k->spikyf * ((hr * hr) / r);
                        px = fmaf(dx * sc, factor, px);
                        py = fmaf(dy * sc, factor, py);
                        pz = fmaf(dz * sc, factor, pz);
                    }
                } else {
                    if (r2 <= k->hh) {
                        float r = sqrtf(r2);
                        if (r >= KERNEL_EPSILON) {
                            float t = k->hh - r2;
                            float corr = -k->corr_k * corr_pow((t * t * t) * k->inv_corr_wdq, cn);
                            float hr = k->h - r;
                            float sc = s->mass[b] * ((hr * hr) / r) * (la + lam[b] + corr);
                            px = fmaf(sc, dx, px);
                            py = fmaf(sc, dy, py);
                            pz = fmaf(sc, dz, pz);
                        }
                    }
                }
            }
        }
        float world[3];
        if (ref) {
            world[0] = (ax + px) * c->scale;
            world[1] = (ay + py) * c->scale;
            world[2] = (az + pz) * c->scale;
        } else {
            float gs = k->spikyf * k->inv_rho0;
            world[0] = (ax + px * gs) * c->scale;
            world[1] = (ay + py * gs) * c->scale;
            world[2] = (az + pz * gs) * c->scale;
            collide_sphere(c, world);
        }
        if (n_tris) collide_triangles(tris, n_tris, world, &vel[3 * a]);
        for (int d = 0; d < 3; ++d) {
            float w = world[d];
            w = fmaxf(c->min_bound[d], w); /* oclsph_kernel.h:371 */
            w = fminf(c->max_bound[d], w);
            ps_out[3 * a + d] = w / c->scale;
        }
    }
}

static inline void cross3(const float *a, const float *b, float *o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

/* Baseline velocity terms (PBF paper eq. 15-17): omega and XSPH, then the
 * vorticity-confinement force.  Sums over fluid neighbours, SPH-normalised with
 * m_j / rho0. */
static void velocity_terms(const state *s, const float *ps, float *vel, float *omega_out) {
    const kc *k = &s->k;
    const size_t n = s->n;
    const float gs = k->spikyf * k->inv_rho0;
    const float ws = k->poly6f * k->inv_rho0;
    const float xc = s->p->xsph_c, ve = s->p->vorticity_epsilon, dt = s->c->dt;
    float *om = (float *)calloc(4 * n, sizeof(float));
    float *vx = (float *)malloc(3 * n * sizeof(float));
#pragma omp parallel for schedule(static)
    for (long ia = 0; ia < (long)n; ++ia) {
        size_t a = (size_t)ia;
        vx[3 * a] = vel[3 * a];
        vx[3 * a + 1] = vel[3 * a + 1];
        vx[3 * a + 2] = vel[3 * a + 2];
        if (s->type[a] == FGB_TYPE_OBSTACLE) continue;
        ranges R;
        neighbour_ranges(&s->g, s->cells, s->cxyz[3 * a], s->cxyz[3 * a + 1], s->cxyz[3 * a + 2], &R);
        const float ax = ps[3 * a], ay = ps[3 * a + 1], az = ps[3 * a + 2];
        const float *va = &vel[3 * a];
        float o[3] = {0.f, 0.f, 0.f}, xs[3] = {0.f, 0.f, 0.f};
        for (int q = 0; q < R.n; ++q) {
            for (uint32_t b = R.r[q][0]; b < R.r[q][1]; ++b) {
                if (s->type[b] == FGB_TYPE_OBSTACLE) continue;
                float d[3] = {ax - ps[3 * b], ay - ps[3 * b + 1], az - ps[3 * b + 2]};
                float r2 = dist2(d[0], d[1], d[2]);
                if (!(r2 <= k->hh)) continue;
                float vab[3] = {vel[3 * b] - va[0], vel[3 * b + 1] - va[1], vel[3 * b + 2] - va[2]};
                float t = k->hh - r2;
                float mw = s->mass[b] * (t * t * t);
                xs[0] = fmaf(mw, vab[0], xs[0]);
                xs[1] = fmaf(mw, vab[1], xs[1]);
                xs[2] = fmaf(mw, vab[2], xs[2]);
                float r = sqrtf(r2);
                if (r >= KERNEL_EPSILON) {
                    float hr = k->h - r;
                    float sc = s->mass[b] * ((hr * hr) / r);
                    float cr[3];
                    cross3(vab, d, cr);
                    o[0] = fmaf(sc, cr[0], o[0]);
                    o[1] = fmaf(sc, cr[1], o[1]);
                    o[2] = fmaf(sc, cr[2], o[2]);
                }
            }
        }
        /* omega = sum_b m_b / rho0 (v_b - v_a) x grad_b W(x_a - x_b) (PBF paper eq. 15),
         * grad_b W = -grad_a W = -spikyf (h - r)^2 d / r */
        float ox = -(o[0] * gs), oy = -(o[1] * gs), oz = -(o[2] * gs);
        om[4 * a] = ox;
        om[4 * a + 1] = oy;
        om[4 * a + 2] = oz;
        om[4 * a + 3] = sqrtf(ox * ox + oy * oy + oz * oz);
        vx[3 * a] = fmaf(xc, xs[0] * ws, va[0]);
        vx[3 * a + 1] = fmaf(xc, xs[1] * ws, va[1]);
        vx[3 * a + 2] = fmaf(xc, xs[2] * ws, va[2]);
    }
#pragma omp parallel for schedule(static)
    for (long ia = 0; ia < (long)n; ++ia) {
        size_t a = (size_t)ia;
        if (s->type[a] == FGB_TYPE_OBSTACLE) continue;
        ranges R;
        neighbour_ranges(&s->g, s->cells, s->cxyz[3 * a], s->cxyz[3 * a + 1], s->cxyz[3 * a + 2], &R);
        const float ax = ps[3 * a], ay = ps[3 * a + 1], az = ps[3 * a + 2];
        const float wa = om[4 * a + 3];
        float e[3] = {0.f, 0.f, 0.f};
        for (int q = 0; q < R.n; ++q) {
            for (uint32_t b = R.r[q][0]; b < R.r[q][1]; ++b) {
                if (s->type[b] == FGB_TYPE_OBSTACLE) continue;
                float d[3] = {ax - ps[3 * b], ay - ps[3 * b + 1], az - ps[3 * b + 2]};
                float r2 = dist2(d[0], d[1], d[2]);
                if (!(r2 <= k->hh)) continue;
                float r = sqrtf(r2);
                if (!(r >= KERNEL_EPSILON)) continue;
                float hr = k->h - r;
                float sc = s->mass[b] * ((hr * hr) / r) * (om[4 * b + 3] - wa);
                e[0] = fmaf(sc, d[0], e[0]);
                e[1] = fmaf(sc, d[1], e[1]);
                e[2] = fmaf(sc, d[2], e[2]);
            }
        }
        float ex = e[0] * gs, ey = e[1] * gs, ez = e[2] * gs;
        float el = sqrtf(ex * ex + ey * ey + ez * ez);
        float N[3] = {0.f, 0.f, 0.f};
        if (el > 0.f) {
            N[0] = ex / el;
            N[1] = ey / el;
            N[2] = ez / el;
        }
        float f[3];
        cross3(N, &om[4 * a], f);
        vel[3 * a] = fmaf(dt, f[0] * ve, vx[3 * a]);
        vel[3 * a + 1] = fmaf(dt, f[1] * ve, vx[3 * a + 1]);
        vel[3 * a + 2] = fmaf(dt, f[2] * ve, vx[3 * a + 2]);
    }
    if (omega_out) memcpy(omega_out, om, 4 * n * sizeof(float));
    free(om);
    free(vx);
}

/* ------------------------------------------------------------------- step */

#define PERMUTE(T, arr, width)                                                   \
    do {                                                                         \
        T *tmp_ = (T *)malloc(n * (width) * sizeof(T));                          \
        for (size_t i_ = 0; i_ < n; ++i_)                                        \
            for (size_t w_ = 0; w_ < (width); ++w_)                              \
                tmp_[i_ * (width) + w_] = (arr)[(size_t)order[i_] * (width) + w_]; \
        memcpy((arr), tmp_, n * (width) * sizeof(T));                            \
        free(tmp_);                                                              \
    } while (0)

int orc_step(const fgb_params *p, const fgb_config *c, size_t n, uint64_t *id, int32_t *type,
             float *mass, float *pos, float *vel, uint32_t *colour, const fgb_triangle *tris,
             size_t n_tris, orc_probe *probe) {
    if (n == 0) return 0;
    state s;
    s.n = n;
    s.p = p;
    s.c = c;
    consts(p, &s.k);
    orc_grid_geometry(p, c, &s.g);
    const float h = p->h;

    float *ps = (float *)malloc(3 * n * sizeof(float));
    float *vk = (float *)malloc(3 * n * sizeof(float));
    uint32_t *key = (uint32_t *)malloc(n * sizeof(uint32_t));
    uint32_t *order = (uint32_t *)malloc(n * sizeof(uint32_t));
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)n; ++i) {
        float v[3] = {vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]};
        predict_one(p, c, type[i], mass[i], &pos[3 * i], v, &ps[3 * i], &vk[3 * i]);
        key[i] = orc_key(&s.g, h, ps[3 * i], ps[3 * i + 1], ps[3 * i + 2]);
    }
    argsort_keys(n, key, order);
    PERMUTE(uint64_t, id, 1);
    PERMUTE(int32_t, type, 1);
    PERMUTE(float, mass, 1);
    PERMUTE(float, pos, 3);
    PERMUTE(float, vk, 3);
    PERMUTE(uint32_t, colour, 1);
    PERMUTE(float, ps, 3);
    PERMUTE(uint32_t, key, 1);

    if (probe && probe->pstar) memcpy(probe->pstar, ps, 3 * n * sizeof(float));
    uint32_t *cells = (uint32_t *)malloc((size_t)s.g.table_n * 2 * sizeof(uint32_t));
    build_cells(n, key, s.g.table_n, cells);
    uint32_t *cxyz = (uint32_t *)malloc(3 * n * sizeof(uint32_t));
    for (size_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) cxyz[3 * i + a] = orc_morton_decode(key[i], a);
    s.cells = cells;
    s.cxyz = cxyz;
    s.type = type;
    s.mass = mass;

    if (p->profile == FGB_PROFILE_REF) diffuse_colours(&s, colour);

    float *lam = (float *)calloc(n, sizeof(float));
    float *rho = (float *)calloc(n, sizeof(float));
    float *ps2 = (float *)malloc(3 * n * sizeof(float));
    for (uint32_t it = 0; it < c->iterations; ++it) {
        lambda_pass(&s, ps, lam, rho);
        delta_pass(&s, ps, lam, ps2, vk, tris, n_tris);
        float *t = ps;
        ps = ps2;
        ps2 = t;
    }

    const float inv_dt = 1.f / c->dt;
    if (p->profile == FGB_PROFILE_REF) {
        /* oclsph_kernel.h:404-416; obstacles keep their state (oclsph.hpp:885-889) */
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)n; ++i) {
            if (type[i] == FGB_TYPE_OBSTACLE) {
                for (int a = 0; a < 3; ++a) vel[3 * i + a] = vk[3 * i + a];
                continue;
            }
            for (int a = 0; a < 3; ++a) {
                float dx = ps[3 * i + a] - pos[3 * i + a] / c->scale;
                pos[3 * i + a] = ps[3 * i + a] * c->scale;
                vel[3 * i + a] = fmaf(dx, inv_dt, vk[3 * i + a]) * p->velocity_damping;
            }
        }
    } else {
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)n; ++i) {
            if (type[i] == FGB_TYPE_OBSTACLE) {
                for (int a = 0; a < 3; ++a) vel[3 * i + a] = vk[3 * i + a];
                continue;
            }
            for (int a = 0; a < 3; ++a) {
                float dx = ps[3 * i + a] - pos[3 * i + a] / c->scale;
                vel[3 * i + a] = dx * inv_dt;
            }
        }
        velocity_terms(&s, ps, vel, probe ? probe->omega : NULL);
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)n; ++i) {
            if (type[i] == FGB_TYPE_OBSTACLE) continue;
            for (int a = 0; a < 3; ++a) pos[3 * i + a] = ps[3 * i + a] * c->scale;
        }
    }

    if (probe) {
        if (probe->keys) memcpy(probe->keys, key, n * sizeof(uint32_t));
        if (probe->order) memcpy(probe->order, order, n * sizeof(uint32_t));
        if (probe->cells) memcpy(probe->cells, cells, (size_t)s.g.table_n * 2 * sizeof(uint32_t));
        if (probe->lambda) memcpy(probe->lambda, lam, n * sizeof(float));
        if (probe->density) memcpy(probe->density, rho, n * sizeof(float));
    }
    free(ps);
    free(ps2);
    free(vk);
    free(key);
    free(order);
    free(cells);
    free(cxyz);
    free(lam);
    free(rho);
    return 0;
}

/* ---------------------------------------------------------- marching cubes */

static inline uint32_t argb_channel(uint32_t c, int ch) { return (c >> (24 - 8 * ch)) & 0xffu; }

static inline uint32_t argb_pack(const float *ch) {
    uint32_t out = 0;
    for (int i = 0; i < 4; ++i) {
        float v = ch[i];
        if (!(v > 0.f)) v = 0.f;
        if (v > 255.f) v = 255.f;
        out |= ((uint32_t)v & 0xffu) << (24 - 8 * i);
    }
    return out;
}

/* Field at every lattice sample (oclsph_kernel.h:421-530 for ref; poly6 density
 * and its normalised negative gradient for baseline), from a grid rebuilt over
 * the given positions. */
static void lattice_field(const fgb_params *p, const fgb_config *c, const orc_grid *g,
                          const orc_lattice *l, size_t n, const int32_t *type, const float *mass,
                          const float *xs /* solver units, sorted */, const float *xw /* world */,
                          const uint32_t *colour, const uint32_t *cells, float *lat,
                          uint32_t *lcol) {
    kc k;
    consts(p, &k);
    const int ref = p->profile == FGB_PROFILE_REF;
    const size_t sy = l->size[1], sz = l->size[2];
    const size_t total = (size_t)l->size[0] * sy * sz;
    const float thr = p->h * c->scale;
    const float infl = p->mc_particle_influence, psize = p->mc_particle_size;
#pragma omp parallel for schedule(dynamic, 256)
    for (long q = 0; q < (long)total; ++q) {
        size_t ix = (size_t)q / (sy * sz), iy = ((size_t)q / sz) % sy, iz = (size_t)q % sz;
        float node[3] = {l->origin[0] + (float)ix * l->step, l->origin[1] + (float)iy * l->step,
                         l->origin[2] + (float)iz * l->step};
        uint32_t cc[3];
        if (ref) {
            cc[0] = (uint32_t)((float)ix / c->resolution);
            cc[1] = (uint32_t)((float)iy / c->resolution);
            cc[2] = (uint32_t)((float)iz / c->resolution);
            for (int a = 0; a < 3; ++a)
                if (cc[a] > g->ext[a]) cc[a] = g->ext[a];
        } else {
            for (int a = 0; a < 3; ++a) cc[a] = quantise(node[a], g->min_ext[a], p->h, g->ext[a]);
        }
        ranges R;
        neighbour_ranges(g, cells, cc[0], cc[1], cc[2], &R);
        float v = 0.f, nx = 0.f, ny = 0.f, nz = 0.f;
        float col[4] = {0.f, 0.f, 0.f, 0.f};
        uint32_t N = 0;
        float aw[3] = {node[0] * c->scale, node[1] * c->scale, node[2] * c->scale};
        for (int r = 0; r < R.n; ++r) {
            for (uint32_t b = R.r[r][0]; b < R.r[r][1]; ++b) {
                if (type[b] == FGB_TYPE_OBSTACLE) continue;
                if (ref) {
                    float lx = xw[3 * b] - aw[0], ly = xw[3 * b + 1] - aw[1], lz = xw[3 * b + 2] - aw[2];
                    float len = sqrtf(lx * lx + ly * ly + lz * lz);
                    if (!(len < thr)) continue;
                    float den = (infl == 0.5f) ? sqrtf(len) : powf(len, infl);
                    float sc = (-infl * psize) / den;
                    nx = fmaf(sc, lx, nx);
                    ny = fmaf(sc, ly, ny);
                    nz = fmaf(sc, lz, nz);
                    v = v + psize / den;
                } else {
                    float dx = node[0] - xs[3 * b], dy = node[1] - xs[3 * b + 1], dz = node[2] - xs[3 * b + 2];
                    float r2 = dx * dx + dy * dy + dz * dz;
                    if (!(r2 <= k.hh)) continue;
                    float t = k.hh - r2;
                    float mt = mass[b] * (t * t);
                    v = fmaf(mt, t, v);
                    nx = fmaf(mt, dx, nx);
                    ny = fmaf(mt, dy, ny);
                    nz = fmaf(mt, dz, nz);
                }
                for (int ch = 0; ch < 4; ++ch) col[ch] += (float)argb_channel(colour[b], ch);
                N++;
            }
        }
        if (!ref) v = v * k.poly6f;
        float nl = sqrtf(nx * nx + ny * ny + nz * nz);
        if (nl > 0.f) {
            nx = nx / nl;
            ny = ny / nl;
            nz = nz / nl;
        }
        lat[4 * q] = v;
        lat[4 * q + 1] = nx;
        lat[4 * q + 2] = ny;
        lat[4 * q + 3] = nz;
        if (lcol) {
            float avg[4] = {0.f, 0.f, 0.f, 0.f};
            if (N)
                for (int ch = 0; ch < 4; ++ch) avg[ch] = col[ch] / (float)N;
            lcol[q] = argb_pack(avg);
        }
    }
}

/* surface.hpp:47-53, including the 1e-5 snapping (compared in double, as there). */
static inline int snap_select(float iso, float v1, float v2) {
    if ((double)fabsf(iso - v1) < 0.00001) return 1;
    if ((double)fabsf(iso - v2) < 0.00001) return 2;
    if ((double)fabsf(v1 - v2) < 0.00001) return 1;
    return 0;
}

static void lerp_vec(float iso, const float *p1, const float *p2, float v1, float v2, float *o) {
    int s = snap_select(iso, v1, v2);
    if (s == 1) {
        o[0] = p1[0]; o[1] = p1[1]; o[2] = p1[2];
        return;
    }
    if (s == 2) {
        o[0] = p2[0]; o[1] = p2[1]; o[2] = p2[2];
        return;
    }
    float mu = (iso - v1) / (v2 - v1);
    for (int a = 0; a < 3; ++a) o[a] = p1[a] + (p2[a] - p1[a]) * mu;
}

static uint32_t lerp_colour(float iso, uint32_t c1, uint32_t c2, float v1, float v2) {
    int s = snap_select(iso, v1, v2);
    if (s == 1) return c1;
    if (s == 2) return c2;
    float mu = (iso - v1) / (v2 - v1);
    float ch[4];
    for (int i = 0; i < 4; ++i) {
        float a = (float)argb_channel(c1, i), b = (float)argb_channel(c2, i);
        ch[i] = a + (b - a) * mu;
    }
    return argb_pack(ch);
}

size_t orc_march(const fgb_params *p, const fgb_config *c, const orc_lattice *l, const float *lat,
                 const uint32_t *lcol, uint8_t *cases, fgb_mesh_triangle *tris, size_t cap) {
    (void)p;
    fgb_mc_tables T;
    fgb_mc_tables_build(&T);
    const size_t sx = l->size[0], sy = l->size[1], sz = l->size[2];
    if (sx < 2 || sy < 2 || sz < 2) return 0;
    const size_t mx = sx - 1, my = sy - 1, mz = sz - 1;
    const size_t cubes = mx * my * mz;
    const float iso = c->isolevel;
    uint32_t *cnt = (uint32_t *)malloc(cubes * sizeof(uint32_t));
    uint8_t *cs = (uint8_t *)malloc(cubes);
#pragma omp parallel for schedule(static)
    for (long q = 0; q < (long)cubes; ++q) {
        size_t x = (size_t)q / (my * mz), y = ((size_t)q / mz) % my, z = (size_t)q % mz;
        uint32_t ci = 0;
        for (int i = 0; i < 8; ++i) {
            size_t idx = ((x + FGB_MC_CORNER_OFFSETS[i][0]) * sy + (y + FGB_MC_CORNER_OFFSETS[i][1])) * sz +
                         (z + FGB_MC_CORNER_OFFSETS[i][2]);
            if (lat[4 * idx] < iso) ci |= 1u << i;
        }
        cs[q] = (uint8_t)ci;
        cnt[q] = T.edge_mask[ci] ? (uint32_t)(T.num_verts[ci] / 3) : 0u;
    }
    size_t *off = (size_t *)malloc((cubes + 1) * sizeof(size_t));
    off[0] = 0;
    for (size_t q = 0; q < cubes; ++q) off[q + 1] = off[q] + cnt[q];
    const size_t total = off[cubes];
    if (cases) memcpy(cases, cs, cubes);
    if (tris) {
#pragma omp parallel for schedule(dynamic, 1024)
        for (long iq = 0; iq < (long)cubes; ++iq) {
            size_t q = (size_t)iq;
            if (!cnt[q] || off[q] >= cap) continue;
            size_t x = q / (my * mz), y = (q / mz) % my, z = q % mz;
            uint32_t ci = cs[q];
            float val[8], pw[8][3], nrm[8][3];
            uint32_t col[8];
            for (int i = 0; i < 8; ++i) {
                size_t ox = x + FGB_MC_CORNER_OFFSETS[i][0], oy = y + FGB_MC_CORNER_OFFSETS[i][1],
                       oz = z + FGB_MC_CORNER_OFFSETS[i][2];
                size_t idx = (ox * sy + oy) * sz + oz;
                val[i] = lat[4 * idx];
                nrm[i][0] = lat[4 * idx + 1];
                nrm[i][1] = lat[4 * idx + 2];
                nrm[i][2] = lat[4 * idx + 3];
                col[i] = lcol ? lcol[idx] : 0xffffffffu;
                /* oclsph.hpp:275: (offset * step + min) * scale */
                pw[i][0] = ((float)ox * l->step + l->origin[0]) * c->scale;
                pw[i][1] = ((float)oy * l->step + l->origin[1]) * c->scale;
                pw[i][2] = ((float)oz * l->step + l->origin[2]) * c->scale;
            }
            float ev[12][3], en[12][3];
            uint32_t ec[12];
            for (int e = 0; e < 12; ++e) {
                if (!(T.edge_mask[ci] & (1u << e))) continue;
                int a = FGB_MC_EDGE_CORNERS[e][0], b = FGB_MC_EDGE_CORNERS[e][1];
                lerp_vec(iso, pw[a], pw[b], val[a], val[b], ev[e]);
                lerp_vec(iso, nrm[a], nrm[b], val[a], val[b], en[e]);
                ec[e] = lerp_colour(iso, col[a], col[b], val[a], val[b]);
            }
            size_t o = off[q];
            for (int t = 0; t < T.num_verts[ci] && o < cap; t += 3, ++o) {
                fgb_mesh_triangle *m = &tris[o];
                for (int j = 0; j < 3; ++j) {
                    int e = T.tri[ci][t + j];
                    m->v[3 * j] = ev[e][0];
                    m->v[3 * j + 1] = ev[e][1];
                    m->v[3 * j + 2] = ev[e][2];
                    m->n[3 * j] = en[e][0];
                    m->n[3 * j + 1] = en[e][1];
                    m->n[3 * j + 2] = en[e][2];
                    m->c[j] = ec[e];
                }
            }
        }
    }
    free(cnt);
    free(cs);
    free(off);
    return total;
}

size_t orc_surface(const fgb_params *p, const fgb_config *c, size_t n, const int32_t *type,
                   const float *mass, const float *pos, const uint32_t *colour, float *lattice,
                   uint32_t *lattice_colour, uint8_t *cases, fgb_mesh_triangle *tris, size_t cap) {
    orc_grid g;
    orc_lattice l;
    orc_grid_geometry(p, c, &g);
    orc_lattice_geometry(p, c, &g, &l);
    const size_t samples = (size_t)l.size[0] * l.size[1] * l.size[2];
    float *xs = (float *)malloc(3 * (n ? n : 1) * sizeof(float));
    uint32_t *key = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    uint32_t *order = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    for (size_t i = 0; i < n; ++i) {
        for (int a = 0; a < 3; ++a) xs[3 * i + a] = pos[3 * i + a] / c->scale;
        key[i] = orc_key(&g, p->h, xs[3 * i], xs[3 * i + 1], xs[3 * i + 2]);
    }
    argsort_keys(n, key, order);
    int32_t *st = (int32_t *)malloc((n ? n : 1) * sizeof(int32_t));
    float *sm = (float *)malloc((n ? n : 1) * sizeof(float));
    float *sxs = (float *)malloc(3 * (n ? n : 1) * sizeof(float));
    float *sxw = (float *)malloc(3 * (n ? n : 1) * sizeof(float));
    uint32_t *sc = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    uint32_t *sk = (uint32_t *)malloc((n ? n : 1) * sizeof(uint32_t));
    for (size_t i = 0; i < n; ++i) {
        size_t o = order[i];
        st[i] = type[o];
        sm[i] = mass[o];
        sc[i] = colour ? colour[o] : 0xffffffffu;
        sk[i] = key[o];
        for (int a = 0; a < 3; ++a) {
            sxs[3 * i + a] = xs[3 * o + a];
            sxw[3 * i + a] = pos[3 * o + a];
        }
    }
    uint32_t *cells = (uint32_t *)malloc((size_t)g.table_n * 2 * sizeof(uint32_t));
    build_cells(n, sk, g.table_n, cells);
    float *lat = lattice ? lattice : (float *)malloc(4 * samples * sizeof(float));
    uint32_t *lcol = lattice_colour ? lattice_colour : (uint32_t *)malloc(samples * sizeof(uint32_t));
    lattice_field(p, c, &g, &l, n, st, sm, sxs, sxw, sc, cells, lat, lcol);
    size_t total = orc_march(p, c, &l, lat, lcol, cases, tris, cap);
    if (!lattice) free(lat);
    if (!lattice_colour) free(lcol);
    free(xs);
    free(key);
    free(order);
    free(st);
    free(sm);
    free(sxs);
    free(sxw);
    free(sc);
    free(sk);
    free(cells);
    return total;
}

/* ------------------------------------------------------------ vertex welding */

typedef struct weld_item {
    uint32_t key[3];
    uint32_t idx;
} weld_item;

static int cmp_weld(const void *a, const void *b) {
    const weld_item *x = (const weld_item *)a, *y = (const weld_item *)b;
    for (int k = 0; k < 3; ++k)
        if (x->key[k] != y->key[k]) return x->key[k] < y->key[k] ? -1 : 1;
    return x->idx < y->idx ? -1 : (x->idx > y->idx);
}

/* geometry.hpp:152-166 (first appearance wins), by sorting (position bytes, index):
 * within a run of equal positions the first item holds the smallest index. */
size_t orc_weld(const fgb_mesh_triangle *tris, size_t n, uint32_t *indices, float *vertices) {
    const size_t nv = 3 * n;
    if (!nv) return 0;
    weld_item *it = (weld_item *)malloc(nv * sizeof(weld_item));
    uint32_t *first = (uint32_t *)malloc(nv * sizeof(uint32_t));
    uint32_t *rank = (uint32_t *)malloc(nv * sizeof(uint32_t));
    for (size_t i = 0; i < nv; ++i) {
        memcpy(it[i].key, &tris[i / 3].v[3 * (i % 3)], 12);
        it[i].idx = (uint32_t)i;
    }
    qsort(it, nv, sizeof(weld_item), cmp_weld);
    for (size_t s = 0; s < nv;) {
        size_t e = s + 1;
        while (e < nv && memcmp(it[e].key, it[s].key, 12) == 0) ++e;
        for (size_t j = s; j < e; ++j) first[it[j].idx] = it[s].idx;
        s = e;
    }
    size_t count = 0;
    for (size_t i = 0; i < nv; ++i) {
        if (first[i] == (uint32_t)i) {
            rank[i] = (uint32_t)count;
            memcpy(&vertices[3 * count], &tris[i / 3].v[3 * (i % 3)], 12);
            ++count;
        }
        indices[i] = rank[first[i]];
    }
    free(it);
    free(first);
    free(rank);
    return count;
}
