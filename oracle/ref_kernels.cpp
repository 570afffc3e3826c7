// ref_kernels.cpp -- TEST INFRASTRUCTURE ONLY: the oracle's checker, never shipped.
//
// Runs the reference's own OpenCL kernel bodies on the CPU, compiled as C++ straight
// from the reference tree, so that tests can pin the oracle's floating-point
// restatement to the reference's code rather than to a reading of it:
//   include/fluid/oclsph_kernel.h:281-303  sph_diffuse
//   include/fluid/oclsph_kernel.h:305-332  sph_lambda
//   include/fluid/oclsph_kernel.h:335-384  sph_delta (+ oclsph_collision.h:7-58)
//   include/fluid/oclsph_kernel.h:404-416  sph_finalise
//   include/fluid/oclsph_kernel.h:421-530  mc_lattice
//   include/fluid/oclsph_kernel.h:545-596  mc_size
//   include/fluid/oclsph_kernel.h:599-735  mc_eval (with lerpAll)
//
// How the OpenCL C compiles as C++ (oracle/Makefile):
//   - the recipe rewrites OpenCL vector literals "(float3)(a, b, c)" into C++
//     constructor calls "float3(a, b, c)" (a C++ compiler reads the former as a cast
//     of a comma expression) and writes the result to oracle/_ref/; nothing else in
//     the file changes;
//   - SPH_H is defined on the command line as the reference's host does it,
//     "-DSPH_H=" + std::to_string(h) (oclsph.hpp:178), for h = 0.1;
//   - the OpenCL vocabulary below: address-space qualifiers vanish, vector types are
//     small structs with component-wise operators, and each built-in is a plain IEEE
//     single-precision function, named here because OpenCL leaves its precision to
//     the device (the reference's fast-math build, clutils.hpp:164-169):
//       mad(a, b, c)        fmaf(a, b, c) (the fused reading; the oracle fuses too)
//       pown(x, n)          x * x * ... left to right
//       pow(x, y)           powf
//       native_divide(a, b) a / b;   native_recip(x) 1 / x
//       fast_length(v)      sqrtf(x*x + y*y + z*z), summed left to right
//       fast_distance(a, b) fast_length(a - b)
//       fast_normalize(v)   each component / fast_length(v)
//       dot(a, b)           a.x*b.x + a.y*b.y + a.z*b.z, left to right
//       mix(a, b, t)        a + (b - a) * t
//       convert_uchar4(f)   truncation toward zero; NaN and values outside [0, 255]
//                           (undefined in OpenCL without _sat) give 0 and 255
//   - work items run one after another; a work-group holds one item, so mc_size's
//     local reduction returns each cube's own count;
//   - sph_delta writes pStar in place while other items read it, a race with no
//     defined result (oclsph_kernel.h:355,374).  The driver runs it as the Jacobi
//     step the oracle follows: each item runs against the unchanged input, and its
//     new pStar is moved to the output afterwards.
// Built by oracle/Makefile into oracle/_ref/ only where the reference tree exists.
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <vector>

namespace oclk {

typedef unsigned int uint;
typedef unsigned char uchar;

struct float3 {
    union {
        struct { float x, y, z, pad_; };
        struct { float s0, s1, s2, s3_; };
    };
    float3() { x = y = z = pad_ = 0.f; }
    explicit float3(float v) { x = y = z = v, pad_ = 0.f; }
    float3(float a, float b, float c) { x = a, y = b, z = c, pad_ = 0.f; }
};
struct float4 {
    union {
        struct { float x, y, z, w; };
        struct { float s0, s1, s2, s3; };
    };
    float4() { x = y = z = w = 0.f; }
    explicit float4(float v) { x = y = z = w = v; }
    float4(float a, float b, float c, float d) { x = a, y = b, z = c, w = d; }
};
struct uint3 {
    uint x, y, z, pad_;
    uint3() : x(0), y(0), z(0), pad_(0) {}
    explicit uint3(uint v) : x(v), y(v), z(v), pad_(0) {}
    uint3(uint a, uint b, uint c) : x(a), y(b), z(c), pad_(0) {}
};
struct uchar4 {
    union {
        struct { uchar x, y, z, w; };
        struct { uchar s0, s1, s2, s3; };
    };
    uchar4() { x = y = z = w = 0; }
    uchar4(uchar a, uchar b, uchar c, uchar d) { x = a, y = b, z = c, w = d; }
};

inline float3 operator+(float3 a, float3 b) { return float3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 operator-(float3 a, float3 b) { return float3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float3 operator*(float3 a, float3 b) { return float3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float3 operator*(float3 a, float s) { return float3(a.x * s, a.y * s, a.z * s); }
inline float3 operator*(float s, float3 a) { return float3(s * a.x, s * a.y, s * a.z); }
inline float3 operator/(float3 a, float s) { return float3(a.x / s, a.y / s, a.z / s); }
inline float3 &operator+=(float3 &a, float3 b) { return a = a + b; }
inline float4 operator+(float4 a, float4 b) { return float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline float4 operator-(float4 a, float4 b) { return float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline float4 operator*(float4 a, float s) { return float4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline float4 operator/(float4 a, float s) { return float4(a.x / s, a.y / s, a.z / s, a.w / s); }
inline float4 &operator+=(float4 &a, float4 b) { return a = a + b; }
inline uint3 operator+(uint3 a, uint3 b) { return uint3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline uint3 operator-(uint3 a, uint3 b) { return uint3(a.x - b.x, a.y - b.y, a.z - b.z); }

inline float mad(float a, float b, float c) { return fmaf(a, b, c); }
inline float3 mad(float3 a, float b, float3 c) { return float3(fmaf(a.x, b, c.x), fmaf(a.y, b, c.y), fmaf(a.z, b, c.z)); }
inline float pown(float x, int n) {
    float r = x;
    for (int i = 1; i < n; ++i) r = r * x;
    return r;
}
inline float pow(float x, float y) { return powf(x, y); }
inline float native_divide(float a, float b) { return a / b; }
inline float native_recip(float a) { return 1.f / a; }
inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float3 cross(float3 a, float3 b) {
    return float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float fast_length(float3 v) { return sqrtf(v.x * v.x + v.y * v.y + v.z * v.z); }
inline float fast_distance(float3 a, float3 b) { return fast_length(a - b); }
inline float3 fast_normalize(float3 v) {
    const float l = fast_length(v);
    return float3(v.x / l, v.y / l, v.z / l);
}
inline float select(float a, float b, bool c) { return c ? b : a; }
inline uint select(uint a, uint b, bool c) { return c ? b : a; }
inline float3 mix(float3 a, float3 b, float t) { return a + (b - a) * t; }
inline float4 mix(float4 a, float4 b, float t) { return a + (b - a) * t; }
inline uint atomic_inc(volatile uint *p) { return (*p)++; }  // items run one at a time
template <class T> inline T min(T a, T b) { return b < a ? b : a; }
template <class T> inline T max(T a, T b) { return a < b ? b : a; }
inline float3 min(float3 a, float3 b) { return float3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
inline float3 max(float3 a, float3 b) { return float3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
inline int clamp(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
inline float4 clamp(float4 v, float lo, float hi) {
    return float4(fminf(fmaxf(v.x, lo), hi), fminf(fmaxf(v.y, lo), hi), fminf(fmaxf(v.z, lo), hi),
                  fminf(fmaxf(v.w, lo), hi));
}
inline float4 convert_float4(uchar4 c) { return float4((float)c.x, (float)c.y, (float)c.z, (float)c.w); }
inline float3 convert_float3(uint3 v) { return float3((float)v.x, (float)v.y, (float)v.z); }
inline uchar to_uchar(float f) {
    if (!(f > 0.f)) return 0;  // NaN and non-positive
    if (f >= 255.f) return 255;
    return (uchar)f;
}
inline uchar4 convert_uchar4(float4 f) { return uchar4(to_uchar(f.x), to_uchar(f.y), to_uchar(f.z), to_uchar(f.w)); }

// one work item at a time; a work-group holds one item
static size_t g_gid[3];
inline size_t get_global_id(int d) { return g_gid[d]; }
inline size_t get_local_id(int) { return 0; }
inline size_t get_local_size(int) { return 1; }
inline size_t get_group_id(int) { return g_gid[0]; }
#define CLK_LOCAL_MEM_FENCE 0
inline void barrier(int) {}

#define global
#define local
#define kernel
#define constant
#define ALIGNED_(x) __attribute__((aligned(x)))
#define M_PI_F 3.14159265358979323846f
#define LIBFLUID_CL_TYPES  // cl_types.h needs the OpenCL headers; its stubs are above

// curves.h first, with a C++ constructor for its uint3, so that to3d is right
#define CURVE_UINT3_TYPE uint3
#define CURVE_UINT3_CTOR(x, y, z) (uint3((x), (y), (z)))
#include "curves.h"
#include "oclsph_kernel_cxx.h"

#undef global
#undef local
#undef kernel
#undef constant
}  // namespace oclk

using namespace oclk;

static uchar4 unpack_argb(uint32_t c) {  // clutil::unpackARGB (clutils.hpp:223-228)
    return uchar4((c >> 24) & 0xff, (c >> 16) & 0xff, (c >> 8) & 0xff, c & 0xff);
}
static uint32_t pack_argb(uchar4 c) {  // clutil::packARGB (clutils.hpp:205-210)
    return ((uint32_t)c.s0 << 24) | ((uint32_t)c.s1 << 16) | ((uint32_t)c.s2 << 8) | (uint32_t)c.s3;
}
static std::vector<float3> load3(const float *p, size_t n) {
    std::vector<float3> v(n);
    for (size_t i = 0; i < n; ++i) v[i] = float3(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
    return v;
}
static void store3(const std::vector<float3> &v, float *p) {
    for (size_t i = 0; i < v.size(); ++i) {
        p[3 * i] = v[i].x;
        p[3 * i + 1] = v[i].y;
        p[3 * i + 2] = v[i].z;
    }
}

// The grid table of oclsph.hpp:744-767: gridTable[k] is the first sorted index whose
// key is >= k, for k < zCurveGridIndexAtCoord(extent).
static std::vector<uint> grid_table(const uint32_t *keys, size_t n, const uint32_t ext[3]) {
    const size_t table_n = zCurveGridIndexAtCoord(ext[0], ext[1], ext[2]);
    std::vector<uint> t(table_n);
    uint gi = 0;
    for (size_t i = 0; i < table_n; ++i) {
        t[i] = gi;
        while (gi != n && keys[gi] == i) gi++;
    }
    return t;
}

// FOR_EACH_NEIGHBOUR__ (oclsph_kernel.h:150-192) reads gridTable at 27 unclamped
// neighbour keys; true when every read of a particle with this key stays in the table.
static bool neighbours_in_table(size_t key, size_t table_n) {
    const size_t x = coordAtZCurveGridIndex0(key), y = coordAtZCurveGridIndex1(key), z = coordAtZCurveGridIndex2(key);
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx)
                if (zCurveGridIndexAtCoord(x + dx, y + dy, z + dz) >= table_n) return false;
    return true;
}

extern "C" {

float refk_h(void) { return (float)SPH_H; }

// One solve of the reference's kernels on particles already predicted and sorted
// (what oclsph.hpp:716-853 hands to runSphKernel): sph_diffuse, `iterations` x
// (sph_lambda, sph_delta), sph_finalise (oclsph.hpp:563-641).
//   keys: sorted z-indices; pstar, position (world), velocity (as copied before the
//   forces, oclsph.hpp:300): 3n; tris: 9 per triangle; cfg: dt, scale, min_bound[3],
//   max_bound[3]; ext: grid extent (oclsph.hpp:386).
// Outputs: pstar_out, position_out, velocity_out (3n), lambda_out (n, last iteration),
// colour_out (n, ARGB after diffusion; obstacles keep theirs, oclsph.hpp:885-889).
// Returns 0, or -1 when a particle's neighbour reads would leave the table.
int refk_solve(uint32_t n, const uint32_t *keys, const int32_t *type, const float *mass, const uint32_t *colour,
               const float *pstar, const float *position, const float *velocity, const float *tris, uint32_t n_tris,
               const float *cfg, uint32_t iterations, const uint32_t *ext, float *pstar_out, float *position_out,
               float *velocity_out, float *lambda_out, uint32_t *colour_out) {
    std::vector<uint> table = grid_table(keys, n, ext);
    const uint table_n = (uint)table.size();
    for (uint32_t i = 0; i < n; ++i)
        if (type[i] != Obstacle && !neighbours_in_table(keys[i], table_n)) return -1;
    ClSphConfig config;
    memset(&config, 0, sizeof config);
    config.dt = cfg[0];
    config.scale = cfg[1];
    config.iteration = iterations;
    config.minBound = float3(cfg[2], cfg[3], cfg[4]);
    config.maxBound = float3(cfg[5], cfg[6], cfg[7]);
    std::vector<uint> zindex(keys, keys + n);
    std::vector<ClSphType> types(n);
    for (uint32_t i = 0; i < n; ++i) types[i] = type[i] ? Obstacle : Fluid;
    std::vector<float> masses(mass, mass + n);
    std::vector<uchar4> cols(n), diffused(n);
    for (uint32_t i = 0; i < n; ++i) cols[i] = unpack_argb(colour[i]);
    std::vector<float3> ps = load3(pstar, n), pos = load3(position, n), vel = load3(velocity, n);
    std::vector<float3> next(n), deltaP(n);
    std::vector<float> lambda(n, 0.f);
    std::vector<ClSphTraiangle> mesh(n_tris ? n_tris : 1);
    for (uint32_t t = 0; t < n_tris; ++t) {
        mesh[t].a = float3(tris[9 * t], tris[9 * t + 1], tris[9 * t + 2]);
        mesh[t].b = float3(tris[9 * t + 3], tris[9 * t + 4], tris[9 * t + 5]);
        mesh[t].c = float3(tris[9 * t + 6], tris[9 * t + 7], tris[9 * t + 8]);
    }
    for (uint32_t a = 0; a < n; ++a) {
        g_gid[0] = a;
        diffused[a] = cols[a];
        sph_diffuse(&config, zindex.data(), table.data(), table_n, types.data(), ps.data(), cols.data(),
                    diffused.data());
    }
    for (uint32_t it = 0; it < iterations; ++it) {
        for (uint32_t a = 0; a < n; ++a) {
            g_gid[0] = a;
            sph_lambda(&config, zindex.data(), table.data(), table_n, types.data(), ps.data(), masses.data(),
                       lambda.data());
        }
        for (uint32_t a = 0; a < n; ++a) {  // Jacobi: every item reads the unchanged input
            g_gid[0] = a;
            const float3 saved = ps[a];
            sph_delta(&config, zindex.data(), table.data(), table_n, types.data(), mesh.data(), n_tris, ps.data(),
                      lambda.data(), pos.data(), vel.data(), deltaP.data());
            next[a] = ps[a];
            ps[a] = saved;
        }
        ps.swap(next);
    }
    for (uint32_t a = 0; a < n; ++a) {
        g_gid[0] = a;
        sph_finalise(&config, types.data(), ps.data(), pos.data(), vel.data());
    }
    store3(ps, pstar_out);
    store3(pos, position_out);
    store3(vel, velocity_out);
    memcpy(lambda_out, lambda.data(), n * sizeof(float));
    for (uint32_t i = 0; i < n; ++i) colour_out[i] = type[i] ? colour[i] : pack_argb(diffused[i]);
    return 0;
}

// mc_lattice over a lattice of sizes[0] x sizes[1] x sizes[2] samples (oclsph.hpp:
// 418-427): keys/type/position (world)/colour sorted by the z-index of the grid the
// field is sampled with; min_ext in solver units; mc: sampleResolution, particleSize,
// particleInfluence, isolevel; scale.  lattice_out: 4 floats per sample (value,
// normal), index3d order (curves.h:16-19); colour_out: ARGB per sample.  A sample the
// kernel skips (oclsph_kernel.h:456-459) keeps zeros.
int refk_lattice(uint32_t n, const uint32_t *keys, const int32_t *type, const float *position,
                 const uint32_t *colour, const uint32_t *ext, const float *min_ext, const uint32_t *sizes,
                 const float *mc, float scale, float *lattice_out, uint32_t *colour_out) {
    std::vector<uint> table = grid_table(keys, n, ext);
    ClSphConfig config;
    memset(&config, 0, sizeof config);
    config.scale = scale;
    ClMcConfig mcc;
    mcc.sampleResolution = mc[0];
    mcc.particleSize = mc[1];
    mcc.particleInfluence = mc[2];
    mcc.isolevel = mc[3];
    std::vector<ClSphType> types(n);
    for (uint32_t i = 0; i < n; ++i) types[i] = type[i] ? Obstacle : Fluid;
    std::vector<float3> pos = load3(position, n);
    std::vector<uchar4> cols(n);
    for (uint32_t i = 0; i < n; ++i) cols[i] = unpack_argb(colour[i]);
    const size_t total = (size_t)sizes[0] * sizes[1] * sizes[2];
    std::vector<float4> pns(total);
    std::vector<uchar4> lcs(total);
    const float3 mn(min_ext[0], min_ext[1], min_ext[2]);
    const uint3 sz(sizes[0], sizes[1], sizes[2]), ex(ext[0], ext[1], ext[2]);
    for (size_t x = 0; x < sizes[0]; ++x)
        for (size_t y = 0; y < sizes[1]; ++y)
            for (size_t z = 0; z < sizes[2]; ++z) {
                g_gid[0] = x, g_gid[1] = y, g_gid[2] = z;
                mc_lattice(&config, &mcc, table.data(), (uint)table.size(), types.data(), mn, sz, ex, pos.data(),
                           cols.data(), pns.data(), lcs.data());
            }
    for (size_t i = 0; i < total; ++i) {
        lattice_out[4 * i] = pns[i].s0;
        lattice_out[4 * i + 1] = pns[i].s1;
        lattice_out[4 * i + 2] = pns[i].s2;
        lattice_out[4 * i + 3] = pns[i].s3;
        colour_out[i] = pack_argb(lcs[i]);
    }
    return 0;
}

// mc_size with one cube per work-group: counts[q] = triangles of cube q, cubes in
// to3d order over (sizes - 1) (oclsph_kernel.h:554-567).
int refk_cube_counts(const uint32_t *sizes, float isolevel, const float *lattice, uint32_t *counts) {
    ClMcConfig mcc;
    memset(&mcc, 0, sizeof mcc);
    mcc.isolevel = isolevel;
    const size_t total = (size_t)sizes[0] * sizes[1] * sizes[2];
    std::vector<float4> values(total);
    for (size_t i = 0; i < total; ++i)
        values[i] = float4(lattice[4 * i], lattice[4 * i + 1], lattice[4 * i + 2], lattice[4 * i + 3]);
    const size_t cubes = (size_t)(sizes[0] - 1) * (sizes[1] - 1) * (sizes[2] - 1);
    const uint3 sz(sizes[0], sizes[1], sizes[2]);
    uint local_sum[1];
    for (size_t q = 0; q < cubes; ++q) {
        g_gid[0] = q;
        mc_size(&mcc, sz, values.data(), local_sum, counts);
    }
    return 0;
}

// mc_eval over every cube with items run in cube order, so the atomic counter hands
// out triangle slots cube-major (cubes in to3d order, TriTable order within a cube).
// lattice/colour as refk_lattice gives them; out: 21 words per triangle (v0 v1 v2,
// n0 n1 n2 as floats, then the three ARGB colours, packARGB), at most cap triangles.
// Returns the triangle count.
size_t refk_mc_eval(const uint32_t *sizes, const float *min_ext, const float *mc, float scale, const float *lattice,
                    const uint32_t *colour, float *out, size_t cap) {
    ClSphConfig config;
    memset(&config, 0, sizeof config);
    config.scale = scale;
    ClMcConfig mcc;
    mcc.sampleResolution = mc[0];
    mcc.particleSize = mc[1];
    mcc.particleInfluence = mc[2];
    mcc.isolevel = mc[3];
    const size_t total = (size_t)sizes[0] * sizes[1] * sizes[2];
    std::vector<float4> pns(total);
    std::vector<uchar4> lcs(total);
    for (size_t i = 0; i < total; ++i) {
        pns[i] = float4(lattice[4 * i], lattice[4 * i + 1], lattice[4 * i + 2], lattice[4 * i + 3]);
        lcs[i] = unpack_argb(colour[i]);
    }
    const size_t cubes = (size_t)(sizes[0] - 1) * (sizes[1] - 1) * (sizes[2] - 1);
    // at most 5 triangles a cube
    std::vector<float3> v[3], nr[3];
    std::vector<uchar4> c[3];
    for (int k = 0; k < 3; ++k) {
        v[k].resize(5 * cubes + 1);
        nr[k].resize(5 * cubes + 1);
        c[k].resize(5 * cubes + 1);
    }
    volatile uint counter = 0;
    const float3 mn(min_ext[0], min_ext[1], min_ext[2]);
    const uint3 sz(sizes[0], sizes[1], sizes[2]);
    for (size_t q = 0; q < cubes; ++q) {
        g_gid[0] = q;
        mc_eval(&config, &mcc, mn, sz, pns.data(), lcs.data(), &counter, 0, v[0].data(), v[1].data(), v[2].data(),
                nr[0].data(), nr[1].data(), nr[2].data(), c[0].data(), c[1].data(), c[2].data());
    }
    const size_t count = counter;
    for (size_t t = 0; t < count && t < cap; ++t) {
        float *o = out + 21 * t;
        for (int k = 0; k < 3; ++k) {
            o[3 * k] = v[k][t].x;
            o[3 * k + 1] = v[k][t].y;
            o[3 * k + 2] = v[k][t].z;
            o[9 + 3 * k] = nr[k][t].x;
            o[9 + 3 * k + 1] = nr[k][t].y;
            o[9 + 3 * k + 2] = nr[k][t].z;
            const uint32_t packed = pack_argb(c[k][t]);
            memcpy(&o[18 + k], &packed, 4);
        }
    }
    return count;
}
}
