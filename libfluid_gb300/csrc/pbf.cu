// pbf.cu -- the Position Based Fluids step as sm_103a gather kernels.
//
// One step (all scenes of a batch in one launch per stage):
//   k_predict_keys   predict p* and its 30-bit Morton key  (oclsph.hpp:289-387)
//   radix sort       (sort.cu)                              (oclsph.hpp:733-743)
//   k_reorder_cells  gather the state into sorted SoA float4 and write each cell's
//                    {start, end} by adjacent difference    (oclsph.hpp:746-767, 822-853)
//   ref only:        k_cell_colours, k_diffuse              (oclsph_kernel.h:281-303)
//   iterations x {k_lambda, k_delta}                        (oclsph_kernel.h:305-384)
//   k_delta(last)    also finalises x / v                   (oclsph_kernel.h:404-416)
//   baseline only:   k_vorticity_xsph, k_vorticity_apply    (PBF paper eq. 15-17)
// Gathers walk the 27 neighbour cells in the reference's order (dz, dy, dx with x
// fastest, oclsph_kernel.h:155-183) and each cell's particles in sorted order, so
// every per-particle sum has one fixed order.  The solve is Jacobi: k_delta reads
// one p* buffer and writes the other (the reference updates p* in place, a race).
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>

#include "fgb_internal.h"

namespace fgb {
namespace {

constexpr int kRef = FGB_PROFILE_REF;

// Squared distance of a pair in the baseline profile's gathers: two fused
// multiply-adds, as the oracle's baseline restatement computes it (the ref profile
// keeps the reference's sum of three products).
__device__ __forceinline__ float dist2(float dx, float dy, float dz) {
    return __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz)));
}

// Predicted position of one particle in solver units (oclsph.hpp:297-323).
__device__ __forceinline__ float3 predict(const Phys &ph, const SceneDev &S, const WellDev *wells, int32_t type,
                                          float4 x, float4 v) {
    float3 ps = make_float3(x.x / S.scale, x.y / S.scale, x.z / S.scale);
    if (type == FGB_TYPE_OBSTACLE) return ps;
    const bool ref = ph.profile == kRef;
    const float mass = x.w;
    float f[3];
    for (int a = 0; a < 3; ++a) f[a] = ref ? mass * S.g[a] : S.g[a];
    const float xa[3] = {x.x, x.y, x.z};
    for (uint32_t w = 0; w < S.n_wells; ++w) {
        const WellDev wl = wells[S.well_first + w];
        float d0 = xa[0] - wl.centre[0], d1 = xa[1] - wl.centre[1], d2 = xa[2] - wl.centre[2];
        float dist = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
        if (dist < 75.f) {
            float u0 = wl.centre[0] - xa[0], u1 = wl.centre[1] - xa[1], u2 = wl.centre[2] - xa[2];
            float ul = sqrtf(u0 * u0 + u1 * u1 + u2 * u2);
            const float u[3] = {u0, u1, u2};
            for (int a = 0; a < 3; ++a) {
                float rhat = u[a] / ul;
                float fw = ref ? ((rhat * wl.force) * mass) / (dist * dist) : (rhat * wl.force) / (dist * dist);
                if (fw < -10.f) fw = -10.f;
                if (fw > 10.f) fw = 10.f;
                f[a] = f[a] + fw;
            }
        }
    }
    const float va[3] = {v.x, v.y, v.z};
    float p[3];
    for (int a = 0; a < 3; ++a) {
        float vn = f[a] * S.dt + va[a];
        p[a] = vn * S.dt + xa[a] / S.scale;
    }
    return make_float3(p[0], p[1], p[2]);
}

__device__ __forceinline__ uint32_t cell_key(const SceneDev &S, float h, float x, float y, float z) {
    return morton3(quantise(x, S.min_ext[0], h, S.ext[0]), quantise(y, S.min_ext[1], h, S.ext[1]),
                   quantise(z, S.min_ext[2], h, S.ext[2]));
}

template <class F>
__device__ __forceinline__ void for_neighbours(const SceneDev &S, const uint2 *__restrict__ cells, uint32_t key,
                                               uint32_t mbits, F &&f) {
    const uint32_t m = morton_of(key, mbits);
    for_neighbour_cells(S, cells, (int)compact10(m), (int)compact10(m >> 1), (int)compact10(m >> 2), f);
}

__global__ void k_predict_keys(const SceneDev *__restrict__ scenes, const WellDev *__restrict__ wells, Phys ph,
                               uint32_t n, uint32_t mbits, const uint32_t *__restrict__ keys_prev,
                               const float4 *__restrict__ x, const float4 *__restrict__ v,
                               const int32_t *__restrict__ type, uint32_t *__restrict__ keys_out,
                               uint32_t *__restrict__ vals_out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t s = scene_of(keys_prev[i], mbits);
        const SceneDev &S = scenes[s];
        const float3 p = predict(ph, S, wells, type[i], x[i], v[i]);
        const uint32_t m = cell_key(S, ph.h, p.x, p.y, p.z);
        keys_out[i] = (mbits >= 32 ? 0u : (s << mbits)) | m;
        vals_out[i] = i;
    }
}

// Gather the state into sorted order, recompute p* there (same bits as
// k_predict_keys), and write each occupied cell's {start, end}.
__global__ void k_reorder_cells(const SceneDev *__restrict__ scenes, const WellDev *__restrict__ wells, Phys ph,
                                uint32_t n, uint32_t mbits, const uint32_t *__restrict__ keys,
                                const uint32_t *__restrict__ vals, const float4 *__restrict__ x0,
                                const float4 *__restrict__ v0, const int32_t *__restrict__ type0,
                                const uint32_t *__restrict__ col0, const uint32_t *__restrict__ slot0,
                                float4 *__restrict__ x1, float4 *__restrict__ v1, int32_t *__restrict__ type1,
                                uint32_t *__restrict__ col1, uint32_t *__restrict__ slot1,
                                float4 *__restrict__ ps, uint2 *__restrict__ cells, uint64_t cells_n,
                                uint32_t *err, uint32_t *mass_range) {
    // the smallest mass's bits and the complement of the largest's, both by atomicMin
    // (one pair per CTA); the masses are all equal when range[0] == ~range[1]
    __shared__ uint32_t s_lo, s_hi;
    if (threadIdx.x == 0) s_lo = s_hi = 0xffffffffu;
    __syncthreads();
    uint32_t lo = 0xffffffffu, hi = 0xffffffffu;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t j = vals[i];
        const uint32_t key = keys[i];
        const uint32_t s = scene_of(key, mbits);
        const SceneDev &S = scenes[s];
        const float4 xj = x0[j], vj = v0[j];
        const int32_t tj = type0[j];
        const float3 p = predict(ph, S, wells, tj, xj, vj);
        x1[i] = xj;
        v1[i] = vj;
        type1[i] = tj;
        col1[i] = col0[j];
        slot1[i] = slot0[j];
        ps[i] = make_float4(p.x, p.y, p.z, xj.w);
        lo = min(lo, __float_as_uint(xj.w));
        hi = min(hi, ~__float_as_uint(xj.w));
        const uint64_t c = (uint64_t)S.table_base + morton_of(key, mbits);
        if (c >= cells_n) {
            raise_error(err, ERR_CELL_RANGE);
            continue;
        }
        if (i == 0 || keys[i - 1] != key) cells[c].x = i;
        if (i + 1 == n || keys[i + 1] != key) cells[c].y = i + 1;
    }
    lo = __reduce_min_sync(0xffffffffu, lo);
    hi = __reduce_min_sync(0xffffffffu, hi);
    if ((threadIdx.x & 31u) == 0) {
        atomicMin(&s_lo, lo);
        atomicMin(&s_hi, hi);
    }
    __syncthreads();
    if (threadIdx.x == 0 && mass_range) {
        atomicMin(&mass_range[0], s_lo);
        atomicMin(&mass_range[1], s_hi);
    }
}


// ---------------------------------------------------------------- gathers
//
// Neighbour lists.  The reference walks the 27 cells of the grid built from p* at
// the start of the step on every pass (oclsph_kernel.h:150-192); only ~16% of the
// ~216 candidates lie within h.  The first lambda pass does that walk and also keeps,
// per particle and in walk order, every candidate within h + skin (a Verlet list).
// Later passes iterate the list instead of the cells.  A list is exact -- it holds
// every candidate that the walk would find within h, in the walk's order -- while
// disp_a + disp_b <= skin for all candidates b, where disp is the distance moved
// since the grid was built: r_now <= h implies r_build <= h + disp_a + disp_b.  Each
// delta pass records disp_a and a per-cell maximum; a particle whose bound fails (or
// whose list overflowed) walks the cells.  Either way the per-particle sums see the
// same candidates in the same order, so results are identical to the walk.

struct GatherArgs {
    const SceneDev *scenes;
    const TriDev *tris;
    Phys ph;
    uint32_t n, mbits;
    const uint32_t *keys;
    const uint2 *cells;
    const int32_t *type;
    uint32_t *nlist;
    uint16_t *ncount;
    uint32_t cap;
    float list_r2, skin;
    const float4 *ps_grid;
    float *disp;
    uint32_t *cellmax;
    uint8_t *valid;
    uint32_t *hlist;
    uint16_t *hcount;
    uint32_t hcap;
    uint8_t *near;  // null: no near rows
    float near_r2, near_skin;
    uint32_t *over;  // build pass: [0] Verlet rows, [1] hit rows that overflowed (null: not counted)
    // null, or: warps of checked passes on near rows [0] / filtering [1]; particles of
    // filtering later lambda passes on their list [2] / walking [3]
    uint32_t *near_stats;
    // the lambda pass's p* with lambda in w, read by the delta pass (null: off), and the
    // batch's smallest and largest mass (float bits) of the step
    float4 *plam;
    float4 *pom;  // the vorticity pass's p* with |omega| in w, read by the apply pass (null: off)
    const uint32_t *mass_range;
    // null: one particle per thread over a flat grid; else this launch's tile counter
    // (zero at launch) for a persistent grid taking tiles of ppt x blockDim particles
    uint32_t *queue;
    uint32_t verlet_off;
    uint32_t ppt;
    // null, or per scene: kPolicyWords words of k_list_policy's state
    uint32_t *list_policy;
    int count_lists;  // this lambda pass samples how many particles could use their list
};

enum ListMode { kBuild = 0, kFresh = 1, kCheck = 2, kStored = 3 };

__device__ __forceinline__ float max_cell_disp(const SceneDev &S, const uint32_t *__restrict__ cellmax,
                                               uint32_t key, uint32_t mbits) {
    const uint32_t m = morton_of(key, mbits);
    const int cx = (int)compact10(m), cy = (int)compact10(m >> 1), cz = (int)compact10(m >> 2);
    const uint32_t *tbl = cellmax + S.table_base;
    uint32_t best = 0;  // non-negative floats order like their bit patterns
    for_cell_indices(S, cx, cy, cz, [&](uint32_t k) { best = max(best, __ldg(&tbl[k])); });
    return __uint_as_float(best);
}

// Whether particle a may use its list for the current positions.
// mcd: the 27 cells' maximum displacement when the caller already has it, else < 0.
template <int MODE>
__device__ __forceinline__ bool use_list(const GatherArgs &A, const SceneDev &S, uint32_t a, uint32_t key,
                                         float mcd = -1.f) {
    if (A.cap == 0 || MODE == kBuild) return false;
    const uint16_t c = A.ncount[a];
    if (c == kListOverflow) return false;
    if (MODE == kFresh) return true;
    if (MODE == kStored) return A.valid[a] != 0;
    if (mcd < 0.f) mcd = max_cell_disp(S, A.cellmax, key, A.mbits);
    const bool ok = A.disp[a] + mcd <= A.skin;
    A.valid[a] = ok ? 1 : 0;
    return ok;
}

// Where a gather finds its neighbours' data.  GlobalSpace: the batch arrays by sorted
// particle index, walks through the cell table.  pos(b): p* of candidate b; x(b): the
// pass's second array; fluid(b): whether b is not an obstacle.
constexpr int kPrefetch = 4;

template <class T>
struct GlobalSpace {
    const float4 *ps;
    const T *ex;
    const int32_t *type;
    static constexpr bool kPacked = false;
    __device__ __forceinline__ float4 pos(uint32_t b) const { return __ldg(&ps[b]); }
    __device__ __forceinline__ T x(uint32_t b) const { return __ldg(&ex[b]); }
    __device__ __forceinline__ bool fluid(uint32_t b) const { return __ldg(&type[b]) != FGB_TYPE_OBSTACLE; }
    // the delta pass's view of a candidate: its mass and its lambda
    __device__ __forceinline__ float mass(const float4 &pb) const { return pb.w; }
    __device__ __forceinline__ float lam(uint32_t b, const float4 &) const { return __ldg(&ex[b]); }
    __device__ __forceinline__ T omega_of(uint32_t b) const { return __ldg(&ex[b]); }
    // Visit the particles of the 27 cells in walk order as f(b, p_b); loads run four
    // candidates ahead of the arithmetic.
    template <class F>
    __device__ __forceinline__ void walk(const GatherArgs &A, const SceneDev &S, uint32_t key, F &f) const {
        const uint32_t m = morton_of(key, A.mbits);
        const uint2 *tbl = A.cells + S.table_base;
        for_cell_indices(S, (int)compact10(m), (int)compact10(m >> 1), (int)compact10(m >> 2), [&](uint32_t k) {
            const uint2 c = __ldg(&tbl[k]);
            visit(c.x, c.y, f);
        });
    }
    template <class F>
    __device__ __forceinline__ void visit(uint32_t lo, uint32_t hi, F &f) const {
        uint32_t b = lo;
        for (; b + kPrefetch <= hi; b += kPrefetch) {
            float4 p[kPrefetch];
#pragma unroll
            for (int k = 0; k < kPrefetch; ++k) p[k] = pos(b + k);
#pragma unroll
            for (int k = 0; k < kPrefetch; ++k) f(b + k, p[k]);
        }
        if (b < hi) {  // the last 1-3 candidates, their loads issued together
            const uint32_t rest = hi - b;
            const float4 p0 = pos(b);
            const float4 p1 = rest > 1 ? pos(b + 1) : p0;
            const float4 p2 = rest > 2 ? pos(b + 2) : p0;
            f(b, p0);
            if (rest > 1) f(b + 1, p1);
            if (rest > 2) f(b + 2, p2);
        }
    }
};

// The delta pass's candidates through the lambda pass's copy of p* with each
// particle's lambda in w (plam): one 16-byte load a neighbour instead of p* and lambda
// apart.  Their masses are then not in w: the ref profile's delta sum uses none, and
// the baseline takes this path only when every particle of the batch has the same
// mass (`m`).
struct PackedSpace : GlobalSpace<float> {
    float m;
    static constexpr bool kPacked = true;
    __device__ __forceinline__ float mass(const float4 &) const { return m; }
    __device__ __forceinline__ float lam(uint32_t, const float4 &pb) const { return pb.w; }
};

// The vorticity-apply pass's candidates through the vorticity pass's copy of p* with
// each particle's |omega| in w (pom): one 16-byte load a neighbour instead of p* and
// omega apart, when every particle of the batch has the same mass (`m`).
struct PackedOmegaSpace : GlobalSpace<float4> {
    float m;
    static constexpr bool kPacked = true;
    __device__ __forceinline__ float mass(const float4 &) const { return m; }
};

// Visit the c entries of particle a's row (particle-major, `cap` entries per row, cap
// a multiple of 4) as f(b, p_b); indices arrive four at a time as one 16-byte load,
// and the four positions are loaded before any arithmetic.
// kSameKernel: the row was written earlier in this kernel, so it is read through L2
// (ld.global.cg) rather than the read-only path.
template <bool kSameKernel = false, class Sp, class F>
__device__ __forceinline__ void for_row(const uint32_t *__restrict__ base, uint32_t cap, uint32_t a, uint32_t c,
                                        const Sp &sp, F &f) {
    const uint4 *row = reinterpret_cast<const uint4 *>(base + (size_t)a * cap);
    auto load = [&](uint32_t j) { return kSameKernel ? __ldcg(row + (j >> 2)) : __ldg(row + (j >> 2)); };
    // software pipeline: the next index vector is in flight while the current four
    // candidates are loaded and processed (rows usually stream from HBM)
    uint4 next = c ? load(0) : make_uint4(0, 0, 0, 0);
    uint32_t j = 0;
    for (; j + 4 <= c; j += 4) {
        const uint4 b = next;
        if (j + 4 < c) next = load(j + 4);
        const float4 p0 = sp.pos(b.x), p1 = sp.pos(b.y), p2 = sp.pos(b.z), p3 = sp.pos(b.w);
        f(b.x, p0);
        f(b.y, p1);
        f(b.z, p2);
        f(b.w, p3);
    }
    if (j < c) {
        const uint4 b = next;
        const uint32_t rest = c - j;
        const float4 p0 = sp.pos(b.x);
        const float4 p1 = rest > 1 ? sp.pos(b.y) : p0;
        const float4 p2 = rest > 2 ? sp.pos(b.z) : p0;
        f(b.x, p0);
        if (rest > 1) f(b.y, p1);
        if (rest > 2) f(b.z, p2);
    }
}

// for_row with the pass's second array gathered beside each position (the delta
// pass's lambda_b, the vorticity passes' v_b and omega_b): the four values load with
// the four positions, ahead of the arithmetic.  f(b, p_b, get) with get() the value.
template <bool kSameKernel = false, class Sp, class F>
__device__ __forceinline__ void for_row_x(const uint32_t *__restrict__ base, uint32_t cap, uint32_t a, uint32_t c,
                                          const Sp &sp, F &f) {
    const uint4 *row = reinterpret_cast<const uint4 *>(base + (size_t)a * cap);
    auto load = [&](uint32_t j) { return kSameKernel ? __ldcg(row + (j >> 2)) : __ldg(row + (j >> 2)); };
    uint4 next = c ? load(0) : make_uint4(0, 0, 0, 0);
    uint32_t j = 0;
    for (; j + 4 <= c; j += 4) {
        const uint4 b = next;
        if (j + 4 < c) next = load(j + 4);
        const float4 p0 = sp.pos(b.x), p1 = sp.pos(b.y), p2 = sp.pos(b.z), p3 = sp.pos(b.w);
        const auto e0 = sp.x(b.x), e1 = sp.x(b.y), e2 = sp.x(b.z), e3 = sp.x(b.w);
        f(b.x, p0, [&] { return e0; });
        f(b.y, p1, [&] { return e1; });
        f(b.z, p2, [&] { return e2; });
        f(b.w, p3, [&] { return e3; });
    }
    if (j < c) {
        const uint4 b = next;
        const uint32_t rest = c - j;
        const float4 p0 = sp.pos(b.x);
        const float4 p1 = rest > 1 ? sp.pos(b.y) : p0;
        const float4 p2 = rest > 2 ? sp.pos(b.z) : p0;
        const auto e0 = sp.x(b.x);
        const auto e1 = rest > 1 ? sp.x(b.y) : e0;
        const auto e2 = rest > 2 ? sp.x(b.z) : e0;
        f(b.x, p0, [&] { return e0; });
        if (rest > 1) f(b.y, p1, [&] { return e1; });
        if (rest > 2) f(b.z, p2, [&] { return e2; });
    }
}

template <class Sp, class F>
__device__ __forceinline__ void for_candidates(const GatherArgs &A, const SceneDev &S, uint32_t a, uint32_t key,
                                               bool list, const Sp &sp, F &&f) {
    if (list) for_row(A.nlist, A.cap, a, A.ncount[a], sp, f);
    else sp.walk(A, S, key, f);
}

// Hit lists.  A lambda pass and the delta pass after it read the same p*, so they
// agree on which candidates lie within h; likewise the two vorticity passes.  The
// first pass of each pair filters its candidates (Verlet list or cell walk) by range
// alone, appending those within h (in walk order) to a per-pass hit list, then runs
// its kernel arithmetic over the hits; the second pass of the pair iterates the same
// hits.  About 35 entries instead of the ~60 of the Verlet list or the ~216 of the
// cell walk, and no lanes idle on a range test during the arithmetic.  Every pass
// still applies its own range tests to each hit, so its sums are bit-identical to a
// walk.  A row that overflows (count > hcap) sends its passes back to the candidates.
// Rows are particle-major like the Verlet lists.
//
// Near rows.  The build pass (the step's first lambda pass) keeps in the hit row
// every candidate within h + near_skin of the grid positions rather than within h,
// and marks the row (near[a]).  By the same bound as the Verlet lists, that row still
// holds every neighbour within h while disp_a + max disp_b <= near_skin, so a later
// lambda pass for which the bound holds runs its arithmetic straight over the row,
// without the range-filter phase, and leaves the row for the delta pass after it.
// The extra entries (~15% at 0.05 h) fail the passes' own range tests, so the sums
// are unchanged.  A pass for which the bound fails (for any lane of the warp) filters
// as before and clears the mark: the row it writes holds the hits of that pass's
// positions only.
struct RowWriter {
    uint4 *row;
    uint32_t cap, count = 0;
    uint4 q;
    __device__ __forceinline__ RowWriter(uint32_t *base, uint32_t cap_, uint32_t a)
        : row(reinterpret_cast<uint4 *>(base + (size_t)a * cap_)), cap(cap_), q(make_uint4(0u, 0u, 0u, 0u)) {}
    // the last four entries, oldest in x: shifted along on every append and stored
    // whole when four new ones have come in
    __device__ __forceinline__ void add(uint32_t b) {
        q.x = q.y;
        q.y = q.z;
        q.z = q.w;
        q.w = b;
        ++count;
        if ((count & 3u) == 0 && count <= cap) row[(count >> 2) - 1] = q;
    }
    // add(b) when `hit`, the vector shifted by selects instead of under a branch: the
    // same entries.  Measured faster in the list build and the vorticity filter (1.1%
    // off the 64 batched scenes' step), no faster in the lambda filter's walks.
    __device__ __forceinline__ void add_if(bool hit, uint32_t b) {
        q.x = hit ? q.y : q.x;
        q.y = hit ? q.z : q.y;
        q.z = hit ? q.w : q.z;
        q.w = hit ? b : q.w;
        count += hit ? 1u : 0u;
        if (hit && (count & 3u) == 0 && count <= cap) row[(count >> 2) - 1] = q;
    }
    // store the last partial vector, its entries moved to the front (the tail entries
    // are stale and never read); returns the row's count, kListOverflow when it did
    // not fit
    __device__ __forceinline__ uint16_t close() {
        const uint32_t r = count & 3u;
        if (r && count <= cap) {
            uint4 t = q;
            if (r == 1) t.x = q.w;
            if (r == 2) t.x = q.z, t.y = q.w;
            if (r == 3) t.x = q.y, t.y = q.z, t.z = q.w;
            row[count >> 2] = t;
        }
        return count > cap ? kListOverflow : (uint16_t)count;
    }
};

struct HitWriter : RowWriter {
    __device__ __forceinline__ HitWriter(const GatherArgs &A, uint32_t a) : RowWriter(A.hlist, A.hcap, a) {}
    __device__ __forceinline__ void close(const GatherArgs &A, uint32_t a) {
        if (cap) A.hcount[a] = RowWriter::close();
    }
};

__device__ __forceinline__ void close_hits_empty(const GatherArgs &A, uint32_t a) {
    if (A.hcap) A.hcount[a] = 0;
}


// The list policy's sample: per scene of the warp, the particles whose list (or near
// row) served this pass and those that walked.
__device__ __forceinline__ void count_list_use(const GatherArgs &A, uint32_t key, bool used) {
    const uint32_t sc = scene_of(key, A.mbits);
    const unsigned m = __activemask();
    const unsigned grp = __match_any_sync(m, sc);
    const unsigned on = __ballot_sync(m, used) & grp;
    if ((threadIdx.x & 31u) == (unsigned)(__ffs(grp) - 1)) {
        if (on) atomicAdd(&A.list_policy[kPolicyWords * sc + 3], (uint32_t)__popc(on));
        if (grp & ~on) atomicAdd(&A.list_policy[kPolicyWords * sc + 4], (uint32_t)__popc(grp & ~on));
    }
}

// One count per warp of a checked pass: whether it ran on its near rows.
__device__ __forceinline__ void count_near(const GatherArgs &A, bool on_rows) {
    if (!A.near_stats) return;
    const unsigned m = __activemask();
    if ((threadIdx.x & 31u) == (unsigned)(__ffs(m) - 1)) atomicAdd(&A.near_stats[on_rows ? 0 : 1], 1u);
}

__device__ __forceinline__ bool have_hits(const GatherArgs &A, uint32_t a) {
    return A.hcap != 0 && A.hcount[a] != kListOverflow;
}

template <class Sp, class F>
__device__ __forceinline__ void for_hits(const GatherArgs &A, uint32_t a, const Sp &sp, F &&f) {
    for_row(A.hlist, A.hcap, a, A.hcount[a], sp, f);
}

// The particles of one gather launch, f(a) for each.  Flat: one particle per thread,
// one CTA per blockDim particles.  Persistent: a grid sized to the GPU whose CTAs take
// tiles of ppt x blockDim consecutive sorted particles -- a block of cells of one
// scene, or of a few small ones -- from an atomic counter until none is left, each
// thread ppt particles of a tile, blockDim apart.  Every particle's work is the same
// either way.
template <bool kTiles, class F>
__device__ __forceinline__ void for_tiles(const GatherArgs &A, F &&f) {
    if constexpr (!kTiles) {
        f(blockIdx.x * blockDim.x + threadIdx.x);
        return;
    }
    __shared__ uint32_t s_tile;
    const uint64_t span = (uint64_t)blockDim.x * A.ppt;
    for (;;) {
        __syncthreads();  // every thread has read the previous tile
        if (threadIdx.x == 0) s_tile = atomicAdd(A.queue, 1u);
        __syncthreads();
        const uint64_t base = (uint64_t)s_tile * span;
        if (base >= A.n) break;
        for (uint32_t k = 0; k < A.ppt; ++k) {
            const uint64_t a = base + (uint64_t)k * blockDim.x + threadIdx.x;
            f(a < A.n ? (uint32_t)a : A.n);  // A.n: past the end, the body returns
        }
    }
}

// Whether this step builds scene sc's Verlet lists and near rows (k_list_policy).
__device__ __forceinline__ bool lists_on(const GatherArgs &A, uint32_t sc) {
    return !A.list_policy || A.list_policy[kPolicyWords * sc] != 0u;
}

// The step's Verlet lists on their own: each particle walks its 27 cells and keeps, in
// walk order, every candidate within h + skin.  The first lambda pass then filters the
// fresh lists (near rows) instead of walking, so the walk carries one row writer and
// no kernel arithmetic.
template <class Sp>
__device__ __forceinline__ void build_body(const GatherArgs &A, uint32_t a, const Sp &sp, const float4 *__restrict__ ps) {
    if (a >= A.n) return;
    if (A.verlet_off || !lists_on(A, scene_of(A.keys[a], A.mbits))) {  // no lists this step: every pass walks
        A.ncount[a] = kListOverflow;
        return;
    }
    if (A.type[a] == FGB_TYPE_OBSTACLE) {
        A.ncount[a] = 0;
        return;
    }
    const uint32_t key = A.keys[a];
    const SceneDev &S = A.scenes[scene_of(key, A.mbits)];
    const float4 pa = ps[a];
    RowWriter built(A.nlist, A.cap, a);
    // membership only (the passes re-test every entry exactly): a contracted r^2,
    // within ~2e-7 of the sum of squares, against a radius rounded up by 1e-5
    for_candidates(A, S, a, key, false, sp, [&](uint32_t b, const float4 &pb) {
        const float dx = pa.x - pb.x, dy = pa.y - pb.y, dz = pa.z - pb.z;
        built.add_if(__fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz))) <= A.list_r2, b);
    });
    A.ncount[a] = built.close();
    if (A.over) {  // one atomic per warp, when rows overflowed
        const unsigned m = __activemask();
        const unsigned lo = __ballot_sync(m, built.count > A.cap);
        if (lo && (threadIdx.x & 31u) == (unsigned)(__ffs(m) - 1)) atomicAdd(&A.over[0], (uint32_t)__popc(lo));
    }
}

template <bool kTiles>
__global__ void __launch_bounds__(256) k_build_lists(GatherArgs A, const float4 *__restrict__ ps) {
    for_tiles<kTiles>(A, [&](uint32_t a) { build_body(A, a, GlobalSpace<char>{ps, nullptr, A.type}, ps); });
}

template <int PROFILE, int MODE, class Sp>
__device__ __forceinline__ void lambda_body(const GatherArgs &A, uint32_t a, const Sp &sp, const float4 *__restrict__ ps,
                                            float *__restrict__ lambda, float *__restrict__ density) {
    if (a >= A.n) return;
    if (A.type[a] == FGB_TYPE_OBSTACLE) {
        lambda[a] = 0.f;
        density[a] = 0.f;
        if (A.plam) {
            const float4 p = ps[a];
            A.plam[a] = make_float4(p.x, p.y, p.z, 0.f);
        }
        if (MODE == kBuild && A.cap) A.ncount[a] = 0;
        close_hits_empty(A, a);
        return;
    }
    const Phys &ph = A.ph;
    const uint32_t key = A.keys[a];
    const SceneDev &S = A.scenes[scene_of(key, A.mbits)];
    const float4 pa = ps[a];
    float rho = 0.f, gx = 0.f, gy = 0.f, gz = 0.f, g2 = 0.f;
    auto body = [&](uint32_t b, const float4 &pb) {
        const float dx = pa.x - pb.x, dy = pa.y - pb.y, dz = pa.z - pb.z;
        if (PROFILE == kRef) {
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (!(r2 <= ph.hh_le)) return;  // sqrtf(r2) > h: no contribution
            const float r = sqrtf(r2);
            if (r <= ph.h) {
                const float t = ph.hh - r * r;
                rho = __fmaf_rn(pa.w, ph.poly6f * (t * t * t), rho);
                if (r >= kKernelEpsilon) {
                    const float hr = ph.h - r;
                    const float sc = ph.spikyf * ((hr * hr) / r);
                    gx = __fmaf_rn(dx * sc, ph.inv_rho0, gx);
                    gy = __fmaf_rn(dy * sc, ph.inv_rho0, gy);
                    gz = __fmaf_rn(dz * sc, ph.inv_rho0, gz);
                }
            }
        } else {
            const float q2 = dist2(dx, dy, dz);
            if (q2 <= ph.hh) {
                const float t = ph.hh - q2;
                rho = __fmaf_rn(pb.w, t * t * t, rho);
                const float r = sqrtf(q2);
                if (r >= kKernelEpsilon) {
                    const float hr = ph.h - r;
                    const float sc = pb.w * ((hr * hr) / r);
                    gx = __fmaf_rn(sc, dx, gx);
                    gy = __fmaf_rn(sc, dy, gy);
                    gz = __fmaf_rn(sc, dz, gz);
                    g2 = __fmaf_rn(sc * sc, q2, g2);
                }
            }
        }
    };
    // a later pass whose near row still holds every neighbour iterates it directly;
    // the choice is made per warp (all lanes or none), as a warp that mixed the two
    // paths would run both one after the other
    float mcd = -1.f;
    bool done = false;
    if (MODE == kCheck && A.near) {
        bool ok = false;
        if (A.near[a] && have_hits(A, a)) {
            mcd = max_cell_disp(S, A.cellmax, key, A.mbits);
            ok = A.disp[a] + mcd <= A.near_skin;
        }
        done = __all_sync(__activemask(), ok);
        count_near(A, done);
        if (done && A.count_lists && A.list_policy) count_list_use(A, key, true);
        if (done) for_hits(A, a, sp, body);
        else A.near[a] = 0;
    }
    if (!done) {
        bool list = use_list<MODE>(A, S, a, key, mcd);
        // ref profile, checked passes: the whole warp walks when any of its lanes must.
        // Its clumped scenes mix lists and walks within warps, which then run both one
        // after the other (the walk gives the same sums: the list is the walk's
        // candidates within h + skin in walk order); the baseline profile is faster with
        // the choice per lane.
        if constexpr (MODE == kCheck && PROFILE == kRef) list = __all_sync(__activemask(), list);
        if (MODE == kCheck && A.count_lists && A.list_policy) count_list_use(A, key, list);
        if (MODE == kCheck && A.near_stats) {
            const unsigned m = __activemask();
            const unsigned on = __ballot_sync(m, list);
            if ((threadIdx.x & 31u) == (unsigned)(__ffs(m) - 1)) {
                atomicAdd(&A.near_stats[2], (uint32_t)__popc(on));
                atomicAdd(&A.near_stats[3], (uint32_t)__popc(m & ~on));
            }
        }
        if (A.hcap == 0 && MODE != kBuild) {
            for_candidates(A, S, a, key, list, sp, body);
        } else {
            // phase 1: range filter (and the Verlet list on the build pass)
            RowWriter built(A.nlist, MODE == kBuild ? A.cap : 0u, a);
            HitWriter hits(A, a);
            const bool near_row =
                (MODE == kBuild || MODE == kFresh) && A.near && lists_on(A, scene_of(key, A.mbits));
            // membership only (the arithmetic re-tests every entry exactly): a contracted
            // r^2, within ~2e-7 of the sum of squares, against radii rounded up by >= 1e-6
            const float hit_r2 = (PROFILE == kRef ? ph.hh_le : ph.hh) * 1.000001f;
            for_candidates(A, S, a, key, list, sp, [&](uint32_t b, const float4 &pb) {
                const float dx = pa.x - pb.x, dy = pa.y - pb.y, dz = pa.z - pb.z;
                const float r2 = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz)));
                if (MODE == kBuild && r2 <= A.list_r2) built.add(b);
                if (r2 <= (near_row ? A.near_r2 : hit_r2)) hits.add(b);
            });
            if (MODE == kBuild && A.cap) A.ncount[a] = built.close();
            hits.close(A, a);
            if ((MODE == kBuild || MODE == kFresh) && A.over) {  // one atomic per warp, when rows overflowed
                const unsigned m = __activemask();
                const unsigned lo = __ballot_sync(m, MODE == kBuild && A.cap && built.count > A.cap);
                const unsigned ho = __ballot_sync(m, A.hcap && hits.count > A.hcap);
                if ((lo | ho) && (threadIdx.x & 31u) == (unsigned)(__ffs(m) - 1)) {
                    if (lo) atomicAdd(&A.over[0], (uint32_t)__popc(lo));
                    if (ho) atomicAdd(&A.over[1], (uint32_t)__popc(ho));
                }
            }
            // the first pass sets every mark (none when this step builds no near rows)
            if ((MODE == kBuild || MODE == kFresh) && A.near) A.near[a] = near_row && A.hcap && hits.count <= A.hcap ? 1 : 0;
            // phase 2: the kernel arithmetic over the hits, in walk order
            if (A.hcap && hits.count <= A.hcap) for_row<true>(A.hlist, A.hcap, a, hits.count, sp, body);
            else for_candidates(A, S, a, key, list, sp, body);
        }
    }
    float dens, lam;
    if (PROFILE == kRef) {
        dens = rho;
        const float norm2 = gx * gx + gy * gy + gz * gz;
        const float C = dens / ph.rho0 - 1.f;
        lam = -C / (norm2 + ph.cfm);
    } else {
        dens = rho * ph.poly6f;
        const float gs = ph.spikyf * ph.inv_rho0;
        const float sx = gx * gs, sy = gy * gs, sz = gz * gs;
        const float denom = (sx * sx + sy * sy + sz * sz) + g2 * (gs * gs);
        const float C = dens * ph.inv_rho0 - 1.f;
        lam = -C / (denom + ph.cfm);
    }
    lambda[a] = lam;
    density[a] = dens;
    if (A.plam) A.plam[a] = make_float4(pa.x, pa.y, pa.z, lam);
}

template <int PROFILE, int MODE, bool kTiles>
__global__ void __launch_bounds__(256) k_lambda(GatherArgs A, const float4 *__restrict__ ps,
                                                float *__restrict__ lambda, float *__restrict__ density) {
    for_tiles<kTiles>(A, [&](uint32_t a) {
        lambda_body<PROFILE, MODE>(A, a, GlobalSpace<char>{ps, nullptr, A.type}, ps, lambda, density);
    });
}

__device__ __forceinline__ float corr_pow(float ratio, float n) {
    if (n == 4.f) {
        const float r2 = ratio * ratio;
        return r2 * r2;
    }
    return powf(ratio, n);
}

__device__ __forceinline__ float dot3(const float *a, const float *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// oclsph_collision.h:7-58 (first containing triangle within 40 world units wins).
__device__ void collide_triangles(const TriDev *__restrict__ tris, uint32_t first, uint32_t count, float *pos,
                                  float *vel) {
    for (uint32_t i = 0; i < count; ++i) {
        const TriDev t = tris[first + i];
        float e1[3], e2[3], nrm[3];
        for (int a = 0; a < 3; ++a) {
            e1[a] = t.b[a] - t.a[a];
            e2[a] = t.c[a] - t.a[a];
        }
        nrm[0] = e1[1] * e2[2] - e1[2] * e2[1];
        nrm[1] = e1[2] * e2[0] - e1[0] * e2[2];
        nrm[2] = e1[0] * e2[1] - e1[1] * e2[0];
        const float len = sqrtf(dot3(nrm, nrm));
        const float nn[3] = {nrm[0] / len, nrm[1] / len, nrm[2] / len};
        const float dist = dot3(nn, t.a) - dot3(nn, pos);
        if (-40.f <= dist && dist <= 40.f) {
            const float p0[3] = {pos[0] + nn[0] * dist, pos[1] + nn[1] * dist, pos[2] + nn[2] * dist};
            float v0[3], v1[3], v2[3];
            for (int a = 0; a < 3; ++a) {
                v0[a] = t.c[a] - t.a[a];
                v1[a] = t.b[a] - t.a[a];
                v2[a] = p0[a] - t.a[a];
            }
            const float d00 = dot3(v0, v0), d01 = dot3(v0, v1), d02 = dot3(v0, v2);
            const float d11 = dot3(v1, v1), d12 = dot3(v1, v2);
            const float inv = 1.f / (d00 * d11 - d01 * d01);
            const float u = (d11 * d02 - d01 * d12) * inv;
            const float w = (d00 * d12 - d01 * d02) * inv;
            if ((u >= 0.f) && (w >= 0.f) && (u + w < 1.f)) {
                const float vn = dot3(vel, nn);
                for (int a = 0; a < 3; ++a) {
                    vel[a] = vel[a] - (nn[a] * 2.f) * vn;
                    pos[a] = p0[a];
                }
                return;
            }
        }
    }
}

__device__ __forceinline__ void collide_sphere(const SceneDev &S, float *pos) {
    if (!S.sphere_enabled) return;
    const float d[3] = {pos[0] - S.sphere[0], pos[1] - S.sphere[1], pos[2] - S.sphere[2]};
    const float r = S.sphere[3];
    const float d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    if (!(d2 < r * r)) return;
    const float dist = sqrtf(d2);
    if (dist > 0.f) {
        const float s = r / dist;
        for (int a = 0; a < 3; ++a) pos[a] = S.sphere[a] + d[a] * s;
    } else {
        pos[0] = S.sphere[0];
        pos[1] = S.sphere[1] + r;
        pos[2] = S.sphere[2];
    }
}


// Final position and velocity of particle a into the caller's arrays (fgb_advance
// with direct host I/O): the step's last kernel stores them beside its own writes.
__device__ __forceinline__ void store_host_motion(const HostParticlesOut *__restrict__ hout, uint32_t a,
                                                  const float4 &xa, const float4 &va) {
    if (!hout) return;
    const uint32_t stride = hout->stride;  // 0: packed arrays, else the caller's records
    float *pp = hout->position, *pv = hout->velocity;
    if (pp) {
        float *q = stride ? (float *)((char *)pp + (size_t)a * stride) : pp + 3 * (size_t)a;
        q[0] = xa.x;
        q[1] = xa.y;
        q[2] = xa.z;
    }
    if (pv) {
        float *q = stride ? (float *)((char *)pv + (size_t)a * stride) : pv + 3 * (size_t)a;
        q[0] = va.x;
        q[1] = va.y;
        q[2] = va.z;
    }
}

template <int PROFILE, int MODE, class Sp>
__device__ __forceinline__ void delta_body(const GatherArgs &A, uint32_t a, const Sp &sp, const float4 *__restrict__ ps_in,
                                           const float *__restrict__ lambda, float4 *__restrict__ ps_out,
                                           float4 *__restrict__ x, float4 *__restrict__ v, int last,
                                           const HostParticlesOut *__restrict__ hout) {
    if (a >= A.n) return;
    const float4 pa = ps_in[a];
    if (A.type[a] == FGB_TYPE_OBSTACLE) {
        ps_out[a] = pa;
        if (A.cap) A.disp[a] = 0.f;
        if (PROFILE == kRef && last) store_host_motion(hout, a, x[a], v[a]);
        return;
    }
    const Phys &ph = A.ph;
    const uint32_t key = A.keys[a];
    const SceneDev &S = A.scenes[scene_of(key, A.mbits)];
    const float la = lambda[a];
    float px = 0.f, py = 0.f, pz = 0.f;
    // lam_b() is lambda of b (gathered beside p_b on rows, loaded on demand on walks)
    auto body = [&](uint32_t b, const float4 &pb, auto lam_b) {
        const float dx = pa.x - pb.x, dy = pa.y - pb.y, dz = pa.z - pb.z;
        if (PROFILE == kRef) {
            const float r2 = dx * dx + dy * dy + dz * dz;
            if (!(r2 <= ph.hh_le)) return;  // sqrtf(r2) > h: no contribution
            const float r = sqrtf(r2);
            float w = 0.f;
            if (r <= ph.h) {
                const float t = ph.hh - r * r;
                w = ph.poly6f * (t * t * t);
            }
            const float corr = -ph.corr_k * corr_pow(w / ph.corr_ref, ph.corr_n);
            const float factor = (la + lam_b() + corr) / ph.rho0;
            if (r >= kKernelEpsilon && r <= ph.h) {
                const float hr = ph.h - r;
                const float sc = ph.spikyf * ((hr * hr) / r);
                px = __fmaf_rn(dx * sc, factor, px);
                py = __fmaf_rn(dy * sc, factor, py);
                pz = __fmaf_rn(dz * sc, factor, pz);
            }
        } else {
            const float q2 = dist2(dx, dy, dz);
            if (q2 <= ph.hh) {
                const float r = sqrtf(q2);
                if (r >= kKernelEpsilon) {
                    const float t = ph.hh - q2;
                    const float corr = -ph.corr_k * corr_pow((t * t * t) * ph.inv_corr_wdq, ph.corr_n);
                    const float hr = ph.h - r;
                    const float sc = sp.mass(pb) * ((hr * hr) / r) * (la + lam_b() + corr);
                    px = __fmaf_rn(sc, dx, px);
                    py = __fmaf_rn(sc, dy, py);
                    pz = __fmaf_rn(sc, dz, pz);
                }
            }
        }
    };
    if (have_hits(A, a)) {
        if constexpr (Sp::kPacked) {
            auto packed = [&](uint32_t b, const float4 &pb) { body(b, pb, [&] { return pb.w; }); };
            for_row(A.hlist, A.hcap, a, A.hcount[a], sp, packed);
        } else {
            for_row_x(A.hlist, A.hcap, a, A.hcount[a], sp, body);
        }
    } else {
        for_candidates(A, S, a, key, use_list<MODE>(A, S, a, key), sp, [&](uint32_t b, const float4 &pb) {
            body(b, pb, [&] { return sp.lam(b, pb); });
        });
    }
    float world[3];
    if (PROFILE == kRef) {
        world[0] = (pa.x + px) * S.scale;
        world[1] = (pa.y + py) * S.scale;
        world[2] = (pa.z + pz) * S.scale;
    } else {
        const float gs = ph.spikyf * ph.inv_rho0;
        world[0] = (pa.x + px * gs) * S.scale;
        world[1] = (pa.y + py * gs) * S.scale;
        world[2] = (pa.z + pz * gs) * S.scale;
        collide_sphere(S, world);
    }
    float4 va = v[a];
    float vel[3] = {va.x, va.y, va.z};
    if (S.tri_count) {
        collide_triangles(A.tris, S.tri_first, S.tri_count, world, vel);
        v[a] = make_float4(vel[0], vel[1], vel[2], va.w);
    }
    float q[3];
    for (int d = 0; d < 3; ++d) {
        float w = world[d];
        w = fmaxf(S.min_b[d], w);
        w = fminf(S.max_b[d], w);
        q[d] = w / S.scale;
    }
    ps_out[a] = make_float4(q[0], q[1], q[2], pa.w);
    if (A.cap) {
        // distance moved since the grid was built, for the list bound of the next pass
        // (the per-cell maxima are cleared before every delta pass)
        const float4 g = A.ps_grid[a];
        const float ex = q[0] - g.x, ey = q[1] - g.y, ez = q[2] - g.z;
        const float d = sqrtf(ex * ex + ey * ey + ez * ez);
        // (a step without lists or near rows checks no bound)
        const uint32_t sc = scene_of(key, A.mbits);
        if (lists_on(A, sc)) {
            A.disp[a] = d;
            atomicMax(&A.cellmax[S.table_base + morton_of(key, A.mbits)], __float_as_uint(d));
        }
        if (last && A.list_policy) {  // one atomic pair per scene of the warp, for k_list_policy
            const unsigned m = __activemask();
            const unsigned grp = __match_any_sync(m, sc);
            const unsigned far = __ballot_sync(m, d > 0.5f * A.skin) & grp;
            if ((threadIdx.x & 31u) == (unsigned)(__ffs(grp) - 1)) {
                if (far) atomicAdd(&A.list_policy[kPolicyWords * sc + 1], (uint32_t)__popc(far));
                atomicAdd(&A.list_policy[kPolicyWords * sc + 2], (uint32_t)__popc(grp));
            }
        }
    }
    if (last) {
        const float4 xa = x[a];
        const float xo[3] = {xa.x, xa.y, xa.z};
        float nv[3], nx[3];
        for (int d = 0; d < 3; ++d) {
            const float dd = q[d] - xo[d] / S.scale;
            if (PROFILE == kRef) {
                nx[d] = q[d] * S.scale;
                nv[d] = __fmaf_rn(dd, S.inv_dt, vel[d]) * ph.damping;
            } else {
                nv[d] = dd * S.inv_dt;
            }
        }
        v[a] = make_float4(nv[0], nv[1], nv[2], va.w);
        if (PROFILE == kRef) {
            x[a] = make_float4(nx[0], nx[1], nx[2], xa.w);
            store_host_motion(hout, a, x[a], v[a]);
        }
    }
}

template <int PROFILE, int MODE, bool kTiles>
__global__ void __launch_bounds__(256)
    k_delta(GatherArgs A, const float4 *__restrict__ ps_in, const float *__restrict__ lambda,
            float4 *__restrict__ ps_out, float4 *__restrict__ x, float4 *__restrict__ v, int last,
            const HostParticlesOut *__restrict__ hout) {
    // the packed copy when the sums need no neighbour mass or all masses are equal
    // (the batch's smallest and largest mass, float bits, from the grid build)
    const bool packed = A.plam && (PROFILE == kRef || A.mass_range[0] == ~A.mass_range[1]);
    for_tiles<kTiles>(A, [&](uint32_t a) {
        if (packed)
            delta_body<PROFILE, MODE>(A, a, PackedSpace{{A.plam, nullptr, A.type}, __uint_as_float(A.mass_range[0])},
                                      ps_in, lambda, ps_out, x, v, last, hout);
        else
            delta_body<PROFILE, MODE>(A, a, GlobalSpace<float>{ps_in, lambda, A.type}, ps_in, lambda, ps_out, x, v,
                                      last, hout);
    });
}

__device__ __forceinline__ void cross3(const float *a, const float *b, float *o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

// Pass A: vorticity omega and the XSPH sum (fluid neighbours only).
template <class Sp>
__device__ __forceinline__ void vorticity_body(const GatherArgs &A, uint32_t a, const Sp &sp, const float4 *__restrict__ ps,
                                               const float4 *__restrict__ v, float4 *__restrict__ omega,
                                               float4 *__restrict__ vx) {
    if (a >= A.n) return;
    const float4 va4 = v[a];
    if (A.type[a] == FGB_TYPE_OBSTACLE) {
        omega[a] = make_float4(0.f, 0.f, 0.f, 0.f);
        vx[a] = va4;
        if (A.pom) {
            const float4 p = ps[a];
            A.pom[a] = make_float4(p.x, p.y, p.z, 0.f);
        }
        close_hits_empty(A, a);
        return;
    }
    const Phys &ph = A.ph;
    const uint32_t key = A.keys[a];
    const SceneDev &S = A.scenes[scene_of(key, A.mbits)];
    const float4 pa = ps[a];
    // the near row, while its bound still holds for the whole warp, serves this pass
    // and the apply pass (it holds obstacles and candidates beyond h, which both
    // passes' own tests skip); near[a] stays set to tell the apply pass
    float mcd = -1.f;
    bool near = false;
    if (A.near) {
        bool ok = false;
        if (A.near[a] && have_hits(A, a)) {
            mcd = max_cell_disp(S, A.cellmax, key, A.mbits);
            ok = A.disp[a] + mcd <= A.near_skin;
        }
        near = __all_sync(__activemask(), ok);
        count_near(A, near);
        if (!near) A.near[a] = 0;
    }
    const bool list = near ? false : use_list<kCheck>(A, S, a, key, mcd);
    const float va[3] = {va4.x, va4.y, va4.z};
    float o[3] = {0.f, 0.f, 0.f}, xs[3] = {0.f, 0.f, 0.f};
    // fluid_known: b came from a filtered hit row, which holds fluid particles only;
    // vel_b() is v of b (gathered beside p_b on rows, loaded on demand on walks)
    auto body = [&](uint32_t b, const float4 &pb, auto vel_b, bool fluid_known) {
        if (!fluid_known && S.obstacles && !sp.fluid(b)) return;
        const float d[3] = {pa.x - pb.x, pa.y - pb.y, pa.z - pb.z};
        const float r2 = dist2(d[0], d[1], d[2]);
        if (!(r2 <= ph.hh)) return;
        const float4 vb = vel_b();
        const float vab[3] = {vb.x - va[0], vb.y - va[1], vb.z - va[2]};
        const float t = ph.hh - r2;
        const float mw = pb.w * (t * t * t);
        xs[0] = __fmaf_rn(mw, vab[0], xs[0]);
        xs[1] = __fmaf_rn(mw, vab[1], xs[1]);
        xs[2] = __fmaf_rn(mw, vab[2], xs[2]);
        const float r = sqrtf(r2);
        if (r >= kKernelEpsilon) {
            const float hr = ph.h - r;
            const float sc = pb.w * ((hr * hr) / r);
            float cr[3];
            cross3(vab, d, cr);
            o[0] = __fmaf_rn(sc, cr[0], o[0]);
            o[1] = __fmaf_rn(sc, cr[1], o[1]);
            o[2] = __fmaf_rn(sc, cr[2], o[2]);
        }
    };
    auto any = [&](uint32_t b, const float4 &pb) {
        body(b, pb, [&] { return sp.x(b); }, false);
    };
    if (near) {
        auto any_row = [&](uint32_t b, const float4 &pb, auto vel_b) { body(b, pb, vel_b, false); };
        for_row_x(A.hlist, A.hcap, a, A.hcount[a], sp, any_row);
    } else if (A.hcap == 0) {
        for_candidates(A, S, a, key, list, sp, any);
    } else {
        // phase 1: fluid candidates within h; phase 2: the arithmetic over them
        HitWriter hits(A, a);
        const float hit_r2 = ph.hh * 1.000001f;  // membership only, as in the lambda filter
        for_candidates(A, S, a, key, list, sp, [&](uint32_t b, const float4 &pb) {
            const float dx = pa.x - pb.x, dy = pa.y - pb.y, dz = pa.z - pb.z;
            const float r2 = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz)));
            hits.add_if(r2 <= hit_r2 && (!S.obstacles || sp.fluid(b)), b);
        });
        hits.close(A, a);
        if (hits.count <= A.hcap) {
            auto fluid = [&](uint32_t b, const float4 &pb, auto vel_b) { body(b, pb, vel_b, true); };
            for_row_x<true>(A.hlist, A.hcap, a, hits.count, sp, fluid);
        } else {
            for_candidates(A, S, a, key, list, sp, any);
        }
    }
    const float gs = ph.spikyf * ph.inv_rho0;
    const float ws = ph.poly6f * ph.inv_rho0;
    // omega = sum_b m_b / rho0 (v_b - v_a) x grad_b W(x_a - x_b), and grad_b W = -grad_a W
    // = -spikyf (h - r)^2 d / r: the sum o carries grad_a's factor, so its sign flips
    const float ox = -(o[0] * gs), oy = -(o[1] * gs), oz = -(o[2] * gs);
    const float om = sqrtf(ox * ox + oy * oy + oz * oz);
    omega[a] = make_float4(ox, oy, oz, om);
    if (A.pom) A.pom[a] = make_float4(pa.x, pa.y, pa.z, om);
    vx[a] = make_float4(__fmaf_rn(ph.xsph_c, xs[0] * ws, va[0]), __fmaf_rn(ph.xsph_c, xs[1] * ws, va[1]),
                        __fmaf_rn(ph.xsph_c, xs[2] * ws, va[2]), va4.w);
}

template <bool kTiles>
__global__ void __launch_bounds__(256)
    k_vorticity_xsph(GatherArgs A, const float4 *__restrict__ ps, const float4 *__restrict__ v,
                     float4 *__restrict__ omega, float4 *__restrict__ vx) {
    for_tiles<kTiles>(A, [&](uint32_t a) { vorticity_body(A, a, GlobalSpace<float4>{ps, v, A.type}, ps, v, omega, vx); });
}

// Pass B: eta = grad |omega|, N = eta / |eta|, f = eps (N x omega); v = vx + dt f.
template <class Sp>
__device__ __forceinline__ void apply_body(const GatherArgs &A, uint32_t a, const Sp &sp, const float4 *__restrict__ ps,
                                           const float4 *__restrict__ omega, const float4 *__restrict__ vx,
                                           float4 *__restrict__ v, float4 *__restrict__ x,
                                           const HostParticlesOut *__restrict__ hout) {
    if (a >= A.n) return;
    if (A.type[a] == FGB_TYPE_OBSTACLE) {
        store_host_motion(hout, a, x[a], v[a]);
        return;
    }
    const Phys &ph = A.ph;
    const uint32_t key = A.keys[a];
    const SceneDev &S = A.scenes[scene_of(key, A.mbits)];
    const float4 pa = ps[a];
    const float4 oa = omega[a];
    float e[3] = {0.f, 0.f, 0.f};
    // fluid_known: b came from a filtered hit row, which holds fluid particles only;
    // om_b() is omega of b (gathered beside p_b on rows, loaded on demand on walks)
    auto body = [&](uint32_t b, const float4 &pb, auto om_b, bool fluid_known) {
        if (!fluid_known && S.obstacles && !sp.fluid(b)) return;
        const float d[3] = {pa.x - pb.x, pa.y - pb.y, pa.z - pb.z};
        const float r2 = dist2(d[0], d[1], d[2]);
        if (!(r2 <= ph.hh)) return;
        const float r = sqrtf(r2);
        if (!(r >= kKernelEpsilon)) return;
        const float hr = ph.h - r;
        const float sc = sp.mass(pb) * ((hr * hr) / r) * (om_b().w - oa.w);
        e[0] = __fmaf_rn(sc, d[0], e[0]);
        e[1] = __fmaf_rn(sc, d[1], e[1]);
        e[2] = __fmaf_rn(sc, d[2], e[2]);
    };
    if (have_hits(A, a)) {
        // a near row (still marked) holds obstacles too; a filtered row fluid only
        const bool fluid_rows = !(A.near && A.near[a]);
        if constexpr (Sp::kPacked) {
            auto row = [&](uint32_t b, const float4 &pb) {
                body(b, pb, [&] { return make_float4(0.f, 0.f, 0.f, pb.w); }, fluid_rows);
            };
            for_row(A.hlist, A.hcap, a, A.hcount[a], sp, row);
        } else {
            auto row = [&](uint32_t b, const float4 &pb, auto om_b) { body(b, pb, om_b, fluid_rows); };
            for_row_x(A.hlist, A.hcap, a, A.hcount[a], sp, row);
        }
    } else {
        for_candidates(A, S, a, key, use_list<kStored>(A, S, a, key), sp, [&](uint32_t b, const float4 &pb) {
            body(b, pb, [&] { return Sp::kPacked ? make_float4(0.f, 0.f, 0.f, pb.w) : sp.omega_of(b); }, false);
        });
    }
    const float gs = ph.spikyf * ph.inv_rho0;
    const float ex = e[0] * gs, ey = e[1] * gs, ez = e[2] * gs;
    const float el = sqrtf(ex * ex + ey * ey + ez * ez);
    float N[3] = {0.f, 0.f, 0.f};
    if (el > 0.f) {
        N[0] = ex / el;
        N[1] = ey / el;
        N[2] = ez / el;
    }
    const float om[3] = {oa.x, oa.y, oa.z};
    float f[3];
    cross3(N, om, f);
    const float4 vxa = vx[a];
    const float ve = ph.vort_eps, dt = S.dt;
    const float4 vn = make_float4(__fmaf_rn(dt, f[0] * ve, vxa.x), __fmaf_rn(dt, f[1] * ve, vxa.y),
                                  __fmaf_rn(dt, f[2] * ve, vxa.z), vxa.w);
    v[a] = vn;
    const float4 xa = x[a];
    const float4 xn = make_float4(pa.x * S.scale, pa.y * S.scale, pa.z * S.scale, xa.w);
    x[a] = xn;
    store_host_motion(hout, a, xn, vn);
}

template <bool kTiles>
__global__ void __launch_bounds__(256)
    k_vorticity_apply(GatherArgs A, const float4 *__restrict__ ps, const float4 *__restrict__ omega,
                      const float4 *__restrict__ vx, float4 *__restrict__ v, float4 *__restrict__ x,
                      const HostParticlesOut *__restrict__ hout) {
    // the vorticity pass's packed copy (p* with |omega| in w) when every mass is equal
    const bool packed = A.pom && A.mass_range[0] == ~A.mass_range[1];
    for_tiles<kTiles>(A, [&](uint32_t a) {
        if (packed)
            apply_body(A, a, PackedOmegaSpace{{A.pom, omega, A.type}, __uint_as_float(A.mass_range[0])}, ps, omega,
                       vx, v, x, hout);
        else
            apply_body(A, a, GlobalSpace<float4>{ps, omega, A.type}, ps, omega, vx, v, x, hout);
    });
}

// Colour diffusion of the ref profile (oclsph_kernel.h:281-303): each fluid particle
// averages the colours of every fluid candidate in its 27 cells (no distance test,
// itself included) and moves toward 1.33x that mean by dt/750, per 8-bit channel,
// clamped to [8, 255] and truncated.  The channel sums are integers below 2^24, exact
// in float in any order, so each cell's sums are formed once (k_cell_colours, at the
// cell's first sorted index) and a particle adds up 27 of them.
__global__ void k_cell_colours(uint32_t n, const uint32_t *__restrict__ keys, const int32_t *__restrict__ type,
                               const uint32_t *__restrict__ col, uint4 *__restrict__ agg,
                               uint32_t *__restrict__ count) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t key = keys[i];
        if (i > 0 && keys[i - 1] == key) continue;
        uint4 s = make_uint4(0, 0, 0, 0);
        uint32_t c = 0;
        for (uint32_t j = i; j < n && keys[j] == key; ++j) {
            if (type[j] == FGB_TYPE_OBSTACLE) continue;
            const uint32_t v = col[j];
            s.x += v & 0xffu;
            s.y += (v >> 8) & 0xffu;
            s.z += (v >> 16) & 0xffu;
            s.w += v >> 24;
            ++c;
        }
        agg[i] = s;
        count[i] = c;
    }
}

// OpenCL mix(x, y, t) = x + (y - x) t, then clamp and convert_uchar (round to zero)
__device__ __forceinline__ uint32_t diffuse_channel(uint32_t own, uint32_t sum, float count, float t) {
    const float x = (float)own;
    const float y = ((float)sum / count) * 1.33f;
    float o = x + (y - x) * t;
    o = fminf(fmaxf(o, 8.f), 255.f);
    return (uint32_t)o;
}

__global__ void k_diffuse(const SceneDev *__restrict__ scenes, uint32_t n, uint32_t mbits,
                          const uint32_t *__restrict__ keys, const uint2 *__restrict__ cells,
                          const int32_t *__restrict__ type, const uint4 *__restrict__ agg,
                          const uint32_t *__restrict__ count, uint32_t *__restrict__ col) {
    for (uint32_t a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x) {
        if (type[a] == FGB_TYPE_OBSTACLE) continue;
        const uint32_t key = keys[a];
        const SceneDev &S = scenes[scene_of(key, mbits)];
        const uint32_t m = morton_of(key, mbits);
        const int cx = (int)compact10(m), cy = (int)compact10(m >> 1), cz = (int)compact10(m >> 2);
        const uint2 *tbl = cells + S.table_base;
        uint4 s = make_uint4(0, 0, 0, 0);
        uint32_t c = 0;
        for_cell_indices(S, cx, cy, cz, [&](uint32_t k) {
            const uint2 r = __ldg(&tbl[k]);
            if (r.x >= r.y) return;
            const uint4 g = __ldg(&agg[r.x]);
            s.x += g.x;
            s.y += g.y;
            s.z += g.z;
            s.w += g.w;
            c += __ldg(&count[r.x]);
        });
        const float t = S.dt / 750.f;
        const float fc = (float)c;
        const uint32_t v = col[a];
        col[a] = diffuse_channel(v & 0xffu, s.x, fc, t) | (diffuse_channel((v >> 8) & 0xffu, s.y, fc, t) << 8) |
                 (diffuse_channel((v >> 16) & 0xffu, s.z, fc, t) << 16) | (diffuse_channel(v >> 24, s.w, fc, t) << 24);
    }
}

// At the end of a step, per scene: whether the next step builds its Verlet lists and
// near rows.  A list holds while its particle and every candidate together moved less
// than the skin.  In a violent flow some particle of nearly every 27-cell
// neighbourhood moves that far within a step, the lists fail their bound at every later
// pass and building them is wasted: the scene's next steps walk instead, until it
// calms.  Sums are the same either way.
__global__ void k_list_policy(uint32_t *policy, uint32_t n_scenes, uint32_t min_use_pct) {
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < n_scenes; s += gridDim.x * blockDim.x) {
        uint32_t *p = policy + kPolicyWords * s;
        if (p[0]) {
            // lists were built: keep them while at least min_use_pct (25) percent of the
            // second pass's particles could use them (the list build and its filter cost
            // about what a quarter of the later walks saves)
            const uint64_t seen = (uint64_t)p[3] + p[4];
            p[0] = seen == 0 || 100ull * p[3] >= (uint64_t)min_use_pct * seen ? 1u : 0u;
            p[5] = 0u;
        } else {
            // walking: build again once the scene has calmed (at most 1% of its particles
            // moved over half the skin), and try every 8th step anyway
            p[5] += 1u;
            p[0] = (uint64_t)p[1] * 100u <= (uint64_t)p[2] || p[5] >= 8u ? 1u : 0u;
        }
        p[1] = p[2] = p[3] = p[4] = 0u;
    }
}

// Keys of the current positions (marching-cubes grid).
__global__ void k_position_keys(const SceneDev *__restrict__ scenes, Phys ph, uint32_t n, uint32_t mbits,
                                const uint32_t *__restrict__ keys_prev, const float4 *__restrict__ x,
                                uint32_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t s = scene_of(keys_prev[i], mbits);
        const SceneDev &S = scenes[s];
        const float4 xi = x[i];
        const uint32_t m = cell_key(S, ph.h, xi.x / S.scale, xi.y / S.scale, xi.z / S.scale);
        keys_out[i] = (mbits >= 32 ? 0u : (s << mbits)) | m;
        vals_out[i] = i;
    }
}

__global__ void k_gather_positions(const SceneDev *__restrict__ scenes, uint32_t n, uint32_t mbits,
                                   const uint32_t *__restrict__ keys, const uint32_t *__restrict__ vals,
                                   const float4 *__restrict__ x, const int32_t *__restrict__ type,
                                   const uint32_t *__restrict__ col, float4 *__restrict__ xs,
                                   int32_t *__restrict__ type_s, uint32_t *__restrict__ col_s,
                                   uint2 *__restrict__ cells, uint64_t cells_n, uint32_t *err) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t j = vals[i];
        const uint32_t key = keys[i];
        const SceneDev &S = scenes[scene_of(key, mbits)];
        xs[i] = x[j];
        type_s[i] = type[j];
        col_s[i] = col[j];
        const uint64_t c = (uint64_t)S.table_base + morton_of(key, mbits);
        if (c >= cells_n) {
            raise_error(err, ERR_CELL_RANGE);
            continue;
        }
        if (i == 0 || keys[i - 1] != key) cells[c].x = i;
        if (i + 1 == n || keys[i + 1] != key) cells[c].y = i + 1;
    }
}

inline unsigned grid_for(uint32_t n, int block) {
    unsigned g = (n + block - 1) / block;
    return g ? g : 1;
}

inline unsigned stream_grid(uint32_t n) {
    unsigned g = (n + 255) / 256;
    const unsigned cap = 152u * 8u;
    if (g > cap) g = cap;
    return g ? g : 1;
}

GatherArgs gather_args(const StepView &s) {
    GatherArgs A;
    A.scenes = s.scenes;
    A.tris = s.tris;
    A.ph = s.ph;
    A.n = s.n;
    A.mbits = s.mbits;
    A.keys = s.keys_sorted;
    A.cells = s.cells;
    A.type = s.type1;
    A.nlist = s.nlist;
    A.ncount = s.ncount;
    A.cap = s.cap;
    A.list_r2 = s.list_r2;
    A.skin = s.skin;
    A.ps_grid = s.ps_grid;
    A.disp = s.disp;
    A.cellmax = s.cellmax;
    A.valid = s.valid;
    A.hlist = s.hlist;
    A.hcount = s.hcount;
    A.hcap = s.hlist ? s.hcap : 0;
    // near rows need the displacement bound (Verlet lists) and hit rows
    A.near = s.cap && A.hcap ? s.near : nullptr;
    A.near_r2 = s.near_r2;
    A.near_skin = s.near_skin;
    A.over = s.over;
    A.near_stats = A.near ? s.near_stats : nullptr;
    A.plam = s.plam;
    A.pom = s.pom;
    A.queue = nullptr;  // per launch, below
    A.list_policy = s.cap ? s.list_policy : nullptr;
    A.count_lists = 0;  // the second lambda pass's launch sets it
    A.ppt = s.ppt ? s.ppt : 1;
    A.verlet_off = s.verlet_off;
    A.mass_range = s.mass_range;
    return A;
}


}  // namespace

namespace {
__global__ void k_fill_u32(uint32_t *__restrict__ p, uint64_t n, uint32_t value) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = value;
}
}  // namespace

namespace {
__global__ void k_iota_u32(uint32_t *__restrict__ p, uint64_t n) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = (uint32_t)i;
}
}  // namespace

void launch_iota_u32(uint32_t *p, uint64_t n, cudaStream_t st) {
    if (!n) return;
    unsigned g = (unsigned)std::min<uint64_t>((n + 255) / 256, 152u * 8u);
    k_iota_u32<<<g, 256, 0, st>>>(p, n);
}

void launch_fill_u32(uint32_t *p, uint64_t n, uint32_t value, cudaStream_t st) {
    if (!n) return;
    unsigned g = (unsigned)std::min<uint64_t>((n + 255) / 256, 152u * 8u);
    k_fill_u32<<<g, 256, 0, st>>>(p, n, value);
}

void launch_predict_keys(const StepView &s, cudaStream_t st) {
    k_predict_keys<<<stream_grid(s.n), 256, 0, st>>>(s.scenes, s.wells, s.ph, s.n, s.mbits, s.keys_prev, s.x0, s.v0,
                                                     s.type0, s.keys_in, s.vals_in);
}

void launch_reorder_cells(const StepView &s, cudaStream_t st) {
    k_reorder_cells<<<stream_grid(s.n), 256, 0, st>>>(s.scenes, s.wells, s.ph, s.n, s.mbits, s.keys_sorted,
                                                      s.vals_sorted, s.x0, s.v0, s.type0, s.col0, s.slot0, s.x1,
                                                      s.v1, s.type1, s.col1, s.slot1, s.ps_grid, s.cells, s.cells_n,
                                                      s.err, s.mass_range);
}

// Grid and tile counter of one gather launch (slot: its place among the step's
// gather launches, each with its own counter).
struct Launch {
    unsigned grid;
    GatherArgs A;
};
Launch gather_launch(const StepView &s, uint32_t slot) {
    Launch L{grid_for(s.n, s.block), gather_args(s)};
    if (s.queue) {
        const uint64_t tiles = ((uint64_t)s.n + (uint64_t)s.block * L.A.ppt - 1) / ((uint64_t)s.block * L.A.ppt);
        const uint64_t resident = (uint64_t)(s.sm_count > 0 ? s.sm_count : 152) * (2048u / (uint32_t)s.block);
        L.grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(tiles, resident));
        L.A.queue = s.queue + slot;
    }
    return L;
}

// Gather launch slots of a step: the list build, then lambda and delta per iteration,
// then the two vorticity passes.
uint32_t slots_of_step(uint32_t iterations) { return 3 + 2 * iterations; }

// Each gather kernel in two forms: a flat grid (one particle per thread) and a
// persistent grid over the launch's tile queue; both compute the same bits.
template <int P, int M>
void run_lambda(const Launch &L, int block, cudaStream_t st, const float4 *ps, float *lambda, float *density) {
    if (L.A.queue) k_lambda<P, M, true><<<L.grid, block, 0, st>>>(L.A, ps, lambda, density);
    else k_lambda<P, M, false><<<L.grid, block, 0, st>>>(L.A, ps, lambda, density);
}

template <int P, int M>
void run_delta(const Launch &L, int block, cudaStream_t st, const float4 *ps_in, const float *lambda, float4 *ps_out,
               float4 *x, float4 *v, int last, const HostParticlesOut *hout) {
    if (L.A.queue) k_delta<P, M, true><<<L.grid, block, 0, st>>>(L.A, ps_in, lambda, ps_out, x, v, last, hout);
    else k_delta<P, M, false><<<L.grid, block, 0, st>>>(L.A, ps_in, lambda, ps_out, x, v, last, hout);
}

void launch_lambda(const StepView &s, const float4 *ps, int iteration, cudaStream_t st) {
    const Launch B = gather_launch(s, 0);
    Launch L = gather_launch(s, 1 + 2 * (uint32_t)iteration);
    L.A.count_lists = iteration == 1;
    const bool ref = s.ph.profile == FGB_PROFILE_REF;
    if (iteration == 0 && L.A.cap) {
        if (B.A.queue) k_build_lists<true><<<B.grid, s.block, 0, st>>>(B.A, ps);
        else k_build_lists<false><<<B.grid, s.block, 0, st>>>(B.A, ps);
        if (ref) run_lambda<FGB_PROFILE_REF, kFresh>(L, s.block, st, ps, s.lambda, s.density);
        else run_lambda<FGB_PROFILE_BASELINE, kFresh>(L, s.block, st, ps, s.lambda, s.density);
    } else if (iteration == 0) {
        if (ref) run_lambda<FGB_PROFILE_REF, kBuild>(L, s.block, st, ps, s.lambda, s.density);
        else run_lambda<FGB_PROFILE_BASELINE, kBuild>(L, s.block, st, ps, s.lambda, s.density);
    } else {
        if (ref) run_lambda<FGB_PROFILE_REF, kCheck>(L, s.block, st, ps, s.lambda, s.density);
        else run_lambda<FGB_PROFILE_BASELINE, kCheck>(L, s.block, st, ps, s.lambda, s.density);
    }
}

void launch_delta(const StepView &s, const float4 *ps_in, float4 *ps_out, int iteration, bool last,
                  cudaStream_t st) {
    const Launch L = gather_launch(s, 2 + 2 * (uint32_t)iteration);
    const bool ref = s.ph.profile == FGB_PROFILE_REF;
    const int l = last ? 1 : 0;
    if (iteration == 0) {
        if (ref) run_delta<FGB_PROFILE_REF, kFresh>(L, s.block, st, ps_in, s.lambda, ps_out, s.x1, s.v1, l, s.hout);
        else run_delta<FGB_PROFILE_BASELINE, kFresh>(L, s.block, st, ps_in, s.lambda, ps_out, s.x1, s.v1, l, s.hout);
    } else {
        if (ref) run_delta<FGB_PROFILE_REF, kStored>(L, s.block, st, ps_in, s.lambda, ps_out, s.x1, s.v1, l, s.hout);
        else run_delta<FGB_PROFILE_BASELINE, kStored>(L, s.block, st, ps_in, s.lambda, ps_out, s.x1, s.v1, l, s.hout);
    }
}

void launch_velocity_terms(const StepView &s, const float4 *ps, cudaStream_t st, const std::function<void()> &between) {
    const Launch X = gather_launch(s, 1 + 2 * s.iterations), Y = gather_launch(s, 2 + 2 * s.iterations);
    if (X.A.queue) k_vorticity_xsph<true><<<X.grid, s.block, 0, st>>>(X.A, ps, s.v1, s.omega, s.vx);
    else k_vorticity_xsph<false><<<X.grid, s.block, 0, st>>>(X.A, ps, s.v1, s.omega, s.vx);
    if (between) between();
    if (Y.A.queue) k_vorticity_apply<true><<<Y.grid, s.block, 0, st>>>(Y.A, ps, s.omega, s.vx, s.v1, s.x1, s.hout);
    else k_vorticity_apply<false><<<Y.grid, s.block, 0, st>>>(Y.A, ps, s.omega, s.vx, s.v1, s.x1, s.hout);
}

void launch_list_policy(const StepView &s, cudaStream_t st) {
    if (s.list_policy && s.cap)
        k_list_policy<<<(s.n_scenes + 255) / 256, 256, 0, st>>>(s.list_policy, s.n_scenes, s.list_min_use);
}

void launch_diffuse(const StepView &s, uint4 *agg, uint32_t *count, cudaStream_t st) {
    k_cell_colours<<<stream_grid(s.n), 256, 0, st>>>(s.n, s.keys_sorted, s.type1, s.col1, agg, count);
    k_diffuse<<<stream_grid(s.n), 256, 0, st>>>(s.scenes, s.n, s.mbits, s.keys_sorted, s.cells, s.type1, agg, count,
                                                s.col1);
}

void launch_position_keys(const StepView &s, const float4 *x, cudaStream_t st) {
    k_position_keys<<<stream_grid(s.n), 256, 0, st>>>(s.scenes, s.ph, s.n, s.mbits, s.keys_prev, x, s.keys_in,
                                                      s.vals_in);
}

void launch_gather_positions(const StepView &s, const float4 *x, const int32_t *type, const uint32_t *col,
                             float4 *xs_sorted, int32_t *type_sorted, uint32_t *col_sorted, cudaStream_t st) {
    k_gather_positions<<<stream_grid(s.n), 256, 0, st>>>(s.scenes, s.n, s.mbits, s.keys_sorted, s.vals_sorted, x,
                                                         type, col, xs_sorted, type_sorted, col_sorted, s.cells,
                                                         s.cells_n, s.err);
}

}  // namespace fgb
