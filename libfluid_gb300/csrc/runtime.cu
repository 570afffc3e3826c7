// runtime.cu -- host runtime behind the C ABI: solver, resident batches, surfaces.
//
// fgb_advance is the drop-in for ocl::SphSolver::advance (include/fluid/oclsph.hpp:
// 661-936): it uploads the caller's particles, runs one step, writes them back in
// Morton order and optionally extracts the surface.  Underneath, every scene lives in
// a batch whose state stays in HBM between steps; a batch of one is the single-scene
// path, so the drop-in, the batched workload and the serving loop share one code path.
//
// Device layout of a batch (n = particles of all scenes; scene k owns the contiguous
// segment [first_k, first_k + count_k) of every array, kept by the sort because the
// scene id sits above the Morton bits of the key):
//   state (two sets, the step gathers one into the other in sorted order):
//     x float4 (position xyz, mass), v float4, type i32, colour u32, slot u32
//   step: keys/vals in + sorted (u32), radix scratch, cell table uint2 {start,end}
//         per Morton key of every scene, p* float4 x2 (Jacobi ping-pong),
//         lambda f32, density f32, omega float4, XSPH velocity float4
//   surface (on first use): sorted positions, lattice float4 + colour u32 per
//         sample, case u8 + offset u32 per cube, triangles
#include <algorithm>
#include <cmath>
#include <limits>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <condition_variable>
#include <functional>
#include <initializer_list>
#include <mutex>
#include <thread>
#include <string>
#include <map>
#include <memory>
#include <vector>

#include <sys/mman.h>
#include <unistd.h>

#include "fgb_internal.h"

namespace fgb {

static thread_local std::string g_last_error;

int fail(int code, const char *msg) {
    g_last_error = msg ? msg : "";
    return code;
}

int fail_cuda(cudaError_t e, const char *where) {
    std::string m = std::string(where) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    g_last_error = m;
    if (e == cudaErrorMemoryAllocation) return FGB_ERR_OOM;
    return FGB_ERR_CUDA;
}

#define FGB_CUDA(call, where)                         \
    do {                                              \
        cudaError_t e_ = (call);                      \
        if (e_ != cudaSuccess) return fail_cuda(e_, where); \
    } while (0)

namespace {

constexpr float kPi = 3.14159265358979323846f;

// Each scene's first triangle after a batched surface: the scanned offset at its
// first cube (the total for a scene without cubes), gathered for one copy to the host.
__global__ void k_scene_first_triangles(const SceneDev *__restrict__ scenes, uint32_t n_scenes,
                                        const uint32_t *__restrict__ offsets, uint64_t cube_total, uint32_t total,
                                        uint32_t *__restrict__ out) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n_scenes; k += gridDim.x * blockDim.x) {
        const uint64_t cb = scenes[k].cube_base;
        out[k] = cb < cube_total ? offsets[cb] : total;
    }
}

// Device blocks of one solver's batches, kept for reuse instead of freed.  Every
// batch of a solver queues its work on the solver's stream, so a block handed back
// while kernels that use it are still queued can go to the next allocation of the
// same solver without a wait: that allocation's users queue behind them
// (fgb_set_stream drains the old stream before it switches).  cudaMalloc and the
// device-wide synchronisation of cudaFree cost ~1.6 and ~1.8 ms for the ~40 arrays
// of a batch, and the serving loop rebuilds a group of scenes several times a
// second.  Blocks come in size classes (four per power of two above 64 KiB) so that
// batches of similar sizes reuse each other's blocks.
class DevPool {
  public:
    ~DevPool() { trim(); }
    static size_t size_class(size_t bytes) {
        if (bytes <= 65536) return (bytes + 511) & ~size_t(511);
        size_t top = 65536;
        while (top * 2 < bytes) top *= 2;  // top < bytes <= 2 top
        const size_t quarter = top / 4;
        return top + (bytes - top + quarter - 1) / quarter * quarter;
    }
    void *get(size_t bytes, cudaError_t *e) {
        const size_t c = size_class(bytes);
        {
            std::lock_guard<std::mutex> lk(mu_);
            auto it = free_.find(c);
            if (it != free_.end()) {
                void *p = it->second;
                free_.erase(it);
                *e = cudaSuccess;
                return p;
            }
        }
        void *p = nullptr;
        *e = cudaMalloc(&p, c);
        if (*e == cudaErrorMemoryAllocation) {  // give the cached blocks back and retry
            (void)cudaGetLastError();
            trim();
            *e = cudaMalloc(&p, c);
        }
        return *e == cudaSuccess ? p : nullptr;
    }
    void put(void *p, size_t bytes) {
        const size_t c = size_class(bytes);
        std::lock_guard<std::mutex> lk(mu_);
        free_.emplace(c, p);
    }
    void trim() {
        std::lock_guard<std::mutex> lk(mu_);
        for (auto &f : free_) cudaFree(f.second);
        free_.clear();
    }
  private:
    std::mutex mu_;
    std::multimap<size_t, void *> free_;
};

// The pool that Dev::alloc draws from on this thread (none: cudaMalloc); set by
// PoolScope in the batch functions that allocate.  A block goes back to the pool
// it came from.
thread_local DevPool *t_pool = nullptr;
struct PoolScope {
    DevPool *prev;
    explicit PoolScope(DevPool *p) : prev(t_pool) { t_pool = p; }
    ~PoolScope() { t_pool = prev; }
};

template <class T>
struct Dev {
    T *p = nullptr;
    size_t n = 0;
    DevPool *pool = nullptr;
    Dev() = default;
    Dev(const Dev &) = delete;
    Dev &operator=(const Dev &) = delete;
    ~Dev() { release(); }
    void release() {
        if (p) {
            if (pool) pool->put(p, n * sizeof(T));
            else cudaFree(p);
        }
        p = nullptr;
        n = 0;
        pool = nullptr;
    }
    cudaError_t alloc(size_t count) {
        release();
        if (count == 0) count = 1;
        cudaError_t e;
        if (t_pool) {
            p = (T *)t_pool->get(count * sizeof(T), &e);
            if (e == cudaSuccess) pool = t_pool;
        } else {
            e = cudaMalloc((void **)&p, count * sizeof(T));
        }
        if (e == cudaSuccess) n = count;
        else p = nullptr;
        return e;
    }
    void swap(Dev &o) {
        std::swap(p, o.p);
        std::swap(n, o.n);
        std::swap(pool, o.pool);
    }
};

template <class T>
struct Pinned {
    T *p = nullptr;
    size_t n = 0;
    ~Pinned() {
        if (p) cudaFreeHost(p);
    }
    cudaError_t ensure(size_t count) {
        if (count <= n && p) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaHostAlloc((void **)&p, std::max<size_t>(count, 1) * sizeof(T), cudaHostAllocDefault);
        if (e == cudaSuccess) n = std::max<size_t>(count, 1);
        return e;
    }
};

uint32_t bits_for(uint32_t v) {
    uint32_t b = 0;
    while ((1u << b) <= v && b < 31) ++b;
    return b;
}

Phys make_phys(const fgb_params &p) {
    Phys ph{};
    const float h = p.h, hh = h * h, hhh = h * h * h;
    ph.h = h;
    ph.hh = hh;
    {
        // sqrtf is correctly rounded and monotonic, so {r2 : sqrtf(r2) <= h} is the
        // floats up to one threshold; the ref profile's range tests compare r2 with it
        // and take the square root only for neighbours within h
        float x = hh;
        while (std::sqrt(x) > h) x = std::nextafter(x, 0.f);
        while (std::sqrt(std::nextafter(x, INFINITY)) <= h) x = std::nextafter(x, INFINITY);
        ph.hh_le = x;
    }
    ph.poly6f = 315.f / (64.f * kPi * (hhh * hhh * hhh));
    ph.spikyf = -(45.f / (kPi * hhh * hhh));
    ph.rho0 = p.rho0;
    ph.inv_rho0 = 1.f / p.rho0;
    ph.cfm = p.cfm_epsilon;
    ph.corr_n = p.corr_n;
    const float dq = p.corr_delta_q * h;
    const float t = hh - dq * dq;
    ph.corr_wdq = t * t * t;
    {
        // poly6(dq) exactly as the oracle's orc_poly6 evaluates it
        const float f = 315.f / (64.f * kPi * (hhh * hhh * hhh));
        const float tt = hh - dq * dq;
        ph.corr_ref = (dq <= h) ? f * (tt * tt * tt) : 0.f;
    }
    ph.inv_corr_ref = ph.corr_ref != 0.f ? 1.f / ph.corr_ref : 0.f;
    ph.inv_corr_wdq = ph.corr_wdq != 0.f ? 1.f / ph.corr_wdq : 0.f;
    ph.corr_k = p.profile == FGB_PROFILE_REF ? p.corr_k : p.corr_k * hh;
    ph.xsph_c = p.xsph_c;
    ph.vort_eps = p.vorticity_epsilon;
    ph.damping = p.velocity_damping;
    ph.mc_size = p.mc_particle_size;
    ph.mc_infl = p.mc_particle_influence;
    ph.profile = p.profile;
    return ph;
}

// Grid and lattice geometry of one scene (same float operations as the oracle).
// The smallest float T with sqrtf(T) >= thr, so that sqrtf(r2) < thr exactly when
// r2 < T (sqrtf is correctly rounded and monotonic): range tests against a length
// then need no square root.
float sqrt_lt_bound(float thr) {
    if (!(thr > 0.f)) return 0.f;  // no r2 has sqrtf(r2) < thr
    if (std::isinf(thr)) return thr;
    float x = thr * thr;
    if (std::isinf(x)) x = std::numeric_limits<float>::max();
    while (x > 0.f && std::sqrt(std::nextafter(x, 0.f)) >= thr) x = std::nextafter(x, 0.f);
    while (std::sqrt(x) < thr) x = std::nextafter(x, INFINITY);
    return x;
}

void scene_geometry(const fgb_params &p, const fgb_config &c, SceneDev &S) {
    const float pad = p.h * 2.f;
    for (int a = 0; a < 3; ++a) {
        const float mn = (c.min_bound[a] / c.scale) - pad;
        const float mx = (c.max_bound[a] / c.scale) + pad;
        S.min_ext[a] = mn;
        const float e = (mx - mn) / p.h;
        uint32_t ei = e > 0.f ? (uint32_t)e : 0u;
        if (ei > 1023u) ei = 1023u;
        S.ext[a] = ei;
    }
    S.dt = c.dt;
    S.inv_dt = 1.f / c.dt;
    S.scale = c.scale;
    for (int a = 0; a < 3; ++a) {
        S.g[a] = c.constant_force[a];
        S.min_b[a] = c.min_bound[a];
        S.max_b[a] = c.max_bound[a];
    }
    S.sphere_enabled = c.sphere_enabled;
    for (int a = 0; a < 4; ++a) S.sphere[a] = c.sphere[a];
    S.resolution = c.resolution;
    S.iso = c.isolevel;
    S.mc_r2_lt = sqrt_lt_bound(p.h * c.scale);
    const float step = c.resolution > 0.f ? p.h / c.resolution : 0.f;
    S.lat_step = step;
    for (int a = 0; a < 3; ++a) {
        if (c.resolution <= 0.f) {
            S.lat[a] = 0;
            S.lat_origin[a] = 0.f;
        } else if (p.profile == FGB_PROFILE_REF) {
            S.lat_origin[a] = S.min_ext[a];
            S.lat[a] = (uint32_t)floorf((float)S.ext[a] * c.resolution) + 1u;
        } else {
            const float lo = c.min_bound[a] / c.scale, hi = c.max_bound[a] / c.scale;
            S.lat_origin[a] = lo;
            S.lat[a] = (uint32_t)floorf((hi - lo) / step + 0.5f) + 1u;
        }
    }
}

std::once_flag g_tables_once[64];

void ensure_tables() {
    int dev = 0;
    cudaGetDevice(&dev);
    std::call_once(g_tables_once[dev & 63], [] { mc_tables_upload(); });
}

}  // namespace
}  // namespace fgb

using namespace fgb;

// Host worker pool for the per-frame pack and unpack loops of upload and download:
// one thread per core, started on first use and parked on a condition variable
// between jobs; the calling thread works too.  A job is f(lo, hi) over [0, n),
// handed out in chunks of 16k items.  Jobs from different threads are serialised.
class HostPool {
  public:
    static HostPool &get() {
        static HostPool pool;
        return pool;
    }
    template <class F>
    void run(uint64_t n, F &&f) {
        const uint64_t chunks = (n + kChunk - 1) / kChunk;
        if (chunks <= 1 || workers_.empty()) {
            if (n) f((uint64_t)0, n);
            return;
        }
        std::lock_guard<std::mutex> job_lock(job_mu_);
        auto job = std::make_shared<Job>();
        job->f = [&f](uint64_t lo, uint64_t hi) { f(lo, hi); };
        job->n = n;
        job->chunks = chunks;
        {
            std::lock_guard<std::mutex> lk(mu_);
            current_ = job;
            ++generation_;
        }
        cv_.notify_all();
        work(*job);
        std::unique_lock<std::mutex> lk(mu_);
        done_cv_.wait(lk, [&] { return job->done.load() == job->chunks; });
        current_.reset();
    }
    ~HostPool() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
            ++generation_;
        }
        cv_.notify_all();
        for (auto &t : workers_) t.join();
    }

  private:
    static constexpr uint64_t kChunk = 1u << 14;
    // One job's state: a worker that wakes late finds every chunk taken and leaves,
    // and run() returns only once every taken chunk has finished.
    struct Job {
        std::function<void(uint64_t, uint64_t)> f;
        uint64_t n = 0, chunks = 0;
        std::atomic<uint64_t> next{0}, done{0};
    };
    HostPool() {
        const unsigned t = std::max(1u, std::thread::hardware_concurrency());
        for (unsigned i = 1; i < t; ++i) workers_.emplace_back([this] { loop(); });
    }
    void work(Job &j) {
        for (;;) {
            const uint64_t c = j.next.fetch_add(1);
            if (c >= j.chunks) return;
            j.f(c * kChunk, std::min(j.n, (c + 1) * kChunk));
            if (j.done.fetch_add(1) + 1 == j.chunks) {
                std::lock_guard<std::mutex> lk(mu_);
                done_cv_.notify_all();
            }
        }
    }
    void loop() {
        uint64_t seen = 0;
        for (;;) {
            std::shared_ptr<Job> job;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return stop_ || generation_ != seen; });
                if (stop_) return;
                seen = generation_;
                job = current_;
            }
            if (job) work(*job);
        }
    }
    std::vector<std::thread> workers_;
    std::mutex job_mu_, mu_;
    std::condition_variable cv_, done_cv_;
    std::shared_ptr<Job> current_;
    uint64_t generation_ = 0;
    bool stop_ = false;
};

template <class F>
static void parallel_for(uint64_t n, F &&f) {
    HostPool::get().run(n, f);
}

// Give the pages of the caller's arrays a frame on the host before a kernel writes
// them over the coherent link.  A GPU store to a page that the host never wrote
// (fresh calloc or mmap memory) faults to the host once per page -- ~17 ms for a
// 1M-particle download into fresh arrays -- whereas one host store per page costs
// ~2 us on a fresh page.  mincore() finds the pages that are not resident (for
// reused arrays: none, at the cost of one system call per array).  For arrays that
// are only outputs, each such page gets a store of 0 into a byte that the kernel then
// overwrites (every element of every array passed is written); a load first would
// cost a second fault (zero page, then copy-on-write).  For arrays that are also
// inputs (fgb_advance works in place), a page that is not resident can still hold
// data -- swapped-out memory, or a file mapping whose page was evicted -- so each
// gets a load of a byte and a store of the same value back: the page is read in
// and made writable without changing what the kernels will read.
struct HostSpan {
    void *p;
    size_t bytes;
};
static int ready_pages(std::initializer_list<HostSpan> spans, bool keep_contents) {
    static const size_t page = (size_t)sysconf(_SC_PAGESIZE) > 0 ? (size_t)sysconf(_SC_PAGESIZE) : 4096;
    std::vector<char *> at;
    std::vector<unsigned char> resident;
    for (const HostSpan &a : spans) {
        if (!a.p || !a.bytes) continue;
        char *p = (char *)a.p, *end = p + a.bytes;
        char *first_page = (char *)((uintptr_t)p / page * page);
        const size_t pages = (size_t)(end - first_page + page - 1) / page;
        resident.assign(pages, 0);
        // a range the host does not map (mincore fails) is left to the kernel as it is
        if (mincore(first_page, (size_t)(end - first_page), resident.data()) != 0) continue;
        for (size_t i = 0; i < pages; ++i)
            if (!(resident[i] & 1)) at.push_back(i ? first_page + i * page : p);
    }
    if (at.empty()) return 0;
    constexpr uint64_t kUnit = 1024;  // a pool chunk covers 16 pages
    parallel_for(at.size() * kUnit, [&](uint64_t lo, uint64_t hi) {
        for (uint64_t i = (lo + kUnit - 1) / kUnit; i * kUnit < hi; ++i) {
            volatile char *q = at[i];
            *q = keep_contents ? *q : (char)0;
        }
    });
    return (int)std::min<size_t>(at.size(), 0x7fffffff);
}
static void prefault_outputs(std::initializer_list<HostSpan> spans) { ready_pages(spans, false); }

// Pieces of the pipelined upload and download: host packing or unpacking of one
// piece overlaps the copies of the others.
static constexpr uint64_t kPieceMin = 1u << 18;
static constexpr uint32_t kMaxRowCap = 1024;  // Verlet and hit rows, entries per particle
static constexpr uint32_t kPieces = 4;

// Autotuner cache key: physics profile and floor(log2(particles)).
static uint32_t tune_bucket(int32_t profile, uint64_t n) {
    uint32_t b = 0;
    while (b < 63 && (2ull << b) <= n) ++b;
    return (uint32_t)profile * 64u + b;
}

struct fgb_solver {
    DevPool pool;  // first member: outlives every block its batches hand back
    fgb_params params;
    Phys ph;
    cudaStream_t own = nullptr;
    cudaStream_t stream = nullptr;
    int device = 0;
    int block = 128;
    // autotuned launch shape per (profile, log2 particle count) bucket
    struct Tuned {
        int block;
        float skin;
        bool persistent;
        uint32_t ppt;
        bool verlet_off;
    };
    std::map<uint32_t, Tuned> tuned;
    // row capacities (Verlet, hit) that batches grew to, per (profile, log2 n) bucket:
    // later batches of the bucket start there
    std::map<uint32_t, std::pair<uint32_t, uint32_t>> caps;
    fgb_batch *cached = nullptr;  // single-scene batch behind fgb_advance
    uint64_t cached_n = 0;
    fgb_config cached_cfg{};
    std::vector<TriDev> cached_tris;
    std::vector<fgb_batch *> batches;  // every live batch; destroyed with the solver
};

struct fgb_batch {
    fgb_solver *solver = nullptr;
    uint32_t n_scenes = 0;
    std::vector<fgb_config> cfg;
    std::vector<uint64_t> counts, first;
    uint64_t n = 0;
    uint64_t capacity = 0;  // particles the per-particle arrays hold (>= n)
    uint32_t mbits = 0, sbits = 0, key_bits = 0, iterations = 0;
    std::vector<SceneDev> h_scenes;
    Dev<SceneDev> d_scenes;
    Dev<WellDev> d_wells;
    Dev<TriDev> d_tris;
    std::vector<std::vector<TriDev>> scene_tris;
    bool tris_dirty = false;
    Phys ph;
    // state
    Dev<float4> x[2], v[2];
    Dev<int32_t> type[2];
    Dev<uint32_t> col[2], slot[2];
    Dev<uint64_t> ids_dev;  // particle ids by upload slot (scene segment), for device-side record packing
    std::vector<uint8_t> ids_stale;  // per scene: ids_dev not yet given the last upload's ids (sync_ids)
    bool direct = false;    // uploads and downloads address the caller's arrays from kernels (hostio.cu)
    Dev<uint32_t> obst_dev; // per scene: obstacle count of the last direct upload
    // direct downloads of fgb_advance: the step graphs record grid_ready once the
    // grid is built, and io_stream writes the fields final from then on (type,
    // colour, id, mass) while the gathers run
    cudaEvent_t grid_ready = nullptr, io_done = nullptr;
    cudaStream_t io_stream = nullptr;
    // and the reorder of each step waits for io_up, recorded by the part of an
    // fgb_advance upload that io_stream does (colours, ids, slots) during the
    // prediction and the sort
    cudaEvent_t io_up = nullptr;
    // the batch behind fgb_advance: the step's last kernel stores final positions and
    // velocities straight into the caller's arrays, named per frame in hout_dev
    bool advance_io = false;
    Dev<HostParticlesOut> hout_dev;
    Pinned<HostParticlesOut> st_hout;
    // rows that overflowed in each step's build pass, copied to st_over at the end of
    // the step; grow_rows() enlarges the capacities when more than 1% did
    // over[2..3]: near-row statistics of the checked passes (FGB_ROW_STATS=1), kept
    // on the device across steps until fgb_batch_row_stats reads and clears them
    Dev<uint32_t> over;
    Pinned<uint32_t> st_over;
    bool row_stats = false;
    // the device error flags (err) as of the end of each step, copied by the step
    // graph; fgb_batch_step, fgb_batch_sync and fgb_advance turn them into a status
    Pinned<uint32_t> st_flags;
    Dev<char> wire;         // packed-record staging (wire.cu)
    int cur = 0;
    // step
    Dev<uint32_t> keys_in, vals_in, keys_sorted, vals_sorted;
    Dev<char> sort_scratch;
    uint64_t sort_scratch_bytes = 0;
    Dev<uint2> cells;
    uint64_t cells_n = 0;
    Dev<float4> ps[2];
    Dev<float4> ps_grid;
    Dev<uint32_t> nlist;
    Dev<uint16_t> ncount;
    Dev<float> disp;
    Dev<uint32_t> cellmax;
    Dev<uint8_t> valid;
    Dev<uint32_t> hlist;
    Dev<uint16_t> hcount;
    uint32_t hit_cap = 64;
    uint32_t list_cap = 96;
    uint32_t verlet_off = 0;
    float skin_frac = 0.2f;
    // persistent gathers: CTAs take tiles of ppt x block particles from per-launch
    // counters (queue, zeroed at the start of every step) instead of a flat grid
    bool persistent = false;
    uint32_t ppt = 1;
    Dev<uint32_t> queue;
    Dev<uint32_t> list_policy;  // per scene: k_list_policy's state
    Dev<uint32_t> scene_firsts;  // per scene: first triangle of the last batched surface
    // FGB_LIST_MIN_USE: percent of a pass's particles using lists that keeps them on;
    // by default 25 with Verlet lists and 10 with near rows alone (measured: the near
    // rows cost little beyond the walk that builds them)
    uint32_t list_min_use = 0;
    bool list_min_use_set = false;
    int sm_count = 0;
    float near_frac = 0.05f;  // near-row skin, fraction of h (0: near rows off)
    Dev<uint8_t> near;
    int block = 128;  // threads per CTA of the gather kernels
    Dev<float> lambda, density;
    Dev<float4> plam;             // the lambda pass's p* with lambda in w (delta reads)
    Dev<float4> pom;              // the vorticity pass's p* with |omega| in w (apply reads)
    Dev<uint32_t> mass_range;     // {min mass, ~max mass} bits of the step
    Dev<float4> omega, vx;
    Dev<uint4> colour_sums;      // ref profile: per-cell channel sums (at the cell's first index)
    Dev<uint32_t> colour_count;
    Dev<uint32_t> err;
    // cell queries: the cell table is the last step's grid until the next upload, edit
    // or surface replaces it
    bool query_ok = false;
    Dev<fgb_query> q_dev;
    Dev<uint32_t> q_out;
    // surface
    bool surf_ready = false;
    uint64_t lat_total = 0, cube_total = 0, brick_total = 0;
    Dev<uint32_t> mc_keys, mc_vals;
    Dev<float4> mc_xs;
    Dev<int32_t> mc_type;
    Dev<uint32_t> mc_col;
    Dev<float4> lattice;
    Dev<uint32_t> lattice_col;
    Dev<uint8_t> cases;
    Dev<uint32_t> offsets;
    Dev<uint32_t> total;
    Dev<char> scan_scratch;
    uint64_t scan_scratch_bytes = 0;
    Dev<fgb_mesh_triangle> tris_out;
    uint32_t surf_scene_begin = 0, surf_scene_end = 0;
    std::vector<uint64_t> surf_tri_first;  // per scene of the last surface_all
    // host
    std::vector<std::vector<uint64_t>> ids;
    Pinned<float4> st_x, st_v;
    Pinned<int32_t> st_type;
    Pinned<uint32_t> st_col, st_slot, st_keys;
    Pinned<uint64_t> st_ids;
    Pinned<uint32_t> st_count;
    std::vector<cudaEvent_t> piece_events;  // pipelined download, one per piece
    uint64_t launches = 0;
    uint64_t launches_per_step = 0;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    bool graphs_ok = false;

    ~fgb_batch() {
        for (auto &g : graph)
            if (g) cudaGraphExecDestroy(g);
        for (auto &ev : events) cudaEventDestroy(ev);
        for (auto &ev : piece_events) cudaEventDestroy(ev);
        if (io_stream) {
            cudaStreamSynchronize(io_stream);
            cudaStreamDestroy(io_stream);
        }
        if (grid_ready) cudaEventDestroy(grid_ready);
        if (io_done) cudaEventDestroy(io_done);
        if (io_up) cudaEventDestroy(io_up);
    }

    cudaStream_t stream() const { return solver->stream; }

    StepView view(int c) {
        StepView s{};
        s.scenes = d_scenes.p;
        s.wells = d_wells.p;
        s.tris = d_tris.p;
        s.n = (uint32_t)n;
        s.n_scenes = n_scenes;
        s.mbits = mbits;
        s.ph = ph;
        s.x0 = x[c].p;
        s.v0 = v[c].p;
        s.type0 = type[c].p;
        s.col0 = col[c].p;
        s.slot0 = slot[c].p;
        s.x1 = x[c ^ 1].p;
        s.v1 = v[c ^ 1].p;
        s.type1 = type[c ^ 1].p;
        s.col1 = col[c ^ 1].p;
        s.slot1 = slot[c ^ 1].p;
        s.keys_prev = keys_sorted.p;
        s.keys_in = keys_in.p;
        s.vals_in = vals_in.p;
        s.keys_sorted = keys_sorted.p;
        s.vals_sorted = vals_sorted.p;
        s.cells = cells.p;
        s.cells_n = cells_n;
        s.ps_a = ps[0].p;
        s.ps_b = ps[1].p;
        s.lambda = lambda.p;
        s.plam = plam.p;
        s.pom = pom.p;
        s.mass_range = mass_range.p;
        s.density = density.p;
        s.omega = omega.p;
        s.vx = vx.p;
        s.err = err.p;
        s.block = block;
        s.queue = persistent ? queue.p : nullptr;
        s.list_policy = list_policy.p;
        s.list_min_use = list_min_use_set ? list_min_use : (verlet_off ? 10u : 25u);
        s.ppt = persistent ? ppt : 1;
        s.verlet_off = verlet_off;
        s.iterations = iterations;
        s.sm_count = sm_count;
        s.nlist = nlist.p;
        s.ncount = ncount.p;
        s.cap = nlist.p ? list_cap : 0;
        const float skin = skin_frac * ph.h;
        const float reach = (ph.h + skin) * 1.00001f;
        s.list_r2 = reach * reach;
        s.skin = skin;
        s.ps_grid = ps_grid.p;
        s.disp = disp.p;
        s.cellmax = cellmax.p;
        s.valid = valid.p;
        s.hlist = hlist.p;
        s.hcount = hcount.p;
        s.hcap = hlist.p ? hit_cap : 0;
        // a near row filtered from a Verlet list is complete out to h + skin only
        const float near_skin = std::min(near_frac, skin_frac) * ph.h;
        const float near_reach = (ph.h + near_skin) * 1.00001f;
        s.near = near_frac > 0.f ? near.p : nullptr;
        s.near_r2 = near_reach * near_reach;
        s.near_skin = near_skin;
        s.hout = advance_io ? hout_dev.p : nullptr;
        s.over = over.p;
        s.near_stats = row_stats && over.p ? over.p + 2 : nullptr;
        return s;
    }

    // Stage timing: CUDA events recorded between the stages of a step (inside the
    // captured graphs as external event nodes).  Stage order: predict, sort,
    // reorder, then lambda/delta per iteration, then the two vorticity passes.
    bool timing = false;
    std::vector<cudaEvent_t> events;
    uint32_t n_stages = 0;

    void mark(uint32_t &k, cudaStream_t st) {
        if (!timing) return;
        if (k < events.size()) cudaEventRecordWithFlags(events[k], st, cudaEventRecordExternal);
        ++k;
    }

    // Enqueue one step that reads state set c and leaves the state in set c^1.
    int record_step(int c) {
        cudaStream_t st = stream();
        StepView s = view(c);
        uint64_t l = 0;
        uint32_t k = 0;
        if (over.p) FGB_CUDA(cudaMemsetAsync(over.p, 0, 2 * sizeof(uint32_t), st), "step: overflow counters");
        mark(k, st);
        launch_predict_keys(s, st);
        l += 1;
        mark(k, st);
        cudaError_t e = radix_sort_pairs(keys_in.p, vals_in.p, keys_sorted.p, vals_sorted.p, n, key_bits,
                                         sort_scratch.p, sort_scratch_bytes, st, err.p, &l);
        if (e != cudaSuccess) return fail_cuda(e, "step: radix sort");
        mark(k, st);
        if (io_up) FGB_CUDA(cudaStreamWaitEvent(st, io_up, cudaEventWaitExternal), "step: upload event");
        FGB_CUDA(cudaMemsetAsync(cells.p, 0, cells_n * sizeof(uint2), st), "step: clear cells");
        if (persistent)
            FGB_CUDA(cudaMemsetAsync(queue.p, 0, slots_of_step(iterations) * sizeof(uint32_t), st),
                     "step: clear tile counters");
        FGB_CUDA(cudaMemsetAsync(mass_range.p, 0xff, 2 * sizeof(uint32_t), st), "step: clear mass range");
        if (cellmax.p) FGB_CUDA(cudaMemsetAsync(cellmax.p, 0, cells_n * sizeof(uint32_t), st), "step: clear cellmax");
        launch_reorder_cells(s, st);
        l += 1;
        if (ph.profile == FGB_PROFILE_REF) {
            launch_diffuse(s, colour_sums.p, colour_count.p, st);
            l += 2;
        }
        if (grid_ready) FGB_CUDA(cudaEventRecordWithFlags(grid_ready, st, cudaEventRecordExternal), "grid event");
        mark(k, st);
        // p* of the grid stays in ps_grid; the iterations ping-pong between ps[0] and ps[1]
        const float4 *pin = ps_grid.p;
        for (uint32_t it = 0; it < iterations; ++it) {
            float4 *pout = ps[it & 1].p;
            launch_lambda(s, pin, (int)it, st);  // the first also builds the Verlet lists (two kernels)
            mark(k, st);
            // the list bound at the next pass needs the neighbours' displacement at that
            // pass only: the cell maxima restart at every delta pass (the step's first
            // starts from the clear above), so an iteration that overshoots does not keep
            // lists invalid after the next one has moved the particles back
            if (it > 0 && cellmax.p)
                FGB_CUDA(cudaMemsetAsync(cellmax.p, 0, cells_n * sizeof(uint32_t), st), "step: clear cellmax");
            launch_delta(s, pin, pout, (int)it, it + 1 == iterations, st);
            mark(k, st);
            l += (it == 0 && s.cap) ? 3 : 2;
            pin = pout;
        }
        if (ph.profile != FGB_PROFILE_REF) {
            launch_velocity_terms(s, pin, st, [&] { mark(k, st); });
            mark(k, st);
            l += 2;
        }
        if (s.list_policy && s.cap) {
            launch_list_policy(s, st);
            l += 1;
        }
        if (over.p)
            FGB_CUDA(cudaMemcpyAsync(st_over.p, over.p, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st),
                     "step: overflow counters");
        FGB_CUDA(cudaMemcpyAsync(st_flags.p, err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st), "step: error flags");
        FGB_CUDA(cudaGetLastError(), "step: launch");
        launches_per_step = l;
        if (timing) n_stages = k ? k - 1 : 0;
        return FGB_OK;
    }

    // Time `per_trial` - 1 steps (after one untimed step) under each candidate
    // launch shape: CTA sizes first at the current skin, then skins at the best CTA
    // size.  Neither knob changes a result (the lists are exact for any skin, and
    // each thread owns one particle), so these are ordinary steps of the batch.
    int autotune(uint32_t per_trial, fgb_tune_result *out) {
        if (per_trial < 2) per_trial = 2;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        FGB_CUDA(cudaEventCreate(&e0), "autotune event");
        FGB_CUDA(cudaEventCreate(&e1), "autotune event");
        uint32_t trials = 0, steps = 0;
        auto trial = [&](int blk, float skin, bool pers, uint32_t per_thread, float *ms, bool voff = false) -> int {
            block = blk;
            skin_frac = skin;
            persistent = pers;
            ppt = per_thread;
            verlet_off = voff ? 1u : 0u;
            // every trial starts from the list policy of a fresh batch (lists on), so
            // that one trial's choices do not carry into the next
            if (list_policy.p) {
                std::vector<uint32_t> init(kPolicyWords * (size_t)n_scenes, 0u);
                for (uint32_t k = 0; k < n_scenes; ++k) init[kPolicyWords * k] = 1u;
                if (cudaMemcpyAsync(list_policy.p, init.data(), init.size() * sizeof(uint32_t),
                                    cudaMemcpyHostToDevice, stream()) != cudaSuccess ||
                    cudaStreamSynchronize(stream()) != cudaSuccess)
                    return fail(FGB_ERR_CUDA, "autotune: list policy");
            }
            for (auto &g : graph)
                if (g) cudaGraphExecDestroy(g), g = nullptr;
            graphs_ok = false;
            int rc = step(1);
            if (!rc) rc = cudaEventRecord(e0, stream()) == cudaSuccess ? FGB_OK : fail(FGB_ERR_CUDA, "autotune");
            if (!rc) rc = step(per_trial - 1);
            if (!rc) rc = cudaEventRecord(e1, stream()) == cudaSuccess ? FGB_OK : fail(FGB_ERR_CUDA, "autotune");
            if (!rc && cudaEventSynchronize(e1) != cudaSuccess) rc = fail(FGB_ERR_CUDA, "autotune sync");
            float t = 0.f;
            if (!rc) cudaEventElapsedTime(&t, e0, e1);
            *ms = t / (float)(per_trial - 1);
            trials++;
            steps += per_trial;
            return rc;
        };
        int rc = FGB_OK;
        int best_block = block;
        float best_skin = skin_frac, best_ms = 3.4e38f, ms = 0.f;
        bool best_pers = false;
        uint32_t best_ppt = 1;
        const float skin0 = skin_frac;
        // flat grids: CTA sizes, then skins; then persistent tile queues of 1 and 2
        // particles per thread at the best of those
        for (int blk : {64, 128, 256}) {
            rc = trial(blk, skin0, false, 1, &ms);
            if (rc) break;
            if (ms < best_ms) best_ms = ms, best_block = blk;
        }
        for (float skin : {0.1f, 0.15f, 0.25f, 0.3f}) {
            if (rc || skin == skin0) continue;
            rc = trial(best_block, skin, false, 1, &ms);
            if (!rc && ms < best_ms) best_ms = ms, best_skin = skin;
        }
        for (uint32_t per_thread : {1u, 2u}) {
            if (rc || !queue.p) continue;
            rc = trial(best_block, best_skin, true, per_thread, &ms);
            if (!rc && ms < best_ms) best_ms = ms, best_pers = true, best_ppt = per_thread;
        }
        // near rows without Verlet lists: trials alternate with and without them (with,
        // without, with, without, with), so a drift of the flow that is linear over the
        // five trials weighs both equally
        bool best_voff = false;
        if (!rc && list_cap && hit_cap) {
            float on = 0.f, off = 0.f, t = 0.f;
            for (int k = 0; k < 5 && !rc; ++k) {
                rc = trial(best_block, best_skin, best_pers, best_ppt, &t, k & 1);
                if (k & 1) off += t / 2.f;
                else on += t / 3.f;
            }
            if (!rc && off < 0.995f * on) best_voff = true, best_ms = off;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        block = best_block;
        skin_frac = best_skin;
        persistent = best_pers;
        ppt = best_ppt;
        verlet_off = best_voff ? 1u : 0u;
        for (auto &g : graph)
            if (g) cudaGraphExecDestroy(g), g = nullptr;
        graphs_ok = false;
        if (rc) return rc;
        solver->tuned[tune_bucket(solver->params.profile, n)] = {best_block, best_skin, best_pers, best_ppt, best_voff};
        if (out) {
            out->block = (uint32_t)best_block;
            out->skin = best_skin;
            out->persistent = best_pers ? 1u : 0u;
            out->particles_per_thread = best_ppt;
            out->verlet = best_voff ? 0u : 1u;
            out->ms_per_step = best_ms;
            out->trials = trials;
            out->steps = steps;
        }
        return FGB_OK;
    }

    int set_timing(bool on) {
        if (on == timing) return FGB_OK;
        timing = on;
        if (on && events.empty()) {
            events.resize(3 + 2 * iterations + 2 + 1);
            for (auto &ev : events) FGB_CUDA(cudaEventCreate(&ev), "timing events");
        }
        for (auto &g : graph)
            if (g) cudaGraphExecDestroy(g), g = nullptr;
        graphs_ok = false;
        return FGB_OK;
    }

    int sync_tris() {
        if (!tris_dirty) return FGB_OK;
        PoolScope scope(&solver->pool);
        std::vector<TriDev> all;
        for (uint32_t k = 0; k < n_scenes; ++k) {
            h_scenes[k].tri_first = (uint32_t)all.size();
            h_scenes[k].tri_count = (uint32_t)scene_tris[k].size();
            all.insert(all.end(), scene_tris[k].begin(), scene_tris[k].end());
        }
        bool moved = false;
        if (all.size() > d_tris.n || !d_tris.p) {
            FGB_CUDA(d_tris.alloc(std::max<size_t>(all.size(), 1)), "colliders");
            moved = true;
        }
        if (!all.empty())
            FGB_CUDA(cudaMemcpyAsync(d_tris.p, all.data(), all.size() * sizeof(TriDev), cudaMemcpyHostToDevice,
                                     stream()),
                     "colliders upload");
        FGB_CUDA(cudaMemcpyAsync(d_scenes.p, h_scenes.data(), n_scenes * sizeof(SceneDev), cudaMemcpyHostToDevice,
                                 stream()),
                 "scene upload");
        FGB_CUDA(cudaStreamSynchronize(stream()), "colliders sync");
        tris_dirty = false;
        if (moved) {  // the collider array pointer is baked into the graphs
            for (auto &g : graph)
                if (g) cudaGraphExecDestroy(g), g = nullptr;
            graphs_ok = false;
        }
        return FGB_OK;
    }

    int build_graphs() {
        cudaStream_t st = stream();
        for (int c = 0; c < 2; ++c) {
            cudaGraph_t g = nullptr;
            FGB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "graph capture begin");
            int rc = record_step(c);
            cudaError_t e = cudaStreamEndCapture(st, &g);
            if (rc != FGB_OK) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            if (e != cudaSuccess) return fail_cuda(e, "graph capture end");
            e = cudaGraphInstantiate(&graph[c], g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return fail_cuda(e, "graph instantiate");
        }
        graphs_ok = true;
        return FGB_OK;
    }

    // Everything the first step would set up: the scene table and the two step
    // graphs, instantiated and uploaded to the device.
    int prepare() {
        int rc = sync_tris();
        if (rc) return rc;
        if (!graphs_ok) {
            rc = build_graphs();
            if (rc) return rc;
            for (auto &g : graph) FGB_CUDA(cudaGraphUpload(g, stream()), "graph upload");
        }
        FGB_CUDA(cudaStreamSynchronize(stream()), "prepare sync");
        return FGB_OK;
    }

    // Rows that overflow send their particles' passes back to the 27-cell walk; when
    // more than 1% of a step's particles overflowed (dense, compressed scenes: the
    // ref profile's constants clump the fluid to ~200-400 neighbours within h), the
    // capacity grows by half (at most 1024) and the solver remembers it for the
    // bucket.  The counts arrive in st_over from steps already run.
    int grow_rows() {
        if (!st_over.p) return FGB_OK;
        const uint64_t lim = std::max<uint64_t>(n / 100, 1);
        const bool gl = list_cap && st_over.p[0] > lim && list_cap < kMaxRowCap;
        const bool gh = hit_cap && st_over.p[1] > lim && hit_cap < kMaxRowCap;
        if (!gl && !gh) return FGB_OK;
        // copies queued by earlier steps would report the old capacities
        FGB_CUDA(cudaStreamSynchronize(stream()), "grow rows sync");
        PoolScope scope(&solver->pool);
        const uint64_t rows = capacity ? capacity : n;
        if (gl) {
            list_cap = std::min<uint32_t>(kMaxRowCap, (list_cap * 3 / 2 + 3u) & ~3u);
            FGB_CUDA(nlist.alloc(rows * list_cap), "grow neighbour lists");
        }
        if (gh) {
            hit_cap = std::min<uint32_t>(kMaxRowCap, (hit_cap * 3 / 2 + 3u) & ~3u);
            FGB_CUDA(hlist.alloc(rows * hit_cap), "grow hit lists");
        }
        st_over.p[0] = st_over.p[1] = 0;
        for (auto &g : graph)
            if (g) cudaGraphExecDestroy(g), g = nullptr;
        graphs_ok = false;
        solver->caps[tune_bucket(solver->params.profile, n)] = {list_cap, hit_cap};
        return FGB_OK;
    }

    int step(uint32_t steps) {
        int rc = grow_rows();
        if (rc) return rc;
        rc = sync_tris();
        if (rc) return rc;
        if (!graphs_ok) {
            rc = build_graphs();
            if (rc) return rc;
        }
        for (uint32_t k = 0; k < steps; ++k) {
            FGB_CUDA(cudaGraphLaunch(graph[cur], stream()), "graph launch");
            cur ^= 1;
            launches += launches_per_step;
        }
        if (steps) query_ok = true;
        return FGB_OK;
    }

    int ensure_surface() {
        if (surf_ready) return FGB_OK;
        PoolScope scope(&solver->pool);
        FGB_CUDA(mc_keys.alloc(n), "surface alloc");
        FGB_CUDA(mc_vals.alloc(n), "surface alloc");
        FGB_CUDA(mc_xs.alloc(n), "surface alloc");
        FGB_CUDA(mc_type.alloc(n), "surface alloc");
        FGB_CUDA(mc_col.alloc(n), "surface alloc");
        FGB_CUDA(lattice.alloc(lat_total), "surface alloc lattice");
        FGB_CUDA(lattice_col.alloc(lat_total), "surface alloc lattice");
        FGB_CUDA(cases.alloc(cube_total), "surface alloc cubes");
        FGB_CUDA(offsets.alloc(cube_total + 1), "surface alloc cubes");
        FGB_CUDA(total.alloc(1), "surface alloc");
        scan_scratch_bytes = scan_u32_scratch_bytes(cube_total);
        FGB_CUDA(scan_scratch.alloc(scan_scratch_bytes), "surface alloc");
        surf_ready = true;
        return FGB_OK;
    }

    // Grid over the current positions, then field + classify + scan for scenes [b, e).
    int surface_count(uint32_t b, uint32_t e, uint64_t *tri_total) {
        int rc = sync_tris();  // the scene table (obstacle counts) as of the last upload
        if (!rc) rc = ensure_surface();
        if (rc) return rc;
        query_ok = false;  // the cell table becomes the grid of the current positions
        cudaStream_t st = stream();
        StepView s = view(cur);
        s.keys_prev = keys_sorted.p;
        launch_position_keys(s, x[cur].p, st);
        launches += 1;
        cudaError_t ce = radix_sort_pairs(keys_in.p, vals_in.p, mc_keys.p, mc_vals.p, n, key_bits, sort_scratch.p,
                                          sort_scratch_bytes, st, err.p, &launches);
        if (ce != cudaSuccess) return fail_cuda(ce, "surface: sort");
        FGB_CUDA(cudaMemsetAsync(cells.p, 0, cells_n * sizeof(uint2), st), "surface: clear cells");
        s.keys_sorted = mc_keys.p;
        s.vals_sorted = mc_vals.p;
        launch_gather_positions(s, x[cur].p, type[cur].p, col[cur].p, mc_xs.p, mc_type.p, mc_col.p, st);
        launches += 1;
        SurfaceView v = surface_view(b, e);
        ce = launch_surface_count(v, st, &launches);
        if (ce != cudaSuccess) return fail_cuda(ce, "surface: count");
        uint32_t t = 0;
        FGB_CUDA(cudaMemcpyAsync(&t, total.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st), "surface: total");
        FGB_CUDA(cudaStreamSynchronize(st), "surface: sync");
        *tri_total = t;
        surf_scene_begin = b;
        surf_scene_end = e;
        return FGB_OK;
    }

    SurfaceView surface_view(uint32_t b, uint32_t e) {
        SurfaceView v{};
        v.scenes = d_scenes.p;
        v.h_scenes = h_scenes.data();
        v.scene_begin = b;
        v.scene_end = e;
        v.mbits = mbits;
        v.ph = ph;
        v.keys_sorted = mc_keys.p;
        v.cells = cells.p;
        v.xs = mc_xs.p;
        v.type = mc_type.p;
        v.col = mc_col.p;
        v.lattice = lattice.p;
        v.lattice_col = lattice_col.p;
        v.cases = cases.p;
        v.offsets = offsets.p;
        v.total = total.p;
        v.lat_begin = h_scenes[b].lat_base;
        v.lat_end = (e < n_scenes) ? h_scenes[e].lat_base : lat_total;
        v.cube_begin = h_scenes[b].cube_base;
        v.cube_end = (e < n_scenes) ? h_scenes[e].cube_base : cube_total;
        v.brick_begin = h_scenes[b].brick_base;
        v.brick_end = (e < n_scenes) ? h_scenes[e].brick_base : brick_total;
        v.scan_scratch = scan_scratch.p;
        v.scan_scratch_bytes = scan_scratch_bytes;
        v.err = err.p;
        return v;
    }

    int surface_emit(uint64_t tri_total) {
        if (tri_total > tris_out.n || !tris_out.p) {
            PoolScope scope(&solver->pool);
            uint64_t cap = std::max<uint64_t>(tri_total + tri_total / 4, 1024);
            FGB_CUDA(tris_out.alloc(cap), "surface: triangles alloc");
        }
        SurfaceView v = surface_view(surf_scene_begin, surf_scene_end);
        cudaError_t ce = launch_surface_emit(v, tris_out.p, tris_out.n, stream(), &launches);
        if (ce != cudaSuccess) return fail_cuda(ce, "surface: emit");
        return FGB_OK;
    }
};

static int mesh_assign(fgb_mesh *m, const fgb_mesh_triangle *dev, uint64_t count, cudaStream_t st) {
    if (!m) return FGB_OK;
    if (count > m->capacity || !m->triangles) {
        free(m->triangles);
        m->triangles = (fgb_mesh_triangle *)malloc(std::max<uint64_t>(count, 1) * sizeof(fgb_mesh_triangle));
        if (!m->triangles) {
            m->capacity = 0;
            m->n = 0;
            return fail(FGB_ERR_OOM, "mesh: host allocation failed");
        }
        m->capacity = std::max<uint64_t>(count, 1);
    }
    m->n = count;
    if (count)
        FGB_CUDA(cudaMemcpyAsync(m->triangles, dev, count * sizeof(fgb_mesh_triangle), cudaMemcpyDeviceToHost, st),
                 "mesh: copy");
    FGB_CUDA(cudaStreamSynchronize(st), "mesh: sync");
    return FGB_OK;
}

// Status of a batch's device error flags: FGB_OK when none is set, else the status
// code of the most serious flag with a message naming them all.
static int flags_status(uint32_t f, const char *where) {
    if (!f) return FGB_OK;
    char msg[256];
    snprintf(msg, sizeof msg,
             "%s: device error flags 0x%x (%s%s%s%s%s); fgb_batch_error_flags reads and clears them", where, f,
             f & ERR_SORT_LOOKBACK ? "sort look-back wait gave up " : "",
             f & ERR_SCAN_LOOKBACK ? "scan look-back wait gave up " : "",
             f & ERR_CELL_RANGE ? "key outside its cell table " : "",
             f & ERR_MESH_CAPACITY ? "more triangles than the buffer holds " : "",
             f & ERR_WELD_TABLE ? "welding table full " : "");
    if (f & (ERR_SORT_LOOKBACK | ERR_SCAN_LOOKBACK)) return fail(FGB_ERR_TIMEOUT, msg);
    if (f & (ERR_MESH_CAPACITY | ERR_WELD_TABLE)) return fail(FGB_ERR_CAPACITY, msg);
    return fail(FGB_ERR_INVALID, msg);
}

// Device error flags as of now (synchronises the batch's stream).
static int batch_flags_now(fgb_batch *b, uint32_t *f) {
    cudaStream_t st = b->stream();
    FGB_CUDA(cudaMemcpyAsync(b->st_flags.p, b->err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st), "error flags");
    FGB_CUDA(cudaStreamSynchronize(st), "error flags");
    *f = b->st_flags.p[0];
    return FGB_OK;
}

// The per-particle arrays a step rebuilds (sort keys, p*, lists, lambda, ...), for
// `cap` particles; their contents do not outlive a step.
// FGB_PACKED=0: the delta and vorticity-apply passes read their neighbours from the
// separate arrays instead of the packed copies (for comparison; same results)
static bool packed_off() {
    const char *e = getenv("FGB_PACKED");
    return e && strcmp(e, "0") == 0;
}

static int alloc_step_arrays(fgb_batch *b, uint64_t cap) {
    PoolScope scope(&b->solver->pool);
    const fgb_params &p = b->solver->params;
    for (int c = 0; c < 2; ++c) FGB_CUDA(b->ps[c].alloc(cap), "batch alloc");
    FGB_CUDA(b->keys_in.alloc(cap), "batch alloc");
    FGB_CUDA(b->vals_in.alloc(cap), "batch alloc");
    FGB_CUDA(b->keys_sorted.alloc(cap), "batch alloc");
    FGB_CUDA(b->vals_sorted.alloc(cap), "batch alloc");
    b->sort_scratch_bytes = radix_scratch_bytes(cap);
    FGB_CUDA(b->sort_scratch.alloc(b->sort_scratch_bytes), "batch alloc");
    FGB_CUDA(b->ps_grid.alloc(cap), "batch alloc");
    if (b->list_cap) {
        FGB_CUDA(b->nlist.alloc(cap * b->list_cap), "batch alloc neighbour lists");
        FGB_CUDA(b->ncount.alloc(cap), "batch alloc");
        FGB_CUDA(b->disp.alloc(cap), "batch alloc");
        FGB_CUDA(b->valid.alloc(cap), "batch alloc");
    }
    if (b->hit_cap) {
        FGB_CUDA(b->hlist.alloc(cap * b->hit_cap), "batch alloc hit lists");
        FGB_CUDA(b->hcount.alloc(cap), "batch alloc");
    }
    if (b->list_cap && b->hit_cap) FGB_CUDA(b->near.alloc(cap), "batch alloc");
    FGB_CUDA(b->lambda.alloc(cap), "batch alloc");
    if (!packed_off()) FGB_CUDA(b->plam.alloc(cap), "batch alloc");
    FGB_CUDA(b->mass_range.alloc(2), "batch alloc");
    FGB_CUDA(b->density.alloc(cap), "batch alloc");
    if (p.profile != FGB_PROFILE_REF) {
        if (!packed_off()) FGB_CUDA(b->pom.alloc(cap), "batch alloc");
        FGB_CUDA(b->omega.alloc(cap), "batch alloc");
        FGB_CUDA(b->vx.alloc(cap), "batch alloc");
    } else {
        FGB_CUDA(b->colour_sums.alloc(cap), "batch alloc");
        FGB_CUDA(b->colour_count.alloc(cap), "batch alloc");
    }
    cudaStream_t st = b->stream();
    FGB_CUDA(cudaMemsetAsync(b->lambda.p, 0, cap * sizeof(float), st), "batch alloc");
    FGB_CUDA(cudaMemsetAsync(b->density.p, 0, cap * sizeof(float), st), "batch alloc");
    b->capacity = cap;
    return FGB_OK;
}

// Uploads and downloads run as kernels that read and write the caller's arrays
// where the device addresses pageable memory through the host's page tables
// (Grace's coherent link); elsewhere, or with FGB_HOST_IO=staged, the host packs
// into pinned staging buffers that the copy engines move.  Both give the same bytes.
static bool host_io_direct() {
    const char *e = getenv("FGB_HOST_IO");
    if (e && strcmp(e, "staged") == 0) return false;
    int dev = 0, pageable = 0, host_tables = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess)
        return false;
    return pageable && host_tables;
}

static int batch_init(fgb_batch *b) {
    PoolScope scope(&b->solver->pool);
    fgb_solver *s = b->solver;
    const fgb_params &p = s->params;
    b->ph = s->ph;
    b->h_scenes.assign(b->n_scenes, SceneDev{});
    uint32_t max_ext = 0;
    uint64_t table = 0, lat = 0, cubes = 0, bricks = 0;
    std::vector<WellDev> wells;
    b->first.resize(b->n_scenes);
    uint64_t off = 0;
    b->iterations = b->cfg[0].iterations;
    for (uint32_t k = 0; k < b->n_scenes; ++k) {
        const fgb_config &c = b->cfg[k];
        if (!(c.scale > 0.f) || !(c.dt > 0.f)) return fail(FGB_ERR_INVALID, "config: scale and dt must be > 0");
        if (c.iterations != b->iterations)
            return fail(FGB_ERR_INVALID, "batch: every scene needs the same iteration count");
        if (c.n_wells > FGB_MAX_WELLS) return fail(FGB_ERR_CAPACITY, "config: more than FGB_MAX_WELLS wells");
        for (int a = 0; a < 3; ++a)
            if (!(c.max_bound[a] >= c.min_bound[a])) return fail(FGB_ERR_INVALID, "config: max_bound < min_bound");
        SceneDev &S = b->h_scenes[k];
        scene_geometry(p, c, S);
        for (int a = 0; a < 3; ++a) max_ext = std::max(max_ext, S.ext[a]);
        S.table_base = (uint32_t)table;
        table += (uint64_t)morton3(S.ext[0], S.ext[1], S.ext[2]) + 1;
        S.first = (uint32_t)off;
        S.count = (uint32_t)b->counts[k];
        b->first[k] = off;
        off += b->counts[k];
        S.n_wells = c.n_wells;
        S.well_first = (uint32_t)wells.size();
        for (uint32_t w = 0; w < c.n_wells; ++w) {
            WellDev wd;
            for (int a = 0; a < 3; ++a) wd.centre[a] = c.wells[w].centre[a];
            wd.force = c.wells[w].force;
            wells.push_back(wd);
        }
        S.lat_base = lat;
        S.cube_base = cubes;
        S.brick_base = bricks;
        bricks += field_bricks(S.lat);
        lat += (uint64_t)S.lat[0] * S.lat[1] * S.lat[2];
        if (S.lat[0] > 1 && S.lat[1] > 1 && S.lat[2] > 1)
            cubes += (uint64_t)(S.lat[0] - 1) * (S.lat[1] - 1) * (S.lat[2] - 1);
    }
    if (b->iterations == 0) return fail(FGB_ERR_INVALID, "config: iterations must be >= 1");
    b->n = off;
    if (b->n > 0x7fffffffull) return fail(FGB_ERR_CAPACITY, "batch: more than 2^31-1 particles");
    if (table > 0xffffffffull) return fail(FGB_ERR_CAPACITY, "batch: cell tables above 2^32 entries");
    b->cells_n = table;
    b->lat_total = lat;
    b->cube_total = cubes;
    b->brick_total = bricks;
    if (cubes > 0xffffffffull) return fail(FGB_ERR_CAPACITY, "batch: more than 2^32-1 marching cubes");
    if (bricks > 0x7fffffffull) return fail(FGB_ERR_CAPACITY, "batch: more than 2^31-1 lattice bricks");
    b->mbits = 3 * bits_for(max_ext);
    b->sbits = bits_for(b->n_scenes - 1);
    b->key_bits = b->mbits + b->sbits;
    if (b->key_bits > 32) return fail(FGB_ERR_CAPACITY, "batch: scene id + Morton key exceed 32 bits");
    if (b->key_bits == 0) b->key_bits = 1;
    const uint64_t n = std::max<uint64_t>(b->n, 1);
    ensure_tables();
    for (int c = 0; c < 2; ++c) {
        FGB_CUDA(b->x[c].alloc(n), "batch alloc");
        FGB_CUDA(b->v[c].alloc(n), "batch alloc");
        FGB_CUDA(b->type[c].alloc(n), "batch alloc");
        FGB_CUDA(b->col[c].alloc(n), "batch alloc");
        FGB_CUDA(b->slot[c].alloc(n), "batch alloc");
    }
    FGB_CUDA(b->ids_dev.alloc(n), "batch alloc");
    FGB_CUDA(b->cells.alloc(std::max<uint64_t>(table, 1)), "batch alloc cells");
    {
        auto it = s->caps.find(tune_bucket(p.profile, n));
        if (it != s->caps.end()) {
            b->list_cap = it->second.first;
            b->hit_cap = it->second.second;
        }
    }
    if (const char *e = getenv("FGB_LIST_CAP")) b->list_cap = (uint32_t)atoi(e);
    b->block = s->block;
    {
        auto it = s->tuned.find(tune_bucket(p.profile, n));
        if (it != s->tuned.end()) {
            b->block = it->second.block;
            b->skin_frac = it->second.skin;
            b->persistent = it->second.persistent;
            b->ppt = it->second.ppt;
            b->verlet_off = it->second.verlet_off ? 1u : 0u;
        }
    }
    if (const char *e = getenv("FGB_LIST_SKIN")) b->skin_frac = (float)atof(e);
    if (const char *e = getenv("FGB_VERLET")) b->verlet_off = atoi(e) == 0;
    if (const char *e = getenv("FGB_PERSISTENT")) b->persistent = atoi(e) != 0;
    if (const char *e = getenv("FGB_PPT")) b->ppt = (uint32_t)std::max(1, std::min(8, atoi(e)));
    cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, s->device);
    FGB_CUDA(b->queue.alloc(slots_of_step(b->iterations)), "batch alloc");
    if (!(getenv("FGB_LIST_POLICY") && strcmp(getenv("FGB_LIST_POLICY"), "0") == 0)) {
        FGB_CUDA(b->list_policy.alloc(kPolicyWords * (uint64_t)b->n_scenes), "batch alloc");
        if (const char *e = getenv("FGB_LIST_MIN_USE")) {
            b->list_min_use = (uint32_t)std::max(0, std::min(101, atoi(e)));
            b->list_min_use_set = true;
        }
        std::vector<uint32_t> init(kPolicyWords * (size_t)b->n_scenes, 0u);
        for (uint32_t k = 0; k < b->n_scenes; ++k) init[kPolicyWords * k] = 1u;  // the first step builds lists
        FGB_CUDA(cudaMemcpy(b->list_policy.p, init.data(), init.size() * sizeof(uint32_t), cudaMemcpyHostToDevice),
                 "batch alloc");
    }
    if (b->list_cap > 4096) b->list_cap = 4096;
    b->list_cap = (b->list_cap + 3u) & ~3u;  // rows move as 16-byte vectors
    if (b->list_cap) FGB_CUDA(b->cellmax.alloc(std::max<uint64_t>(table, 1)), "batch alloc");
    if (const char *e = getenv("FGB_HIT_CAP")) b->hit_cap = (uint32_t)atoi(e);
    if (const char *e = getenv("FGB_NEAR_SKIN")) b->near_frac = (float)atof(e);
    if (b->hit_cap > 4096) b->hit_cap = 4096;
    b->hit_cap = (b->hit_cap + 3u) & ~3u;  // rows move as 16-byte vectors
    int rc = alloc_step_arrays(b, n);
    if (rc) return rc;
    FGB_CUDA(b->err.alloc(1), "batch alloc");
    FGB_CUDA(b->st_flags.ensure(1), "batch alloc");
    b->st_flags.p[0] = 0;
    if (b->list_cap || b->hit_cap) {
        FGB_CUDA(b->over.alloc(6), "batch alloc");
        FGB_CUDA(cudaMemset(b->over.p, 0, 6 * sizeof(uint32_t)), "batch alloc");
        const char *e = getenv("FGB_ROW_STATS");
        b->row_stats = e && strcmp(e, "1") == 0;
        FGB_CUDA(b->st_over.ensure(2), "batch alloc");
        b->st_over.p[0] = b->st_over.p[1] = 0;
    }
    FGB_CUDA(b->d_scenes.alloc(b->n_scenes), "batch alloc");
    FGB_CUDA(b->d_wells.alloc(std::max<size_t>(wells.size(), 1)), "batch alloc");
    FGB_CUDA(b->d_tris.alloc(1), "batch alloc");
    cudaStream_t st = b->stream();
    FGB_CUDA(cudaMemsetAsync(b->err.p, 0, sizeof(uint32_t), st), "batch init");
    if (!wells.empty())
        FGB_CUDA(cudaMemcpyAsync(b->d_wells.p, wells.data(), wells.size() * sizeof(WellDev), cudaMemcpyHostToDevice, st),
                 "batch init");
    FGB_CUDA(cudaMemcpyAsync(b->d_scenes.p, b->h_scenes.data(), b->n_scenes * sizeof(SceneDev),
                             cudaMemcpyHostToDevice, st),
             "batch init");
    // scene ids in the high key bits before the first step
    FGB_CUDA(b->st_keys.ensure(n), "batch init");
    for (uint32_t k = 0; k < b->n_scenes; ++k)
        for (uint64_t i = 0; i < b->counts[k]; ++i)
            b->st_keys.p[b->first[k] + i] = b->mbits >= 32 ? 0u : (k << b->mbits);
    FGB_CUDA(cudaMemcpyAsync(b->keys_sorted.p, b->st_keys.p, b->n * sizeof(uint32_t), cudaMemcpyHostToDevice, st),
             "batch init");
    FGB_CUDA(cudaStreamSynchronize(st), "batch init");
    b->ids.assign(b->n_scenes, {});
    b->ids_stale.assign(b->n_scenes, 0);
    b->direct = host_io_direct();
    if (b->direct) {
        FGB_CUDA(b->obst_dev.alloc(b->n_scenes), "batch alloc");
        FGB_CUDA(b->st_count.ensure(1), "batch alloc");
        FGB_CUDA(cudaEventCreateWithFlags(&b->grid_ready, cudaEventDisableTiming), "batch events");
        FGB_CUDA(cudaEventCreateWithFlags(&b->io_done, cudaEventDisableTiming), "batch events");
        FGB_CUDA(cudaStreamCreateWithFlags(&b->io_stream, cudaStreamNonBlocking), "batch stream");
        FGB_CUDA(cudaEventCreateWithFlags(&b->io_up, cudaEventDisableTiming), "batch events");
        FGB_CUDA(cudaEventRecord(b->io_up, b->io_stream), "batch events");  // complete until an advance
    }
    b->scene_tris.assign(b->n_scenes, {});
    return FGB_OK;
}

// Give ids_dev the ids of every scene uploaded since the last call (the wire
// packers, scene copies and source/drain edits read it; steps do not).
static int sync_ids(fgb_batch *b) {
    cudaStream_t st = b->stream();
    for (uint32_t k = 0; k < b->n_scenes; ++k) {
        if (!b->ids_stale[k]) continue;
        const uint64_t n = b->counts[k];
        if (n) {
            FGB_CUDA(cudaStreamSynchronize(st), "ids sync");
            FGB_CUDA(b->st_ids.ensure(n), "ids staging");
            const uint64_t *src = b->ids[k].data();
            parallel_for(n, [&](uint64_t lo, uint64_t hi) {
                for (uint64_t i = lo; i < hi; ++i) b->st_ids.p[i] = src[i];
            });
            FGB_CUDA(cudaMemcpyAsync(b->ids_dev.p + b->first[k], b->st_ids.p, n * sizeof(uint64_t),
                                     cudaMemcpyHostToDevice, st),
                     "ids upload");
            FGB_CUDA(cudaStreamSynchronize(st), "ids sync");
        }
        b->ids_stale[k] = 0;
    }
    return FGB_OK;
}

// What every upload ends with: the scene table learns whether the scene holds
// obstacles, and the scene's key prefix is set in case a surface call precedes
// the first step.
static void upload_done(fgb_batch *b, uint32_t k, uint32_t obstacles) {
    b->query_ok = false;
    if (b->h_scenes[k].obstacles != obstacles) {
        b->h_scenes[k].obstacles = obstacles;
        b->tris_dirty = true;  // re-uploads the scene table before the next step
    }
    launch_fill_u32(b->keys_sorted.p + b->first[k], b->counts[k], b->mbits >= 32 ? 0u : (k << b->mbits), b->stream());
}

// One kernel reads the caller's arrays and writes the scene segment (ids go to
// ids_dev, which is then the only copy).  Returns once the kernel has finished,
// so the caller may reuse its arrays.
static int batch_upload_direct(fgb_batch *b, uint32_t k, const fgb_particles *xs) {
    const uint64_t n = xs->n, f = b->first[k];
    const int c = b->cur;
    cudaStream_t st = b->stream();
    FGB_CUDA(cudaMemsetAsync(b->obst_dev.p + k, 0, sizeof(uint32_t), st), "upload");
    const HostParticlesIn in{xs->position, xs->velocity, xs->mass, xs->type, xs->colour, xs->id};
    launch_pack_from_host(in, n, b->x[c].p + f, b->v[c].p + f, b->type[c].p + f, b->col[c].p + f, b->slot[c].p + f,
                          b->ids_dev.p + f, b->obst_dev.p + k, st);
    FGB_CUDA(cudaGetLastError(), "upload kernel");
    FGB_CUDA(cudaMemcpyAsync(b->st_count.p, b->obst_dev.p + k, sizeof(uint32_t), cudaMemcpyDeviceToHost, st),
             "upload");
    FGB_CUDA(cudaStreamSynchronize(st), "upload sync");
    b->ids[k].clear();
    b->ids_stale[k] = 0;
    upload_done(b, k, b->st_count.p[0]);
    return FGB_OK;
}

static int batch_upload(fgb_batch *b, uint32_t k, const fgb_particles *xs) {
    if (k >= b->n_scenes) return fail(FGB_ERR_INVALID, "upload: scene out of range");
    if (!xs || xs->n != b->counts[k]) return fail(FGB_ERR_INVALID, "upload: particle count differs from the batch");
    const uint64_t n = xs->n, f = b->first[k];
    if (n && (!xs->position || !xs->velocity || !xs->mass || !xs->type))
        return fail(FGB_ERR_INVALID, "upload: null particle array");
    if (b->direct) return batch_upload_direct(b, k, xs);
    FGB_CUDA(b->st_x.ensure(n), "upload staging");
    FGB_CUDA(b->st_v.ensure(n), "upload staging");
    FGB_CUDA(b->st_type.ensure(n), "upload staging");
    FGB_CUDA(b->st_col.ensure(n), "upload staging");
    cudaStream_t st = b->stream();
    FGB_CUDA(cudaStreamSynchronize(st), "upload sync");
    b->ids[k].resize(n);
    std::atomic<uint32_t> obstacle_count{0};
    uint64_t *ids = b->ids[k].data();
    const int c = b->cur;
    // piece by piece: pack on the host threads, then queue the piece's copies, which
    // run while the next piece is packed
    const uint64_t piece = std::max<uint64_t>(kPieceMin, (n + kPieces - 1) / kPieces);
    for (uint64_t p0 = 0; p0 < n; p0 += piece) {
        const uint64_t m = std::min(n - p0, piece);
        parallel_for(m, [&](uint64_t lo, uint64_t hi) {
            uint32_t obst = 0;
            for (uint64_t i = p0 + lo; i < p0 + hi; ++i) {
                b->st_x.p[i] =
                    make_float4(xs->position[3 * i], xs->position[3 * i + 1], xs->position[3 * i + 2], xs->mass[i]);
                b->st_v.p[i] = make_float4(xs->velocity[3 * i], xs->velocity[3 * i + 1], xs->velocity[3 * i + 2], 0.f);
                b->st_type.p[i] = xs->type[i];
                b->st_col.p[i] = xs->colour ? xs->colour[i] : 0xffffffffu;
                ids[i] = xs->id ? xs->id[i] : i;
                obst += xs->type[i] == FGB_TYPE_OBSTACLE;
            }
            obstacle_count += obst;
        });
        const uint64_t d = f + p0;
        FGB_CUDA(cudaMemcpyAsync(b->x[c].p + d, b->st_x.p + p0, m * sizeof(float4), cudaMemcpyHostToDevice, st),
                 "upload");
        FGB_CUDA(cudaMemcpyAsync(b->v[c].p + d, b->st_v.p + p0, m * sizeof(float4), cudaMemcpyHostToDevice, st),
                 "upload");
        FGB_CUDA(cudaMemcpyAsync(b->type[c].p + d, b->st_type.p + p0, m * sizeof(int32_t), cudaMemcpyHostToDevice, st),
                 "upload");
        FGB_CUDA(cudaMemcpyAsync(b->col[c].p + d, b->st_col.p + p0, m * sizeof(uint32_t), cudaMemcpyHostToDevice, st),
                 "upload");
    }
    // slot = place at upload; the ids reach the device only when a device-side
    // consumer asks for them (sync_ids)
    launch_iota_u32(b->slot[c].p + f, n, st);
    b->ids_stale[k] = 1;
    upload_done(b, k, obstacle_count.load());
    // the staging buffers are only rewritten after a synchronisation (the next
    // upload's, or a download's), so the copies may still be running on return
    return FGB_OK;
}

// Device-to-device copy of one resident scene into another batch (the serving loop
// moves running scenes into a new batch when its membership changes).  The segment
// keeps its particle order, so the scene's next steps are bit-identical to what the
// old batch -- or the scene alone -- would compute.
static int batch_copy_scene(fgb_batch *dst, uint32_t dk, fgb_batch *src, uint32_t sk) {
    if (dk >= dst->n_scenes || sk >= src->n_scenes) return fail(FGB_ERR_INVALID, "copy_scene: scene out of range");
    if (dst->counts[dk] != src->counts[sk]) return fail(FGB_ERR_INVALID, "copy_scene: particle counts differ");
    const uint64_t n = src->counts[sk], fd = dst->first[dk], fs = src->first[sk];
    cudaStream_t st = dst->stream();
    int rc = sync_ids(src);
    if (rc) return rc;
    FGB_CUDA(cudaStreamSynchronize(src->stream()), "copy_scene sync");
    dst->ids_stale[dk] = 0;  // the copy below brings the ids
    dst->query_ok = false;
    const int cd = dst->cur, cs = src->cur;
    if (dst->h_scenes[dk].obstacles != src->h_scenes[sk].obstacles) {
        dst->h_scenes[dk].obstacles = src->h_scenes[sk].obstacles;
        dst->tris_dirty = true;
    }
    if (n) {
        FGB_CUDA(cudaMemcpyAsync(dst->x[cd].p + fd, src->x[cs].p + fs, n * sizeof(float4), cudaMemcpyDeviceToDevice, st),
                 "copy_scene");
        FGB_CUDA(cudaMemcpyAsync(dst->v[cd].p + fd, src->v[cs].p + fs, n * sizeof(float4), cudaMemcpyDeviceToDevice, st),
                 "copy_scene");
        FGB_CUDA(cudaMemcpyAsync(dst->type[cd].p + fd, src->type[cs].p + fs, n * sizeof(int32_t),
                                 cudaMemcpyDeviceToDevice, st),
                 "copy_scene");
        FGB_CUDA(cudaMemcpyAsync(dst->col[cd].p + fd, src->col[cs].p + fs, n * sizeof(uint32_t),
                                 cudaMemcpyDeviceToDevice, st),
                 "copy_scene");
        FGB_CUDA(cudaMemcpyAsync(dst->slot[cd].p + fd, src->slot[cs].p + fs, n * sizeof(uint32_t),
                                 cudaMemcpyDeviceToDevice, st),
                 "copy_scene");
        FGB_CUDA(cudaMemcpyAsync(dst->ids_dev.p + fd, src->ids_dev.p + fs, n * sizeof(uint64_t),
                                 cudaMemcpyDeviceToDevice, st),
                 "copy_scene");
        launch_fill_u32(dst->keys_sorted.p + fd, n, dst->mbits >= 32 ? 0u : (dk << dst->mbits), st);
    }
    if (src->direct && !dst->direct) {  // dst keeps its ids on the host
        dst->ids[dk].assign(n, 0);
        if (n)
            FGB_CUDA(cudaMemcpyAsync(dst->ids[dk].data(), src->ids_dev.p + fs, n * sizeof(uint64_t),
                                     cudaMemcpyDeviceToHost, st),
                     "copy_scene ids");
    } else {
        dst->ids[dk] = src->ids[sk];
    }
    if (dst->scene_tris[dk].size() != src->scene_tris[sk].size() ||
        (!src->scene_tris[sk].empty() && memcmp(dst->scene_tris[dk].data(), src->scene_tris[sk].data(),
                                                src->scene_tris[sk].size() * sizeof(TriDev)) != 0)) {
        dst->scene_tris[dk] = src->scene_tris[sk];
        dst->tris_dirty = true;
    }
    FGB_CUDA(cudaStreamSynchronize(st), "copy_scene sync");
    return FGB_OK;
}

// Device bytes a batch allocates for one scene (admission control of the serving
// loop): per-particle arrays, the scene's cell table, and the surface buffers when a
// mesh is wanted (triangles estimated at one per 20 cubes).  list_words: Verlet-list
// plus hit-list entries per particle.
static uint64_t scene_footprint(const fgb_params &p, const fgb_config &c, uint64_t n, bool mesh,
                                uint32_t list_words) {
    SceneDev S{};
    scene_geometry(p, c, S);
    const uint64_t table = (uint64_t)morton3(S.ext[0], S.ext[1], S.ext[2]) + 1;
    uint64_t per_particle = 64 + 24 + 16 + 8 + 1 + 48 + 8 + 4ull * list_words + 2 + 2 + 4 + 1;
    per_particle += p.profile != FGB_PROFILE_REF ? 32 + 32 : 20 + 16;  // + the packed neighbour copies
    uint64_t bytes = per_particle * n + 12 * table;
    if (mesh && S.lat[0] > 1 && S.lat[1] > 1 && S.lat[2] > 1) {
        const uint64_t samples = (uint64_t)S.lat[0] * S.lat[1] * S.lat[2];
        const uint64_t cubes = (uint64_t)(S.lat[0] - 1) * (S.lat[1] - 1) * (S.lat[2] - 1);
        bytes += 32 * n + 20 * samples + 5 * cubes + sizeof(fgb_mesh_triangle) * (cubes / 20);
    }
    return bytes;
}

static int batch_download(fgb_batch *b, uint32_t k, fgb_particles *xs) {
    if (k >= b->n_scenes) return fail(FGB_ERR_INVALID, "download: scene out of range");
    if (!xs || xs->n != b->counts[k]) return fail(FGB_ERR_INVALID, "download: particle count differs");
    const uint64_t n = xs->n, f = b->first[k];
    if (b->direct) {
        const int c = b->cur;
        cudaStream_t st = b->stream();
        prefault_outputs({{xs->position, 12 * n}, {xs->velocity, 12 * n}, {xs->mass, 4 * n}, {xs->type, 4 * n},
                          {xs->colour, 4 * n}, {xs->id, 8 * n}});
        const HostParticlesOut out{xs->position, xs->velocity, xs->mass, xs->type, xs->colour, xs->id};
        launch_unpack_to_host(out, n, b->x[c].p + f, b->v[c].p + f, b->type[c].p + f, b->col[c].p + f,
                              b->slot[c].p + f, b->ids_dev.p + f, st);
        FGB_CUDA(cudaGetLastError(), "download kernel");
        FGB_CUDA(cudaStreamSynchronize(st), "download sync");
        return FGB_OK;
    }
    FGB_CUDA(b->st_x.ensure(n), "download staging");
    FGB_CUDA(b->st_v.ensure(n), "download staging");
    FGB_CUDA(b->st_type.ensure(n), "download staging");
    FGB_CUDA(b->st_col.ensure(n), "download staging");
    FGB_CUDA(b->st_slot.ensure(n), "download staging");
    cudaStream_t st = b->stream();
    const int c = b->cur;
    // every piece's copies are queued first, each followed by an event; the host
    // threads unpack a piece as soon as its event has passed
    const uint64_t piece = std::max<uint64_t>(kPieceMin, (n + kPieces - 1) / kPieces);
    uint32_t pieces = 0;
    for (uint64_t p0 = 0; p0 < n; p0 += piece, ++pieces) {
        const uint64_t m = std::min(n - p0, piece), d = f + p0;
        if (b->piece_events.size() <= pieces) {
            cudaEvent_t e;
            FGB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "download events");
            b->piece_events.push_back(e);
        }
        FGB_CUDA(cudaMemcpyAsync(b->st_x.p + p0, b->x[c].p + d, m * sizeof(float4), cudaMemcpyDeviceToHost, st),
                 "download");
        FGB_CUDA(cudaMemcpyAsync(b->st_v.p + p0, b->v[c].p + d, m * sizeof(float4), cudaMemcpyDeviceToHost, st),
                 "download");
        FGB_CUDA(cudaMemcpyAsync(b->st_type.p + p0, b->type[c].p + d, m * sizeof(int32_t), cudaMemcpyDeviceToHost, st),
                 "download");
        FGB_CUDA(cudaMemcpyAsync(b->st_col.p + p0, b->col[c].p + d, m * sizeof(uint32_t), cudaMemcpyDeviceToHost, st),
                 "download");
        FGB_CUDA(cudaMemcpyAsync(b->st_slot.p + p0, b->slot[c].p + d, m * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                 st),
                 "download");
        FGB_CUDA(cudaEventRecord(b->piece_events[pieces], st), "download event");
    }
    const std::vector<uint64_t> &ids = b->ids[k];
    uint32_t q = 0;
    for (uint64_t p0 = 0; p0 < n; p0 += piece, ++q) {
        const uint64_t m = std::min(n - p0, piece);
        FGB_CUDA(cudaEventSynchronize(b->piece_events[q]), "download sync");
        parallel_for(m, [&](uint64_t lo, uint64_t hi) {
            for (uint64_t i = p0 + lo; i < p0 + hi; ++i) {
                const float4 X = b->st_x.p[i], V = b->st_v.p[i];
                if (xs->position) {
                    xs->position[3 * i] = X.x;
                    xs->position[3 * i + 1] = X.y;
                    xs->position[3 * i + 2] = X.z;
                }
                if (xs->mass) xs->mass[i] = X.w;
                if (xs->velocity) {
                    xs->velocity[3 * i] = V.x;
                    xs->velocity[3 * i + 1] = V.y;
                    xs->velocity[3 * i + 2] = V.z;
                }
                if (xs->type) xs->type[i] = b->st_type.p[i];
                if (xs->colour) xs->colour[i] = b->st_col.p[i];
                const uint32_t sl = b->st_slot.p[i];
                if (xs->id) xs->id[i] = sl < ids.size() ? ids[sl] : sl;
            }
        });
    }
    FGB_CUDA(cudaStreamSynchronize(st), "download sync");
    return FGB_OK;
}

// Live handles: destroy calls check membership so that a stale or repeated
// destroy is an error instead of a double free.
static std::mutex g_handles_mu;
static std::vector<const void *> g_handles;

static void handle_add(const void *p) {
    std::lock_guard<std::mutex> lk(g_handles_mu);
    g_handles.push_back(p);
}
static bool handle_live(const void *p) {
    std::lock_guard<std::mutex> lk(g_handles_mu);
    return std::find(g_handles.begin(), g_handles.end(), p) != g_handles.end();
}
static bool handle_forget(const void *p) {
    std::lock_guard<std::mutex> lk(g_handles_mu);
    auto it = std::find(g_handles.begin(), g_handles.end(), p);
    if (it == g_handles.end()) return false;
    g_handles.erase(it);
    return true;
}

static void destroy_batch(fgb_batch *b) {
    if (!b) return;
    handle_forget(b);
    if (b->solver) {
        auto &v = b->solver->batches;
        v.erase(std::remove(v.begin(), v.end(), b), v.end());
        if (b->solver->cached == b) b->solver->cached = nullptr;
    }
    delete b;
}

extern "C" {

int fgb_version(void) { return FGB_VERSION; }

const char *fgb_last_error(void) { return g_last_error.c_str(); }

int fgb_struct_sizes(uint64_t *out, int n) {
    const uint64_t sizes[] = {sizeof(fgb_params), sizeof(fgb_config),        sizeof(fgb_particles),
                              sizeof(fgb_triangle), sizeof(fgb_mesh_triangle), sizeof(fgb_mesh),
                              sizeof(fgb_grid_info), sizeof(fgb_well),          sizeof(fgb_serve_options),
                              sizeof(fgb_serve_result), sizeof(fgb_serve_stats), sizeof(fgb_tune_result),
                              sizeof(fgb_source),       sizeof(fgb_drain),       sizeof(fgb_query),
                              sizeof(fgb_query_result), sizeof(fgb_records)};
    const int m = (int)(sizeof(sizes) / sizeof(sizes[0]));
    for (int i = 0; i < n && i < m; ++i) out[i] = sizes[i];
    return m;
}

void fgb_params_default(fgb_params *p, int32_t profile, float h) {
    if (!p) return;
    memset(p, 0, sizeof *p);
    p->h = h;
    p->profile = profile;
    p->corr_n = 4.f;
    p->mc_particle_size = 25.f;     // oclsph.hpp:672
    p->mc_particle_influence = 0.5f; // oclsph.hpp:673
    p->vorticity_epsilon = 0.0005f;  // oclsph_kernel.h:29
    if (profile == FGB_PROFILE_REF) { // oclsph_kernel.h:20-31
        p->rho0 = 6378.f;
        p->cfm_epsilon = 600.f;
        p->corr_k = 0.0001f;
        p->corr_delta_q = 0.3f;
        p->xsph_c = 0.00001f;
        p->velocity_damping = 0.49f;
    } else {
        p->rho0 = 1000.f;
        p->cfm_epsilon = 100.f;
        p->corr_k = 0.1f;
        p->corr_delta_q = 0.2f;
        p->xsph_c = 0.01f;
        p->velocity_damping = 1.f;
    }
}

void fgb_config_default(fgb_config *c, int32_t profile) {
    if (!c) return;
    memset(c, 0, sizeof *c);
    c->scale = 1.f;
    c->resolution = 2.f;
    if (profile == FGB_PROFILE_REF) {
        // samples/main.cpp:398-404 (solverStep 1, isolevel 100, gravity along y)
        c->dt = 0.0083f;
        c->isolevel = 100.f;
        c->iterations = 5;
        c->constant_force[1] = 9.8f;
        c->surface = 1;
    } else {
        c->dt = 1.f / 120.f;
        c->isolevel = 500.f;
        c->iterations = 4;
        c->constant_force[1] = -9.81f;
    }
    for (int a = 0; a < 3; ++a) c->max_bound[a] = 1.f;
}

int fgb_create(const fgb_params *params, fgb_solver **out) {
    if (!params || !out) return fail(FGB_ERR_INVALID, "create: null argument");
    if (!(params->h > 0.f)) return fail(FGB_ERR_INVALID, "create: h must be > 0");
    if (params->profile != FGB_PROFILE_REF && params->profile != FGB_PROFILE_BASELINE)
        return fail(FGB_ERR_INVALID, "create: unknown profile");
    if (!(params->rho0 > 0.f)) return fail(FGB_ERR_INVALID, "create: rho0 must be > 0");
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0)
        return fail(FGB_ERR_CUDA, "create: no CUDA device (this library has no CPU fallback)");
    fgb_solver *s = new fgb_solver();
    s->params = *params;
    s->ph = make_phys(*params);
    cudaGetDevice(&s->device);
    e = cudaStreamCreateWithFlags(&s->own, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete s;
        return fail_cuda(e, "create: stream");
    }
    s->stream = s->own;
    ensure_tables();
    handle_add(s);
    *out = s;
    return FGB_OK;
}

int fgb_destroy(fgb_solver *s) {
    if (!s) return FGB_OK;
    if (!handle_forget(s)) return fail(FGB_ERR_INVALID, "destroy: not a live solver (destroyed twice?)");
    if (s->own) cudaStreamSynchronize(s->own);
    while (!s->batches.empty()) destroy_batch(s->batches.back());
    if (s->own) {
        cudaStreamSynchronize(s->own);
        cudaStreamDestroy(s->own);
    }
    delete s;
    return FGB_OK;
}

int fgb_set_stream(fgb_solver *s, void *cuda_stream) {
    if (!s) return fail(FGB_ERR_INVALID, "set_stream: null solver");
    cudaStream_t st = cuda_stream ? (cudaStream_t)cuda_stream : s->own;
    if (st == s->stream) return FGB_OK;
    // blocks in the solver's pool may still be in use by work queued on the old
    // stream; the new stream's work must not overtake it
    FGB_CUDA(cudaStreamSynchronize(s->stream), "set_stream sync");
    s->stream = st;
    if (s->cached) {
        for (auto &g : s->cached->graph)
            if (g) cudaGraphExecDestroy(g), g = nullptr;
        s->cached->graphs_ok = false;
    }
    return FGB_OK;
}

int fgb_batch_create(fgb_solver *s, uint32_t n_scenes, const uint64_t *counts, const fgb_config *configs,
                     fgb_batch **out) {
    if (!s || !counts || !configs || !out || n_scenes == 0) return fail(FGB_ERR_INVALID, "batch_create: bad argument");
    fgb_batch *b = new fgb_batch();
    b->solver = s;
    b->n_scenes = n_scenes;
    b->counts.assign(counts, counts + n_scenes);
    b->cfg.assign(configs, configs + n_scenes);
    int rc = batch_init(b);
    if (rc != FGB_OK) {
        delete b;
        return rc;
    }
    s->batches.push_back(b);
    handle_add(b);
    *out = b;
    return FGB_OK;
}

int fgb_batch_destroy(fgb_batch *b) {
    if (!b) return FGB_OK;
    if (!handle_live(b)) return fail(FGB_ERR_INVALID, "batch_destroy: not a live batch (its solver was destroyed?)");
    cudaStreamSynchronize(b->stream());
    destroy_batch(b);
    return FGB_OK;
}

int fgb_batch_upload(fgb_batch *b, uint32_t scene, const fgb_particles *xs) {
    if (!b) return fail(FGB_ERR_INVALID, "upload: null batch");
    return batch_upload(b, scene, xs);
}

int fgb_batch_set_colliders(fgb_batch *b, uint32_t scene, const fgb_triangle *tris, size_t n) {
    if (!b || scene >= b->n_scenes || (n && !tris)) return fail(FGB_ERR_INVALID, "set_colliders: bad argument");
    std::vector<TriDev> t(n);
    for (size_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            t[i].a[a] = tris[i].a[a];
            t[i].b[a] = tris[i].b[a];
            t[i].c[a] = tris[i].c[a];
        }
    std::vector<TriDev> &old = b->scene_tris[scene];
    if (old.size() == t.size() && (t.empty() || memcmp(old.data(), t.data(), t.size() * sizeof(TriDev)) == 0))
        return FGB_OK;
    old.swap(t);
    b->tris_dirty = true;
    return FGB_OK;
}

int fgb_batch_step(fgb_batch *b, uint32_t steps) {
    if (!b) return fail(FGB_ERR_INVALID, "step: null batch");
    if (b->n == 0) return FGB_OK;
    // flags raised by steps that have finished (copied by their graphs): the state is
    // suspect, so nothing more is queued until fgb_batch_error_flags clears them
    int rc = flags_status(b->st_flags.p[0], "step");
    if (rc) return rc;
    return b->step(steps);
}

int fgb_batch_download(fgb_batch *b, uint32_t scene, fgb_particles *xs) {
    if (!b) return fail(FGB_ERR_INVALID, "download: null batch");
    return batch_download(b, scene, xs);
}

int fgb_batch_surface(fgb_batch *b, uint32_t scene, fgb_mesh *mesh_out) {
    if (!b || scene >= b->n_scenes) return fail(FGB_ERR_INVALID, "surface: bad argument");
    if (b->h_scenes[scene].lat[0] < 2) {
        if (mesh_out) mesh_out->n = 0;
        return FGB_OK;
    }
    uint64_t t = 0;
    int rc = b->surface_count(scene, scene + 1, &t);
    if (rc) return rc;
    rc = b->surface_emit(t);
    if (rc) return rc;
    rc = mesh_assign(mesh_out, b->tris_out.p, t, b->stream());
    uint32_t f = 0;
    if (!rc) rc = batch_flags_now(b, &f);
    return rc ? rc : flags_status(f, "surface");
}

int fgb_batch_surface_all(fgb_batch *b, uint64_t *counts) {
    if (!b) return fail(FGB_ERR_INVALID, "surface_all: null batch");
    uint64_t t = 0;
    int rc = b->surface_count(0, b->n_scenes, &t);
    if (rc) return rc;
    rc = b->surface_emit(t);
    if (rc) return rc;
    // per-scene triangle ranges: offsets at each scene's first cube, gathered on the
    // device and copied in one piece
    std::vector<uint32_t> firsts(b->n_scenes);
    b->surf_tri_first.assign(b->n_scenes + 1, 0);
    cudaStream_t st = b->stream();
    if (b->scene_firsts.n < b->n_scenes || !b->scene_firsts.p) {
        PoolScope scope(&b->solver->pool);
        FGB_CUDA(b->scene_firsts.alloc(b->n_scenes), "surface_all: alloc");
    }
    k_scene_first_triangles<<<(b->n_scenes + 255) / 256, 256, 0, st>>>(b->d_scenes.p, b->n_scenes, b->offsets.p,
                                                                       b->cube_total, (uint32_t)t, b->scene_firsts.p);
    FGB_CUDA(cudaGetLastError(), "surface_all: offsets");
    FGB_CUDA(cudaMemcpyAsync(firsts.data(), b->scene_firsts.p, b->n_scenes * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                             st),
             "surface_all: offsets");
    FGB_CUDA(cudaStreamSynchronize(st), "surface_all: sync");
    uint32_t f = 0;
    rc = batch_flags_now(b, &f);
    if (!rc) rc = flags_status(f, "surface_all");
    if (rc) return rc;
    for (uint32_t k = 0; k < b->n_scenes; ++k) b->surf_tri_first[k] = firsts[k];
    b->surf_tri_first[b->n_scenes] = t;
    for (uint32_t k = 0; k < b->n_scenes; ++k)
        if (counts) counts[k] = b->surf_tri_first[k + 1] - b->surf_tri_first[k];
    return FGB_OK;
}

extern "C++" {
namespace fgb {
int batch_resident(fgb_batch *b, uint32_t k, ResidentScene *out) {
    if (!b || !out || k >= b->n_scenes) return fail(FGB_ERR_INVALID, "resident scene: bad argument");
    int rc = sync_ids(b);
    if (rc) return rc;
    const int c = b->cur;
    out->first = b->first[k];
    out->n = b->counts[k];
    out->x = b->x[c].p;
    out->v = b->v[c].p;
    out->type = b->type[c].p;
    out->col = b->col[c].p;
    out->slot = b->slot[c].p;
    out->ids = b->ids_dev.p;
    out->stream = b->stream();
    out->tris = nullptr;
    out->tri_count = 0;
    if (b->surf_tri_first.size() == b->n_scenes + 1) {
        out->tris = b->tris_out.p + b->surf_tri_first[k];
        out->tri_count = b->surf_tri_first[k + 1] - b->surf_tri_first[k];
    }
    return FGB_OK;
}

void *batch_wire_scratch(fgb_batch *b, uint64_t bytes) {
    PoolScope scope(&b->solver->pool);
    if (b->wire.n < bytes && b->wire.alloc(bytes) != cudaSuccess) return nullptr;
    return b->wire.p;
}
}  // namespace fgb
}  // extern "C++"

int fgb_batch_surface_fetch(fgb_batch *b, uint32_t scene, fgb_mesh *mesh_out) {
    if (!b || scene >= b->n_scenes || b->surf_tri_first.size() != b->n_scenes + 1)
        return fail(FGB_ERR_INVALID, "surface_fetch: call fgb_batch_surface_all first");
    const uint64_t f = b->surf_tri_first[scene], e = b->surf_tri_first[scene + 1];
    return mesh_assign(mesh_out, b->tris_out.p + f, e - f, b->stream());
}

int fgb_batch_sync(fgb_batch *b) {
    if (!b) return fail(FGB_ERR_INVALID, "sync: null batch");
    FGB_CUDA(cudaStreamSynchronize(b->stream()), "sync");
    return flags_status(b->st_flags.p[0], "sync");  // as of the last step's end
}

int fgb_batch_prepare(fgb_batch *b) {
    if (!b) return fail(FGB_ERR_INVALID, "prepare: null batch");
    return b->prepare();
}

int fgb_batch_host_io(const fgb_batch *b, int *direct) {
    if (!b || !direct) return fail(FGB_ERR_INVALID, "host_io: bad argument");
    *direct = b->direct ? 1 : 0;
    return FGB_OK;
}

int fgb_batch_error_flags(fgb_batch *b, uint32_t *flags) {
    if (!b || !flags) return fail(FGB_ERR_INVALID, "error_flags: bad argument");
    cudaStream_t st = b->stream();
    FGB_CUDA(cudaMemcpyAsync(flags, b->err.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st), "error_flags");
    FGB_CUDA(cudaMemsetAsync(b->err.p, 0, sizeof(uint32_t), st), "error_flags");
    FGB_CUDA(cudaStreamSynchronize(st), "error_flags");
    b->st_flags.p[0] = 0;
    return FGB_OK;
}

int fgb_batch_row_stats(fgb_batch *b, uint32_t *stats, uint32_t n) {
    if (!b || (n && !stats)) return fail(FGB_ERR_INVALID, "row_stats: bad argument");
    for (uint32_t k = 0; k < n; ++k) stats[k] = 0;
    if (!b->row_stats || !b->over.p) return FGB_OK;
    uint32_t h[4] = {0, 0, 0, 0};
    cudaStream_t st = b->stream();
    FGB_CUDA(cudaMemcpyAsync(h, b->over.p + 2, sizeof(h), cudaMemcpyDeviceToHost, st), "row_stats");
    FGB_CUDA(cudaMemsetAsync(b->over.p + 2, 0, sizeof(h), st), "row_stats");
    FGB_CUDA(cudaStreamSynchronize(st), "row_stats");
    for (uint32_t k = 0; k < n && k < 4; ++k) stats[k] = h[k];
    return FGB_OK;
}

uint64_t fgb_batch_launch_count(const fgb_batch *b) { return b ? b->launches : 0; }

int fgb_batch_autotune(fgb_batch *b, uint32_t steps_per_trial, fgb_tune_result *out) {
    if (!b) return fail(FGB_ERR_INVALID, "autotune: null batch");
    if (b->n == 0) return FGB_OK;
    return b->autotune(steps_per_trial, out);
}

int fgb_batch_set_timing(fgb_batch *b, int on) {
    if (!b) return fail(FGB_ERR_INVALID, "set_timing: null batch");
    return b->set_timing(on != 0);
}

int fgb_batch_stage_times(fgb_batch *b, float *ms, uint32_t max, uint32_t *count) {
    if (!b || !count) return fail(FGB_ERR_INVALID, "stage_times: bad argument");
    if (!b->timing || b->n_stages == 0) return fail(FGB_ERR_INVALID, "stage_times: timing is off or no step ran");
    FGB_CUDA(cudaStreamSynchronize(b->stream()), "stage_times: sync");
    *count = b->n_stages;
    for (uint32_t i = 0; i < b->n_stages && i < max; ++i)
        FGB_CUDA(cudaEventElapsedTime(&ms[i], b->events[i], b->events[i + 1]), "stage_times");
    return FGB_OK;
}

int fgb_batch_probe_size(fgb_batch *b, uint32_t what, uint64_t *bytes) {
    if (!b || !bytes) return fail(FGB_ERR_INVALID, "probe: bad argument");
    const uint64_t n = b->n;
    switch (what) {
    case FGB_PROBE_KEYS:
    case FGB_PROBE_ORDER:
    case FGB_PROBE_LAMBDA:
    case FGB_PROBE_DENSITY: *bytes = n * 4; break;
    case FGB_PROBE_CELLS: *bytes = b->cells_n * 8; break;
    case FGB_PROBE_LATTICE: *bytes = b->lat_total * 16; break;
    case FGB_PROBE_CUBE_CASES: *bytes = b->cube_total; break;
    case FGB_PROBE_LIST_COUNT: *bytes = n * 2; break;
    case FGB_PROBE_LIST_VALID: *bytes = n; break;
    case FGB_PROBE_DISPLACEMENT: *bytes = n * 4; break;
    case FGB_PROBE_NEAR_ROW: *bytes = n; break;
    default: return fail(FGB_ERR_INVALID, "probe: unknown array");
    }
    return FGB_OK;
}

int fgb_batch_probe(fgb_batch *b, uint32_t what, void *host_out, uint64_t bytes) {
    uint64_t want = 0;
    int rc = fgb_batch_probe_size(b, what, &want);
    if (rc) return rc;
    if (bytes != want || (!host_out && bytes)) return fail(FGB_ERR_INVALID, "probe: wrong size");
    const void *src = nullptr;
    switch (what) {
    case FGB_PROBE_KEYS: src = b->keys_sorted.p; break;
    case FGB_PROBE_ORDER: src = b->slot[b->cur].p; break;
    case FGB_PROBE_LAMBDA: src = b->lambda.p; break;
    case FGB_PROBE_DENSITY: src = b->density.p; break;
    case FGB_PROBE_CELLS: src = b->cells.p; break;
    case FGB_PROBE_LATTICE: src = b->lattice.p; break;
    case FGB_PROBE_CUBE_CASES: src = b->cases.p; break;
    case FGB_PROBE_LIST_COUNT: src = b->ncount.p; break;
    case FGB_PROBE_LIST_VALID: src = b->valid.p; break;
    case FGB_PROBE_DISPLACEMENT: src = b->disp.p; break;
    case FGB_PROBE_NEAR_ROW: src = b->near.p; break;
    }
    if (!src) return fail(FGB_ERR_INVALID, "probe: array not allocated yet");
    cudaStream_t st = b->stream();
    if (bytes) FGB_CUDA(cudaMemcpyAsync(host_out, src, bytes, cudaMemcpyDeviceToHost, st), "probe");
    FGB_CUDA(cudaStreamSynchronize(st), "probe");
    return FGB_OK;
}

extern "C++" {
uint32_t fgb::scene_morton_bits(const fgb_solver *s, const fgb_config *cfg) {
    SceneDev S{};
    scene_geometry(s->params, *cfg, S);
    return 3 * bits_for(std::max(S.ext[0], std::max(S.ext[1], S.ext[2])));
}
}

int fgb_batch_copy_scene(fgb_batch *dst, uint32_t dst_scene, fgb_batch *src, uint32_t src_scene) {
    if (!dst || !src) return fail(FGB_ERR_INVALID, "copy_scene: null batch");
    if (dst->solver != src->solver) return fail(FGB_ERR_INVALID, "copy_scene: batches of different solvers");
    return batch_copy_scene(dst, dst_scene, src, src_scene);
}

int fgb_batch_sources_drains(fgb_batch *b, uint32_t k, const fgb_source *sources, uint32_t n_sources,
                             const fgb_drain *drains, uint32_t n_drains, uint64_t *count) {
    if (!b || !count || k >= b->n_scenes) return fail(FGB_ERR_INVALID, "sources_drains: bad argument");
    if ((n_sources && !sources) || (n_drains && !drains)) return fail(FGB_ERR_INVALID, "sources_drains: null array");
    const fgb_config &c = b->cfg[k];
    PoolScope scope(&b->solver->pool);
    b->query_ok = false;
    // emission (oclsph.hpp:678-691), with the drain test of 694-705 applied to the
    // new particles right away, as the reference erases after emitting
    const float spacing = (b->solver->params.h * c.scale / 2);
    auto drained = [&](const float *pos) {
        for (uint32_t d = 0; d < n_drains; ++d) {
            const float dx = drains[d].centre[0] - pos[0], dy = drains[d].centre[1] - pos[1],
                        dz = drains[d].centre[2] - pos[2];
            if (std::sqrt(dx * dx + dy * dy + dz * dz) < drains[d].width) return true;
        }
        return false;
    };
    std::vector<float4> ex, ev;
    std::vector<uint64_t> eid;
    std::vector<uint32_t> ecol;
    for (uint32_t q = 0; q < n_sources; ++q) {
        const fgb_source &src = sources[q];
        const float size = (float)std::sqrt((double)src.rate);
        const int width = (int)std::floor(size), depth = (int)std::ceil(size);
        const float off[3] = {src.centre[0] - ((float)width / 2.f) * spacing, src.centre[1] - (0.f / 2.f) * spacing,
                              src.centre[2] - ((float)depth / 2.f) * spacing};
        for (int x = 0; x < width; ++x)
            for (int z = 0; z < depth; ++z) {
                const float pos[3] = {off[0] + (float)x * spacing, off[1] + 0.f * spacing, off[2] + (float)z * spacing};
                if (drained(pos)) continue;
                ex.push_back(make_float4(pos[0], pos[1], pos[2], 1.f));
                ev.push_back(make_float4(src.velocity[0], src.velocity[1], src.velocity[2], 0.f));
                eid.push_back(src.tag);
                ecol.push_back(src.colour);
            }
    }
    const uint64_t E = ex.size(), n0 = b->n;
    cudaStream_t st = b->stream();
    int rc0 = sync_ids(b);
    if (rc0) return rc0;
    FGB_CUDA(cudaStreamSynchronize(st), "sources_drains sync");
    // survivors: drain flags, their exclusive scan
    Dev<uint32_t> keep, rank, total;
    Dev<char> scratch;
    Dev<fgb_drain> d_drains;
    Dev<SceneMove> d_moves;
    const uint64_t sb = scan_u32_scratch_bytes(n0);
    FGB_CUDA(keep.alloc(n0), "sources_drains alloc");
    FGB_CUDA(rank.alloc(n0), "sources_drains alloc");
    FGB_CUDA(total.alloc(1), "sources_drains alloc");
    FGB_CUDA(scratch.alloc(sb), "sources_drains alloc");
    FGB_CUDA(d_drains.alloc(std::max<uint32_t>(n_drains, 1)), "sources_drains alloc");
    FGB_CUDA(d_moves.alloc(b->n_scenes), "sources_drains alloc");
    if (n_drains)
        FGB_CUDA(cudaMemcpyAsync(d_drains.p, drains, n_drains * sizeof(fgb_drain), cudaMemcpyHostToDevice, st),
                 "sources_drains drains");
    const int cs = b->cur, cn = cs ^ 1;
    launch_drain_flags(n0, b->mbits, k, b->keys_sorted.p, b->x[cs].p, b->type[cs].p, d_drains.p, n_drains, keep.p, st);
    uint32_t kept_all = 0;
    if (n0) {
        cudaError_t e = scan_u32(keep.p, rank.p, total.p, n0, scratch.p, sb, st, b->err.p, nullptr);
        if (e != cudaSuccess) return fail_cuda(e, "sources_drains scan");
        FGB_CUDA(cudaMemcpyAsync(&kept_all, total.p, sizeof kept_all, cudaMemcpyDeviceToHost, st), "sources_drains");
        FGB_CUDA(cudaStreamSynchronize(st), "sources_drains sync");
    }
    const uint64_t kept_k = kept_all - (n0 - b->counts[k]);
    // the new layout
    std::vector<uint64_t> counts = b->counts, first(b->n_scenes);
    counts[k] = kept_k + E;
    std::vector<SceneMove> moves(b->n_scenes);
    uint64_t n1 = 0;
    for (uint32_t s = 0; s < b->n_scenes; ++s) {
        first[s] = n1;
        moves[s] = SceneMove{b->first[s], n1};
        n1 += counts[s];
    }
    if (n1 > 0x7fffffffull) return fail(FGB_ERR_CAPACITY, "sources_drains: more than 2^31-1 particles");
    const bool grow = n1 > b->capacity;
    const uint64_t cap = grow ? std::max<uint64_t>(n1, b->capacity + b->capacity / 4) : b->capacity;
    if (grow) {
        FGB_CUDA(b->x[cn].alloc(cap), "sources_drains grow");
        FGB_CUDA(b->v[cn].alloc(cap), "sources_drains grow");
        FGB_CUDA(b->type[cn].alloc(cap), "sources_drains grow");
        FGB_CUDA(b->col[cn].alloc(cap), "sources_drains grow");
        FGB_CUDA(b->slot[cn].alloc(cap), "sources_drains grow");
    }
    Dev<uint64_t> ids1;
    FGB_CUDA(ids1.alloc(cap), "sources_drains alloc");
    FGB_CUDA(cudaMemcpyAsync(d_moves.p, moves.data(), b->n_scenes * sizeof(SceneMove), cudaMemcpyHostToDevice, st),
             "sources_drains moves");
    launch_edit_scatter(n0, b->mbits, k, E, b->keys_sorted.p, keep.p, rank.p, d_moves.p, b->x[cs].p, b->v[cs].p,
                        b->type[cs].p, b->col[cs].p, b->slot[cs].p, b->ids_dev.p, b->x[cn].p, b->v[cn].p,
                        b->type[cn].p, b->col[cn].p, b->slot[cn].p, ids1.p, st);
    FGB_CUDA(cudaGetLastError(), "sources_drains scatter");
    if (E) {  // the emitted particles, after the scene's survivors
        FGB_CUDA(b->st_x.ensure(E), "sources_drains staging");
        FGB_CUDA(b->st_v.ensure(E), "sources_drains staging");
        FGB_CUDA(b->st_type.ensure(E), "sources_drains staging");
        FGB_CUDA(b->st_col.ensure(E), "sources_drains staging");
        FGB_CUDA(b->st_slot.ensure(E), "sources_drains staging");
        FGB_CUDA(b->st_ids.ensure(E), "sources_drains staging");
        for (uint64_t e = 0; e < E; ++e) {
            b->st_x.p[e] = ex[e];
            b->st_v.p[e] = ev[e];
            b->st_type.p[e] = FGB_TYPE_FLUID;
            b->st_col.p[e] = ecol[e];
            b->st_slot.p[e] = (uint32_t)(kept_k + e);
            b->st_ids.p[e] = eid[e];
        }
        const uint64_t d = first[k] + kept_k;
        FGB_CUDA(cudaMemcpyAsync(b->x[cn].p + d, b->st_x.p, E * sizeof(float4), cudaMemcpyHostToDevice, st), "emit");
        FGB_CUDA(cudaMemcpyAsync(b->v[cn].p + d, b->st_v.p, E * sizeof(float4), cudaMemcpyHostToDevice, st), "emit");
        FGB_CUDA(cudaMemcpyAsync(b->type[cn].p + d, b->st_type.p, E * sizeof(int32_t), cudaMemcpyHostToDevice, st),
                 "emit");
        FGB_CUDA(cudaMemcpyAsync(b->col[cn].p + d, b->st_col.p, E * sizeof(uint32_t), cudaMemcpyHostToDevice, st),
                 "emit");
        FGB_CUDA(cudaMemcpyAsync(b->slot[cn].p + d, b->st_slot.p, E * sizeof(uint32_t), cudaMemcpyHostToDevice, st),
                 "emit");
        FGB_CUDA(cudaMemcpyAsync(ids1.p + d, b->st_ids.p, E * sizeof(uint64_t), cudaMemcpyHostToDevice, st), "emit");
    }
    FGB_CUDA(cudaStreamSynchronize(st), "sources_drains sync");
    if (grow) {  // the old set and the per-step arrays, at the new capacity
        FGB_CUDA(b->x[cs].alloc(cap), "sources_drains grow");
        FGB_CUDA(b->v[cs].alloc(cap), "sources_drains grow");
        FGB_CUDA(b->type[cs].alloc(cap), "sources_drains grow");
        FGB_CUDA(b->col[cs].alloc(cap), "sources_drains grow");
        FGB_CUDA(b->slot[cs].alloc(cap), "sources_drains grow");
        int rc = alloc_step_arrays(b, cap);
        if (rc) return rc;
    }
    b->ids_dev.swap(ids1);
    b->cur = cn;
    b->counts = counts;
    b->first = first;
    b->n = n1;
    for (uint32_t s = 0; s < b->n_scenes; ++s) {
        b->h_scenes[s].first = (uint32_t)first[s];
        b->h_scenes[s].count = (uint32_t)counts[s];
        // every scene's key prefix for the next step's scene lookup
        launch_fill_u32(b->keys_sorted.p + first[s], counts[s], b->mbits >= 32 ? 0u : (s << b->mbits), st);
    }
    b->tris_dirty = true;   // re-uploads the scene table
    b->surf_ready = false;  // surface buffers are sized by the particle count
    b->surf_tri_first.clear();
    for (auto &g : b->graph)
        if (g) cudaGraphExecDestroy(g), g = nullptr;
    b->graphs_ok = false;
    // the scene's ids by its new slots, for staged downloads
    b->ids[k].assign(b->direct ? 0 : counts[k], 0);
    if (counts[k] && !b->direct)
        FGB_CUDA(cudaMemcpyAsync(b->ids[k].data(), b->ids_dev.p + first[k], counts[k] * sizeof(uint64_t),
                                 cudaMemcpyDeviceToHost, st),
                 "sources_drains ids");
    FGB_CUDA(cudaStreamSynchronize(st), "sources_drains sync");
    *count = counts[k];
    return FGB_OK;
}

int fgb_scene_footprint(const fgb_solver *s, const fgb_config *cfg, uint64_t n, int want_mesh, uint64_t *bytes) {
    if (!s || !cfg || !bytes) return fail(FGB_ERR_INVALID, "footprint: bad argument");
    uint32_t cap = 96, hits = 64;
    if (const char *e = getenv("FGB_LIST_CAP")) cap = (uint32_t)atoi(e);
    if (const char *e = getenv("FGB_HIT_CAP")) hits = (uint32_t)atoi(e);
    *bytes = scene_footprint(s->params, *cfg, n, want_mesh != 0, cap + hits);
    return FGB_OK;
}

int fgb_batch_grid_info(fgb_batch *b, uint32_t scene, fgb_grid_info *out) {
    if (!b || !out || scene >= b->n_scenes) return fail(FGB_ERR_INVALID, "grid_info: bad argument");
    const SceneDev &S = b->h_scenes[scene];
    for (int a = 0; a < 3; ++a) {
        out->min_extent[a] = S.min_ext[a];
        out->extent[a] = S.ext[a];
        out->lattice[a] = S.lat[a];
        out->lattice_origin[a] = S.lat_origin[a];
    }
    out->table_offset = S.table_base;
    out->table_size = (uint64_t)morton3(S.ext[0], S.ext[1], S.ext[2]) + 1;
    out->morton_bits = b->mbits;
    out->scene_bits = b->sbits;
    out->lattice_step = S.lat_step;
    return FGB_OK;
}

// Cell queries of scene k against the grid of the batch's last step (query.cu); the
// results of points whose cell holds fluid, in query order.  Synchronous.
static int batch_query(fgb_batch *b, uint32_t k, const fgb_query *q, size_t nq, fgb_query_result *out,
                       size_t *n_out) {
    *n_out = 0;
    if (!nq) return FGB_OK;
    if (!b->query_ok)
        return fail(FGB_ERR_INVALID, "query: the cell table is not a step's grid (no step since the last upload, "
                                     "edit or surface)");
    if (nq > 0xffffffffull) return fail(FGB_ERR_CAPACITY, "query: more than 2^32-1 queries");
    cudaStream_t st = b->stream();
    if (b->q_dev.n < nq || !b->q_dev.p) {
        PoolScope scope(&b->solver->pool);
        FGB_CUDA(b->q_dev.alloc(nq), "query alloc");
        FGB_CUDA(b->q_out.alloc(2 * nq), "query alloc");
    }
    FGB_CUDA(cudaMemcpyAsync(b->q_dev.p, q, nq * sizeof(fgb_query), cudaMemcpyHostToDevice, st), "query upload");
    const int cur = b->cur;
    // the sorted types of the step, and the colours it started from (before its
    // diffusion) through the sort's order
    launch_queries(b->d_scenes.p, k, b->ph.h, b->cells.p, b->type[cur].p, b->vals_sorted.p, b->col[cur ^ 1].p,
                   b->q_dev.p, (uint32_t)nq, b->q_out.p, b->q_out.p + nq, st);
    FGB_CUDA(cudaGetLastError(), "query kernel");
    std::vector<uint32_t> res(2 * nq);
    FGB_CUDA(cudaMemcpyAsync(res.data(), b->q_out.p, 2 * nq * sizeof(uint32_t), cudaMemcpyDeviceToHost, st),
             "query download");
    FGB_CUDA(cudaStreamSynchronize(st), "query sync");
    size_t m = 0;
    for (size_t i = 0; i < nq; ++i) {
        if (!res[i]) continue;  // oclsph.hpp:789: only points whose cell holds fluid
        fgb_query_result &r = out[m++];
        r.id = q[i].id;
        for (int a = 0; a < 3; ++a) r.point[a] = q[i].point[a];
        r.neighbours = res[i];
        r.average_colour = res[nq + i];
    }
    *n_out = m;
    return FGB_OK;
}

// fgb_advance with direct host I/O: one frame with a single wait at its end.  The
// upload and the download are split by when the step needs (or finishes) each field:
//   main stream: positions, velocities, masses, types in (obstacles counted into the
//                scene table) -> step, whose last kernel also stores the final
//                positions and velocities into the caller's arrays -> [surface]
//   io_stream:   colours, ids, slots in (the step's reorder waits for them) ->
//                after the grid is built: types, colours, ids, masses out
// The frame's device error flags (raised by its step) as its status.
static int advance_flags(fgb_batch *b) { return flags_status(b->st_flags.p[0], "advance"); }

static int advance_direct(fgb_batch *b, const fgb_config *cfg, fgb_particles *xs, fgb_mesh *mesh_out) {
    const uint64_t n = xs->n;
    if (!xs->position || !xs->velocity || !xs->mass || !xs->type)
        return fail(FGB_ERR_INVALID, "advance: null particle array");
    int rc = b->sync_tris();  // the scene table before the upload counts obstacles into it
    if (rc) return rc;
    cudaStream_t st = b->stream(), io = b->io_stream;
    const int c = b->cur, next = c ^ 1;
    uint32_t *obstacles = &b->d_scenes.p[0].obstacles;
    const HostParticlesIn in{xs->position, xs->velocity, xs->mass, xs->type, xs->colour, xs->id};
    // the arrays are inputs and outputs: their pages are readied, contents kept, before
    // any kernel of the frame reads or stores into them
    ready_pages({{xs->position, 12 * n}, {xs->velocity, 12 * n}, {xs->mass, 4 * n}, {xs->type, 4 * n},
                 {xs->colour, 4 * n}, {xs->id, 8 * n}},
                true);
    FGB_CUDA(cudaMemsetAsync(obstacles, 0, sizeof(uint32_t), st), "advance: upload");
    launch_pack_motion(in, n, b->x[c].p, b->v[c].p, b->type[c].p, obstacles, st);
    FGB_CUDA(cudaGetLastError(), "advance: upload kernel");
    // the rest follows on io_stream once the link is free, beside the prediction and
    // the sort
    FGB_CUDA(cudaEventRecord(b->io_done, st), "advance: upload event");
    FGB_CUDA(cudaStreamWaitEvent(io, b->io_done, 0), "advance: upload event");
    launch_pack_static(in, n, b->col[c].p, b->slot[c].p, b->ids_dev.p, io);
    FGB_CUDA(cudaGetLastError(), "advance: upload kernel");
    FGB_CUDA(cudaEventRecord(b->io_up, io), "advance: upload event");
    launch_fill_u32(b->keys_sorted.p, n, 0u, st);  // scene 0's key prefix for the prediction
    b->ids[0].clear();
    b->ids_stale[0] = 0;
    // the step's last kernel stores positions and velocities into the caller's arrays
    b->st_hout.p[0] = HostParticlesOut{xs->position, xs->velocity, nullptr, nullptr, nullptr, nullptr};
    FGB_CUDA(cudaMemcpyAsync(b->hout_dev.p, b->st_hout.p, sizeof(HostParticlesOut), cudaMemcpyHostToDevice, st),
             "advance: output arrays");
    rc = b->step(1);
    if (rc) return rc;
    // io_stream writes the fields that are final once the grid is built
    const HostParticlesOut fixed{nullptr, nullptr, xs->mass, xs->type, xs->colour, xs->id};
    FGB_CUDA(cudaStreamWaitEvent(io, b->grid_ready, 0), "advance: io wait");
    launch_unpack_static(fixed, n, b->ps_grid.p, b->type[next].p, b->col[next].p, b->slot[next].p, b->ids_dev.p, io);
    FGB_CUDA(cudaGetLastError(), "advance: download kernel");
    FGB_CUDA(cudaEventRecord(b->io_done, io), "advance: io event");
    if (cfg->surface && mesh_out) {
        rc = fgb_batch_surface(b, 0, mesh_out);
        if (rc) return rc;
    }
    FGB_CUDA(cudaMemcpyAsync(b->st_count.p, obstacles, sizeof(uint32_t), cudaMemcpyDeviceToHost, st),
             "advance: obstacle count");
    FGB_CUDA(cudaStreamWaitEvent(st, b->io_done, 0), "advance: io join");
    FGB_CUDA(cudaStreamSynchronize(st), "advance: sync");
    b->h_scenes[0].obstacles = b->st_count.p[0];  // the device table has it already
    return advance_flags(b);
}

// The solver's single-scene batch for a frame of n particles under cfg, created when
// the count or the configuration changed, with the frame's colliders and cleared
// error flags.
static int frame_batch(fgb_solver *s, const fgb_config *cfg, uint64_t n, const fgb_triangle *colliders,
                       size_t n_colliders, fgb_batch **out) {
    // `surface` only says whether this frame also extracts a surface: it does not
    // change the resident scene, so frames that differ in it reuse the same batch
    fgb_config key = *cfg;
    key.surface = s->cached_cfg.surface;
    const bool same = s->cached && s->cached_n == n && memcmp(&s->cached_cfg, &key, sizeof(fgb_config)) == 0;
    if (!same) {
        if (s->cached) destroy_batch(s->cached);
        s->cached = nullptr;
        int rc = fgb_batch_create(s, 1, &n, cfg, &s->cached);
        if (rc) return rc;
        s->cached_n = n;
        s->cached_cfg = *cfg;
        fgb_batch *nb = s->cached;
        if (nb->direct) {  // before the first step captures the graphs
            PoolScope scope(&s->pool);
            FGB_CUDA(nb->hout_dev.alloc(1), "advance alloc");
            FGB_CUDA(nb->st_hout.ensure(1), "advance alloc");
            FGB_CUDA(cudaMemsetAsync(nb->hout_dev.p, 0, sizeof(HostParticlesOut), nb->stream()), "advance alloc");
            nb->advance_io = true;
        }
    }
    fgb_batch *b = s->cached;
    int rc = fgb_batch_set_colliders(b, 0, colliders, n_colliders);
    if (rc) return rc;
    // a frame's flags are its own: the particles are uploaded afresh every frame (the
    // previous frame has finished, so the pinned copy is not being written)
    b->st_flags.p[0] = 0;
    FGB_CUDA(cudaMemsetAsync(b->err.p, 0, sizeof(uint32_t), b->stream()), "advance: error flags");
    *out = b;
    return FGB_OK;
}

int fgb_advance(fgb_solver *s, const fgb_config *cfg, fgb_particles *xs, const fgb_triangle *colliders,
                size_t n_colliders, fgb_mesh *mesh_out) {
    if (!s || !cfg || !xs) return fail(FGB_ERR_INVALID, "advance: null argument");
    if (n_colliders && !colliders) return fail(FGB_ERR_INVALID, "advance: null colliders");
    if (mesh_out) mesh_out->n = 0;
    if (xs->n == 0) return FGB_OK;  // oclsph.hpp:711-715 returns an empty result
    fgb_batch *b = nullptr;
    int rc = frame_batch(s, cfg, xs->n, colliders, n_colliders, &b);
    if (rc) return rc;
    if (b->advance_io && b->io_stream) return advance_direct(b, cfg, xs, mesh_out);
    rc = batch_upload(b, 0, xs);
    if (rc) return rc;
    rc = b->step(1);
    if (rc) return rc;
    if (cfg->surface && mesh_out) {
        rc = fgb_batch_surface(b, 0, mesh_out);
        if (rc) return rc;
    }
    rc = batch_download(b, 0, xs);
    return rc ? rc : advance_flags(b);
}

// fgb_advance_records with direct host I/O: one kernel reads the caller's records
// before the step (a tile of records staged in shared memory), the step's last
// kernel stores the final positions and velocities into them, and io_stream writes
// type, colour, id and mass once the grid is built, while the gathers run.  The
// queries are answered between the step and the surface, while the cell table is
// the step's grid.
static int advance_records_direct(fgb_batch *b, const fgb_config *cfg, const HostRecords &r, uint64_t n,
                                  const fgb_query *queries, size_t n_queries, fgb_query_result *results,
                                  size_t *n_results, fgb_mesh *mesh_out) {
    int rc = b->sync_tris();  // the scene table before the upload counts obstacles into it
    if (rc) return rc;
    cudaStream_t st = b->stream();
    const int c = b->cur, next = c ^ 1;
    uint32_t *obstacles = &b->d_scenes.p[0].obstacles;
    // the records are inputs and outputs: their pages are readied, contents kept,
    // before any kernel of the frame reads or stores into them
    ready_pages({{r.base, n * r.stride}}, true);
    FGB_CUDA(cudaMemsetAsync(obstacles, 0, sizeof(uint32_t), st), "advance: upload");
    launch_pack_records(r, n, b->x[c].p, b->v[c].p, b->type[c].p, b->col[c].p, b->slot[c].p, b->ids_dev.p, obstacles,
                        st);
    FGB_CUDA(cudaGetLastError(), "advance: upload kernel");
    FGB_CUDA(cudaEventRecord(b->io_up, st), "advance: upload event");  // every field is in
    launch_fill_u32(b->keys_sorted.p, n, 0u, st);  // scene 0's key prefix for the prediction
    b->ids[0].clear();
    b->ids_stale[0] = 0;
    b->query_ok = false;
    // no field stores from the step's last kernel: the records go back whole below
    b->st_hout.p[0] = record_fields(r, false, false);
    FGB_CUDA(cudaMemcpyAsync(b->hout_dev.p, b->st_hout.p, sizeof(HostParticlesOut), cudaMemcpyHostToDevice, st),
             "advance: output records");
    rc = b->step(1);
    if (rc) return rc;
    launch_unpack_records(r, n, b->x[next].p, b->v[next].p, b->type[next].p, b->col[next].p, b->slot[next].p,
                          b->ids_dev.p, st);
    FGB_CUDA(cudaGetLastError(), "advance: download kernel");
    if (n_queries) {
        rc = batch_query(b, 0, queries, n_queries, results, n_results);
        if (rc) return rc;
    }
    if (cfg->surface && mesh_out) {
        rc = fgb_batch_surface(b, 0, mesh_out);
        if (rc) return rc;
    }
    FGB_CUDA(cudaMemcpyAsync(b->st_count.p, obstacles, sizeof(uint32_t), cudaMemcpyDeviceToHost, st),
             "advance: obstacle count");
    FGB_CUDA(cudaStreamSynchronize(st), "advance: sync");
    b->h_scenes[0].obstacles = b->st_count.p[0];  // the device table has it already
    return advance_flags(b);
}

int fgb_advance_records(fgb_solver *s, const fgb_config *cfg, fgb_records *xs, const fgb_triangle *colliders,
                        size_t n_colliders, const fgb_query *queries, size_t n_queries, fgb_query_result *results,
                        size_t *n_results, fgb_mesh *mesh_out) {
    if (!s || !cfg || !xs) return fail(FGB_ERR_INVALID, "advance_records: null argument");
    if (n_colliders && !colliders) return fail(FGB_ERR_INVALID, "advance_records: null colliders");
    if (n_queries && (!queries || !results || !n_results))
        return fail(FGB_ERR_INVALID, "advance_records: queries need results and n_results");
    if (n_results) *n_results = 0;
    if (mesh_out) mesh_out->n = 0;
    const uint32_t st = xs->stride;
    auto field_ok = [&](int32_t off, uint32_t bytes, bool required) {
        if (off < 0) return !required;
        return (off % 4) == 0 && (uint64_t)off + bytes <= st;
    };
    if (st == 0 || st % 4 || st > kMaxRecordStride || ((uintptr_t)xs->base % 4) ||
        (xs->id_bytes != 4 && xs->id_bytes != 8) || !field_ok(xs->position, 12, true) ||
        !field_ok(xs->velocity, 12, true) || !field_ok(xs->mass, 4, true) || !field_ok(xs->type, 4, true) ||
        !field_ok(xs->colour, 4, false) || !field_ok(xs->id, xs->id_bytes, false))
        return fail(FGB_ERR_INVALID, "advance_records: the record layout must have a stride of at most 128 bytes, "
                                     "4-byte aligned fields within it, and position, velocity, mass and type");
    if (xs->n && !xs->base) return fail(FGB_ERR_INVALID, "advance_records: null records");
    if (xs->n == 0) return FGB_OK;  // oclsph.hpp:711-715 returns an empty result
    fgb_batch *b = nullptr;
    int rc = frame_batch(s, cfg, xs->n, colliders, n_colliders, &b);
    if (rc) return rc;
    const HostRecords r{(char *)xs->base, st, xs->id_bytes, xs->id, xs->type, xs->mass, xs->position, xs->velocity,
                        xs->colour};
    const uint64_t n = xs->n;
    if (b->advance_io && b->io_stream)
        return advance_records_direct(b, cfg, r, n, queries, n_queries, results, n_results, mesh_out);
    // staged: the records to and from packed arrays on the host threads, around the
    // packed-array frame
    std::vector<uint64_t> id(n);
    std::vector<int32_t> type(n);
    std::vector<float> mass(n), pos(3 * n), vel(3 * n);
    std::vector<uint32_t> col(n);
    auto word = [&](uint64_t i, int32_t off) { return (const void *)(r.base + i * st + off); };
    parallel_for(n, [&](uint64_t lo, uint64_t hi) {
        for (uint64_t i = lo; i < hi; ++i) {
            memcpy(&pos[3 * i], word(i, r.off_position), 12);
            memcpy(&vel[3 * i], word(i, r.off_velocity), 12);
            memcpy(&mass[i], word(i, r.off_mass), 4);
            memcpy(&type[i], word(i, r.off_type), 4);
            col[i] = 0xffffffffu;
            if (r.off_colour >= 0) memcpy(&col[i], word(i, r.off_colour), 4);
            id[i] = i;
            if (r.off_id >= 0) {
                if (r.id_bytes == 8) {
                    memcpy(&id[i], word(i, r.off_id), 8);
                } else {
                    uint32_t v;
                    memcpy(&v, word(i, r.off_id), 4);
                    id[i] = v;
                }
            }
        }
    });
    fgb_particles p{n, id.data(), type.data(), mass.data(), pos.data(), vel.data(), col.data()};
    rc = batch_upload(b, 0, &p);
    if (!rc) rc = b->step(1);
    if (!rc && n_queries) rc = batch_query(b, 0, queries, n_queries, results, n_results);
    if (!rc && cfg->surface && mesh_out) rc = fgb_batch_surface(b, 0, mesh_out);
    if (!rc) rc = batch_download(b, 0, &p);
    if (rc) return rc;
    parallel_for(n, [&](uint64_t lo, uint64_t hi) {
        for (uint64_t i = lo; i < hi; ++i) {
            char *rec = r.base + i * st;
            memset(rec, 0, st);  // whole records, as the direct path writes them
            memcpy(rec + r.off_position, &pos[3 * i], 12);
            memcpy(rec + r.off_velocity, &vel[3 * i], 12);
            memcpy(rec + r.off_mass, &mass[i], 4);
            memcpy(rec + r.off_type, &type[i], 4);
            if (r.off_colour >= 0) memcpy(rec + r.off_colour, &col[i], 4);
            if (r.off_id >= 0) {
                if (r.id_bytes == 8) {
                    memcpy(rec + r.off_id, &id[i], 8);
                } else {
                    const uint32_t v = (uint32_t)id[i];
                    memcpy(rec + r.off_id, &v, 4);
                }
            }
        }
    });
    return advance_flags(b);
}

int fgb_batch_query(fgb_batch *b, uint32_t scene, const fgb_query *queries, size_t n, fgb_query_result *results,
                    size_t *n_results) {
    if (!b || !n_results || scene >= b->n_scenes || (n && (!queries || !results)))
        return fail(FGB_ERR_INVALID, "query: bad argument");
    return batch_query(b, scene, queries, n, results, n_results);
}

int fgb_host_ready_pages(void *p, size_t bytes, int keep_contents, uint64_t *touched) {
    if (bytes && !p) return fail(FGB_ERR_INVALID, "ready_pages: null pointer");
    const int t = ready_pages({{p, bytes}}, keep_contents != 0);
    if (touched) *touched = (uint64_t)t;
    return FGB_OK;
}

void fgb_mesh_free(fgb_mesh *m) {
    if (!m) return;
    free(m->triangles);
    m->triangles = nullptr;
    m->n = 0;
    m->capacity = 0;
}

}  // extern "C"
