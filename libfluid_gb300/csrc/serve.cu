// serve.cu -- resident serving loop with continuous batching.
//
// Requests (a scene, a step count, optionally a final surface) arrive at any time.
// A worker thread admits waiting requests in arrival order while their device
// footprint fits the HBM budget and keeps every admitted scene resident on the
// device.  Admitted scenes are spread over groups of at most tick_particles
// particles; one tick advances one group (one launch per stage for all its scenes,
// fgb_batch_step), taking the groups round robin: by one step, or by several when the
// group is small (tick_steps).  A tick's latency is linear in its particle-steps
// (~0.3 ms + 3.2 ns a particle-step on GB300), so the groups are
// kept as few and as even as the scenes allow: a new scene joins the lightest group
// it fits, and whenever the largest group holds more than 1.5x the smallest (or more
// than ceil(total / tick_particles) groups exist) the scenes are re-spread largest
// first onto the lightest group (LPT); a group that ends up with the same scenes keeps
// its batch.  When a group's membership changes,
// its scenes are copied device-to-device into a new batch from wherever they live
// (fgb_batch_copy_scene keeps their particle order, so a scene's result is
// bit-identical alone and in any mix).  Finished scenes optionally run marching
// cubes, their final state is copied to the host, and their memory is released.
//
// Budget accounting: rebuilding a group holds its old and new batch at once, so
// admission keeps the sum of active footprints within half the budget.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "fgb_internal.h"

namespace {

using fgb::fail;

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

uint32_t bits_of(uint32_t v) {
    uint32_t b = 0;
    while ((1u << b) <= v && b < 31) ++b;
    return b;
}

struct Request {
    uint64_t ticket = 0;
    fgb_config cfg{};
    uint32_t steps = 0, remaining = 0;
    bool want_mesh = false;
    uint64_t n = 0, footprint = 0;
    uint32_t mbits = 0;
    std::vector<uint64_t> id;
    std::vector<int32_t> type;
    std::vector<float> mass, pos, vel;
    std::vector<uint32_t> col;
    double t_submit = 0, t_admit = -1, t_done = -1;
    int32_t status = FGB_SERVE_WAITING;
    uint64_t triangles = 0;
    fgb_mesh mesh{nullptr, 0, 0};

    fgb_particles view() {
        return fgb_particles{n, id.data(), type.data(), mass.data(), pos.data(), vel.data(), col.data()};
    }
    ~Request() { fgb_mesh_free(&mesh); }
};

}  // namespace

// Scenes that are stepped together: one batch (one launch per stage for all of
// them).  A group holds at most tick_particles particles (a larger scene is a group
// on its own), so every tick does about the same amount of work whatever the mix of
// active requests -- the step latency stays flat while requests come and go.
struct ServeGroup {
    fgb_batch *batch = nullptr;
    std::vector<Request *> scenes;  // scene k of `batch` is scenes[k]
    std::vector<Request *> want;    // membership for the next tick
    uint64_t particles = 0;         // of `want`
    uint32_t mbits = 0;             // largest Morton key width in `want`
};

struct fgb_server {
    fgb_solver *solver = nullptr;
    fgb_serve_options opt{};
    int device = 0;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Request *> waiting;                       // admitted in arrival order
    std::vector<Request *> live;                         // admitted and still running
    std::map<uint64_t, std::unique_ptr<Request>> requests;
    uint64_t used = 0, next_ticket = 1;
    bool stop = false;
    double t0 = 0;
    // worker-only state
    std::vector<std::unique_ptr<ServeGroup>> groups;
    size_t next_group = 0;  // round-robin position
    double spread = 1.5;    // largest group / smallest group kept without re-spreading
    std::thread worker;
    // statistics (under mu)
    uint64_t ticks = 0, particle_steps = 0, completed = 0, rejected = 0, failed = 0, rebuilds = 0;
    double busy = 0, rebuild_time = 0;
    std::vector<double> step_latency;
    std::vector<uint64_t> step_particles;  // particles of each tick, beside step_latency
    std::vector<uint32_t> step_scenes;     // scenes (requests) stepped by each tick
    std::vector<uint32_t> step_count;      // steps each tick advanced its group by
    std::vector<double> step_start;        // start of each tick, seconds since creation
    std::string last_error;

    double t() const { return now_s() - t0; }

    // Admit waiting requests (mu held); returns the newly admitted ones.
    std::vector<Request *> admit() {
        const uint64_t cap_bytes = opt.budget_bytes / 2;
        std::vector<Request *> fresh;
        while (!waiting.empty()) {
            Request *r = waiting.front();
            if (r->footprint > cap_bytes) {  // could never fit
                waiting.pop_front();
                r->status = -FGB_ERR_BUDGET;
                r->t_done = t();
                rejected++;
                continue;
            }
            if (opt.one_at_a_time && !live.empty()) break;
            if (live.size() >= opt.max_active) break;
            if (used + r->footprint > cap_bytes) break;
            waiting.pop_front();
            used += r->footprint;
            r->status = FGB_SERVE_ACTIVE;
            r->t_admit = t();
            live.push_back(r);
            fresh.push_back(r);
        }
        return fresh;
    }

    // Whether r may join a group of `particles` particles, `count` scenes and Morton
    // width `mbits` (room in the tick, and scene-id bits above the Morton key).
    bool fits(uint64_t particles, size_t count, uint32_t mbits, const Request *r) const {
        if (!count) return true;
        if (opt.one_at_a_time) return false;
        if (particles + r->n > opt.tick_particles) return false;
        return std::max(mbits, r->mbits) + bits_of((uint32_t)count) <= 32;
    }

    // The lightest group with room for r, else a new group.
    void place(Request *r) {
        ServeGroup *best = nullptr;
        for (auto &g : groups)
            if (!g->want.empty() && fits(g->particles, g->want.size(), g->mbits, r) &&
                (!best || g->particles < best->particles))
                best = g.get();
        if (!best) {
            groups.push_back(std::make_unique<ServeGroup>());
            best = groups.back().get();
        }
        best->want.push_back(r);
        best->particles += r->n;
        best->mbits = std::max(best->mbits, r->mbits);
    }

    // Re-spread the scenes whenever the groups are uneven (see the top of the file);
    // a group whose scenes stay the same keeps its batch.
    void rebalance() {
        if (opt.one_at_a_time) return;
        std::vector<ServeGroup *> used;
        uint64_t total = 0, lo = ~0ull, hi = 0;
        for (auto &g : groups)
            if (!g->want.empty()) {
                used.push_back(g.get());
                total += g->particles;
                lo = std::min(lo, g->particles);
                hi = std::max(hi, g->particles);
            }
        if (used.size() < 2) return;
        const uint64_t need = (total + opt.tick_particles - 1) / opt.tick_particles;
        // groups as few as the particles need, and within `spread` of each other: keep
        // them (every change of membership is a rebuild)
        if (used.size() <= need && (double)hi <= spread * (double)lo) return;
        // LPT: largest scene first, onto the lightest group it fits
        std::vector<Request *> all;
        for (ServeGroup *g : used) all.insert(all.end(), g->want.begin(), g->want.end());
        std::sort(all.begin(), all.end(), [](const Request *a, const Request *b) {
            return a->n != b->n ? a->n > b->n : a->ticket < b->ticket;
        });
        struct Bin {
            std::vector<Request *> scenes;
            uint64_t particles = 0;
            uint32_t mbits = 0;
        };
        std::vector<Bin> bins(std::max<uint64_t>(need, 1));
        for (Request *r : all) {
            Bin *best = nullptr;
            for (Bin &b : bins)
                if (fits(b.particles, b.scenes.size(), b.mbits, r) && (!best || b.particles < best->particles))
                    best = &b;
            if (!best) {
                bins.emplace_back();
                best = &bins.back();
            }
            best->scenes.push_back(r);
            best->particles += r->n;
            best->mbits = std::max(best->mbits, r->mbits);
        }
        // each bin goes to the old group it shares the most particles with, so that
        // as many groups as possible keep their batch
        std::vector<bool> taken(used.size(), false);
        std::vector<ServeGroup *> owner(bins.size(), nullptr);
        for (size_t b = 0; b < bins.size(); ++b) {
            uint64_t best_shared = 0;
            for (size_t g = 0; g < used.size(); ++g) {
                if (taken[g]) continue;
                uint64_t shared = 0;
                for (Request *r : bins[b].scenes)
                    if (std::find(used[g]->want.begin(), used[g]->want.end(), r) != used[g]->want.end()) shared += r->n;
                if (shared > best_shared) best_shared = shared, owner[b] = used[g];
            }
            if (owner[b]) taken[std::find(used.begin(), used.end(), owner[b]) - used.begin()] = true;
        }
        for (size_t g = 0; g < used.size(); ++g)
            if (!taken[g]) {
                used[g]->want.clear();
                used[g]->particles = 0;
                used[g]->mbits = 0;
            }
        for (size_t b = 0; b < bins.size(); ++b) {
            ServeGroup *g = owner[b];
            if (!g) {
                groups.push_back(std::make_unique<ServeGroup>());
                g = groups.back().get();
            }
            // the same scenes in another order need no rebuild
            std::vector<Request *> a = bins[b].scenes, c = g->scenes;
            std::sort(a.begin(), a.end());
            std::sort(c.begin(), c.end());
            g->want = a == c ? g->scenes : bins[b].scenes;
            g->particles = bins[b].particles;
            g->mbits = bins[b].mbits;
        }
    }

    // Make g.batch hold exactly g.want; scenes already resident (in any group's
    // current batch, found through `where`) move on the device.  The old batch is
    // handed to `retired`: other groups' rebuilds may still copy from it.
    struct Home {
        fgb_batch *batch;
        uint32_t scene;
    };
    int rebuild(ServeGroup &g, const std::map<Request *, Home> &where, std::vector<fgb_batch *> &retired) {
        const double r0 = now_s();
        fgb_batch *nb = nullptr;
        if (!g.want.empty()) {
            std::vector<uint64_t> counts;
            std::vector<fgb_config> cfgs;
            for (Request *r : g.want) {
                counts.push_back(r->n);
                cfgs.push_back(r->cfg);
            }
            int rc = fgb_batch_create(solver, (uint32_t)g.want.size(), counts.data(), cfgs.data(), &nb);
            if (rc) return rc;
            for (size_t k = 0; k < g.want.size(); ++k) {
                Request *r = g.want[k];
                auto it = where.find(r);
                if (it != where.end()) {
                    rc = fgb_batch_copy_scene(nb, (uint32_t)k, it->second.batch, it->second.scene);
                } else {
                    fgb_particles v = r->view();
                    rc = fgb_batch_upload(nb, (uint32_t)k, &v);
                }
                if (rc) {
                    fgb_batch_destroy(nb);
                    return rc;
                }
            }
            // graph capture and the scene table belong to the rebuild, not the next tick
            int rc2 = fgb_batch_prepare(nb);
            if (rc2) {
                fgb_batch_destroy(nb);
                return rc2;
            }
        }
        if (g.batch) retired.push_back(g.batch);
        g.batch = nb;
        g.scenes = g.want;
        std::lock_guard<std::mutex> lk(mu);
        rebuilds++;
        rebuild_time += now_s() - r0;
        return FGB_OK;
    }

    // Fail every active scene of g and empty it.
    void fail_group(ServeGroup &g, int rc) {
        {
            std::lock_guard<std::mutex> lk(mu);
            last_error = fgb_last_error();
            for (Request *r : g.want) {
                if (r->status != FGB_SERVE_ACTIVE) continue;
                r->status = -rc;
                r->t_done = t();
                used -= r->footprint;
                failed++;
            }
            std::vector<Request *> keep;
            for (Request *r : live)
                if (r->status == FGB_SERVE_ACTIVE) keep.push_back(r);
            live.swap(keep);
            cv.notify_all();
        }
        if (g.batch) fgb_batch_destroy(g.batch);
        g.batch = nullptr;
        g.scenes.clear();
        g.want.clear();
        g.particles = 0;
    }

    // Steps of the next tick of g.  A tick costs about kTickFixed + n particles of
    // work (0.3 ms + 3.2 ns a particle on GB300, measured), so a group below half of
    // tick_particles takes k steps with k (n + kTickFixed) <= tick_particles +
    // kTickFixed: every tick then does between half and all of a full group's work,
    // and its latency stays within a factor of two whatever the load.  k never takes
    // a scene past its last step, and a tick that would leave a scene a remainder
    // shorter than k takes the remainder's share now (two even ticks, not a long one
    // and a short one).
    static constexpr uint64_t kTickFixed = 98304;
    uint32_t tick_steps(const ServeGroup &g) const {
        if (opt.one_at_a_time || opt.max_steps_per_tick <= 1) return 1;
        uint64_t n = 0;
        uint32_t rest = UINT32_MAX;
        for (const Request *r : g.scenes) {
            n += r->n;
            rest = std::min(rest, r->remaining);
        }
        uint64_t k = (opt.tick_particles + kTickFixed) / (n + kTickFixed);
        k = std::max<uint64_t>(1, std::min<uint64_t>(k, opt.max_steps_per_tick));
        if (k >= rest) return rest;
        if (rest < 2 * k) k = (rest + 1) / 2;
        return (uint32_t)k;
    }

    // One tick: step group g tick_steps(g) times; finished scenes run their surface
    // and go home.
    void tick(ServeGroup &g) {
        const uint32_t k = tick_steps(g);
        const double s0 = now_s();
        int rc = fgb_batch_step(g.batch, k);
        if (!rc) rc = fgb_batch_sync(g.batch);
        const double s1 = now_s();
        if (rc) return fail_group(g, rc);
        std::vector<Request *> done;
        for (size_t j = 0; j < g.scenes.size(); ++j) {
            Request *r = g.scenes[j];
            r->remaining -= k;
            if (r->remaining) continue;
            if (r->want_mesh) {
                rc = fgb_batch_surface(g.batch, (uint32_t)j, &r->mesh);
                if (rc) return fail_group(g, rc);
                r->triangles = r->mesh.n;
            }
            fgb_particles v = r->view();
            rc = fgb_batch_download(g.batch, (uint32_t)j, &v);
            if (rc) return fail_group(g, rc);
            done.push_back(r);
        }
        if (!done.empty()) {
            std::vector<Request *> keep;
            g.particles = 0;
            g.mbits = 0;
            for (Request *r : g.want)
                if (std::find(done.begin(), done.end(), r) == done.end()) {
                    keep.push_back(r);
                    g.particles += r->n;
                    g.mbits = std::max(g.mbits, r->mbits);
                }
            g.want.swap(keep);
        }
        std::lock_guard<std::mutex> lk(mu);
        step_latency.push_back(s1 - s0);
        step_start.push_back(s0 - t0);
        busy += s1 - s0;
        ticks++;
        uint64_t tick_n = 0;
        for (Request *r : g.scenes) tick_n += r->n;
        particle_steps += tick_n * k;
        step_particles.push_back(tick_n);
        step_scenes.push_back((uint32_t)g.scenes.size());
        step_count.push_back(k);
        for (Request *r : done) {
            r->status = FGB_SERVE_DONE;
            r->t_done = t();
            used -= r->footprint;
            completed++;
        }
        if (!done.empty()) {
            std::vector<Request *> keep;
            for (Request *r : live)
                if (r->status == FGB_SERVE_ACTIVE) keep.push_back(r);
            live.swap(keep);
        }
        cv.notify_all();
    }

    void run() {
        cudaSetDevice(device);
        for (;;) {
            std::vector<Request *> fresh;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return stop || !waiting.empty() || !live.empty(); });
                if (stop) break;
                fresh = admit();
            }
            for (Request *r : fresh) place(r);
            rebalance();
            // bring the changed groups up to date (scenes move between batches on the
            // device), then release the batches nothing uses any more
            std::map<Request *, Home> where;
            for (auto &g : groups)
                for (size_t k = 0; k < g->scenes.size(); ++k) where[g->scenes[k]] = Home{g->batch, (uint32_t)k};
            std::vector<fgb_batch *> retired;
            for (auto &g : groups)
                if (g->want != g->scenes) {
                    const int rc = rebuild(*g, where, retired);
                    if (rc) {
                        // the old batch may still hold scenes that other groups copy
                        if (g->batch) retired.push_back(g->batch);
                        g->batch = nullptr;
                        g->scenes.clear();
                        fail_group(*g, rc);
                    }
                }
            for (fgb_batch *b : retired) fgb_batch_destroy(b);
            std::vector<std::unique_ptr<ServeGroup>> kept;
            for (auto &g : groups)
                if (!g->want.empty()) kept.push_back(std::move(g));
            groups.swap(kept);
            // round robin over the groups that hold scenes
            ServeGroup *pick = nullptr;
            for (size_t i = 0; i < groups.size() && !pick; ++i) {
                ServeGroup *g = groups[(next_group + i) % groups.size()].get();
                if (g->batch && !g->scenes.empty()) {
                    pick = g;
                    next_group = (next_group + i + 1) % groups.size();
                }
            }
            if (pick) tick(*pick);
        }
        for (auto &g : groups)
            if (g->batch) fgb_batch_destroy(g->batch);
        groups.clear();
    }
};

extern "C" {

int fgb_serve_create(fgb_solver *s, const fgb_serve_options *opt, fgb_server **out) {
    if (!s || !out) return fail(FGB_ERR_INVALID, "serve_create: null argument");
    fgb_server *sv = new fgb_server();
    sv->solver = s;
    if (opt) sv->opt = *opt;
    if (!sv->opt.budget_bytes) sv->opt.budget_bytes = 150ull << 30;
    if (!sv->opt.max_active) sv->opt.max_active = 256;
    if (!sv->opt.tick_particles) sv->opt.tick_particles = 2097152;
    if (!sv->opt.max_steps_per_tick) sv->opt.max_steps_per_tick = 16;
    if (const char *e = getenv("FGB_SERVE_SPREAD")) sv->spread = std::max(1.0, atof(e));
    cudaGetDevice(&sv->device);
    sv->t0 = now_s();
    sv->worker = std::thread([sv] { sv->run(); });
    *out = sv;
    return FGB_OK;
}

int fgb_serve_submit(fgb_server *sv, const fgb_config *cfg, const fgb_particles *xs, uint32_t steps,
                     int want_mesh, uint64_t *ticket) {
    if (!sv || !cfg || !xs || !ticket) return fail(FGB_ERR_INVALID, "serve_submit: null argument");
    if (steps == 0) return fail(FGB_ERR_INVALID, "serve_submit: steps must be >= 1");
    if (xs->n == 0 || !xs->position || !xs->velocity || !xs->mass || !xs->type)
        return fail(FGB_ERR_INVALID, "serve_submit: empty or incomplete particle arrays");
    auto r = std::make_unique<Request>();
    r->cfg = *cfg;
    r->steps = r->remaining = steps;
    r->want_mesh = want_mesh != 0;
    r->n = xs->n;
    int rc = fgb_scene_footprint(sv->solver, cfg, xs->n, want_mesh, &r->footprint);
    if (rc) return rc;
    // Morton bits of the scene's grid: admission keeps scene id + key within 32 bits
    r->mbits = fgb::scene_morton_bits(sv->solver, cfg);
    r->id.assign(xs->n, 0);
    r->type.assign(xs->type, xs->type + xs->n);
    r->mass.assign(xs->mass, xs->mass + xs->n);
    r->pos.assign(xs->position, xs->position + 3 * xs->n);
    r->vel.assign(xs->velocity, xs->velocity + 3 * xs->n);
    r->col.assign(xs->n, 0xffffffffu);
    for (uint64_t i = 0; i < xs->n; ++i) {
        r->id[i] = xs->id ? xs->id[i] : i;
        if (xs->colour) r->col[i] = xs->colour[i];
    }
    std::lock_guard<std::mutex> lk(sv->mu);
    r->ticket = sv->next_ticket++;
    r->t_submit = sv->t();
    *ticket = r->ticket;
    sv->waiting.push_back(r.get());
    sv->requests[r->ticket] = std::move(r);
    sv->cv.notify_all();
    return FGB_OK;
}

int fgb_serve_poll(fgb_server *sv, uint64_t ticket, fgb_serve_result *out) {
    if (!sv || !out) return fail(FGB_ERR_INVALID, "serve_poll: null argument");
    std::lock_guard<std::mutex> lk(sv->mu);
    auto it = sv->requests.find(ticket);
    if (it == sv->requests.end()) return fail(FGB_ERR_INVALID, "serve_poll: unknown ticket");
    const Request &r = *it->second;
    out->ticket = r.ticket;
    out->n = r.n;
    out->steps = r.steps;
    out->status = r.status;
    out->triangles = r.triangles;
    out->t_submit = r.t_submit;
    out->t_admit = r.t_admit;
    out->t_done = r.t_done;
    return FGB_OK;
}

int fgb_serve_fetch(fgb_server *sv, uint64_t ticket, fgb_particles *xs, fgb_mesh *mesh) {
    if (!sv) return fail(FGB_ERR_INVALID, "serve_fetch: null server");
    std::unique_ptr<Request> r;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        auto it = sv->requests.find(ticket);
        if (it == sv->requests.end()) return fail(FGB_ERR_INVALID, "serve_fetch: unknown ticket");
        const int32_t st = it->second->status;
        if (st == FGB_SERVE_WAITING || st == FGB_SERVE_ACTIVE) return fail(FGB_ERR_INVALID, "serve_fetch: not done");
        r = std::move(it->second);
        sv->requests.erase(it);
    }
    if (r->status != FGB_SERVE_DONE) return fail(-r->status, "serve_fetch: request failed or was rejected");
    if (xs) {
        if (xs->n != r->n) return fail(FGB_ERR_INVALID, "serve_fetch: particle count differs");
        if (xs->id) memcpy(xs->id, r->id.data(), r->n * sizeof(uint64_t));
        if (xs->type) memcpy(xs->type, r->type.data(), r->n * sizeof(int32_t));
        if (xs->mass) memcpy(xs->mass, r->mass.data(), r->n * sizeof(float));
        if (xs->position) memcpy(xs->position, r->pos.data(), 3 * r->n * sizeof(float));
        if (xs->velocity) memcpy(xs->velocity, r->vel.data(), 3 * r->n * sizeof(float));
        if (xs->colour) memcpy(xs->colour, r->col.data(), r->n * sizeof(uint32_t));
    }
    if (mesh) {
        fgb_mesh_free(mesh);
        *mesh = r->mesh;  // ownership moves to the caller
        r->mesh = fgb_mesh{nullptr, 0, 0};
    }
    return FGB_OK;
}

int fgb_serve_get_stats(fgb_server *sv, fgb_serve_stats *out) {
    if (!sv || !out) return fail(FGB_ERR_INVALID, "serve_stats: null argument");
    std::lock_guard<std::mutex> lk(sv->mu);
    out->ticks = sv->ticks;
    out->particle_steps = sv->particle_steps;
    out->completed = sv->completed;
    out->rejected = sv->rejected;
    out->failed = sv->failed;
    out->active = sv->live.size();
    out->waiting = sv->waiting.size();
    out->used_bytes = sv->used;
    out->budget_bytes = sv->opt.budget_bytes;
    out->rebuilds = sv->rebuilds;
    out->busy_seconds = sv->busy;
    out->rebuild_seconds = sv->rebuild_time;
    out->elapsed_seconds = sv->t();
    return FGB_OK;
}

int fgb_serve_step_latencies(fgb_server *sv, double *out, uint64_t max, uint64_t *count) {
    if (!sv || !count) return fail(FGB_ERR_INVALID, "serve_step_latencies: null argument");
    std::lock_guard<std::mutex> lk(sv->mu);
    *count = sv->step_latency.size();
    for (uint64_t i = 0; out && i < max && i < sv->step_latency.size(); ++i) out[i] = sv->step_latency[i];
    return FGB_OK;
}

int fgb_serve_tick_scenes(fgb_server *sv, uint32_t *out, uint64_t max, uint64_t *count) {
    if (!sv || !count) return fail(FGB_ERR_INVALID, "serve_tick_scenes: null argument");
    std::lock_guard<std::mutex> lk(sv->mu);
    *count = sv->step_scenes.size();
    for (uint64_t i = 0; out && i < max && i < sv->step_scenes.size(); ++i) out[i] = sv->step_scenes[i];
    return FGB_OK;
}

int fgb_serve_tick_steps(fgb_server *sv, uint32_t *out, uint64_t max, uint64_t *count) {
    if (!sv || !count) return fail(FGB_ERR_INVALID, "serve_tick_steps: null argument");
    std::lock_guard<std::mutex> lk(sv->mu);
    *count = sv->step_count.size();
    for (uint64_t i = 0; out && i < max && i < sv->step_count.size(); ++i) out[i] = sv->step_count[i];
    return FGB_OK;
}

int fgb_serve_tick_particles(fgb_server *sv, uint64_t *out, uint64_t max, uint64_t *count) {
    if (!sv || !count) return fail(FGB_ERR_INVALID, "serve_tick_particles: null argument");
    std::lock_guard<std::mutex> lk(sv->mu);
    *count = sv->step_particles.size();
    for (uint64_t i = 0; out && i < max && i < sv->step_particles.size(); ++i) out[i] = sv->step_particles[i];
    return FGB_OK;
}

int fgb_serve_tick_starts(fgb_server *sv, double *out, uint64_t max, uint64_t *count) {
    if (!sv || !count) return fail(FGB_ERR_INVALID, "serve_tick_starts: null argument");
    std::lock_guard<std::mutex> lk(sv->mu);
    *count = sv->step_start.size();
    for (uint64_t i = 0; out && i < max && i < sv->step_start.size(); ++i) out[i] = sv->step_start[i];
    return FGB_OK;
}

int fgb_serve_drain(fgb_server *sv, double timeout_seconds) {
    if (!sv) return fail(FGB_ERR_INVALID, "serve_drain: null server");
    std::unique_lock<std::mutex> lk(sv->mu);
    const bool ok = sv->cv.wait_for(lk, std::chrono::duration<double>(timeout_seconds),
                                    [&] { return sv->waiting.empty() && sv->live.empty(); });
    if (!ok) return fail(FGB_ERR_TIMEOUT, "serve_drain: requests still pending at the timeout");
    return FGB_OK;
}

int fgb_serve_destroy(fgb_server *sv) {
    if (!sv) return FGB_OK;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
    }
    sv->cv.notify_all();
    if (sv->worker.joinable()) sv->worker.join();
    delete sv;
    return FGB_OK;
}

}  // extern "C"

