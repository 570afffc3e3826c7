// cudasph.hpp -- cuda::SphSolver, the drop-in for libfluid's ocl::SphSolver
// (tom91136/libfluid include/fluid/oclsph.hpp:150-939) behind the unchanged
// interface fluid::SphSolver<size_t, float>::advance (include/fluid/fluid.hpp:222-232).
//
// Include libfluid's own fluid.hpp (with GLM) or, without GLM, the source-compatible
// "fluid_gb300/compat/fluid.hpp" first; then this header; link libfluidgb.so.
//
// What stays on the host, as in the reference's advance: sources and drains
// (oclsph.hpp:675-708), which resize the vector.  Everything else -- the particles'
// upload and write-back (read and written in place in the vector), prediction, the
// Morton grid, the constraint iterations, the velocity update, the cell queries
// (oclsph.hpp:770-791) and marching cubes -- runs on the GPU through the C ABI in
// fluid_gb300.h.  Failures
// throw std::runtime_error carrying the library's message, as the reference throws.
#ifndef FLUID_GB300_CUDASPH_HPP
#define FLUID_GB300_CUDASPH_HPP

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <vector>

#include "../fluid_gb300.h"

namespace cuda {

class SphSolver : public fluid::SphSolver<size_t, float> {
public:
    // h is fixed per solver as in ocl::SphSolver(h, kernelPath, device); the profile
    // selects the reference's constants (FGB_PROFILE_REF, the default) or the
    // baseline PBF (FGB_PROFILE_BASELINE).
    explicit SphSolver(float h, int profile = FGB_PROFILE_REF) {
        fgb_params p;
        fgb_params_default(&p, profile, h);
        init(p);
    }
    explicit SphSolver(const fgb_params &params) { init(params); }
    ~SphSolver() override { fgb_destroy(solver_); }
    SphSolver(const SphSolver &) = delete;
    SphSolver &operator=(const SphSolver &) = delete;

    fgb_solver *handle() const { return solver_; }

    // An analytic static sphere collider (world units) for the frames that follow;
    // radius <= 0 removes it.  No counterpart in fluid::Config, whose colliders are
    // triangle meshes: the benchmark's 1M dam break has a sphere.
    void sphere(float cx, float cy, float cz, float radius) {
        sphere_[0] = cx;
        sphere_[1] = cy;
        sphere_[2] = cz;
        sphere_[3] = radius;
    }

    fluid::Result<float> advance(const fluid::Config<float> &config, std::vector<fluid::Particle<size_t, float>> &xs,
                                 const std::vector<fluid::MeshCollider<float>> &colliders) override {
        emit_sources(config, xs);
        apply_drains(config, xs);
        if (xs.empty()) return fluid::Result<float>({}, {});  // oclsph.hpp:711-715

        // the particles are read and written where they lie: the library addresses the
        // vector's records through their field offsets (no copy into separate arrays)
        using P = fluid::Particle<size_t, float>;
        static_assert(sizeof(fluid::Type) == 4, "fluid::Type must be a 4-byte enum");
        static_assert(sizeof(P) % 4 == 0 && sizeof(P) <= 128, "fluid::Particle layout");
        fgb_records view;
        view.base = xs.data();
        view.n = xs.size();
        view.stride = (uint32_t)sizeof(P);
        view.id_bytes = (uint32_t)sizeof(size_t);
        view.id = (int32_t)offsetof(P, id);
        view.type = (int32_t)offsetof(P, type);
        view.mass = (int32_t)offsetof(P, mass);
        view.position = (int32_t)offsetof(P, position);
        view.velocity = (int32_t)offsetof(P, velocity);
        view.colour = (int32_t)offsetof(P, colour);

        fgb_config c;
        fgb_config_default(&c, FGB_PROFILE_REF);
        c.dt = config.dt;
        c.scale = config.scale;
        c.resolution = config.resolution;
        c.isolevel = config.isolevel;
        c.iterations = (uint32_t)config.iteration;
        c.surface = config.resolution > 0.f ? 1u : 0u;  // the reference always extracts a surface
        c.constant_force[0] = config.constantForce.x;
        c.constant_force[1] = config.constantForce.y;
        c.constant_force[2] = config.constantForce.z;
        c.min_bound[0] = config.minBound.x;
        c.min_bound[1] = config.minBound.y;
        c.min_bound[2] = config.minBound.z;
        c.max_bound[0] = config.maxBound.x;
        c.max_bound[1] = config.maxBound.y;
        c.max_bound[2] = config.maxBound.z;
        c.sphere_enabled = sphere_[3] > 0.f ? 1 : 0;
        for (int a = 0; a < 4; ++a) c.sphere[a] = sphere_[a];
        if (config.wells.size() > FGB_MAX_WELLS) throw std::runtime_error("libfluidgb: more than 16 wells");
        c.n_wells = (uint32_t)config.wells.size();
        for (size_t w = 0; w < config.wells.size(); ++w) {
            c.wells[w].centre[0] = config.wells[w].centre.x;
            c.wells[w].centre[1] = config.wells[w].centre.y;
            c.wells[w].centre[2] = config.wells[w].centre.z;
            c.wells[w].force = config.wells[w].force;
        }
        tris_.clear();
        for (const auto &m : colliders)
            for (const auto &t : m.triangles)
                tris_.push_back(fgb_triangle{{t.v0.x, t.v0.y, t.v0.z}, {t.v1.x, t.v1.y, t.v1.z}, {t.v2.x, t.v2.y, t.v2.z}});

        // queries of the frame (oclsph.hpp:770-791), answered on the device from the
        // step's grid
        queries_.resize(config.queries.size());
        for (size_t q = 0; q < config.queries.size(); ++q) {
            queries_[q].id = (uint64_t)config.queries[q].id;
            queries_[q].point[0] = config.queries[q].point.x;
            queries_[q].point[1] = config.queries[q].point.y;
            queries_[q].point[2] = config.queries[q].point.z;
        }
        results_.resize(queries_.size());
        size_t n_results = 0;
        fgb_mesh mesh{nullptr, 0, 0};
        // the library writes the particles back in Morton order (oclsph.hpp:875-891)
        int rc = fgb_advance_records(solver_, &c, &view, tris_.empty() ? nullptr : tris_.data(), tris_.size(),
                                     queries_.empty() ? nullptr : queries_.data(), queries_.size(),
                                     results_.empty() ? nullptr : results_.data(), &n_results, &mesh);
        if (rc != FGB_OK) {
            fgb_mesh_free(&mesh);
            throw std::runtime_error(std::string("libfluidgb: ") + fgb_last_error());
        }
        std::vector<fluid::QueryResult<float>> query_results;
        query_results.reserve(n_results);
        for (size_t q = 0; q < n_results; ++q) {
            const fgb_query_result &r = results_[q];
            query_results.emplace_back((size_t)r.id, fluid::tvec3<float>(r.point[0], r.point[1], r.point[2]),
                                       (size_t)r.neighbours, r.average_colour);
        }
        std::vector<geometry::MeshTriangle<float>> triangles(mesh.n);
        for (size_t t = 0; t < mesh.n; ++t) {
            const fgb_mesh_triangle &m = mesh.triangles[t];
            auto &o = triangles[t];
            o.v0 = fluid::tvec3<float>(m.v[0], m.v[1], m.v[2]);
            o.v1 = fluid::tvec3<float>(m.v[3], m.v[4], m.v[5]);
            o.v2 = fluid::tvec3<float>(m.v[6], m.v[7], m.v[8]);
            o.n0 = fluid::tvec3<float>(m.n[0], m.n[1], m.n[2]);
            o.n1 = fluid::tvec3<float>(m.n[3], m.n[4], m.n[5]);
            o.n2 = fluid::tvec3<float>(m.n[6], m.n[7], m.n[8]);
            o.c.x = m.c[0];
            o.c.y = m.c[1];
            o.c.z = m.c[2];
        }
        fgb_mesh_free(&mesh);
        return fluid::Result<float>(triangles, query_results);
    }

private:
    fgb_solver *solver_ = nullptr;
    float h_ = 0.1f;
    float sphere_[4] = {0.f, 0.f, 0.f, 0.f};
    std::vector<fgb_triangle> tris_;
    std::vector<fgb_query> queries_;
    std::vector<fgb_query_result> results_;

    void init(const fgb_params &p) {
        h_ = p.h;
        if (fgb_create(&p, &solver_) != FGB_OK) throw std::runtime_error(std::string("libfluidgb: ") + fgb_last_error());
    }

    // oclsph.hpp:678-691: a sqrt(rate) x sqrt(rate) sheet of particles, spacing h*scale/2
    void emit_sources(const fluid::Config<float> &config, std::vector<fluid::Particle<size_t, float>> &xs) const {
        const float spacing = (h_ * config.scale / 2);
        for (const auto &source : config.sources) {
            const float size = std::sqrt((float)source.rate);
            const int width = (int)std::floor(size);
            const int depth = (int)std::ceil(size);
            const auto offset = source.centre - (fluid::tvec3<float>((float)width, 0.f, (float)depth) / 2.f * spacing);
            for (int x = 0; x < width; ++x)
                for (int z = 0; z < depth; ++z) {
                    const auto pos = offset + fluid::tvec3<float>((float)x, 0.f, (float)z) * spacing;
                    xs.emplace_back(source.tag, fluid::Type::Fluid, 1.f, source.colour, pos, source.velocity);
                }
        }
    }

    // oclsph.hpp:693-706: drains erase fluid particles within `width` of their centre
    static void apply_drains(const fluid::Config<float> &config, std::vector<fluid::Particle<size_t, float>> &xs) {
        if (config.drains.empty()) return;
        xs.erase(std::remove_if(xs.begin(), xs.end(),
                                [&config](const fluid::Particle<size_t, float> &x) {
                                    if (x.type == fluid::Type::Obstacle) return false;
                                    for (const auto &d : config.drains)
                                        if (glm::distance(d.centre, x.position) < d.width) return true;
                                    return false;
                                }),
                 xs.end());
    }
};

}  // namespace cuda

#endif  // FLUID_GB300_CUDASPH_HPP
