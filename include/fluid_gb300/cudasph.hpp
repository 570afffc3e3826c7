// cudasph.hpp -- cuda::SphSolver, the drop-in for libfluid's ocl::SphSolver
// (tom91136/libfluid include/fluid/oclsph.hpp:150-939) behind the unchanged
// interface fluid::SphSolver<size_t, float>::advance (include/fluid/fluid.hpp:222-232).
//
// Include libfluid's own fluid.hpp (with GLM) or, without GLM, the source-compatible
// "fluid_gb300/compat/fluid.hpp" first; then this header; link libfluidgb.so.
//
// What stays on the host, as in the reference's advance: sources and drains
// (oclsph.hpp:675-708) and query results (oclsph.hpp:770-791).  Everything else --
// prediction, the Morton grid, the constraint iterations, the velocity update and
// marching cubes -- runs on the GPU through the C ABI in fluid_gb300.h.  Failures
// throw std::runtime_error carrying the library's message, as the reference throws.
#ifndef FLUID_GB300_CUDASPH_HPP
#define FLUID_GB300_CUDASPH_HPP

#include <algorithm>
#include <cmath>
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

    fluid::Result<float> advance(const fluid::Config<float> &config, std::vector<fluid::Particle<size_t, float>> &xs,
                                 const std::vector<fluid::MeshCollider<float>> &colliders) override {
        emit_sources(config, xs);
        apply_drains(config, xs);
        if (xs.empty()) return fluid::Result<float>({}, {});  // oclsph.hpp:711-715

        const size_t n = xs.size();
        id_.resize(n);
        type_.resize(n);
        mass_.resize(n);
        colour_.resize(n);
        pos_.resize(3 * n);
        vel_.resize(3 * n);
        for (size_t i = 0; i < n; ++i) {
            const auto &p = xs[i];
            id_[i] = (uint64_t)p.id;
            type_[i] = p.type == fluid::Type::Obstacle ? FGB_TYPE_OBSTACLE : FGB_TYPE_FLUID;
            mass_[i] = p.mass;
            colour_[i] = p.colour;
            pos_[3 * i] = p.position.x;
            pos_[3 * i + 1] = p.position.y;
            pos_[3 * i + 2] = p.position.z;
            vel_[3 * i] = p.velocity.x;
            vel_[3 * i + 1] = p.velocity.y;
            vel_[3 * i + 2] = p.velocity.z;
        }
        fgb_particles view{n, id_.data(), type_.data(), mass_.data(), pos_.data(), vel_.data(), colour_.data()};

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

        fgb_mesh mesh{nullptr, 0, 0};
        int rc = fgb_advance(solver_, &c, &view, tris_.empty() ? nullptr : tris_.data(), tris_.size(), &mesh);
        if (rc != FGB_OK) {
            fgb_mesh_free(&mesh);
            throw std::runtime_error(std::string("libfluidgb: ") + fgb_last_error());
        }
        // write-back in Morton order (oclsph.hpp:875-891)
        for (size_t i = 0; i < n; ++i) {
            auto &p = xs[i];
            p.id = (size_t)id_[i];
            p.type = type_[i] == FGB_TYPE_OBSTACLE ? fluid::Type::Obstacle : fluid::Type::Fluid;
            p.mass = mass_[i];
            p.colour = colour_[i];
            p.position = fluid::tvec3<float>(pos_[3 * i], pos_[3 * i + 1], pos_[3 * i + 2]);
            p.velocity = fluid::tvec3<float>(vel_[3 * i], vel_[3 * i + 1], vel_[3 * i + 2]);
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
        return fluid::Result<float>(triangles, queries(config, xs));
    }

private:
    fgb_solver *solver_ = nullptr;
    float h_ = 0.1f;
    std::vector<uint64_t> id_;
    std::vector<int32_t> type_;
    std::vector<float> mass_, pos_, vel_;
    std::vector<uint32_t> colour_;
    std::vector<fgb_triangle> tris_;

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

    // oclsph.hpp:770-791: fluid particles in the query point's grid cell and their
    // mean ARGB colour (here over the advanced positions)
    std::vector<fluid::QueryResult<float>> queries(const fluid::Config<float> &config,
                                                   const std::vector<fluid::Particle<size_t, float>> &xs) const {
        std::vector<fluid::QueryResult<float>> out;
        if (config.queries.empty()) return out;
        const float pad = h_ * 2.f;
        const float mn[3] = {config.minBound.x / config.scale - pad, config.minBound.y / config.scale - pad,
                             config.minBound.z / config.scale - pad};
        auto cell = [&](const fluid::tvec3<float> &p, long c[3]) {
            const float v[3] = {p.x / config.scale, p.y / config.scale, p.z / config.scale};
            for (int a = 0; a < 3; ++a) c[a] = (long)std::floor((v[a] - mn[a]) / h_);
        };
        for (const auto &q : config.queries) {
            long qc[3];
            cell(q.point, qc);
            size_t count = 0;
            double acc[4] = {0, 0, 0, 0};
            for (const auto &p : xs) {
                if (p.type != fluid::Type::Fluid) continue;
                long pc[3];
                cell(p.position, pc);
                if (pc[0] != qc[0] || pc[1] != qc[1] || pc[2] != qc[2]) continue;
                ++count;
                for (int ch = 0; ch < 4; ++ch) acc[ch] += (double)((p.colour >> (24 - 8 * ch)) & 0xffu);
            }
            if (!count) continue;
            uint32_t argb = 0;
            for (int ch = 0; ch < 4; ++ch) argb |= ((uint32_t)(acc[ch] / (double)count) & 0xffu) << (24 - 8 * ch);
            out.emplace_back(q.id, q.point, count, argb);
        }
        return out;
    }
};

}  // namespace cuda

#endif  // FLUID_GB300_CUDASPH_HPP
