// Packs the same particles with cuda::wire (header-only, fluid types) and with the C
// ABI's fgb_wire_particles (SoA arrays), and triangles with both; exits 0 when the
// byte streams are identical.  Needs no GPU.
#include <cstdio>
#include <cstring>
#include <vector>

#include "fluid_gb300/wire.hpp"

int main() {
    std::vector<fluid::Particle<size_t, float>> xs;
    for (size_t i = 0; i < 50; ++i) {
        const float f = 0.25f * (float)i;
        xs.emplace_back(1000 + 7 * i, i % 3 ? fluid::Fluid : fluid::Obstacle, 0.5f + f, (uint32_t)(0xFF000000u + i),
                        glm::tvec3<float>(f, -f, 2 * f), glm::tvec3<float>(-f, 1.f, f * f));
    }
    std::vector<char> a(cuda::wire::particles_bytes(xs.size()));
    cuda::wire::writeParticles(a.data(), a.size(), xs, 42);

    std::vector<uint64_t> id;
    std::vector<int32_t> type;
    std::vector<float> mass, pos, vel;
    std::vector<uint32_t> col;
    for (const auto &p : xs) {
        id.push_back(p.id);
        type.push_back(p.type);
        mass.push_back(p.mass);
        col.push_back(p.colour);
        pos.insert(pos.end(), {p.position.x, p.position.y, p.position.z});
        vel.insert(vel.end(), {p.velocity.x, p.velocity.y, p.velocity.z});
    }
    fgb_particles v{xs.size(), id.data(), type.data(), mass.data(), pos.data(), vel.data(), col.data()};
    std::vector<char> b(a.size());
    uint64_t used = 0;
    if (fgb_wire_particles(&v, 42, b.data(), b.size(), &used) != FGB_OK || used != a.size()) return 2;
    if (std::memcmp(a.data(), b.data(), a.size()) != 0) return 3;

    std::vector<geometry::MeshTriangle<float>> ts;
    std::vector<fgb_mesh_triangle> raw;
    for (int i = 0; i < 9; ++i) {
        const float f = (float)i;
        geometry::MeshTriangle<float> t(glm::tvec3<float>(f, 1, 2), glm::tvec3<float>(3, f, 5),
                                        glm::tvec3<float>(6, 7, f), glm::tvec3<float>(0, 1, 0),
                                        glm::tvec3<float>(1, 0, 0), glm::tvec3<float>(0, 0, 1));
        t.c = glm::tvec3<uint32_t>(0xFF000000u + i, 2, 3);
        ts.push_back(t);
        fgb_mesh_triangle r;
        const float vv[9] = {f, 1, 2, 3, f, 5, 6, 7, f}, nn[9] = {0, 1, 0, 1, 0, 0, 0, 0, 1};
        std::memcpy(r.v, vv, sizeof vv);
        std::memcpy(r.n, nn, sizeof nn);
        r.c[0] = 0xFF000000u + i;
        r.c[1] = 2;
        r.c[2] = 3;
        raw.push_back(r);
    }
    std::vector<char> c(cuda::wire::triangles_bytes(ts.size())), d(c.size());
    cuda::wire::writeTriangles(c.data(), c.size(), ts, 9);
    fgb_mesh m{raw.data(), raw.size(), raw.size()};
    if (fgb_wire_triangles(&m, 9, d.data(), d.size(), &used) != FGB_OK || used != c.size()) return 4;
    if (std::memcmp(c.data(), d.data(), c.size()) != 0) return 5;

    std::vector<fluid::QueryResult<float>> qs{fluid::QueryResult<float>(5, glm::tvec3<float>(1, 2, 3), 12, 7u)};
    std::vector<char> q(cuda::wire::queries_bytes(1));
    if (cuda::wire::writeQueries(q.data(), q.size(), qs, 1) != 24 + 32) return 6;
    std::printf("ok %zu %zu %zu\n", a.size(), c.size(), q.size());
    return 0;
}
