// C ABI of the scene builders and of the C++ drop-in solvers (include/spgx_scenes.h).
#include <memory>
#include <tuple>

#include "../../csrc/api_internal.h"
#include "spg/scenes.h"
#include "spg/sim/solver/gpuSolvers.h"
#include "spgx_scenes.h"

struct spgx_scene {
    std::vector<spg::ParticleGroup> groups;
    spg::gpu::PackedScene packed;
};

namespace {

spgx_status finish(std::unique_ptr<spgx_scene> s, spgx_scene **out)
{
    spg::gpu::pack(s->groups, s->packed);
    *out = s.release();
    return SPGX_OK;
}

// Copies loaded mesh arrays and checks the anchor list.
template <class Cell>
bool meshInputs(const double *vertices, int32_t n_vertices, const int32_t *cells, int32_t n_cells, int32_t n_anchors,
                const int32_t *anchors, std::vector<spg::Vector3> &V, std::vector<Cell> &C, std::vector<int> &ids)
{
    constexpr int K = static_cast<int>(std::tuple_size<Cell>::value);
    if (n_vertices < 1 || n_cells < 1 || !vertices || !cells || n_anchors < 0 || (n_anchors > 0 && !anchors)) {
        spgx::set_error("invalid mesh arguments");
        return false;
    }
    V.resize(size_t(n_vertices));
    for (int i = 0; i < n_vertices; ++i) V[i] = {vertices[3 * i], vertices[3 * i + 1], vertices[3 * i + 2]};
    C.resize(size_t(n_cells));
    for (int c = 0; c < n_cells; ++c)
        for (int k = 0; k < K; ++k) C[c][k] = cells[size_t(c) * K + k];
    ids.assign(anchors, anchors + n_anchors);
    for (int id : ids)
        if (id < 0 || id >= n_vertices) {
            spgx::set_error("anchor index out of range");
            return false;
        }
    return true;
}

}  // namespace

extern "C" {

spgx_status spgx_scene_cloth(double mass, float width, float height, int32_t rows, int32_t cols, double young,
                             double poisson, double bending_k, double anchor_k, int32_t n_anchors,
                             const int32_t *anchors, int32_t rest_initial, spgx_scene **out)
{
    SPGX_GUARD_BEGIN
    if (!out || rows < 2 || cols < 2 || (n_anchors > 0 && !anchors)) {
        spgx::set_error("invalid cloth parameters");
        return SPGX_ERR_INVALID_ARG;
    }
    std::vector<int> ids;
    if (n_anchors < 0)
        ids = {0, rows - 1};
    else
        ids.assign(anchors, anchors + n_anchors);
    for (int id : ids)
        if (id < 0 || id >= rows * cols) {
            spgx::set_error("anchor index out of range");
            return SPGX_ERR_INVALID_ARG;
        }
    auto s = std::make_unique<spgx_scene>();
    s->groups.push_back(spg::scenes::createCloth(mass, width, height, rows, cols, young, poisson, bending_k, anchor_k,
                                                 ids, rest_initial != 0));
    return finish(std::move(s), out);
    SPGX_GUARD_END
}

spgx_status spgx_scene_spring_cloth(double mass, float width, float height, int32_t rows, int32_t cols,
                                    double spring_k, double bending_k, double anchor_k, double jitter, uint64_t seed,
                                    spgx_scene **out)
{
    SPGX_GUARD_BEGIN
    if (!out || rows < 2 || cols < 2) {
        spgx::set_error("invalid cloth parameters");
        return SPGX_ERR_INVALID_ARG;
    }
    auto s = std::make_unique<spgx_scene>();
    s->groups.push_back(
        spg::scenes::createSpringCloth(mass, width, height, rows, cols, spring_k, bending_k, anchor_k, jitter, seed));
    return finish(std::move(s), out);
    SPGX_GUARD_END
}

spgx_status spgx_scene_tet_beam(double mass, float sx, float sy, float sz, int32_t nx, int32_t ny, int32_t nz,
                                double young, double poisson, double anchor_k, int32_t split, spgx_scene **out)
{
    SPGX_GUARD_BEGIN
    if (!out || nx < 2 || ny < 2 || nz < 2) {
        spgx::set_error("invalid beam parameters");
        return SPGX_ERR_INVALID_ARG;
    }
    auto s = std::make_unique<spgx_scene>();
    s->groups.push_back(
        spg::scenes::createTetrahedralBeam(mass, sx, sy, sz, nx, ny, nz, young, poisson, anchor_k, split));
    return finish(std::move(s), out);
    SPGX_GUARD_END
}

spgx_status spgx_scene_patch_batch(int32_t n_patches, int32_t n_min, int32_t n_max, double mu_lo, double mu_hi,
                                   double kb_lo, double kb_hi, double mass, double anchor_k, uint64_t seed,
                                   spgx_scene **out)
{
    SPGX_GUARD_BEGIN
    if (!out || n_patches < 0 || n_min < 2 || n_max < n_min) {
        spgx::set_error("invalid batch parameters");
        return SPGX_ERR_INVALID_ARG;
    }
    auto s = std::make_unique<spgx_scene>();
    s->groups = spg::scenes::createPatchBatch(n_patches, n_min, n_max, mu_lo, mu_hi, kb_lo, kb_hi, mass, anchor_k, seed);
    return finish(std::move(s), out);
    SPGX_GUARD_END
}

spgx_status spgx_scene_triangle_mesh(const double *vertices, int32_t n_vertices, const int32_t *faces, int32_t n_faces,
                                     double mass, double spring_k, double bending_k, double anchor_k,
                                     int32_t n_anchors, const int32_t *anchors, spgx_scene **out)
{
    SPGX_GUARD_BEGIN
    std::vector<spg::Vector3> V;
    std::vector<spg::Int3> F;
    std::vector<int> ids;
    if (!out || !meshInputs(vertices, n_vertices, faces, n_faces, n_anchors, anchors, V, F, ids))
        return SPGX_ERR_INVALID_ARG;
    auto s = std::make_unique<spgx_scene>();
    s->groups.push_back(spg::scenes::createTriangleMeshShell(V, F, mass, spring_k, bending_k, anchor_k, ids));
    return finish(std::move(s), out);
    SPGX_GUARD_END
}

spgx_status spgx_scene_tet_mesh(const double *vertices, int32_t n_vertices, const int32_t *tets, int32_t n_tets,
                                double mass, double young, double poisson, double anchor_k, int32_t n_anchors,
                                const int32_t *anchors, spgx_scene **out)
{
    SPGX_GUARD_BEGIN
    std::vector<spg::Vector3> V;
    std::vector<spg::Int4> T;
    std::vector<int> ids;
    if (!out || !meshInputs(vertices, n_vertices, tets, n_tets, n_anchors, anchors, V, T, ids))
        return SPGX_ERR_INVALID_ARG;
    auto s = std::make_unique<spgx_scene>();
    s->groups.push_back(spg::scenes::createTetMeshSolid(V, T, mass, young, poisson, anchor_k, ids));
    return finish(std::move(s), out);
    SPGX_GUARD_END
}

spgx_status spgx_scene_get_desc(spgx_scene *scene, const spgx_scene_desc **out)
{
    if (!scene || !out) {
        spgx::set_error("invalid argument");
        return SPGX_ERR_INVALID_ARG;
    }
    *out = &scene->packed.desc;
    return SPGX_OK;
}

spgx_status spgx_scene_rest_positions(spgx_scene *scene, int32_t object, double *x0)
{
    if (!scene || !x0 || object < 0 || object >= static_cast<int>(scene->groups.size())) {
        spgx::set_error("invalid argument");
        return SPGX_ERR_INVALID_ARG;
    }
    const auto &g = scene->groups[object];
    for (int i = 0; i < g.size(); ++i)
        for (int a = 0; a < 3; ++a) x0[3 * i + a] = g.positions0()[i][a];
    return SPGX_OK;
}

void spgx_scene_destroy(spgx_scene *scene) { delete scene; }

spgx_status spgx_scene_run_gpu_vbd(spgx_scene *scene, const spgx_vbd_params *params, int32_t steps, double *x_out)
{
    SPGX_GUARD_BEGIN
    if (!scene || !params || steps < 0 || !x_out || scene->groups.empty()) {
        spgx::set_error("invalid argument");
        return SPGX_ERR_INVALID_ARG;
    }
    spg::solver::GpuVBD solver;
    for (const auto &g : scene->groups) solver.addObject(g);
    solver.setDt(params->dt);
    solver.setNumSubsteps(params->substeps);
    solver.setGravity({params->gravity[0], params->gravity[1], params->gravity[2]});
    solver.setIterations(params->iterations);
    solver.setLaunch(params->lanes_per_vertex, params->block_size);
    for (int s = 0; s < steps; ++s) solver.step();
    const auto &g = solver.particleGroups()[0];
    for (int i = 0; i < g.size(); ++i)
        for (int a = 0; a < 3; ++a) x_out[3 * i + a] = g.positions()[i][a];
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_scene_run_gpu_xpbd(spgx_scene *scene, const spgx_xpbd_params *params, int32_t steps, double *x_out)
{
    SPGX_GUARD_BEGIN
    if (!scene || !params || steps < 0 || !x_out || scene->groups.empty()) {
        spgx::set_error("invalid argument");
        return SPGX_ERR_INVALID_ARG;
    }
    spg::solver::GpuXPBD solver;
    for (const auto &g : scene->groups) solver.addObject(g);
    solver.setDt(params->dt);
    solver.setNumSubsteps(params->substeps);
    solver.setGravity({params->gravity[0], params->gravity[1], params->gravity[2]});
    for (int s = 0; s < steps; ++s) solver.step();
    const auto &g = solver.particleGroups()[0];
    for (int i = 0; i < g.size(); ++i)
        for (int a = 0; a < 3; ++a) x_out[3 * i + a] = g.positions()[i][a];
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_scene_run_gpu_implicit(spgx_scene *scene, const spgx_implicit_params *params, int32_t steps,
                                        double *x_out)
{
    SPGX_GUARD_BEGIN
    if (!scene || !params || steps < 0 || !x_out || scene->groups.empty()) {
        spgx::set_error("invalid argument");
        return SPGX_ERR_INVALID_ARG;
    }
    spg::solver::GpuImplicit solver(static_cast<spgx_implicit_method>(params->method));
    for (const auto &g : scene->groups) solver.addObject(g);
    solver.setDt(params->dt);
    solver.setNumSubsteps(params->substeps);
    solver.setGravity({params->gravity[0], params->gravity[1], params->gravity[2]});
    for (int s = 0; s < steps; ++s) solver.step();
    const auto &g = solver.particleGroups()[0];
    for (int i = 0; i < g.size(); ++i)
        for (int a = 0; a < 3; ++a) x_out[3 * i + a] = g.positions()[i][a];
    return SPGX_OK;
    SPGX_GUARD_END
}

}  // extern "C"
