/*
 * spgx_scenes.h — headless scene builders and the C++ drop-in solver classes behind a C ABI.
 *
 * The reference builds its scenes in its GUI application (apps/solverCompare.cpp:118-498,
 * Polyscope/OpenGL) through ParticleGroup::addParticle and each energy's addStencil /
 * preparePrecomputations. These entry points run the same construction with the library's
 * Eigen-free spg:: classes and hand back the packed spgx_scene_desc that GpuVBD / GpuXPBD
 * (spg::solver::BaseSolver subclasses) pass to spgx_vbd_create / spgx_xpbd_create.
 * No device is needed except for spgx_scene_run_gpu_vbd / _xpbd.
 */
#ifndef SPGX_SCENES_H
#define SPGX_SCENES_H

#include "spgx.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct spgx_scene spgx_scene;

/* createCloth (solverCompare.cpp:367-498): n_anchors < 0 pins vertices 0 and rows - 1 as
 * the reference does; rest_initial != 0 starts from the flat rest state. */
spgx_status spgx_scene_cloth(double mass, float width, float height, int32_t rows, int32_t cols, double young,
                             double poisson, double bending_k, double anchor_k, int32_t n_anchors,
                             const int32_t *anchors, int32_t rest_initial, spgx_scene **out);
/* Jittered spring cloth (springs on all edges, bending on interior edges, row 0 anchored). */
spgx_status spgx_scene_spring_cloth(double mass, float width, float height, int32_t rows, int32_t cols,
                                    double spring_k, double bending_k, double anchor_k, double jitter, uint64_t seed,
                                    spgx_scene **out);
/* createTetrahedralBeam (solverCompare.cpp:260-330) with SNH tets, split 5 or 6 per cell. */
spgx_status spgx_scene_tet_beam(double mass, float sx, float sy, float sz, int32_t nx, int32_t ny, int32_t nz,
                                double young, double poisson, double anchor_k, int32_t split, spgx_scene **out);
/* Batch of independent square patches (one object each). */
spgx_status spgx_scene_patch_batch(int32_t n_patches, int32_t n_min, int32_t n_max, double mu_lo, double mu_hi,
                                   double kb_lo, double kb_hi, double mass, double anchor_k, uint64_t seed,
                                   spgx_scene **out);
/* A shell on a triangle mesh (e.g. from spgx_load_obj): lumped masses from the rest areas,
 * springs on every edge, discrete bending on interior edges, anchors on the listed vertices.
 * vertices: 3 * n_vertices doubles (rest = initial state); faces: 3 * n_faces indices. */
spgx_status spgx_scene_triangle_mesh(const double *vertices, int32_t n_vertices, const int32_t *faces, int32_t n_faces,
                                     double mass, double spring_k, double bending_k, double anchor_k,
                                     int32_t n_anchors, const int32_t *anchors, spgx_scene **out);
/* A solid on a tetrahedral mesh (e.g. from spgx_load_msh): lumped masses from the rest
 * volumes, Stable Neo-Hookean tets, anchors on the listed vertices. tets: 4 * n_tets indices,
 * each with positive rest volume. */
spgx_status spgx_scene_tet_mesh(const double *vertices, int32_t n_vertices, const int32_t *tets, int32_t n_tets,
                                double mass, double young, double poisson, double anchor_k, int32_t n_anchors,
                                const int32_t *anchors, spgx_scene **out);
/* Packed descriptor of the scene (valid until spgx_scene_destroy). */
spgx_status spgx_scene_get_desc(spgx_scene *scene, const spgx_scene_desc **out);
/* Rest positions (ParticleGroup::positions0) of one object, 3 * n_vertices doubles. */
spgx_status spgx_scene_rest_positions(spgx_scene *scene, int32_t object, double *x0);
void spgx_scene_destroy(spgx_scene *scene);

/* Runs `steps` steps of spg::solver::GpuVBD on the scene's ParticleGroups with the given
 * parameters (dt, substeps, gravity and iterations are applied through the BaseSolver
 * setters) and copies object 0's final positions to x_out (3 * n_vertices). */
spgx_status spgx_scene_run_gpu_vbd(spgx_scene *scene, const spgx_vbd_params *params, int32_t steps, double *x_out);
/* Same with spg::solver::GpuXPBD. */
spgx_status spgx_scene_run_gpu_xpbd(spgx_scene *scene, const spgx_xpbd_params *params, int32_t steps, double *x_out);
/* Same with spg::solver::GpuImplicit for params->method (the global solvers). */
spgx_status spgx_scene_run_gpu_implicit(spgx_scene *scene, const spgx_implicit_params *params, int32_t steps,
                                        double *x_out);

/* ---- Mesh input (spg::io::loadObj / loadMsh, spg/source/geom/io/{obj,msh}.cpp) ----------
 * spgx_load_obj: the vertices of the whole file (as float, widened to double) and the
 * triangles of its first shape, quads split along the shorter diagonal.
 * spgx_load_msh: the nodes and tetrahedra of a Gmsh 2.2 (ASCII) or 4.1 (ASCII or binary)
 * file; blocks of other element types are skipped.
 * Query the sizes with spgx_mesh_info, copy out with spgx_mesh_copy (vertices: 3 doubles per
 * vertex; cells: cell_size indices per cell, 3 for OBJ and 4 for MSH), then destroy. */
typedef struct spgx_mesh spgx_mesh;
spgx_status spgx_load_obj(const char *path, spgx_mesh **out);
spgx_status spgx_load_msh(const char *path, spgx_mesh **out);
spgx_status spgx_mesh_info(const spgx_mesh *mesh, int64_t *n_vertices, int64_t *n_cells, int32_t *cell_size);
spgx_status spgx_mesh_copy(const spgx_mesh *mesh, double *vertices, int32_t *cells);
spgx_status spgx_mesh_destroy(spgx_mesh *mesh);

#ifdef __cplusplus
}
#endif

#endif /* SPGX_SCENES_H */
