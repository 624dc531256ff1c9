// Test-only, needs a GPU: drives spg::solver::GpuVBD through the reference application's
// picking sequence (apps/solverCompare.cpp:717-726 adds a one-stencil SpringAnchorEnergy and
// flags a topology update, :1524 moves it with updateAnchor every frame, :1499 removes it).
#include <cstring>
#include <memory>

#include "spg/scenes.h"
#include "spg/sim/solver/gpuSolvers.h"

using namespace spg;

extern "C" int run_picking(int n, int kernel, int lanes, int iterations, double dt, int steps, int pick_vertex,
                           int pick_start, int pick_end, const double *path, double stiffness, double *x_out,
                           int *rebuilds)
{
    try {
        const float w = 2.0f * float(n - 1) / 512.0f;
        solver::GpuVBD s;
        s.addObject(scenes::createSpringCloth(0.1 * w * w, w, w, n, n, 1e4, 1e-4, 1e5, 0.1, 12345));
        s.setDt(dt);
        s.setGravity({0, 0, -9.81});
        s.setIterations(iterations);
        s.setKernel(kernel);
        s.setLaunch(lanes, 0);
        std::shared_ptr<SpringAnchorEnergy> pick;
        spgx_vbd *h = nullptr;
        *rebuilds = 0;
        for (int step = 0; step < steps; ++step) {
            auto &g = s.particleGroups()[0];
            if (step == pick_start) {
                pick = std::make_shared<SpringAnchorEnergy>();
                pick->addStencil({pick_vertex}, g.positions()[pick_vertex], stiffness);
                g.addEnergy(pick);
                s.requirePrecomputationUpdate();
            }
            if (pick && step > pick_start) pick->updateAnchor(0, {path[3 * step], path[3 * step + 1], path[3 * step + 2]});
            if (pick && step == pick_end) {
                g.removeEnergy(pick);
                pick.reset();
                s.requirePrecomputationUpdate();
            }
            s.step();
            if (h && s.handle() != h) ++*rebuilds;
            h = s.handle();
        }
        const auto &g = s.particleGroups()[0];
        for (int i = 0; i < g.size(); ++i)
            for (int a = 0; a < 3; ++a) x_out[3 * i + a] = g.positions()[i][a];
        return 0;
    } catch (...) {
        return 1;
    }
}
