// Learned warm start of a VBD step: per-vertex features of the displacement history, the
// MLP's predicted correction to the inertial guess, and the residual-based acceptance.
//
// Units: displacements are scaled by 1 / l with l = h^2 * kWarmG0 (the distance standard
// gravity moves a body in one substep), so the features of a given motion do not depend on h.
//
// Features of vertex i (24 floats), with d_in = y - x_n (inertial displacement),
// d1 = x_n - x_{n-1}, d2 = x_{n-1} - x_{n-2}, lap(u)_i = mean over the one-ring j of u_j - u_i:
//   0-2  d_in / l          3-5  d1 / l           6-8   d2 / l
//   9-11 lap(d1) / l       12-14 lap(d2) / l     15-17 g / kWarmG0
//   18   anchored flag     19   anchored fraction of the one-ring
//   20   one-ring size / 8 21   |d1| / l         22    |lap(d1)| / l     23  1
// The one-ring is every vertex sharing a mesh edge, a triangle or a tet with i (the two
// opposite vertices of a bending stencil are not neighbours of each other).
// Recorded target: (x* - y) / l, the converged position's offset from the inertial guess.
// Network output: the correction c to the extrapolated guess, x_w = x_n + 2 d1 - d2 + l c
// (the last step's acceleration carried over, plus the learned remainder), so the network is
// trained on (x* - y) / l - (d1 - d2 - h^2 g) / l = target - (f[3:6] - f[6:9] - f[15:18]).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "devbuf.h"
#include "layout.h"

namespace spgx {

constexpr int kWarmFeatures = 24;
constexpr double kWarmG0 = 9.81;
// Sweeps run from each of the learned and the extrapolated guess before they are compared. On
// the 513^2 cloth (time to 1e-5 over three steps) 10 kept the network's guess in no step, 20
// in one of three, 30 in two, 40 in all three at the lowest time (50 ms; 60 and 80: 57, 64 ms).
constexpr int kWarmProbeSweeps = 40;
// Default one-ring smoothing passes over the network's correction field.
constexpr int kWarmSmoothPasses = 20;

struct Mlp;

// One-ring CSR in internal vertex order plus per-vertex static features
// {anchored, anchored fraction of the one-ring, one-ring size / 8, 0}.
void build_vertex_neighbours(const SceneLayout &L, std::vector<int32_t> &off, std::vector<int32_t> &nbr,
                             std::vector<F4> &stat);

// Initial-guess modes of spgx_vbd_set_warm_start.
enum WarmMode { kWarmInertial = 0, kWarmLearned = 1, kWarmExtrapolate = 2 };

struct WarmStart {
    bool history{false};  // history buffers exist and are maintained every substep
    int mode{kWarmInertial};
    const Mlp *mlp{nullptr};
    int smooth{kWarmSmoothPasses};  // one-ring smoothing passes over the network's correction field
    DevBuf nbr_off, nbr, stat, vhist, feats, out, out2, wres;
};

// feats = features of every vertex at the start of the substep (after the inertial predict).
void launch_warm_features(const WarmStart &W, const float4 *vel, int nv, double h, const double *g, cudaStream_t st);
// W.smooth passes of out <- (out + one-ring mean of out) / 2 (the network's correction field
// keeps its smooth part and loses per-vertex noise, which the stiff springs amplify).
void launch_warm_smooth(const WarmStart &W, int nv, cudaStream_t st);
// delta = tgt + h (v_n - v_{n-1}) - h^2 g + l * out for every vertex (the learned guess).
void launch_warm_apply(const WarmStart &W, float4 *pos, const float4 *tgt, const float4 *vel, int nv, double h,
                       const double *g, cudaStream_t st);
// delta = tgt + h (v_n - v_{n-1}) - h^2 g (the previous step's acceleration carried over).
void launch_warm_extrapolate(const WarmStart &W, float4 *pos, const float4 *tgt, const float4 *vel, int nv, double h,
                             const double *g, cudaStream_t st);
// Starts the substep from the guess with the lowest residual: the candidate in the positions
// (squared residual wres[1]), y (wres[0]) or, with three_way, the extrapolated guess
// (wres[2]). Counts the pick in counters[3] (learned) or counters[4] (extrapolated).
void launch_warm_select(const WarmStart &W, float4 *pos, const float4 *tgt, const float4 *vel, int nv, double h,
                        const double *g, bool three_way, int *counters, cudaStream_t st);
// The learned guess's probe: when wres[1] (its residual after the probe sweeps) is below
// wres[2] (the extrapolated guess's), the positions go back to the learned probe's state
// saved in `saved` (base and delta per vertex); counts the pick in counters[3] or [4].
void launch_warm_probe_select(const WarmStart &W, float4 *pos, const float4 *saved, int nv, int *counters,
                              cudaStream_t st);
// targets = (x - y) / l for every vertex (training data of the converged step).
void launch_warm_targets(const float4 *pos, const float4 *tgt, int nv, double h, float *targets, cudaStream_t st);

}  // namespace spgx
