// Particle state shared by the VBD and XPBD solver handles: device buffers in the layout
// described in device_common.cuh, pinned host mirrors, and the host<->device state calls
// (ParticleGroup positions/velocities, particleGroup.h:51-56; BaseSolver::reset).
#pragma once

#include <cuda_runtime.h>

#include "devbuf.h"
#include "device_common.cuh"
#include "layout.h"

namespace spgx {

struct ParticleState {
    int nv{0};
    DevBuf d_pos, d_tgt, d_dold, d_vel, d_invm;
    DevBuf d_ext2int;   // concatenated external index -> internal index
    DevBuf d_stage;     // FP64 staging of one object's positions and velocities
    size_t stage_doubles{0};
    bool replaced{false};  // set() wrote positions or velocities since the last take_replaced()

    // Allocates the buffers and uploads the scene's initial positions and velocities:
    // base = fl(x), delta = fl(x - base); target = current delta with the mass in w.
    spgx_status init(const SceneLayout &L);
    // Host <-> device state of one object in its external order. The FP64 host arrays are
    // copied as they are and converted on the device (base/delta split, velocity rounding,
    // external <-> internal order), in stream order with the solver's work.
    spgx_status get(const SceneLayout &L, int obj, double *x, double *v, cudaStream_t stream);
    spgx_status set(const SceneLayout &L, int obj, const double *x, const double *v, cudaStream_t stream);
    spgx_status reset(const SceneLayout &L, cudaStream_t stream);
    // The state lives on the device only; kept for the solvers' call sites.
    spgx_status upload_if_dirty(cudaStream_t) { return SPGX_OK; }
    void mark_device_advanced() {}
    bool take_replaced()
    {
        const bool r = replaced;
        replaced = false;
        return r;
    }

    float4 *pos() const { return d_pos.as<float4>(); }
    float4 *tgt() const { return d_tgt.as<float4>(); }
    float4 *dold() const { return d_dold.as<float4>(); }
    float4 *vel() const { return d_vel.as<float4>(); }
    float *invm() const { return d_invm.as<float>(); }
};

// Substep kernels shared by both solvers (see state.cu).
void launch_begin_substep(const ParticleState &P, double h, const double *g, cudaStream_t st);
// With vhist given, also stores v_n = (velocity after the inertial predict) - h g into vhist
// before the velocity update (the displacement history of the learned warm start).
void launch_end_substep(const ParticleState &P, double h, cudaStream_t st, float4 *vhist = nullptr,
                        const double *g = nullptr);

}  // namespace spgx
