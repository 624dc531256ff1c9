// VBD solver handle behind the spgx_vbd_* C ABI.
#pragma once

#include <cuda_runtime.h>

#include "devbuf.h"
#include "device_common.cuh"
#include "layout.h"
#include "state.h"
#include "vbd_tile.cuh"
#include "warm.h"

namespace spgx {

// Device element tables of one scene (shared by the VBD handle's kernels).
struct ElementBuffers {
    DevBuf anchors, springs, spring_cmp, bend_idx, bend_prm, stvk_idx, stvk_D, stvk_Ka, stvk_Kb, stvk_Ca, stvk_Cb,
        stvk_Cc, snh_idx, snh_p0, snh_p1, snh_p2, snh_cmp, anchor_cmp;
    DevBuf gen_off, gen_adj, gen_idx, gen_info, gen_prm;
    spgx_status upload(const ElementTables &E, DevTables &T);
    // Energies of types 6-14 (no-op without them).
    spgx_status upload_generic(const SceneLayout &L, DevTables &T);
};

struct VbdSolver {
    SceneLayout L;
    spgx_vbd_params P{};
    double h_sub{0.01};
    int device{0};
    int kernel{1};  // 1: lanes-per-vertex kernel, 2: shared-memory tile kernel, 3: dataflow tiles
    int lanes{1};
    int block{128};
    cudaStream_t stream{nullptr};
    cudaEvent_t ev0{nullptr}, ev1{nullptr};
    cudaGraphExec_t graph_exec{nullptr};
    bool graph_valid{false};

    ParticleState X;
    ElementBuffers EB;
    DevBuf d_hdr, d_adj, d_counters, d_resid, d_backup;
    HostBuf h_counters;
    DevTables T{};
    DevState S{};
    TileLayout TL;
    DevBuf tb_hdr, tb_halo, tb_records, tb_vrec;
    TileView TV{};
    size_t tile_smem{0};
    DevBuf fl_fhdr, fl_nbrp, fl_epoch, fl_ticket;
    FlowView FV{};
    int flow_blocks_per_sm[4]{};  // per lanes variant 1, 2, 4, 8
    int num_sms{0};
    mutable int flow_epoch{0};    // sweeps the dataflow kernel has completed on this handle
    mutable cudaError_t flow_launch_error{cudaSuccess};
    WarmStart W;
    DevBuf d_pick_v, d_pick_a;  // dynamic anchors, SPGX_MAX_PICKS slots

    VbdSolver() = default;
    VbdSolver(const VbdSolver &) = delete;
    VbdSolver &operator=(const VbdSolver &) = delete;
    ~VbdSolver();

    spgx_status init(const spgx_scene_desc *scene, const spgx_vbd_params *params);
    static spgx_status check_params(const spgx_vbd_params *p);
    spgx_status set_params(const spgx_vbd_params *params);
    spgx_status configure_launch();
    spgx_status setup_tiles(int tile_vertices);
    spgx_status setup_flow();
    spgx_status reset_flow();
    spgx_status take_flow_launch_error();
    spgx_status build_graph();
    spgx_status residual_norm(double *out);
    spgx_status profile_sweeps(int iterations, double *color_ms);
    // One step. With features/targets given (one substep only), also returns every vertex's
    // warm-start features at the start of the step and its target (x* - y) / l at the end.
    spgx_status step(spgx_step_stats *stats, float *features = nullptr, float *targets = nullptr);
    spgx_status enable_history();
    spgx_status upload_state();
    spgx_status set_warm_start(const Mlp *mlp, int mode);
    int launch_warm(cudaStream_t st);
    // Sweeps each probe of the learned guess runs (0 in the other modes).
    int warm_probe_sweeps() const
    {
        if (W.mode != kWarmLearned) return 0;
        return std::min(kWarmProbeSweeps, P.tolerance > 0 ? P.max_iterations : P.iterations);
    }
    // Replaces the dynamic anchors (picking) between steps.
    spgx_status set_picks(int n, const int32_t *object, const int32_t *vertex, const double *target, const double *k);
};

}  // namespace spgx
