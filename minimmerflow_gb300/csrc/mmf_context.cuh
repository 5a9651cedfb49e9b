// mmf_context.cuh -- the solver context of the C ABI (private to the library's
// translation units).
#pragma once

#include <cuda_runtime.h>

#include "../../include/mmf_gb300.h"
#include "mmf_launch.cuh"
#include "mmf_nvtx.h"

namespace mmf {
cudaError_t mlp_indicator(mmf_mlp *p, const GridParams &gp, const double *U, float thr, float *prob,
                          unsigned char *flags, cudaStream_t s, float *Q, unsigned char *raw, IndicatorStep is);
}

using namespace mmf;

struct mmf_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    mmf_grid grid;
    GridParams gp;
    double *U = nullptr, *R = nullptr, *W = nullptr;   // SoA [5][plane]
    double *S = nullptr;                               // scratch state (compute_rhs)
    double *aos = nullptr;                             // AoS staging [plane][5]
    long long *raw_to_cell = nullptr;                  // null = identity
    Ctrl *ctrl = nullptr;
    double *rhs_maxeig = nullptr;
    cudaGraphExec_t graph_many = nullptr, graph_one = nullptr;
    long long launches = 0;
    double cfl = 0.0;
    bool time_ready = false;
    bool w_zero = false;      // 2D state with identically zero z-momentum
    int *flag = nullptr;      // device scratch flag
    // order 2
    double *Sl = nullptr;               // slopes, dim x 5 planes
    unsigned char *lim_flag = nullptr;  // per cell: limit (1) / central slope (0) in LIMIT_FLAGGED mode
    unsigned char *lim_active = nullptr;// per cell: the limiter changed a slope (stage 1 of the last step)
    int limit_mode = LIMIT_ALL;
    mmf_mlp *indicator = nullptr;       // learned indicator run at the start of every step
    float ind_threshold = 0.5f;
    float *ind_q = nullptr;             // the indicator's FP32 primitive planes (5 x plane)
    int ind_period = 1;                 // the indicator runs every ind_period steps (1 or 2)
    int *ind_tick = nullptr;            // device step counter of the period
    unsigned char *ind_raw = nullptr;   // the network's flags before the dilation (period 2)
    // pipelined host round trip (mmf_advance_host): a copy stream, one event
    // per band and direction, pinned host words for the flag and the control block
    static constexpr int MAX_BANDS = 16;
    cudaStream_t copy_stream = nullptr;
    cudaStream_t tr_stream = nullptr;            // upload transpositions, highest priority
    cudaStream_t band_stream[MAX_BANDS] = {};   // band b at priority b (band 0 first)
    cudaEvent_t ev_up[MAX_BANDS] = {}, ev_tr[MAX_BANDS] = {}, ev_s1[MAX_BANDS] = {}, ev_dn[MAX_BANDS] = {};
    cudaEvent_t ev_s2b[MAX_BANDS] = {};          // order 1: stage 2 of band b done; order 2: stage-1 slopes of bands 0..b done
    cudaEvent_t ev_start = nullptr, ev_s2 = nullptr, ev_flag = nullptr;
    int *h_flag = nullptr;
    Ctrl *h_ctrl = nullptr;
    // optional per-step log (mmf_set_step_log): 3 doubles per step, a ring
    double *steplog = nullptr;
    long long steplog_cap = 0;

    cudaError_t stage(int st, const double *U_in, double *out) { return stage_gp(st, gp, U_in, out, stream); }
    // a stage over the rows (2D) / planes (3D) that 'g' covers, on stream 'on'
    cudaError_t stage_gp(int st, const GridParams &g, const double *U_in, double *out, cudaStream_t on)
    {
        StageArgs sa;
        sa.U = U_in;
        sa.R = R;
        sa.W = W;
        sa.out = out;
        sa.ctrl = ctrl;
        sa.rhs_maxeig = rhs_maxeig;
        ++launches;
        return (grid.arith == MMF_ARITH_FAST && st != STAGE_RHS) ? mmf::launch_stage_fast(st, g, sa, on, w_zero)
                                                                : mmf::launch_stage_exact(st, g, sa, on);
    }
    cudaError_t o2(int op, int st, const double *state, double *out, unsigned char *active)
    {
        return o2_gp(op, st, gp, state, out, active, stream, 0, gp.plane);
    }
    // an order-2 operation with the decomposition 'g' (stage launches over its
    // chunks) and, for the slopes, the grid cells [cell0, cell1), on stream 'on'
    cudaError_t o2_gp(int op, int st, const GridParams &g, const double *state, double *out, unsigned char *active,
                      cudaStream_t on, long long cell0, long long cell1)
    {
        StageArgs sa;
        sa.U = U; sa.R = R; sa.W = W; sa.out = out; sa.ctrl = ctrl; sa.rhs_maxeig = rhs_maxeig;
        O2Args oa;
        oa.state = state; oa.S = Sl; oa.flag = lim_flag; oa.active = active; oa.limit_mode = limit_mode;
        oa.ctrl = ctrl; oa.stage = st;
        oa.cell0 = cell0;
        oa.cell1 = cell1;
        // a step's stage-1 slopes advance the indicator's step counter
        oa.tick = (op == O2_SLOPES && st == STAGE_1 && indicator && ind_period > 1) ? ind_tick : nullptr;
        ++launches;
        return (grid.arith == MMF_ARITH_FAST && st != STAGE_RHS) ? mmf::launch_o2_fast(op, st, g, sa, oa, W, on, w_zero)
                                                                : mmf::launch_o2_exact(op, st, g, sa, oa, W, on);
    }
    cudaError_t rk_step()
    {
        cudaError_t e;
        if (grid.order == 2) {
            // stage 1: slopes(U), R = RHS(U); stage 2: W1 = U + dt R / V, slopes(W1), R := W2;
            // stage 3: slopes(W2), U := 1/3 U + 2/3 (W2 + dt RHS(W2) / V)
            if (indicator) {
                launches += ind_period > 1 ? 3 : 2;   // primitives, features + MLP (, dilation)
                if ((e = mlp_indicator(indicator, gp, U, ind_threshold, nullptr, lim_flag, stream, ind_q,
                                       ind_period > 1 ? ind_raw : nullptr, IndicatorStep{ind_period, ind_tick})) !=
                    cudaSuccess)
                    return e;
            }
            if ((e = o2(O2_SLOPES, STAGE_1, U, nullptr, lim_active)) != cudaSuccess) return e;
            if ((e = o2(O2_STAGE, STAGE_1, U, R, nullptr)) != cudaSuccess) return e;
            if ((e = o2(O2_FORM_W1, STAGE_2, U, W, nullptr)) != cudaSuccess) return e;
            if ((e = o2(O2_SLOPES, STAGE_2, W, nullptr, nullptr)) != cudaSuccess) return e;
            if ((e = o2(O2_STAGE, STAGE_2, W, R, nullptr)) != cudaSuccess) return e;
            if ((e = o2(O2_SLOPES, STAGE_3, R, nullptr, nullptr)) != cudaSuccess) return e;
            return o2(O2_STAGE, STAGE_3, R, U, nullptr);
        }
        if ((e = stage(STAGE_1, U, R)) != cudaSuccess) return e;
        if ((e = stage(STAGE_2, U, W)) != cudaSuccess) return e;
        return stage(STAGE_3, U, U);
    }
    int launches_per_step() const { return grid.order == 2 ? (indicator ? (ind_period > 1 ? 10 : 9) : 7) : 3; }
    // the next step runs the indicator (after a change of the state or of the time control)
    void indicator_restart()
    {
        if (ind_tick) cudaMemsetAsync(ind_tick, 0, sizeof(int), stream);
    }
};


namespace mmf {
// After the state changed on the device: pick the 2D kernels without
// z-momentum when that plane is identically zero (defined in mmf_capi.cu).
int refresh_w_zero(mmf_ctx *c);
}
