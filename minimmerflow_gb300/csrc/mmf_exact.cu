// mmf_exact.cu -- reference-arithmetic instantiation of the stage kernels and
// the pointwise kernels of the reference's unit-level functions.  Built with
// -fmad=false so no multiply-add is contracted: the results are the
// reference's CPU results bit for bit.
#include "mmf_batch.cuh"
#include "mmf_launch.cuh"

namespace mmf {

cudaError_t launch_stage_exact(int stage, const GridParams &gp, const StageArgs &sa, cudaStream_t s)
{
    return launch_stage<ExactArith>(stage, gp, sa, s);
}

void prime_tile3d_exact() { prime_tile3d_slots<ExactArith>(); }

cudaError_t launch_screen_selftest_exact(int dim, long long n, const double *uc, const double *sig, int *dec,
                                        unsigned char *ref, cudaStream_t s)
{
    return launch_screen_selftest<ExactArith>(dim, n, uc, sig, dec, ref, s);
}

cudaError_t launch_o2_exact(int op, int stage, const GridParams &gp, const StageArgs &sa, const O2Args &oa,
                            double *W1, cudaStream_t s)
{
    return launch_o2<ExactArith>(op, stage, gp, sa, oa, W1, s);
}

cudaError_t launch_batch_o2_exact(int op, int stage, const CaseDesc *cases, const int *item_case, int nitems,
                                  Ctrl *cctrl, const StageArgs &base, const double *state, const O2Batch &ob,
                                  double *W1, int blocks, cudaStream_t s)
{
    return launch_batch_o2<ExactArith>(op, stage, cases, item_case, nitems, cctrl, base, state, ob, W1, blocks, s);
}

int batch_slope_blocks_per_sm_exact()
{
    return batch_slopes_blocks_per_sm<ExactArith>();
}

int batch_max_blocks_per_sm_exact(int order)
{
    return order == 2 ? batch_o2_blocks_per_sm<ExactArith>() : batch_blocks_per_sm<ExactArith>();
}

cudaError_t launch_batch_exact(int stage, const CaseDesc *cases, const int *item_case, int nitems, Ctrl *cctrl,
                               const StageArgs &base, int blocks, cudaStream_t s)
{
    return launch_batch<ExactArith>(stage, cases, item_case, nitems, cctrl, base, blocks, s);
}

// One thread per item; arrays are AoS [n][5] (normals [n][3]).
__global__ void pointwise_kernel(int op, long long n, const double *a, const double *b, const double *nrm, int bc,
                                 const double *dir_prim, double *out, double *out2)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *ai = a + NF * i;
    double *oi = out + NF * i;
    double dp[NF];
    switch (op) {
    case OP_CONS2PRIM: ExactArith::cons2prim(ai, oi); break;           // utils.cpp:48-63
    case OP_PRIM2CONS: ExactArith::prim2cons(ai, oi); break;           // utils.cpp:71-83
    case OP_FLUXES: ExactArith::eval_fluxes(ai, b + NF * i, nrm + 3 * i, oi); break; // euler.cpp:83-113
    case OP_SPLITTING: {                                                // euler.cpp:42-73
        const double *cl = ai, *cr = b + NF * i, *nn = nrm + 3 * i;
        double pl[NF], pr[NF], fl[NF], fr[NF];
        ExactArith::cons2prim(cl, pl);
        ExactArith::cons2prim(cr, pr);
        ExactArith::eval_fluxes(cl, pl, nn, fl);
        ExactArith::eval_fluxes(cr, pr, nn, fr);
        double lamL = fabs(ExactArith::normal_velocity(pl, nn)) + sqrt(GAMMA * pl[4]);
        double lamR = fabs(ExactArith::normal_velocity(pr, nn)) + sqrt(GAMMA * pr[4]);
        out2[i] = ExactArith::face(cl, fl, lamL, cr, fr, lamR, oi);
        break;
    }
    case OP_BC:                                                         // euler.cpp:261-376
        for (int k = 0; k < NF; ++k) dp[k] = dir_prim ? dir_prim[k] : 0.0;
        {
            double dc[NF];
            ExactArith::prim2cons(dp, dc);
            ghost_state<ExactArith>(bc, nrm + 3 * i, ai, dc, oi);
        }
        break;
    default: break;
    }
}

cudaError_t launch_pointwise_exact(int op, long long n, const double *a, const double *b, const double *nrm,
                                   int bc, const double *dir_prim, double *out, double *out2, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    const unsigned blocks = (unsigned)((n + 127) / 128);
    pointwise_kernel<<<blocks, 128, 0, s>>>(op, n, a, b, nrm, bc, dir_prim, out, out2);
    return cudaPeekAtLastError();
}

} // namespace mmf
