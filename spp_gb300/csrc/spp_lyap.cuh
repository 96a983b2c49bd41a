/* spp_lyap.cuh -- device state of the tangent-space (Lyapunov) estimator. */
#ifndef SPP_LYAP_CUH
#define SPP_LYAP_CUH
#include "spp_internal.cuh"

struct LyapState {
  int K;                  /* number of tangent vectors (<= SPP_LYAP_MAX) */
  int n;
  float* t0;              /* tangent vectors at the start of the step, [K][3][n] by particle id */
  float* ua;              /* stage inputs (RK2/RK4) */
  float* ub;
  float* acc;             /* RK4 slope sums */
  float* uslot;           /* two buffers of the stage inputs' heading components in slot order,
                             [2][n][K padded to 4]: stage s reads buffer s % 2, writes the other */
  double* partial;        /* Gram partials [SPP_GRAM_BLOCKS][SPP_GRAM_ENTRIES] */
  double* rinv;           /* R^{-1}, [SPP_LYAP_MAX][SPP_LYAP_MAX] */
  double* log_stretch;    /* running sums of log R_aa, FP64 */
  uint32_t* error;        /* set when the Gram matrix is not positive definite */
};

struct TanStage {
  const float4* cur;      /* base state of this stage (slot order) */
  const float* uin;       /* tangent stage input */
  float* uout;            /* next stage input */
  const float* us_in;     /* this stage's heading components in slot order */
  float* us_out;          /* the next stage's, written here (NULL in the last stage) */
  int stage, nstages;
};

void launch_tangent_stage(const SppConsts& k, const DevState& d, const LyapState& L, int stage,
                          int nstages, const float4* cur, cudaStream_t s, int64_t* launches);
void launch_renormalize(const LyapState& L, int accumulate, cudaStream_t s, int64_t* launches);
void launch_tangent_init(const LyapState& L, uint64_t seed, uint32_t system, cudaStream_t s);
/* floats of LyapState::uslot for K vectors of n particles */
size_t tangent_slot_floats(int K, int n);

#endif
