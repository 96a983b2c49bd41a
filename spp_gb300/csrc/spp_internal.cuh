/*
 * spp_internal.cuh -- device data layout and kernel entry points.
 *
 * HBM layout of one system (structure of arrays, all in cell order: particles
 * are counting-sorted by the Morton key of their cell at every list rebuild):
 *   pos     float4 (x, y, cos theta, sin theta)  read by neighbours, 16 B
 *   half    float4 stage state of Runge-Kutta stages (RK4 ping-pongs with half2)
 *   theta   float, img int2 (box crossings), id uint32 (slot -> particle id)
 *   kacc    float4 RK4 slope accumulator (fx, fy, tau, -)
 *   ref     float2 positions at the last neighbour-list build
 *   nbr     int32 [cap][n] neighbour slots, column-major so that a warp's
 *           32 consecutive particles read 128 contiguous bytes per list slot
 *   nn      int32 list lengths
 *   cell_count / cell_start  uint32 per Morton key
 * A small control block (Ctl) in device memory carries the step counter and
 * the device-side rebuild decision, so captured graphs replay without host
 * round trips.
 */
#ifndef SPP_INTERNAL_CUH
#define SPP_INTERNAL_CUH

#include <cuda_runtime.h>
#include <stdint.h>
#include "spp_physics.h"

#define SPP_BLOCK 256

struct Ctl {
  uint32_t step;          /* absolute step index (Philox counter word) */
  uint32_t dmax2_bits;    /* max squared displacement since the last build (float bits) */
  uint32_t blocks_done;   /* last-block detection */
  uint32_t need_rebuild;  /* decision of the last step */
  uint32_t list_need;     /* largest neighbour count met by a build (overflow if > cap) */
  uint32_t fx_overflow;   /* a pair term left the fixed-point range */
  uint32_t max_nn;        /* largest list length of the last build */
  uint32_t n_rebuilds;
  uint32_t frozen;        /* set on list overflow: later stages skip until the host recovers */
  uint32_t smax2_bits;    /* max squared displacement during the current step (float bits) */
  uint32_t late_rebuilds; /* rebuilds decided after some particle had already moved > skin/2 */
  uint32_t bad_nonfinite; /* smallest index of an uploaded particle with a non-finite value (or ~0) */
  uint32_t bad_range;     /* smallest index of an uploaded position outside [-L, L) (or ~0) */
  uint32_t long_n;        /* lists longer than the in-block sort queued by the last build */
  uint32_t bad_index;     /* SPP_CHECKED builds: a kernel met an index out of range */
  uint32_t bulk_timeouts; /* warps whose bulk copy of list rows did not arrive in time (they read global memory) */
};

/* SPP_CHECKED builds check every list, cell and slot index a hot kernel
 * uses; an index out of [0, bound) sets Ctl.bad_index (the next sync
 * returns SPP_ERR_BOUNDS) and the caller skips the access.  Without
 * SPP_CHECKED the check is the constant true. */
#ifdef SPP_CHECKED
__device__ __forceinline__ bool spp_index_ok(Ctl* ctl, long long idx, long long bound) {
  if (idx >= 0 && idx < bound) return true;
  atomicOr(&ctl->bad_index, 1u);
  return false;
}
#else
__device__ __forceinline__ bool spp_index_ok(Ctl*, long long, long long) { return true; }
#endif

struct DevState {
  int n;
  int cap;
  int D;                  /* cells per side */
  int morton_bits;
  uint32_t n_keys;        /* 4^morton_bits */
  float4* pos;
  float4* half;
  float4* half2;
  float* theta;
  int2* img;
  uint32_t* id;
  uint32_t* inv;          /* particle id -> slot (ring neighbours of membrane beads) */
  float4* kacc;
  float* dth;             /* rotational noise of the current step (multi-stage integrators) */
  float2* ref;
  float4* pos_alt;
  float* theta_alt;
  int2* img_alt;
  uint32_t* id_alt;
  uint32_t* key;
  uint32_t* rank;
  uint32_t* cell_count;
  uint32_t* cell_start;
  uint32_t* scan_tmp;     /* block sums of the scan */
  int32_t* nbr;
  int32_t* nn;
  int32_t* long_q;        /* particles whose list k_sort_long orders (n entries) */
  unsigned long long* nn_lanes; /* list entries per id % 4, 16 bits each (lanes > 1), else NULL */
  int32_t* tumble;        /* run-and-tumble state by particle id (SPP_NOISE_TUMBLE), else NULL */
  Ctl* ctl;
  double* red;            /* reduction scratch (polarization) */
};

/* api.cu: the device state, constants and stream of an uploaded system
 * (observables.cu), and the host-launch counter */
int spp_internal_view(SppSystem* s, DevState* d, SppConsts* k, cudaStream_t* st);
void spp_internal_count_launches(SppSystem* s, int n);
/* api.cu: the marked-frame buffers of spp_ring_motion (n entries each, by
 * particle id; allocated on first use) and the mark's step (-1: none) */
int spp_internal_mark(SppSystem* s, double2** xy, float** th, int64_t** step);
/* api.cu: the absolute step counter (waits for the stream); -1 on error */
int64_t spp_internal_step(SppSystem* s);
/* api.cu: the time step as given (double) */
double spp_internal_dt(SppSystem* s);

/* api.cu: sets the message spp_last_error() returns on the calling thread */
void spp_internal_set_error(const char* msg);

/* kernels_cells.cu */
void launch_bin_count(const SppConsts& k, const DevState& d, cudaStream_t s, int64_t* launches);
void launch_scan(const DevState& d, cudaStream_t s, int64_t* launches);
/* exclusive scan of n <= scan_max_elements() counts; block_tmp holds
 * ceil(n / 4096) entries */
void launch_scan_u32(const uint32_t* in, uint32_t n, uint32_t* block_tmp, uint32_t* out,
                     cudaStream_t s, int64_t* launches);
uint32_t scan_max_elements();
void launch_scatter(const DevState& d, cudaStream_t s, int64_t* launches);
void launch_build_list(const SppConsts& k, const DevState& d, int with_list, cudaStream_t s,
                       int64_t* launches);
void launch_pairs_count(const SppConsts& k, const DevState& d, float r2, unsigned long long* counter,
                        int32_t* pi, int32_t* pj, long long cap, cudaStream_t s);
void launch_cells(const SppConsts& k, const DevState& d, int D, int rule, int32_t* cx, int32_t* cy,
                  cudaStream_t s);
/* Also checks the inputs (finite, positions in [-L, L)) into Ctl::bad_*;
 * img_xy (may be NULL): 2n int32 box-crossing counters, x then y. */
void launch_init_state(const SppConsts& k, const DevState& d, const float* x, const float* y,
                       const float* th, const int32_t* img_xy, cudaStream_t s);
/* img_xy: 2n int32, x counters then y counters (particle-id order) */
void launch_gather_state(const SppConsts& k, const DevState& d, float* x, float* y, float* th,
                         int32_t* img_xy, cudaStream_t s);

/* kernels_step.cu */
void prepare_abp_stage();
void launch_abp_stage(const SppConsts& k, const DevState& d, int stage, int nstages,
                      cudaGraphConditionalHandle cond, int use_cond, cudaStream_t s,
                      int64_t* launches);
void launch_vicsek_step(const SppConsts& k, const DevState& d, cudaStream_t s, int64_t* launches);
/* Whole Vicsek steps of a small system in one thread-block cluster
 * (k_vicsek_small): at most SPP_SMALL_MAX_N particles, fewer than 65536
 * cells, and SPP_SMALL_MAX_SMEM bytes of cell-ordered copy plus cell table
 * per CTA. */
#define SPP_SMALL_MAX_N 16384
#define SPP_SMALL_MAX_SMEM (224 * 1024)
bool vicsek_small_fits(const SppConsts& k, const DevState& d);
int launch_vicsek_small(const SppConsts& k, const DevState& d, int nsteps, cudaStream_t s, int64_t* launches);
void launch_polarization(const DevState& d, cudaStream_t s);
/* the two fixed-point heading sums added into sums[0..1] (zeroed by the caller) */
void launch_polarization_into(const DevState& d, unsigned long long* sums, cudaStream_t s);

#endif
