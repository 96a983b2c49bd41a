/* spp_batch.cuh -- device layout of a batch of independent systems. */
#ifndef SPP_BATCH_CUH
#define SPP_BATCH_CUH
#include "spp_internal.cuh"

/* One row of the per-system offset table. */
struct BatchSys {
  SppConsts k;            /* the system's constants (box, noise, Philox key and system id) */
  uint32_t p_off, n;      /* particle range [p_off, p_off + n) */
  uint32_t c_off, D;      /* cell range [c_off, c_off + D*D), row-major D x D grid */
  uint32_t active;        /* 0: retired or finished, copied through without work */
  uint32_t steps;         /* steps taken (the system's Philox step counter) */
};

/* Per-system accumulators of the polarization P. */
struct BatchStats {
  double w1, w2, w3, w4;  /* sums of P^1..P^4 over the first `window` steps */
  double s1, s2, s4;      /* sums of P, P^2, P^4 after `stationary_from` steps */
  long long ns;           /* number of stationary samples */
  double p_last;          /* P of the last step */
  long long sx, sy;       /* fixed-point heading sums of the current step (units 2^-27) */
};

/* Per system: where it sits in the compact launch space of the active
 * systems (rebuilt by the host when the set of active systems changes). */
struct SysAct {
  uint32_t a_coff;        /* first cell of the system in the compact cell space */
  int32_t a_corr;         /* slot = compact particle index + a_corr */
};

struct DevBatch {
  int n_total, n_sys;
  int window, stationary_from, max_steps;
  BatchSys* sys;
  BatchStats* stats;
  uint32_t* sys_of;       /* particle slot -> system (static: binning stays inside a system's range) */
  float4 *pos, *pos_alt;
  float *theta, *theta_alt;
  int2 *img, *img_alt;
  int4* fx_alt;           /* fixed-point (cos hi, cos lo, sin hi, sin lo) of the cell-ordered copy */
  uint32_t *id, *id_alt;  /* particle id within its system */
  uint32_t *key, *rank;
  uint32_t *cell_count, *cell_start, *scan_tmp;
  Ctl* ctl;
  /* compact launch space: the particles and cells of the systems that were
   * active when the host last looked; binning, scan, scatter and step run
   * over these only */
  int n_act, n_act_keys;
  uint32_t* act_sys;      /* compact particle index -> system */
  SysAct* sact;           /* [n_sys] */
  uint32_t* flags;        /* [n_sys] snapshot of the active flags (k_batch_flags) */
};
#endif
