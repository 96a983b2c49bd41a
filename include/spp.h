/*
 * spp.h -- C ABI of the GB300 (sm_103a) per-step particle update.
 *
 * The reference (hamidallaei/SPP) has no binary interface.  Its hot path is a
 * set of header-only C++ classes selected at compile time: Box
 * (parallel/box.h:15-58, serial/box.h:15-61), the Particle models
 * (shared/particle.h) and Cell (shared/cell.h:8-41), configured through
 * mutable globals (shared/parameters.h:60-99) and static setters
 * (shared/particle.h:106-121, 524-557).  This header replaces that surface
 * with plain functions on an opaque handle.  Each entry point names the
 * reference member it stands in for.
 *
 * Conventions
 *   - Box is [-L, L) x [-L, L) with L the half-width, as Lx in the reference
 *     (shared/c2dvector.h:67-73, shared/parameters.h:71-74).
 *   - Every function returns an int status (SPP_OK == 0).  The reference
 *     prints and calls exit(0) or MPI_Abort instead (shared/cell.h:45-49,
 *     parallel/box.h:224-228, parallel/node.h:696).
 *   - The handle owns all device memory; the caller owns host buffers.  One
 *     handle is driven from one host thread and one CUDA stream.
 *   - Host arrays are indexed by particle id (the order of upload), no matter
 *     how the device reorders particles internally.
 */
#ifndef SPP_H
#define SPP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPP_ABI_VERSION 1

enum SppStatus {
  SPP_OK = 0,
  SPP_ERR_INVALID = 1,     /* bad argument or parameter combination */
  SPP_ERR_ALLOC = 2,       /* device or host allocation failed */
  SPP_ERR_CUDA = 3,        /* a CUDA runtime call failed */
  SPP_ERR_OVERFLOW = 4,    /* neighbour-list or fixed-point range exceeded */
  SPP_ERR_TIMEOUT = 5,     /* a bounded device wait gave up */
  SPP_ERR_UNSUPPORTED = 6, /* model/integrator pair not built */
  SPP_ERR_NUMERIC = 7,     /* non-finite value detected */
  SPP_ERR_BOUNDS = 8       /* a kernel met an index out of range (builds with SPP_CHECKED) */
};

/* Particle models (shared/particle.h). */
enum SppModel {
  SPP_MODEL_VICSEK = 0,            /* theta_i <- arg(sum_{|r_ij|<r} e^{i theta_j}) + eta xi, self included */
  SPP_MODEL_VICSEK_REF_ANGLE = 1,  /* VicsekParticle, shared/particle.h:145-189 (raw-angle average) */
  SPP_MODEL_VICSEK_REF_VECTOR = 2, /* VicsekParticle2, shared/particle.h:193-250 */
  SPP_MODEL_CONTINUOUS = 3,        /* ContinuousParticle, shared/particle.h:254-378 */
  SPP_MODEL_ABP = 4,               /* RepulsiveParticle, shared/particle.h:499-786 */
  SPP_MODEL_BEADS = 5              /* ActiveBrownianChain nb=1 + ring membranes, shared/particle.h:792-1056 */
};

enum SppIntegrator { SPP_INT_EULER = 1, SPP_INT_RK2 = 2, SPP_INT_RK4 = 4 };

enum SppForceLaw {
  SPP_FORCE_NONE = 0,
  SPP_FORCE_HARMONIC = 1,  /* k (1 - d / r_rep) along dr/d for d < r_rep (r_rep = 2a) */
  SPP_FORCE_R12_TRUNC = 2  /* R12_Repulsive_Truncated, shared/force-fields.h:14-39 */
};

enum SppAlignMode {
  SPP_ALIGN_REFERENCE = 0, /* g sin(theta_j - theta_i) / (pi R_a^2), shared/particle.h:752 */
  SPP_ALIGN_MEAN = 1       /* (g / n_i) sum sin(theta_j - theta_i), n_i counts self (shared/particle.h:561) */
};

/* Rotational noise of the swimmers of SPP_MODEL_BEADS. */
enum SppRotNoise {
  SPP_NOISE_GAUSSIAN = 0,  /* sqrt(2 Dr dt) N(0,1) per step (ActiveBrownianChain::Noise_Gen, particle.h:891-894) */
  SPP_NOISE_TUMBLE = 1     /* run and tumble (RTPChain::Noise_Gen, particle.h:1085-1103) */
};

enum SppBinRule {
  SPP_BIN_GEOMETRIC = 0,   /* cell = floor((x + L) D / 2L) */
  SPP_BIN_REFERENCE = 1    /* cell = (int)((int)(x + L) * D / 2L), serial/box.h:116-117 */
};

/* Runtime parameters; replaces the compile-time switches and globals of
 * shared/parameters.h and the static setters of shared/particle.h.
 * spp_params_init() fills the reference's defaults for a model. */
typedef struct SppParams {
  uint32_t struct_size;   /* sizeof(SppParams); checked by spp_create */
  int32_t model;          /* enum SppModel */
  int32_t integrator;     /* enum SppIntegrator */
  int32_t force_law;      /* enum SppForceLaw */
  int32_t align_mode;     /* enum SppAlignMode */
  int32_t n;              /* number of bodies */
  uint64_t seed;          /* Philox key */
  uint32_t system_id;     /* Philox counter word for a system inside a batch */
  int32_t n_rings;        /* SPP_MODEL_BEADS: ring membranes (bodies 0 .. n_rings*ring_size-1) */
  int32_t ring_size;      /* beads per ring */
  int32_t list_capacity;  /* neighbour-list slots per particle; 0 = automatic */
  double L;               /* half-width of the periodic box (Lx) */
  double dt;              /* time step (dt) */
  double v0;              /* self-propulsion speed (speed / F0) */
  double Dr;              /* rotational diffusion; noise sigma = sqrt(2 Dr dt) (Set_Dr, particle.h:106-110) */
  double eta;             /* Vicsek noise amplitude (noise_amplitude of the Vicsek models) */
  double g;               /* alignment strength */
  double alpha;           /* ContinuousParticle alpha */
  double r_align;         /* alignment radius */
  double r_rep;           /* repulsion cutoff */
  double k_rep;           /* repulsion amplitude (k, or A_p for R12) */
  double sigma_rep;       /* R12 sigma */
  double skin;            /* Verlet skin; list radius = max(r_align, r_rep) + skin */
  double beta_push;       /* VicsekParticle2::beta (particle.h:249) */
  double r_push;          /* VicsekParticle2::rc (particle.h:250) */
  double mu;              /* translational mobility of beads (m_parallel = m_perpendicular, particle.h:861-863) */
  double k_perp;          /* rotational mobility of beads (k_perpendicular) */
  double torque0;         /* intrinsic torque (ActiveBrownianChain::torque0) */
  double k_bond;          /* ring bond stiffness (Spring amplitude, force-fields.h:87-97) */
  double bond_rest;       /* ring bond rest length */
  double kappa_bend;      /* bending stiffness on consecutive bond angles */
  int32_t rot_noise;      /* enum SppRotNoise (swimmers of SPP_MODEL_BEADS) */
  int32_t gather_lanes;   /* threads per particle in the Verlet-list neighbour sums of the
                           * ABP and continuous models: 0 = automatic (4 up to 16,384
                           * particles, else 1), or 1 or 4 (spp_autotune chooses);
                           * single-bead SPP_MODEL_BEADS systems take 0 (one lane), 1 or
                           * 4; the other models take 0 or 1.  The lane count fixes the
                           * order in which neighbour terms are added, so it is part of
                           * the result */
  double tumble_rate;     /* RTPChain::lambda: a tumble starts with probability rate * dt per step */
  double tumble_time;     /* RTPChain::t_tumble: a tumble lasts while its elapsed time < t_tumble */
  double tumble_torque;   /* RTPChain::torque_tumble: dtheta = k_perp dt (+-1) torque_tumble per step */
  /* Multi-bead swimmers of SPP_MODEL_BEADS (ActiveBrownianChain with nb > 1,
   * shared/particle.h:856-876, 964-1012).  With chain_beads = 1 every body is
   * a single bead and the fields below are unused. */
  int32_t chain_beads;    /* beads per swimmer (nb), 1 .. SPP_MAX_CHAIN_BEADS */
  int32_t reserved2;
  double bead_separation; /* ActiveBrownianChain::separation: distance between a swimmer's beads */
  double sigma_chain;     /* ActiveBrownianChain::sigma_p: R12 sigma of bead pairs that involve a chain */
  double r_chain;         /* ActiveBrownianChain::repulsion_radius: their cutoff */
  /* Closed box with walls (the reference built without
   * PERIODIC_BOUNDARY_CONDITION, shared/parameters.h:6): no wrap and no
   * minimum image; the four box walls of Box::Init_Topology
   * (parallel/box.h:92-101) plus n_walls extra segments (Geometry::Add_Wall,
   * shared/geometry.h:34-47) act on every particle each stage
   * (parallel/box.h:296-302).  Built for SPP_MODEL_ABP (Wall::Interact
   * (RepulsiveParticle*), shared/wall.h:215-265) and SPP_MODEL_CONTINUOUS
   * (Wall::Interact(ContinuousParticle*), :192-213). */
  int32_t boundary;       /* enum SppBoundary */
  int32_t n_walls;        /* extra wall segments, 0 .. SPP_MAX_WALLS - 4 */
  double walls[4][4];     /* x1, y1, x2, y2 of the extra segments (point_1 -> point_2) */
  double A_w;             /* RepulsiveParticle::A_w: wall repulsion amplitude */
  double sigma_w;         /* RepulsiveParticle::sigma_w: its screening length */
  double r_c_w;           /* RepulsiveParticle::r_c_w: its cutoff */
  double r_f_w;           /* RepulsiveParticle::r_f_w: range of the wall alignment torque */
  double g_w;             /* RepulsiveParticle::g_w: wall alignment strength */
  double g_w_cont;        /* ContinuousParticle::gw: wall torque strength of the continuous model */
} SppParams;

/* Boundary of the box. */
enum SppBoundary {
  SPP_BOUNDARY_PERIODIC = 0,  /* periodic box [-L, L)^2 */
  SPP_BOUNDARY_WALLS = 1,     /* closed box: the box walls plus SppParams.walls */
  SPP_BOUNDARY_CIRCLE = 2     /* circular box of radius L (the reference built with CIRCULAR_BOX,
                                 parallel/box.h:285-294): no wrap, no walls; a particle beyond
                                 r = L - 1 turns away from the circle by the torque
                                 40 g (v x r)_z / (2 pi r (L - r)).  SPP_MODEL_ABP and
                                 SPP_MODEL_CONTINUOUS, n_walls = 0 */
};
#define SPP_MAX_WALLS 8

/* Largest chain_beads. */
#define SPP_MAX_CHAIN_BEADS 8

typedef struct SppObservables {
  int64_t step;           /* steps taken since upload */
  double t;               /* step * dt */
  double px, py;          /* mean heading vector (1/N) sum (cos, sin) */
  double polarization;    /* |(px, py)| (Node::Compute_Polarization, parallel/node.h:1565-1591) */
  int64_t n_rebuilds;     /* Verlet-list / cell rebuilds so far */
  int32_t n;
  int32_t list_capacity;
  int32_t max_neighbors;  /* largest list length at the last rebuild */
  int32_t cells_per_side;
  int64_t late_rebuilds;  /* list rebuilds decided only after some particle had moved more than
                             skin/2 since the previous build: pairs may have been missed (the
                             time step is too large for the skin) */
  int64_t list_regrowths; /* neighbour-list overflows met so far: each one grew the list and re-ran
                             the frozen steps */
  int64_t bulk_timeouts;  /* warps of the stage kernel whose bulk copy of list rows into shared
                             memory did not complete within the wait limit; they read the list from
                             global memory instead (same results; a diagnostic, expected 0) */
} SppObservables;

typedef struct SppSystem SppSystem;

/* ---- library ---- */
int spp_abi_version(void);
const char* spp_status_string(int status);
/* Last error message of the calling thread ("" if none). */
const char* spp_last_error(void);
/* Fill defaults for a model: the static initialisers of shared/particle.h
 * (e.g. RepulsiveParticle A_p=2, sigma_p=1, R_a=1.1, r_c=1.2, :774-786). */
int spp_params_init(SppParams* p, int model);
/* Mobilities of a swimmer of nb beads (ActiveBrownianChain::Set_nb,
 * shared/particle.h:856-876): out = {m_parallel, m_perpendicular,
 * k_perpendicular}.  nb = 1 gives {0.5, 0.5, 1}; nb > 1 the prolate-body
 * formulas of the aspect ratio 1 / ((separation (nb - 1) / sigma) + 1).  A
 * chain swimmer's speed is v0 = m_parallel F0, its intrinsic angular
 * velocity k_perpendicular torque0 (Set_R0: torque0 = m_parallel F0 /
 * (k_perpendicular R0)). */
int spp_chain_mobility(int nb, double separation, double sigma, double* out3);

/* ---- one system ---- */
/* Box constructor + Init (parallel/box.h:69-88, 123-151): validates the
 * parameters and allocates every device buffer.  No particles yet. */
int spp_create(const SppParams* p, SppSystem** out);
/* Releases the device buffers (the reference never frees, box.h:66,87). */
int spp_destroy(SppSystem* s);
/* Use the given cudaStream_t for all work on this handle (NULL: the handle's own). */
int spp_set_stream(SppSystem* s, void* cuda_stream);
/* Positions and headings, in particle-id order; replaces Positioning_Particles
 * / Sync / Load (parallel/box.h:106-119, 155-218, 222-243).  img_x/img_y
 * (may be NULL = zero) are box-crossing counters carried over from a
 * snapshot.  Bins the particles and builds the neighbour list (Update_Cells
 * + Update_Neighbor_List).  Sets the step counter (the Philox counter word)
 * to step0, so reloading a snapshot reproduces the same noise. */
int spp_upload_state(SppSystem* s, const float* x, const float* y, const float* theta,
                     const int32_t* img_x, const int32_t* img_y, int n, int64_t step0);
/* Gathers state back in particle-id order (Save, parallel/box.h:246-267, and
 * the Root_Gather of operator<<, :476-502).  img_x/img_y (may be NULL) count
 * box crossings: r_original = r + 2L * img. */
int spp_download_state(SppSystem* s, float* x, float* y, float* theta, int32_t* img_x,
                       int32_t* img_y, int n);
/* Run-and-tumble state (SPP_NOISE_TUMBLE) per particle id: RTPChain::
 * tumble_flag and tumble_elapesed_time (shared/particle.h:1063-1064) as one
 * integer, 0 while running and +-c during the c-th step of a tumble turning
 * by +-tumble_torque.  spp_upload_state starts every swimmer running;
 * spp_upload_tumble (after it) restores a saved state, so that a snapshot
 * of state + tumble + step counter resumes bit for bit.  SPP_ERR_INVALID
 * for systems without run and tumble and for out-of-range values. */
int spp_download_tumble(SppSystem* s, int32_t* state, int n);
int spp_upload_tumble(SppSystem* s, const int32_t* state, int n);
/* Multi_Step(nsteps) (parallel/box.h:394-439): nsteps full integrator steps.
 * The neighbour list is rebuilt on device when a particle has moved more
 * than skin/2 since the last build.  Asynchronous on the handle's stream;
 * errors raised on the device are reported by the next spp_sync. */
int spp_step(SppSystem* s, int nsteps);
/* Waits for the handle's stream and reports device-side status. */
int spp_sync(SppSystem* s);
/* Polarization and counters (Save_Polarization, parallel/box.h:467-473). */
int spp_observables(SppSystem* s, SppObservables* out);
/* Parity hook: the unique pairs (i < j, particle ids) with |r_ij| < r under
 * the kernels' FP32 predicate, found through the device cell list
 * (Cell::Neighbor_List, shared/cell.h:74-103).  r must not exceed the list
 * radius.  *n_pairs receives the full count even when it exceeds cap. */
int spp_pairs(SppSystem* s, double r, int32_t* pi, int32_t* pj, int cap, int64_t* n_pairs);
/* Parity hook: cell coordinates of every particle (id order) for a grid of
 * D x D cells under the given SppBinRule (Box::Update_Cells, serial/box.h:107-134). */
int spp_cells(SppSystem* s, int D, int rule, int32_t* cell_x, int32_t* cell_y, int n);

/* ---- order parameters and pair statistics ----
 * The reference computes these offline from saved frames:
 * Compute_Order_Parameters (analyze/analyze.h:121-146) with the error bar of
 * Stat::Compute / Find_Correlation_Length (analyze/statistics.h:35-82), and
 * Pair_Distribution (analyze/analyze.h:365-424).  Here the frames come from
 * the device. */
typedef struct SppOrderStats {
  int64_t samples;
  double mean, mean_square, variance, std, min, max;
  double corr_len;          /* first lag whose normalised autocorrelation is < 0.01 (T/2 - 1 if none) */
  double error;             /* sqrt(variance * corr_len / samples) */
  double sigma2;            /* variance * area (analyze.h:144) */
  double p4_mean;           /* mean of P^4 */
  double binder;            /* 1 - <P^4> / (3 <P^2>^2) */
  double binder_reference;  /* 1 - <P^4> / (3 <P^2>), as analyze.h:145 writes it */
} SppOrderStats;
/* Statistics of a polarization series p[0..T-1] (host computation, T >= 2);
 * area = the box area (2L)^2 for sigma2. */
int spp_order_parameters(const double* p, int T, double area, SppOrderStats* out);
/* Advances the system nframes x every steps and records P after every
 * `every` steps (px, py may be NULL).  P is the exact fixed-point heading sum
 * of spp_observables. */
int spp_polarization_series(SppSystem* s, int nframes, int every, double* p, double* px, double* py);
/* Radial pair histogram of the current state: counts[b] = number of ordered
 * pairs (i != j) with minimum-image distance d < r_max and
 * b = min(nbins - 1, (int)(d / (r_max / nbins))) in FP32.  r_max <= 2L/3,
 * 1 <= nbins <= 4096.  g(r) = counts[b] / (N rho pi ((r+dr)^2 - r^2)). */
int spp_radial_distribution(SppSystem* s, double r_max, int nbins, uint64_t* counts);
/* Pair_Distribution (analyze/analyze.h:365-424) of the current state: for
 * ordered pairs (j, k), j != k, the plain (not minimum-image) difference
 * dr = r_k - r_j in the frame of j's heading, t_y = v_j . dr and
 * t_x = v_j.y dr.x - v_j.x dr.y; pairs with |t_x| < lx and |t_y| < ly add
 * one to counts[x * gy + y], x = (int)(gx ((t_x / lx) + 1) / 2),
 * y = (int)(gy ((t_y / ly) + 1) / 2), in FP32.  sqrt(lx^2 + ly^2) <= 2L/3,
 * 1 <= gx, gy and gx * gy <= 65536. */
int spp_pair_distribution(SppSystem* s, double lx, double ly, int gx, int gy, uint64_t* counts);
/* Shape of each ring vesicle of a bead model (Box::Compute_All_Variables,
 * parallel/beadbox.h:325-434, which does this for the one membrane of a
 * box): centre of mass, gyration tensor xx = <x^2> - <x>^2 (and yy, xy),
 * its eigenvalues, Rg = sqrt(xx + yy) and asphericity
 * Delta = ((l1 - l2) / (l1 + l2))^2, of the ring's beads (mb_) and of the
 * swimmers of the ring (sw_: the swimmers_per_ring consecutive swimmers
 * placed in it), from the unwrapped positions.  out[n_rings]. */
typedef struct SppRingShape {
  double mb_cm_x, mb_cm_y, mb_xx, mb_yy, mb_xy, mb_lambda1, mb_lambda2, mb_Rg, mb_Delta;
  double sw_cm_x, sw_cm_y, sw_xx, sw_yy, sw_xy, sw_lambda1, sw_lambda2, sw_Rg, sw_Delta;
} SppRingShape;
int spp_ring_shapes(SppSystem* s, SppRingShape* out, int n_rings);
/* The motion terms of Box::Compute_All_Variables (parallel/beadbox.h:325-434)
 * per ring vesicle, between the frame of the last mark and now.  The
 * reference keeps r_original, theta and t of a saved frame
 * (Save_Particles_Positions, :315-322); spp_ring_motion_mark saves the same
 * on the device.  spp_ring_motion then gives, with v = (r - r_old) / (t -
 * t_old) and the swimmers' spin = (theta - theta_old, folded to [-pi, pi))
 * / (t - t_old): the centre-of-mass velocities, the angular momenta about
 * the centres (the swimmers' in the membrane's frame, as the reference
 * writes it), the rotation rates mb_l / (mb_xx + mb_yy) and sw_l / (sw_xx +
 * sw_yy + |mb_cm - sw_cm|^2), and the mean swimmer spin; then it marks the
 * current frame, as the reference does.  SPP_ERR_INVALID without a mark or
 * if no step was taken since it. */
typedef struct SppRingMotion {
  double mb_v_cm_x, mb_v_cm_y, mb_l, mb_omega;
  double sw_v_cm_x, sw_v_cm_y, sw_l, sw_omega, sw_spin;
} SppRingMotion;
int spp_ring_motion_mark(SppSystem* s);
int spp_ring_motion(SppSystem* s, SppRingMotion* out, int n_rings);

/* ---- batches of independent systems (parameter sweeps) ----
 * Replaces the task farm of serial/mpi-main.cpp:157-176 (one MPI rank per
 * realisation, run one after another): every system of a sweep shares one
 * set of device arrays and one launch per phase of a step.  Vicsek-family
 * models.  Per system the device keeps the polarization P each step, its
 * first four moments over a start-up window and its mean over the
 * stationary part of the run (Compute_Order_Parameters, analyze/analyze.h:
 * 121-146, computed online). */
typedef struct SppSweepStats {
  int64_t steps;            /* steps taken by this system */
  int32_t active;           /* 1 while stepping; 0 once retired or finished */
  int32_t reserved;
  int64_t window_steps;     /* steps inside the start-up window */
  double p_mean, p_var, p_kurt;   /* moments of P over the window (kurtosis = m4 / var^2) */
  int64_t stationary_steps; /* samples of P after stationary_from */
  double p_stationary;      /* their mean */
  double p2_stationary;     /* mean of P^2 */
  double p_last;
  double p4_stationary;     /* mean of P^4 */
  double binder;            /* 1 - <P^4> / (3 <P^2>^2) over the stationary samples */
  double binder_reference;  /* 1 - <P^4> / (3 <P^2>), as analyze/analyze.h:145 writes it */
} SppSweepStats;

typedef struct SppBatch SppBatch;
/* systems[s] describes system s (model, n, L, eta, v0, dt, r_align, seed,
 * system_id -- the Philox counter word keeping systems independent). */
int spp_batch_create(const SppParams* systems, int n_systems, SppBatch** out);
int spp_batch_destroy(SppBatch* b);
/* Start-up window for the moments, start of the stationary average, and the
 * step count after which a system stops (0 = never). */
int spp_batch_set_windows(SppBatch* b, int window_steps, int stationary_from, int max_steps);
/* Positions and headings of all systems concatenated in system order;
 * resets every system's step counter and statistics. */
int spp_batch_upload(SppBatch* b, const float* x, const float* y, const float* theta, int total_n);
int spp_batch_step(SppBatch* b, int nsteps);
int spp_batch_poll(SppBatch* b, SppSweepStats* out, int n_systems);
/* Stops the listed systems (retired by the sweep's stopping rule). */
int spp_batch_retire(SppBatch* b, const int32_t* systems, int count);
/* Restarts retired systems where they stopped (not those past max_steps). */
int spp_batch_resume(SppBatch* b, const int32_t* systems, int count);
int spp_batch_download(SppBatch* b, float* x, float* y, float* theta, int32_t* img_x,
                       int32_t* img_y, int total_n);
int64_t spp_batch_kernel_launches(SppBatch* b);
/* spp_batch_step bracketed by CUDA events on the batch's stream (ms). */
int spp_batch_time_steps(SppBatch* b, int nsteps, double* ms);

/* ---- sweep surrogate: ensemble MLP (no counterpart in the reference) ----
 * E independent networks in -> 128 -> 128 -> 1 (GELU), BF16 weights with
 * FP32 masters, FP32 accumulation, trained full-batch with Adam on the
 * device by the library's own forward/backward kernels.  Parameters per
 * member (spp_mlp_num_params floats): W1[128][in] b1[128] W2[128][128]
 * b2[128] W3[128] b3; arrays over members are [E][P]. */
typedef struct SppMlp SppMlp;
int spp_mlp_create(int ensemble, int in_dim, SppMlp** out);
int spp_mlp_destroy(SppMlp* m);
int spp_mlp_num_params(SppMlp* m);
/* Sets the FP32 masters (and their BF16 copies); resets Adam's moments. */
int spp_mlp_set_params(SppMlp* m, const float* theta);
int spp_mlp_get_params(SppMlp* m, float* theta);
/* y[E][B] for inputs x[B][in]. */
int spp_mlp_predict(SppMlp* m, const float* x, int B, float* y);
/* Gradient [E][P] of each member's weighted squared error
 * L_e = sum_s w[e][s] (y_e(x_s) - t_s)^2 / sum_s w[e][s], and L_e itself.
 * weights[E][B] may be NULL (the mean-squared error); a member's weights are
 * finite, >= 0 and not all zero (a zero weight leaves a sample out of that
 * member's fit, as in K-fold bagging). */
int spp_mlp_grad(SppMlp* m, const float* x, const float* t, const float* weights, int B, float* grad,
                 float* loss);
/* iters Adam steps (beta 0.9 / 0.999, eps 1e-8) at learning rate lr on the
 * full batch with the loss of spp_mlp_grad; loss[E] (may be NULL) after the
 * last step. */
int spp_mlp_train(SppMlp* m, const float* x, const float* t, const float* weights, int B, int iters, float lr,
                  float* loss);

/* ---- tangent-space Lyapunov spectrum (continuous model) ----
 * Replaces LyapunovBox (parallel/lyapunovbox.h:11-28): Init_Deviation
 * (:32-42), Evolution_Reorthonormalize (:128-194) and Lyapunov_Exponent
 * (:197-255).  The reference evolves k finite perturbations of size 1e-7 as
 * full clones of the system; here k tangent vectors follow the linearised
 * integrator (RK2/RK4 of SPP_MODEL_CONTINUOUS with alpha = 0, no
 * repulsion) and are renormalised every renorm_every steps in FP64
 * (Gram-Schmidt in Cholesky-QR form, as VectorSet::Renormalize,
 * shared/vector-set.h:118-127), the log of each stretch summed in FP64. */
/* k <= 8 tangent vectors of dimension 3n, N(0,1) entries from the Philox
 * stream keyed by seed, orthonormalised; resets the log-stretch sums. */
int spp_lyap_init(SppSystem* s, int k, uint64_t seed);
/* Replaces the tangent vectors ([k][x|y|theta][n], particle-id order)
 * without renormalising them; resets the sums. */
int spp_lyap_set_vectors(SppSystem* s, const float* v, int k);
/* nsteps steps of the base and tangent dynamics, renormalising after every
 * renorm_every steps and at the end. */
int spp_lyap_step(SppSystem* s, int nsteps, int renorm_every);
/* Exponents lambda_a = (sum of log stretches) / elapsed time, a < k. */
int spp_lyap_exponents(SppSystem* s, double* lambda, int k, double* elapsed);
/* The current (orthonormal) tangent vectors, [k][x|y|theta][n]. */
int spp_lyap_vectors(SppSystem* s, float* v, int k);

/* ---- measurement helpers (no reference counterpart) ---- */
typedef struct SppProfile {
  int64_t steps;          /* steps advanced by the profiling run */
  int64_t stage_launches; /* force/integrator stage kernels timed */
  double stage_ms;        /* summed CUDA-event time of those launches */
  int64_t rebuilds;       /* list rebuilds that happened during the run */
  double rebuild_ms;      /* summed CUDA-event time of the rebuild sequences */
  double total_ms;        /* event time from the first to the last launch */
} SppProfile;
/* Advances nsteps steps with direct (non-graph) launches, bracketing every
 * stage kernel and every rebuild sequence with CUDA events on the handle's
 * stream.  The state advances exactly as under spp_step. */
int spp_profile(SppSystem* s, int nsteps, SppProfile* out);
/* spp_step(nsteps) bracketed by CUDA events on the handle's stream; waits for
 * completion and returns the elapsed device time in *ms.  The end event is
 * recorded after any list-overflow recovery has finished the requested
 * steps, so recovered steps are timed as well (the host round trip of a
 * recovery included). */
int spp_time_steps(SppSystem* s, int nsteps, double* ms);
/* ---- autotuner of the launch shape (no counterpart in the reference) ----
 * The reference fixes its cell and list geometry from compile-time globals
 * (shared/parameters.h:93-99).  spp_autotune() times the candidate shapes
 * of a Verlet-list system (SPP_MODEL_ABP, _CONTINUOUS, _BEADS) on the device
 * and writes the fastest into *p:
 *   SPP_TUNE_LANES  gather_lanes in {1, 4} (ABP, continuous and single-bead
 *                   bead models): threads
 *                   per particle in the neighbour sums.  Changes the order of
 *                   the neighbour additions, hence the low bits of the result.
 *   SPP_TUNE_SKIN   skin in {0.5, 1, 1.5, 2} x p->skin: list length against
 *                   rebuild frequency.  Every neighbour list is summed in
 *                   particle-id order, so the trajectory does not depend on
 *                   the skin; candidates whose trial missed a rebuild
 *                   (late_rebuilds > 0) are not chosen.  (Lyapunov runs: the
 *                   skin moves the list-overflow recoveries, each of which
 *                   adds a renormalisation point, so the exponents agree
 *                   across skins to rounding, not bit for bit.)
 * Each candidate is a fresh system given (x, y, theta) (host arrays of
 * p->n values in particle-id order), stepped trial_steps steps untimed
 * (graph capture, list growth), then trial_steps steps timed with CUDA
 * events (spp_time_steps).  The
 * report lists every candidate in the order tried.  Takes the device memory
 * of one system at a time. */
#define SPP_TUNE_LANES 1
#define SPP_TUNE_SKIN 2
#define SPP_TUNE_MAX_CANDIDATES 8
typedef struct SppTuneCandidate {
  int32_t gather_lanes;
  int32_t status;         /* SPP_OK, or the status that ruled the candidate out */
  double skin;
  double ms_per_step;     /* timed device time per step (0 if not measured) */
  int64_t late_rebuilds;  /* rebuilds that came later than the skin allows, in the trial */
} SppTuneCandidate;
typedef struct SppTuneReport {
  int32_t n_candidates;
  int32_t best;           /* index of the chosen candidate */
  SppTuneCandidate c[SPP_TUNE_MAX_CANDIDATES];
} SppTuneReport;
int spp_autotune(SppParams* p, const float* x, const float* y, const float* theta, int trial_steps,
                 int what, SppTuneReport* report);
/* Number of kernels this handle has launched (graph replays count each
 * kernel node they run). */
int64_t spp_kernel_launches(SppSystem* s);
/* The cudaStream_t the handle launches on. */
void* spp_stream(SppSystem* s);

/* ---- pair search that allocates nothing (no counterpart in the reference) ----
 * For callers that cannot allocate GPU memory themselves or through this
 * library: a component running under another owner's fixed memory budget
 * (a host framework with its own pool), or a latency-critical loop where a
 * cudaMalloc/cudaFree would synchronise the device.  The caller passes its
 * own device buffers: x, y (n positions, already wrapped into [-L, L)),
 * pi, pj (room for cap pairs) and count (one int64).  The unique pairs
 * (i < j, indices into x/y) with |r_ij| < r under the FP32 predicate of
 * spp_pairs() are written there, and *count receives the total, which may
 * exceed cap.  Work is enqueued on `stream` (a cudaStream_t, NULL for the
 * default stream); the results are ready once that stream has completed.
 * Scratch is one static device array of about 1.8 MB that every GPU loading
 * this library holds until the process exits; n <= SPP_NOALLOC_MAX_N and at
 * most SPP_NOALLOC_MAX_CELLS_PER_SIDE^2 cells, larger n is rejected with
 * SPP_ERR_INVALID.  The first call in a CUDA context (each device's primary
 * context, a context the caller made current, or a new primary context after
 * cudaDeviceReset) looks up the array's device address in that context
 * (cudaGetSymbolAddress) and remembers it by the context's id; make that
 * first call before any stream capture (a first call inside a capture is
 * refused with SPP_ERR_INVALID).  Calls share the array: calls that overlap
 * on the GPU race and must be ordered by the caller; the host-side set-up
 * is safe from several threads.  Allocates nothing: no cudaMalloc, cudaFree
 * or allocating library routine is called. */
#define SPP_NOALLOC_MAX_N 65536
#define SPP_NOALLOC_MAX_CELLS_PER_SIDE 256
int spp_pairs_noalloc(const float* x, const float* y, int n, double L, double r, int32_t* pi,
                      int32_t* pj, int64_t cap, int64_t* count, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SPP_H */
