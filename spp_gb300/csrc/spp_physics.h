/*
 * spp_physics.h -- per-pair and per-particle FP32 arithmetic of the step.
 *
 * Written once, compiled into the sm_103a kernels and into the CPU mirror
 * (oracle/spp_mirror32.c), so that the mirror reproduces the kernels' bits
 * and can prove that binning, neighbour lists, particle reordering and graph
 * replay neither lose nor add anything.  The result does not depend on the
 * order the neighbours are visited in: the Verlet-list models sum in FP32 in
 * ascending neighbour id (their lists are sorted by id at every build), and
 * the Vicsek models in exact split int32 fixed point (spp_fp32.h).
 *
 * All interactions are written in gather form (particle i sums the terms it
 * receives from each neighbour j).  The reference visits every pair once and
 * applies Newton's third law to both particles (shared/cell.h:112-128); the
 * gather form computes the same sums without write conflicts between threads.
 */
#ifndef SPP_PHYSICS_H
#define SPP_PHYSICS_H

#include "spp_fp32.h"
#include "../../include/spp.h"

/* Constants of one system, rounded once from the double parameters. */
typedef struct SppConsts {
  int32_t model, integrator, force_law, align_mode;
  uint64_t seed;
  uint32_t system;
  int32_t n;
  float L, L2;                 /* half width, box length */
  float dt, half_dt, dt6;
  float v0, v0dt;
  float sigma;                 /* rotational noise sqrt(2 Dr dt) */
  float eta;
  float g, g_over_area;        /* g / (pi R_a^2) */
  float ral2;                  /* alignment radius squared */
  float rrep2, inv_rrep, k_rep, sigma_rep, c13;
  float k_over_rrep;           /* k_rep / r_rep (harmonic law: t = k_rep r - k_rep / r_rep) */
  float one_minus_alpha_over_pi, alpha_over_pi;
  float beta_push, r_push, rpush2;
  float rlist, rlist2;         /* Verlet list radius */
  float half_skin;             /* rebuild threshold on displacements */
  float interior;              /* |x|,|y| below this: no list neighbour is across the boundary */
  /* ring membranes + swimmers (SPP_MODEL_BEADS) */
  int32_t n_beads;             /* bodies [0, n_beads) are membrane beads */
  int32_t ring_size;
  float mu;                    /* translational mobility (m_parallel = m_perpendicular) */
  float ang_drift;             /* k_perp * torque0: intrinsic angular velocity of swimmers */
  float k_bond, bond_rest, kappa;
  /* run and tumble (SPP_NOISE_TUMBLE): a tumble starts when the 24-bit
   * uniform of the start draw is < tumble_u24, i.e. exactly when the
   * reference's double u < rate * dt; it lasts tumble_steps steps, the count
   * of dt additions after which the reference's double elapsed time first
   * reaches t_tumble; each tumbling step turns by +-tumble_dth */
  int32_t tumble;
  uint32_t tumble_u24;
  int32_t tumble_steps;
  float tumble_dth;
  /* multi-bead swimmers (chain_nb > 1): bead a of a swimmer with heading v
   * sits at v chain_off[a] from its centre; bead pairs involving a chain
   * use R12 with chain_sigma / chain_rc2 / chain_c13 (the membrane constants
   * above stay for bead-bead pairs); chain_reach2 bounds the centre distance
   * of two bodies that have any bead pair within the cutoff */
  int32_t chain_nb;
  float chain_off[SPP_MAX_CHAIN_BEADS];
  float chain_sigma, chain_rc2, chain_c13, chain_reach2;
  float chain_f0;              /* F0 = v0 / m_parallel */
  float chain_mperp, chain_dm; /* m_perpendicular, m_parallel - m_perpendicular */
  float chain_k;               /* k_perpendicular */
  float chain_torque0;
  /* lanes per particle in the neighbour sums of the Verlet-list kernels
   * (1, or SPP_GATHER_LANES for the ABP / continuous models: by default up
   * to SPP_LANES_MAX_N particles, where one thread per particle leaves the
   * GPU idle; SppParams.gather_lanes overrides): a neighbour belongs to lane id % lanes; each lane sums its
   * neighbours in id order and the lane sums combine as
   * (p0 + p1) + (p2 + p3) */
  int32_t lanes;
  /* closed box (SPP_BOUNDARY_WALLS): no wrap, no minimum image, and the
   * n_walls segments below act on every particle; segment w starts at
   * (wall_x1, wall_y1), runs along the unit vector (wall_ex, wall_ey) for
   * wall_len */
  int32_t closed;
  int32_t n_walls;
  int32_t circle;              /* circular box (SPP_BOUNDARY_CIRCLE): closed, no walls */
  float circ_k;                /* 40 g / (2 pi): the circle's torque prefactor */
  float wall_x1[SPP_MAX_WALLS], wall_y1[SPP_MAX_WALLS], wall_x2[SPP_MAX_WALLS], wall_y2[SPP_MAX_WALLS];
  float wall_ex[SPP_MAX_WALLS], wall_ey[SPP_MAX_WALLS], wall_len[SPP_MAX_WALLS];
  float wall_theta[SPP_MAX_WALLS];   /* Wall::theta, the direction angle (wall.h:38-41) */
  float wall_A, wall_sigma, wall_rc, wall_rf, wall_g_over_pi;
  float wall_cut;              /* e^(-r_c/sigma) (1/r_c^2 + 1/(sigma r_c)), the truncation shift */
  float wall_gcont_over_2pi;   /* ContinuousParticle::gw / (2 pi) */
  uint32_t philox_ks[20];      /* Philox round keys of seed (spp_philox_round_keys) */
} SppConsts;

/* spp_draw(k->seed, k->system, pid, step, stream) from the precomputed
 * round keys: the same four words. */
SPP_HD spp_u32x4 spp_draw_k(const SppConsts* k, uint32_t pid, uint32_t step, uint32_t stream) {
  return spp_philox4x32_10_ks(pid, step, stream, k->system, k->philox_ks);
}

#define SPP_GATHER_LANES 4
#ifndef SPP_LANES_MAX_N
#define SPP_LANES_MAX_N 16384
#endif

/* ActiveBrownianChain::Set_nb (shared/particle.h:856-876): {m_parallel,
 * m_perpendicular, k_perpendicular} of a swimmer of nb beads. */
static inline void spp_chain_mobility_d(int nb, double sep, double sigma, double* m) {
  if (nb <= 1) {
    m[0] = 0.5; m[1] = 0.5; m[2] = 1.0;
    return;
  }
  const double ar = 1.0 / ((sep * (nb - 1) / sigma) + 1.0);
  const double e2 = 1.0 - ar * ar;
  const double e = sqrt(e2);
  const double lg = log((1.0 + e) / (1.0 - e));
  m[0] = 1.0;
  m[1] = 0.5 * (2.0 * e + (3.0 * e2 - 1.0) * lg) / ((1.0 + e2) * lg - 2.0 * e);
  m[2] = 6.0 / (1.0 + ar * ar) / sigma / sigma;
}

/* Largest centre distance at which two bodies still interact: the pair
 * cutoff, alignment and push radii, and for chains the bead cutoff plus the
 * two half-lengths (nb - 1) separation / 2. */
static inline double spp_interaction_range(const SppParams* p) {
  double rc = p->model == SPP_MODEL_BEADS ? 0.0 : p->r_align;
  if (p->force_law != SPP_FORCE_NONE && p->r_rep > rc) rc = p->r_rep;
  if (p->model == SPP_MODEL_VICSEK_REF_VECTOR && p->r_push > rc) rc = p->r_push;
  if (p->model == SPP_MODEL_BEADS && p->chain_beads > 1 && p->force_law != SPP_FORCE_NONE) {
    const double reach = (p->chain_beads - 1) * p->bead_separation + p->r_chain;
    if (reach > rc) rc = reach;
  }
  return rc;
}

/* Host-side: round the double parameters to the kernels' floats. */
static inline void spp_consts_from_params(SppConsts* k, const SppParams* p) {
  k->model = p->model; k->integrator = p->integrator;
  k->force_law = p->force_law; k->align_mode = p->align_mode;
  k->seed = p->seed; k->system = p->system_id; k->n = p->n;
  spp_philox_round_keys(p->seed, k->philox_ks);
  k->L = (float)p->L; k->L2 = (float)(2.0 * p->L);
  k->dt = (float)p->dt; k->half_dt = (float)(0.5 * p->dt); k->dt6 = (float)(p->dt / 6.0);
  k->v0 = (float)p->v0; k->v0dt = (float)(p->v0 * p->dt);
  k->sigma = (float)sqrt(2.0 * p->Dr * p->dt);
  /* ContinuousParticle::Move (shared/particle.h:273-274) adds the Gaussian to
   * the torque and multiplies the sum by dt, so its Euler noise is sigma * dt. */
  if (p->model == SPP_MODEL_CONTINUOUS && p->integrator == SPP_INT_EULER)
    k->sigma = (float)(sqrt(2.0 * p->Dr * p->dt) * p->dt);
  k->eta = (float)p->eta;
  k->g = (float)p->g;
  k->g_over_area = p->r_align > 0 ? (float)(p->g / (3.14159265358979323846 * p->r_align * p->r_align)) : 0.0f;
  k->ral2 = (float)(p->r_align * p->r_align);
  if (p->force_law == SPP_FORCE_NONE || p->r_rep <= 0) {
    k->rrep2 = 0.0f; k->inv_rrep = 0.0f;
  } else {
    k->rrep2 = (float)(p->r_rep * p->r_rep);
    k->inv_rrep = (float)(1.0 / p->r_rep);
  }
  k->k_rep = (float)p->k_rep;
  k->k_over_rrep = (p->force_law == SPP_FORCE_NONE || p->r_rep <= 0) ? 0.0f : (float)(p->k_rep / p->r_rep);
  k->sigma_rep = (float)p->sigma_rep;
  {
    float q = (p->r_rep > 0) ? k->sigma_rep / (float)p->r_rep : 0.0f;
    float q2 = q * q, q4 = q2 * q2, q8 = q4 * q4;
    k->c13 = (q8 * q4) * q;
  }
  k->one_minus_alpha_over_pi = (float)((1.0 - p->alpha) / 3.14159265358979323846);
  k->alpha_over_pi = (float)(p->alpha / 3.14159265358979323846);
  k->beta_push = (float)p->beta_push;
  k->r_push = (float)p->r_push;
  k->rpush2 = (float)(p->r_push * p->r_push);
  {
    double rc = spp_interaction_range(p);
    double rl = rc + (p->skin > 0 ? p->skin : 0.0);
    k->rlist = (float)rl;
    k->rlist2 = (float)(rl * rl);
    k->half_skin = (float)(0.5 * (p->skin > 0 ? p->skin : 0.0));
    k->n_beads = p->model == SPP_MODEL_BEADS ? p->n_rings * p->ring_size : 0;
    k->ring_size = p->ring_size;
    k->mu = (float)p->mu;
    k->ang_drift = (float)(p->k_perp * p->torque0);
    k->k_bond = (float)p->k_bond;
    k->bond_rest = (float)p->bond_rest;
    k->kappa = (float)p->kappa_bend;
    k->interior = (float)(p->L - 2.0 * (rl + (p->skin > 0 ? p->skin : 0.0)));
  }
  k->tumble = (p->model == SPP_MODEL_BEADS && p->rot_noise == SPP_NOISE_TUMBLE) ? 1 : 0;
  k->tumble_u24 = 0u;
  k->tumble_steps = 0;
  k->tumble_dth = 0.0f;
  if (k->tumble) {
    const double thr = ceil((p->tumble_rate * p->dt) * 16777216.0);  /* 2^24 */
    k->tumble_u24 = thr <= 0.0 ? 0u : (thr >= 16777216.0 ? 16777216u : (uint32_t)thr);
    double e = 0.0;
    int32_t c = 0;
    while (e < p->tumble_time && c < 0x7fffffff) {
      e += p->dt;
      ++c;
    }
    k->tumble_steps = c;
  }
  {
    /* gather_lanes: 0 = automatic, else 1 or SPP_GATHER_LANES (ABP,
     * continuous and single-bead bead models; spp_create rejects the rest).
     * Automatic: four lanes for ABP and continuous systems of up to
     * SPP_LANES_MAX_N particles, else one. */
    const int auto_model = p->model == SPP_MODEL_ABP || p->model == SPP_MODEL_CONTINUOUS;
    const int lane_model = auto_model || (p->model == SPP_MODEL_BEADS && p->chain_beads <= 1);
    if (!lane_model || p->gather_lanes == 1)
      k->lanes = 1;
    else if (p->gather_lanes == SPP_GATHER_LANES)
      k->lanes = SPP_GATHER_LANES;
    else
      k->lanes = auto_model && p->n <= SPP_LANES_MAX_N ? SPP_GATHER_LANES : 1;
  }
  k->closed = p->boundary == SPP_BOUNDARY_WALLS || p->boundary == SPP_BOUNDARY_CIRCLE ? 1 : 0;
  k->n_walls = 0;
  k->circle = p->boundary == SPP_BOUNDARY_CIRCLE ? 1 : 0;
  k->circ_k = (float)(40.0 * p->g / (2.0 * 3.14159265358979323846));
  for (int w = 0; w < SPP_MAX_WALLS; ++w) {
    k->wall_x1[w] = k->wall_y1[w] = k->wall_x2[w] = k->wall_y2[w] = 0.0f;
    k->wall_ex[w] = k->wall_ey[w] = k->wall_len[w] = k->wall_theta[w] = 0.0f;
  }
  k->wall_A = k->wall_sigma = k->wall_rc = k->wall_rf = k->wall_g_over_pi = 0.0f;
  k->wall_cut = 0.0f;
  k->wall_gcont_over_2pi = 0.0f;
  if (k->closed && !k->circle) {
    /* Box::Init_Topology (parallel/box.h:97-101), then the extra segments */
    double seg[SPP_MAX_WALLS][4] = {{-p->L, -p->L, -p->L, p->L},
                                    {-p->L, p->L, p->L, p->L},
                                    {p->L, p->L, p->L, -p->L},
                                    {p->L, -p->L, -p->L, -p->L}};
    int nw = 4;
    for (int w = 0; w < p->n_walls && nw < SPP_MAX_WALLS; ++w, ++nw)
      for (int c = 0; c < 4; ++c) seg[nw][c] = p->walls[w][c];
    k->n_walls = nw;
    for (int w = 0; w < nw; ++w) {
      /* Wall::Init (shared/wall.h:27-41) */
      const double dx = seg[w][2] - seg[w][0], dy = seg[w][3] - seg[w][1];
      const double len = sqrt(dx * dx + dy * dy);
      k->wall_x1[w] = (float)seg[w][0];
      k->wall_y1[w] = (float)seg[w][1];
      k->wall_x2[w] = (float)seg[w][2];
      k->wall_y2[w] = (float)seg[w][3];
      {
        /* Wall::Init: atan of the direction, +pi when it points to -x, then
         * theta -= 2 pi (int)(theta / pi) */
        double th = atan((dy / len) / (dx / len));
        if (dx / len < 0.) th += 3.14159265358979323846;
        th -= 2 * 3.14159265358979323846 * (int)(th / 3.14159265358979323846);
        k->wall_theta[w] = (float)th;
      }
      k->wall_ex[w] = (float)(dx / len);
      k->wall_ey[w] = (float)(dy / len);
      k->wall_len[w] = (float)len;
    }
    k->wall_A = (float)p->A_w;
    k->wall_sigma = (float)p->sigma_w;
    k->wall_rc = (float)p->r_c_w;
    k->wall_rf = (float)p->r_f_w;
    k->wall_g_over_pi = (float)(p->g_w / 3.14159265358979323846);
    if (p->r_c_w > 0 && p->sigma_w > 0)
      k->wall_cut = (float)(exp(-p->r_c_w / p->sigma_w) *
                            (1.0 / (p->r_c_w * p->r_c_w) + 1.0 / (p->sigma_w * p->r_c_w)));
    k->wall_gcont_over_2pi = (float)(p->g_w_cont / (2.0 * 3.14159265358979323846));
  }
  k->chain_nb = (p->model == SPP_MODEL_BEADS && p->chain_beads > 1) ? p->chain_beads : 1;
  for (int a = 0; a < SPP_MAX_CHAIN_BEADS; ++a)
    k->chain_off[a] = a < k->chain_nb ? (float)(p->bead_separation * ((1 - k->chain_nb) / 2.0 + a)) : 0.0f;
  {
    double m[3];
    spp_chain_mobility_d(k->chain_nb, p->bead_separation, p->sigma_chain, m);
    const int chain = k->chain_nb > 1;
    k->chain_sigma = chain ? (float)p->sigma_chain : 0.0f;
    k->chain_rc2 = chain && p->force_law != SPP_FORCE_NONE ? (float)(p->r_chain * p->r_chain) : 0.0f;
    {
      float q = chain && p->r_chain > 0 ? k->chain_sigma / (float)p->r_chain : 0.0f;
      float q2 = q * q, q4 = q2 * q2, q8 = q4 * q4;
      k->chain_c13 = (q8 * q4) * q;
    }
    /* 1e-3 above the exact bound: a pure pre-test, never tighter than the
     * FP32 bead separations it guards */
    const double reach = ((k->chain_nb - 1) * p->bead_separation + p->r_chain) * 1.001;
    k->chain_reach2 = chain ? (float)(reach * reach) : 0.0f;
    k->chain_f0 = chain ? (float)(p->v0 / m[0]) : 0.0f;
    k->chain_mperp = chain ? (float)m[1] : 0.0f;
    k->chain_dm = chain ? (float)(m[0] - m[1]) : 0.0f;
    k->chain_k = chain ? (float)m[2] : 0.0f;
    k->chain_torque0 = chain ? (float)p->torque0 : 0.0f;
    /* RTPChain::Noise_Gen turns by k_perpendicular dt torque_tumble: the
     * swimmers' own k_perpendicular */
    if (k->tumble)
      k->tumble_dth = (float)(((chain ? m[2] : p->k_perp) * p->dt) * p->tumble_torque);
  }
}

/* Sort key of neighbour id in the Verlet lists: the id itself with one
 * lane, else (id % 4, id / 4), which groups each lane's neighbours into one
 * id-ordered segment (ids < 2^30 with 4 lanes). */
SPP_HD uint32_t spp_list_order(const SppConsts* k, uint32_t id) {
  return k->lanes == 1 ? id : ((id & 3u) << 30) | (id >> 2);
}

/* The fixed combination of the four lane sums (the butterfly of xor
 * shuffles 1 then 2 computes exactly this on every lane). */
SPP_HD float spp_lane_sum4(float p0, float p1, float p2, float p3) { return (p0 + p1) + (p2 + p3); }

/* Accumulator for the sums particle i receives. */
typedef struct SppAcc {
  spp_fx ax, ay;    /* force (ABP) or heading vector sum (Vicsek) */
  spp_fx at;        /* torque / angle sum */
  int32_t cnt;      /* neighbours within the alignment radius (self excluded) */
  int32_t ovf;      /* a term left the fixed-point range */
} SppAcc;

SPP_HD void spp_acc_zero(SppAcc* a) {
  a->ax.hi = a->ax.lo = 0; a->ay.hi = a->ay.lo = 0; a->at.hi = a->at.lo = 0;
  a->cnt = 0; a->ovf = 0;
}

SPP_HD void spp_fx_add_guarded(spp_fx* acc, float t, int32_t* ovf) {
  if (!spp_fx_ok(t)) { *ovf = 1; return; }
  spp_fx_add(acc, t);
}

/* Minimum-image separation r_i - r_j and its squared length (the plain
 * difference in a closed box; `closed` is k->closed, a compile-time
 * constant in the specialised kernels). */
SPP_HD float spp_sep_cl(const SppConsts* k, int closed, float xi, float yi, float xj, float yj,
                        float* dx, float* dy) {
  if (closed) {
    *dx = xi - xj;
    *dy = yi - yj;
  } else {
    *dx = spp_min_image_f(xi - xj, k->L, k->L2);
    *dy = spp_min_image_f(yi - yj, k->L, k->L2);
  }
  return fmaf(*dx, *dx, *dy * *dy);
}
SPP_HD float spp_sep(const SppConsts* k, float xi, float yi, float xj, float yj, float* dx,
                     float* dy) {
  return spp_sep_cl(k, k->closed, xi, yi, xj, yj, dx, dy);
}

/* A coordinate after a move: wrapped into [-L, L) (image counter updated)
 * in a periodic box, left as it is in a closed one. */
SPP_HD float spp_move_coord(const SppConsts* k, int closed, float x, int* img) {
  return closed ? x : spp_wrap_coord_f(x, k->L, k->L2, img);
}

/* Accumulator of the Verlet-list models.  Their neighbour lists are sorted
 * by particle id at every build, so the terms arrive in ascending id order
 * and plain FP32 sums are reproducible (the CPU mirror sums the same
 * contributors in the same order). */
typedef struct SppAccF {
  float fx, fy;     /* received force */
  float sc, ss;     /* sums of cos theta_j and sin theta_j over the aligning neighbours:
                       sum_j sin(theta_j - theta_i) = cos theta_i ss - sin theta_i sc */
  float tq;         /* torque terms that do not factor that way (the alpha term of the
                       continuous model, lever-arm torques of chains) */
  int32_t cnt;      /* neighbours within the alignment radius (self excluded) */
  int32_t ovf;      /* an R12 term left the checked range */
} SppAccF;

SPP_HD void spp_accf_zero(SppAccF* a) {
  a->fx = 0.0f; a->fy = 0.0f; a->ss = 0.0f; a->sc = 0.0f; a->tq = 0.0f; a->cnt = 0; a->ovf = 0;
}

/* Alignment-term kinds of the gather loop. */
#define SPP_KIND_ABP 0          /* sin(theta_j - theta_i), neighbour count */
#define SPP_KIND_CONT 1         /* (1 - alpha)/pi sin(...)                  */
#define SPP_KIND_CONT_ALPHA 2   /* ... - alpha (dr x v_i) / (pi d)          */
#define SPP_KIND_BEADS 3        /* repulsion only (ActiveBrownianChain nb = 1) */
#define SPP_KIND_CHAIN 4        /* beads with multi-bead swimmers (nb > 1) */

SPP_HD int spp_pair_kind(const SppConsts* k) {
  if (k->model == SPP_MODEL_BEADS) return k->chain_nb > 1 ? SPP_KIND_CHAIN : SPP_KIND_BEADS;
  if (k->model != SPP_MODEL_CONTINUOUS) return SPP_KIND_ABP;
  return k->alpha_over_pi != 0.0f ? SPP_KIND_CONT_ALPHA : SPP_KIND_CONT;
}

/* The separation of a pair (minimum image where wrap is set) and its
 * square. */
SPP_HD float spp_pair_sep(const SppConsts* k, int wrap, float xi, float yi, float xj, float yj,
                          float* dx, float* dy) {
  if (wrap) return spp_sep_cl(k, 0, xi, yi, xj, yj, dx, dy);
  /* both particles far from the boundary, or a closed box: the plain difference */
  const spp_f2 dr = spp_sub2(spp_f2_make(xi, yi), spp_f2_make(xj, yj));
  *dx = dr.x;
  *dy = dr.y;
  return fmaf(dr.x, dr.x, dr.y * dr.y);
}

/* Whether the term of (law, kind) needs r = 1/d. */
SPP_HD int spp_pair_needs_r(int law, int kind) {
  return law != SPP_FORCE_NONE || kind == SPP_KIND_CONT_ALPHA;
}

/* RepulsiveParticle::Interact (shared/particle.h:728-757) / ContinuousParticle::
 * Interact (:296-338), as received by i from j.  (c, s) = (cos, sin) theta.
 * law and kind are compile-time constants in the kernels (template
 * arguments), so the branches on them vanish there; the CPU mirror passes
 * k->force_law and spp_pair_kind(k) and evaluates the same arithmetic.
 * Callers present the neighbours j in ascending particle id.
 * Every term is evaluated and then masked (no data-dependent branches, so a
 * warp's lanes stay converged); a masked term adds exactly nothing: t = 0
 * gives fmaf(0, dx, f) = f, and the alignment sums are predicated adds.
 * With r = 1/d from spp_rsqrtf:
 *   harmonic  k (1 - d / r_rep) dr / d  ->  t = k r - k / r_rep,  F = t dr
 *   R12       A ((sigma/d)^13 - (sigma/r_c)^13) dr / d  ->  t = A (q^13 - c^13) r, q = sigma r
 * The alignment term sin(theta_j - theta_i) = s_j c_i - c_j s_i factors:
 * the loop sums s_j and c_j and spp_align_sum combines them once. */
/* The term of one pair from its separation (dx, dy), d2 and r =
 * spp_rsqrtf(d2) (r is not read where spp_pair_needs_r is 0). */
SPP_HD void spp_pair_abp_apply(const SppConsts* k, int law, int kind, SppAccF* a, float dx, float dy,
                               float d2, float r, float ci, float si, float cj, float sj, int valid) {
  const int aligns = (kind != SPP_KIND_BEADS && kind != SPP_KIND_CHAIN);
  const int in_rep = valid && (law != SPP_FORCE_NONE) && (d2 < k->rrep2) && (d2 > 0.0f);
  const int in_al = valid && aligns && d2 < k->ral2;
  if (law != SPP_FORCE_NONE) {
    float t;
    if (law == SPP_FORCE_HARMONIC) {
      t = fmaf(k->k_rep, r, -k->k_over_rrep);
      t = in_rep ? t : 0.0f;
    } else {
      const float q = k->sigma_rep * r;
      const float q2 = q * q, q4 = q2 * q2, q8 = q4 * q4;
      const float q13 = (q8 * q4) * q;
      t = in_rep ? (k->k_rep * (q13 - k->c13)) * r : 0.0f;
      if (!(fabsf(t * dx) < SPP_FX_RANGE && fabsf(t * dy) < SPP_FX_RANGE)) { a->ovf = 1; t = 0.0f; }
    }
    const spp_f2 f = spp_fma2s(t, spp_f2_make(dx, dy), spp_f2_make(a->fx, a->fy));
    a->fx = f.x;
    a->fy = f.y;
  }
  if (aligns) {
    a->cnt += in_al;
    if (in_al) {
      const spp_f2 cs = spp_add2(spp_f2_make(a->sc, a->ss), spp_f2_make(cj, sj));
      a->sc = cs.x;
      a->ss = cs.y;
    }
    if (kind == SPP_KIND_CONT_ALPHA && in_al && d2 > 0.0f)
      a->tq = a->tq - (k->alpha_over_pi * (dx * si - dy * ci)) * r;
  }
}

SPP_HD void spp_pair_abp_lkwv(const SppConsts* k, int law, int kind, int wrap, SppAccF* a, float xi,
                              float yi, float ci, float si, float xj, float yj, float cj, float sj,
                              int valid) {
  float dx, dy;
  const float d2 = spp_pair_sep(k, wrap, xi, yi, xj, yj, &dx, &dy);
  const float r = spp_pair_needs_r(law, kind) ? spp_rsqrtf(d2) : 0.0f;
  spp_pair_abp_apply(k, law, kind, a, dx, dy, d2, r, ci, si, cj, sj, valid);
}

/* The pair term of a list entry that exists (valid = 0 masks a padding
 * entry of a kernel's grouped loads: it then adds exactly nothing). */
SPP_HD void spp_pair_abp_lkw(const SppConsts* k, int law, int kind, int wrap, SppAccF* a, float xi,
                             float yi, float ci, float si, float xj, float yj, float cj, float sj) {
  spp_pair_abp_lkwv(k, law, kind, wrap, a, xi, yi, ci, si, xj, yj, cj, sj, 1);
}

/* The alignment torque sum of the ABP and continuous kinds from the
 * accumulated sums: sum_j sin(theta_j - theta_i), times (1 - alpha)/pi for
 * the continuous model, plus the terms kept in tq (alpha term). */
SPP_HD float spp_align_sum(const SppConsts* k, const SppAccF* a, float ci, float si) {
  float S = fmaf(ci, a->ss, -(si * a->sc));
  if (k->model == SPP_MODEL_CONTINUOUS) S = fmaf(k->one_minus_alpha_over_pi, S, a->tq);
  return S;
}

SPP_HD void spp_pair_abp(const SppConsts* k, SppAccF* a, float xi, float yi, float ci, float si,
                         float xj, float yj, float cj, float sj) {
  spp_pair_abp_lkw(k, k->force_law, spp_pair_kind(k), !k->closed, a, xi, yi, ci, si, xj, yj, cj, sj);
}

/* ActiveBrownianChain::Interact (shared/particle.h:964-1012) as received by
 * body i from body j; nbi, nbj are their bead counts (1 for membrane beads
 * and single-bead swimmers).  Two single beads interact by the membrane law
 * (sigma_m, repulsion_radius_m: the bead kind of spp_pair_abp_lkw).
 * Otherwise each bead pair (a, b), a outer, at s_i = v_i off[a] and
 * s_j = v_j off[b] from the centres, whose separation dr = (dr0 + s_i) - s_j
 * is inside the chain cutoff adds the R12 force F (sigma_p,
 * repulsion_radius) to i and the lever-arm torque s_i x F = s_i.x F.y -
 * s_i.y F.x.  A single bead sits at its centre (s = 0): it neither shifts
 * the separation nor receives torque. */
SPP_HD void spp_pair_chain(const SppConsts* k, int law, int wrap, SppAccF* a, int nbi, int nbj,
                           float xi, float yi, float ci, float si, float xj, float yj, float cj,
                           float sj) {
  if (nbi == 1 && nbj == 1) {
    spp_pair_abp_lkw(k, law, SPP_KIND_BEADS, wrap, a, xi, yi, ci, si, xj, yj, cj, sj);
    return;
  }
  if (law == SPP_FORCE_NONE) return;
  float dx0, dy0, d02;
  if (wrap) {
    d02 = spp_sep_cl(k, 0, xi, yi, xj, yj, &dx0, &dy0);
  } else {
    dx0 = xi - xj;
    dy0 = yi - yj;
    d02 = fmaf(dx0, dx0, dy0 * dy0);
  }
  if (!(d02 < k->chain_reach2)) return;
  for (int p = 0; p < nbi; ++p) {
    float stx = 0.0f, sty = 0.0f, ex = dx0, ey = dy0;
    if (nbi > 1) {
      stx = ci * k->chain_off[p];
      sty = si * k->chain_off[p];
      ex = dx0 + stx;
      ey = dy0 + sty;
    }
    for (int q = 0; q < nbj; ++q) {
      float dx = ex, dy = ey;
      if (nbj > 1) {
        dx = ex - cj * k->chain_off[q];
        dy = ey - sj * k->chain_off[q];
      }
      const float d2 = fmaf(dx, dx, dy * dy);
      if (!(d2 < k->chain_rc2 && d2 > 0.0f)) continue;
      const float r = spp_rsqrtf(d2);
      const float u = k->chain_sigma * r;
      const float u2 = u * u, u4 = u2 * u2, u8 = u4 * u4;
      const float u13 = (u8 * u4) * u;
      float t = (k->k_rep * (u13 - k->chain_c13)) * r;
      if (!(fabsf(t * dx) < SPP_FX_RANGE && fabsf(t * dy) < SPP_FX_RANGE)) { a->ovf = 1; t = 0.0f; }
      const float Fx = t * dx, Fy = t * dy;
      a->fx = a->fx + Fx;
      a->fy = a->fy + Fy;
      if (nbi > 1) a->tq = a->tq + (stx * Fy - sty * Fx);
    }
  }
}

/* Velocity and angular velocity of a chain swimmer (ActiveBrownianChain::
 * Reset / Move*, shared/particle.h:878-962): the force f = F0 v + F, with v
 * = (ci, si) the heading the forces were evaluated at, moves it at
 *   m_perp f + (m_par - m_perp) (f . w) w
 * where w is the heading of the position update (v itself in the
 * Runge-Kutta stages; Move() turns first and projects on the new heading),
 * and it turns at k_perp (torque0 + lever-arm torques). */
SPP_HD void spp_chain_velocity(const SppConsts* k, const SppAccF* a, float ci, float si, float wc,
                               float ws, float* vx, float* vy, float* om) {
  const float ftx = k->chain_f0 * ci + a->fx;
  const float fty = k->chain_f0 * si + a->fy;
  const float fw = ftx * wc + fty * ws;
  const float g = k->chain_dm * fw;
  *vx = k->chain_mperp * ftx + g * wc;
  *vy = k->chain_mperp * fty + g * ws;
  *om = k->chain_k * (k->chain_torque0 + a->tq);
}

/* The walls of a closed box acting on a particle at (x, y) with heading
 * (c, s), summed in wall order into force (wfx, wfy) and torque wtq.
 *   SPP_MODEL_ABP, Wall::Interact(RepulsiveParticle*) (shared/wall.h:
 *     215-265): dr = Distance_Vector (the perpendicular from the segment, or
 *     from its nearer end beyond it, :127-148), d = |dr|;
 *     for d < r_c_w the force along dr/d of strength
 *       A_w (e^(-d/sigma_w) (1/d^2 + 1/(sigma_w d)) - the same at r_c_w);
 *     for d < r_f_w beside the segment, heading towards it (dr . v < 0), the
 *     torque -(g_w/pi) sin(theta - theta_w), negated when cos(theta -
 *     theta_w) < 0 (i.e. pi/2 < theta - theta_w < 3pi/2 mod 2pi);
 *   SPP_MODEL_CONTINUOUS, Wall::Interact(ContinuousParticle*) (:192-213):
 *     dr the perpendicular from the wall's line, for |dr|^2 < 1 the torque
 *     gw (v x dr) / (2 pi |dr|^2).
 * (cos theta_w, sin theta_w) is the wall's unit direction (Wall::Init
 * reduces theta_w to the same angle, :36-40). */
SPP_HD void spp_wall_terms(const SppConsts* k, float x, float y, float c, float s, float* wfx,
                           float* wfy, float* wtq) {
  float fx = 0.0f, fy = 0.0f, tq = 0.0f;
  for (int w = 0; w < k->n_walls; ++w) {
    const float ex = k->wall_ex[w], ey = k->wall_ey[w];
    const float r1x = x - k->wall_x1[w], r1y = y - k->wall_y1[w];
    const float proj = fmaf(r1x, ex, r1y * ey);
    if (k->model == SPP_MODEL_CONTINUOUS) {
      const float dx = r1x - ex * proj, dy = r1y - ey * proj;
      const float d2 = fmaf(dx, dx, dy * dy);
      if (d2 < 1.0f && d2 > 0.0f)
        tq = tq + k->wall_gcont_over_2pi * ((c * dy - s * dx) / d2);
      continue;
    }
    const int beside = proj < k->wall_len[w] && proj > 0.0f;
    float dx, dy;
    if (beside) {
      dx = r1x - ex * proj;
      dy = r1y - ey * proj;
    } else {
      const float r2x = x - k->wall_x2[w], r2y = y - k->wall_y2[w];
      const float d21 = fmaf(r1x, r1x, r1y * r1y), d22 = fmaf(r2x, r2x, r2y * r2y);
      dx = d22 < d21 ? r2x : r1x;
      dy = d22 < d21 ? r2y : r1y;
    }
    const float d2 = fmaf(dx, dx, dy * dy);
    const float d = sqrtf(d2);
    if (d < k->wall_rc && d2 > 0.0f) {
      const float u = -d / k->wall_sigma;
      const float e = u > -80.0f ? spp_expf(u) : 0.0f;   /* spp_expf covers |x| < 80 */
      const float mag = k->wall_A * (e * (1.0f / d2 + 1.0f / (k->wall_sigma * d)) - k->wall_cut);
      fx = fx + (dx / d) * mag;
      fy = fy + (dy / d) * mag;
    }
    if (d < k->wall_rf && beside && fmaf(dx, c, dy * s) < 0.0f) {
      float t = k->wall_g_over_pi * (s * ex - c * ey);   /* (g_w / pi) sin(theta - theta_w) */
      if (fmaf(c, ex, s * ey) < 0.0f) t = -t;
      tq = tq - t;
    }
  }
  *wfx = fx;
  *wfy = fy;
  *wtq = tq;
}

/* The circular box (Box::Interact, parallel/box.h:285-294, CIRCULAR_BOX
 * without PERIODIC_BOUNDARY_CONDITION): a particle at distance r > L - 1
 * from the centre turns away from the circle of radius L by
 *   40 g (v_y x - v_x y) / (2 pi r (L - r)),
 * added to its torque with the pair terms (the continuous model's Move
 * multiplies that sum by g once more, particle.h:273). */
SPP_HD float spp_circle_torque(const SppConsts* k, float x, float y, float c, float s) {
  const float r = sqrtf(fmaf(x, x, y * y));
  if (!(r > k->L - 1.0f)) return 0.0f;
  return k->circ_k * (fmaf(s, x, -(c * y)) / (r * (k->L - r)));
}

/* Self-propulsion plus received force, and the torque (RepulsiveParticle::
 * Reset :559-564 and the alignment normalisations), plus, with walls
 * (k->n_walls > 0, a closed box; a compile-time constant in the specialised
 * kernels), the walls at the particle's position (x, y), added after the pair sums
 * as the reference adds them (parallel/box.h:296-302).  The continuous
 * model's wall torque enters before the factor g, which
 * ContinuousParticle::Move applies to the whole torque (particle.h:273). */
SPP_HD void spp_abp_forces(const SppConsts* k, int walls, const SppAccF* a, float xi, float yi,
                           float ci, float si, float* fx, float* fy, float* tau) {
  float wfx = 0.0f, wfy = 0.0f, wtq = 0.0f;
  if (walls) {
    spp_wall_terms(k, xi, yi, ci, si, &wfx, &wfy, &wtq);
    if (k->circle) wtq = wtq + spp_circle_torque(k, xi, yi, ci, si);
  }
  *fx = fmaf(k->v0, ci, a->fx);
  *fy = fmaf(k->v0, si, a->fy);
  float S = spp_align_sum(k, a, ci, si);
  if (k->model == SPP_MODEL_CONTINUOUS) {
    if (walls) S = S + wtq;
    *tau = k->g * S;
  } else if (k->align_mode == SPP_ALIGN_MEAN) {
    *tau = (k->g * S) / (float)(a->cnt + 1);
  } else {
    *tau = S * k->g_over_area;
  }
  if (walls && k->model != SPP_MODEL_CONTINUOUS) {
    *fx = *fx + wfx;
    *fy = *fy + wfy;
    *tau = *tau + wtq;
  }
}

/* RTPChain::Noise_Gen (shared/particle.h:1085-1103) on an integer state: 0
 * while running, +-c while tumbling (c = dt additions to the elapsed time so
 * far).  Returns the step's dtheta and updates the state. */
SPP_HD float spp_tumble_noise(const SppConsts* k, uint32_t pid, uint32_t step, int32_t* state) {
  int32_t s = *state;
  if (s == 0) {
    const uint32_t u = spp_draw_k(k, pid, step, SPP_RNG_TUMBLE).v[0] >> 8;
    if (u < k->tumble_u24) {
      /* 2 * gsl_rng_uniform_int(r, 2) - 1: -1 when the uniform is < 1/2 */
      const uint32_t v = spp_draw_k(k, pid, step, SPP_RNG_TUMBLE_SIGN).v[0] >> 8;
      s = v < (1u << 23) ? -1 : 1;
    }
  } else {
    const int32_t c = s < 0 ? -s : s;
    if (c < k->tumble_steps) s = s < 0 ? s - 1 : s + 1;
    else s = 0;
  }
  *state = s;
  return s == 0 ? 0.0f : (s < 0 ? -k->tumble_dth : k->tumble_dth);
}

/* The rotational-noise increment of particle pid at a step. */
SPP_HD float spp_rot_noise(const SppConsts* k, uint32_t pid, uint32_t step) {
  spp_u32x4 d = spp_draw_k(k, pid, step, SPP_RNG_ROT_NOISE);
  return k->sigma * spp_normal_f(d.v[0], d.v[1]);
}

/* One Runge-Kutta stage update from the start-of-step state (x0, y0, th0):
 *   th = wrap(th0 + h_t * tau + frac * dth),  x = wrap(x0 + h_x * fx).
 * Move_Runge_Kutta2_1/2 (shared/particle.h:589-631) use (h, frac) =
 * (dt/2, 1/2) then (dt, 1); RK4 (:633-726) uses (dt/2, 1/2), (dt/2, 1/2),
 * (dt, 1) and finally dt/6 times the weighted sum of the four slopes. */
SPP_HD void spp_stage_update(float h, float frac_noise, float x0, float y0, float th0, float fx,
                             float fy, float tau, float dth, const SppConsts* k, float* x, float* y,
                             float* th, float* c, float* s, int* imgx, int* imgy, int closed) {
  float t = fmaf(h, tau, th0) + frac_noise * dth;
  t = spp_wrap_angle_f(t);
  spp_sincosf(t, s, c);
  *th = t;
  *x = spp_move_coord(k, closed, fmaf(fx, h, x0), imgx);
  *y = spp_move_coord(k, closed, fmaf(fy, h, y0), imgy);
}

/* Euler move (RepulsiveParticle::Move, shared/particle.h:571-587: the step
 * along the force of the old heading; ContinuousParticle::Move, :268-280:
 * along the new heading): theta is not wrapped there. */
SPP_HD float spp_euler_theta(const SppConsts* k, float th0, float tau, float dth) {
  return fmaf(k->dt, tau, th0) + dth;
}
SPP_HD void spp_euler_update(float x0, float y0, float th0, float fx, float fy, float tau, float dth,
                             const SppConsts* k, float* x, float* y, float* th, float* c, float* s,
                             int* imgx, int* imgy, int closed) {
  float t = spp_euler_theta(k, th0, tau, dth);
  spp_sincosf(t, s, c);
  *th = t;
  if (k->model == SPP_MODEL_CONTINUOUS) {
    /* ContinuousParticle::Move (shared/particle.h:268-280) turns first and
     * then steps along the new heading: r += v (speed dt) */
    *x = spp_move_coord(k, closed, fmaf(*c, k->v0dt, x0), imgx);
    *y = spp_move_coord(k, closed, fmaf(*s, k->v0dt, y0), imgy);
    return;
  }
  *x = spp_move_coord(k, closed, fmaf(fx, k->dt, x0), imgx);
  *y = spp_move_coord(k, closed, fmaf(fy, k->dt, y0), imgy);
}

/* ------------------------------------------------------------------ */
/* Vicsek family                                                       */
/* ------------------------------------------------------------------ */
/* Configured rule: sum e^{i theta_j} over |r_ij| < r, self included (the
 * self term comes from the d2 = 0 visit of j = i). */
SPP_HD void spp_pair_vicsek(const SppConsts* k, SppAcc* a, float xi, float yi, float xj, float yj,
                            float cj, float sj, float thj, int self) {
  float dx, dy;
  float d2 = spp_sep(k, xi, yi, xj, yj, &dx, &dy);
  if (k->model == SPP_MODEL_VICSEK) {
    if (d2 < k->ral2) {
      spp_fx_add(&a->ax, cj);
      spp_fx_add(&a->ay, sj);
      a->cnt += 1;
    }
    return;
  }
  if (self) return;
  if (k->model == SPP_MODEL_VICSEK_REF_ANGLE) { /* VicsekParticle::Interact, particle.h:171-188 */
    if (d2 < k->ral2) {
      a->cnt += 1;
      spp_fx_add_guarded(&a->at, thj, &a->ovf);
    }
    return;
  }
  /* VicsekParticle2::Interact, particle.h:221-246 */
  if (d2 < k->ral2) {
    a->cnt += 1;
    spp_fx_add(&a->ax, cj);
    spp_fx_add(&a->ay, sj);
    if (d2 < k->rpush2 && d2 > 0.0f) {
      const float r = spp_rsqrtf(d2);
      const float d = d2 * r;
      float fa = k->beta_push / (1.0f + spp_expf(d / k->r_push - 2.0f));
      float t = fa * r;
      spp_fx_add_guarded(&a->ax, t * dx, &a->ovf);
      spp_fx_add_guarded(&a->ay, t * dy, &a->ovf);
    }
  }
}

/* New heading and position of particle i (VicsekParticle::Move :148-163,
 * VicsekParticle2::Move :198-213, configured rule). xi_u is the Philox word
 * of the Vicsek noise stream. */
/* Wall::Interact(VicsekParticle*) (shared/wall.h:163-190) of every wall of a
 * closed box: a particle whose foot on the segment lies inside it and whose
 * distance from it is below 1 counts the wall as a neighbour and adds, as
 * the reference writes it, its own heading relative to the wall's direction
 * folded to [-pi/2, pi/2] (dtheta = theta - theta_w, dtheta -= 2 pi
 * (int)(dtheta / pi), and once more after adding pi when |dtheta| > pi/2)
 * to the angle sum that VicsekParticle::Move averages.  Into the exact
 * fixed-point angle sum. */
SPP_HD void spp_vicsek_walls(const SppConsts* k, SppAcc* a, float x, float y, float th) {
  for (int w = 0; w < k->n_walls; ++w) {
    const float ex = k->wall_ex[w], ey = k->wall_ey[w];
    const float r1x = x - k->wall_x1[w], r1y = y - k->wall_y1[w];
    const float proj = fmaf(r1x, ex, r1y * ey);
    if (!(proj < k->wall_len[w] && proj > 0.0f)) continue;
    const float dx = r1x - ex * proj, dy = r1y - ey * proj;
    if (!(fmaf(dx, dx, dy * dy) < 1.0f)) continue;
    float dth = th - k->wall_theta[w];
    dth = fmaf(-SPP_TWO_PI_F, truncf(dth / SPP_PI_F), dth);
    if (dth > 0.5f * SPP_PI_F || dth < -0.5f * SPP_PI_F) {
      dth = dth + SPP_PI_F;
      dth = fmaf(-SPP_TWO_PI_F, truncf(dth / SPP_PI_F), dth);
    }
    a->cnt += 1;
    spp_fx_add_guarded(&a->at, dth, &a->ovf);
  }
}

SPP_HD void spp_vicsek_update(const SppConsts* k, const SppAcc* a, float x0, float y0, float th0,
                              float c0, float s0, uint32_t xi_bits, float* x, float* y, float* th,
                              float* c, float* s, int* imgx, int* imgy) {
  float xi = spp_uniform_pm_pi_f(xi_bits);
  float t;
  if (k->model == SPP_MODEL_VICSEK) {
    t = spp_atan2f(spp_fx_value(a->ay), spp_fx_value(a->ax)) + k->eta * xi;
    t = spp_wrap_angle_f(t);
  } else if (k->model == SPP_MODEL_VICSEK_REF_ANGLE) {
    float avg = a->cnt > 0 ? spp_fx_value(a->at) / (float)a->cnt : th0;
    t = avg + k->eta * xi;
  } else {
    float ax = a->cnt == 0 ? c0 : spp_fx_value(a->ax);
    float ay = a->cnt == 0 ? s0 : spp_fx_value(a->ay);
    float sx, cx;
    spp_sincosf(xi, &sx, &cx);
    float amp = (float)a->cnt * k->eta;
    ax = ax + amp * cx;
    ay = ay + amp * sx;
    t = spp_atan2f(ay, ax);
  }
  spp_sincosf(t, s, c);
  *th = t;
  *x = spp_move_coord(k, k->closed, fmaf(k->v0dt, *c, x0), imgx);
  *y = spp_move_coord(k, k->closed, fmaf(k->v0dt, *s, y0), imgy);
}

/* ------------------------------------------------------------------ */
/* tangent dynamics (Lyapunov spectrum of the continuous model)        */
/* ------------------------------------------------------------------ */
/* Maximum number of tangent vectors carried per system. */
#define SPP_LYAP_MAX 8

/* The continuous model with alpha = 0 (ContinuousParticle, shared/
 * particle.h:296-338): dr_i/dt = v0 (cos th_i, sin th_i),
 * dth_i/dt = g (1 - alpha)/pi sum_{|r_ij| < R} sin(th_j - th_i).  Its
 * Jacobian-vector product, the cutoff's step ignored (zero almost
 * everywhere), is
 *   d(dx_i)/dt  = -v0 sin th_i dth_i,    d(dy_i)/dt = v0 cos th_i dth_i,
 *   d(dth_i)/dt = g (1 - alpha)/pi sum_j cos(th_j - th_i) (dth_j - dth_i).
 * The reference estimates exponents with finite perturbations of the full
 * dynamics instead (parallel/lyapunovbox.h:128-194); this is the linearised
 * counterpart.  Per-pair term for one tangent vector: */
SPP_HD float spp_tangent_coupling(float ci, float si, float cj, float sj) {
  return cj * ci + sj * si; /* cos(th_j - th_i) */
}

/* One integrator stage of one tangent component, the derivative of the
 * base stage updates (spp_stage_update / spp_euler_update): slope is the
 * JVP at the stage state, t0 the component at the start of the step, acc
 * the RK4 slope sum, uout the input of the next stage. */
SPP_HD void spp_tangent_stage_update(const SppConsts* k, int stage, int nst, float slope, float* t0,
                                     float* acc, float* uout) {
  if (nst == 1) {
    *t0 = fmaf(k->dt, slope, *t0);
  } else if (nst == 2) {
    if (stage == 0) *uout = fmaf(k->half_dt, slope, *t0);
    else *t0 = fmaf(k->dt, slope, *t0);
  } else {
    if (stage == 0) { *acc = slope; *uout = fmaf(k->half_dt, slope, *t0); }
    else if (stage == 1) { *acc = *acc + 2.0f * slope; *uout = fmaf(k->half_dt, slope, *t0); }
    else if (stage == 2) { *acc = *acc + 2.0f * slope; *uout = fmaf(k->dt, slope, *t0); }
    else { *t0 = fmaf(k->dt6, *acc + slope, *t0); }
  }
}

/* Gram-matrix layout of the FP64 renormalisation: entries (a, b), b <= a,
 * packed row by row. */
#define SPP_GRAM_ENTRIES (SPP_LYAP_MAX * (SPP_LYAP_MAX + 1) / 2)
#ifndef SPP_GRAM_BLOCKS
#define SPP_GRAM_BLOCKS 64
#endif
#define SPP_GRAM_THREADS 256
SPP_HD int spp_gram_index(int a, int b) { return a * (a + 1) / 2 + b; }

/* Cholesky G = R^T R (R upper triangular) of a K x K Gram matrix in packed
 * form, then Rinv = R^{-1}.  Returns 0 on success, 1 if G is not positive
 * definite (dependent vectors).  log_r[a] = log R_aa, the stretch of vector
 * a in the Gram-Schmidt sense (the same R as classical Gram-Schmidt,
 * shared/vector-set.h:118-127, computes). */
SPP_HD int spp_cholesky_inverse(int K, const double* G, double* Rinv, double* log_r) {
  double R[SPP_LYAP_MAX][SPP_LYAP_MAX];
  for (int a = 0; a < K; ++a)
    for (int b = 0; b < K; ++b) R[a][b] = 0.0;
  /* one FP64 division per diagonal entry (FP64 division is a long
   * dependent sequence on this GPU): the rest multiply by the reciprocal */
  double inv[SPP_LYAP_MAX];
  for (int j = 0; j < K; ++j) {
    double d = G[spp_gram_index(j, j)];
    for (int q = 0; q < j; ++q) d -= R[q][j] * R[q][j];
    if (!(d > 0.0)) return 1;
    const double rjj = sqrt(d);
    R[j][j] = rjj;
    inv[j] = 1.0 / rjj;
    for (int c = j + 1; c < K; ++c) {
      double v = G[spp_gram_index(c, j)];
      for (int q = 0; q < j; ++q) v -= R[q][j] * R[q][c];
      R[j][c] = v * inv[j];
    }
    log_r[j] = log(rjj);
  }
  /* upper-triangular inverse, column by column */
  for (int a = 0; a < K; ++a)
    for (int b = 0; b < K; ++b) Rinv[a * SPP_LYAP_MAX + b] = 0.0;
  for (int c = 0; c < K; ++c) {
    Rinv[c * SPP_LYAP_MAX + c] = inv[c];
    for (int r = c - 1; r >= 0; --r) {
      double v = 0.0;
      for (int q = r + 1; q <= c; ++q) v += R[r][q] * Rinv[q * SPP_LYAP_MAX + c];
      Rinv[r * SPP_LYAP_MAX + c] = -v * inv[r];
    }
  }
  return 0;
}

/* ------------------------------------------------------------------ */
/* ring membranes (SPP_MODEL_BEADS)                                    */
/* ------------------------------------------------------------------ */
/* Ring forces on bead m from its bonds and from the bending of the three
 * bond angles it takes part in.  px/py hold ring beads m-2 .. m+2 (index 2
 * is bead m).
 *   bonds: Spring (shared/force-fields.h:87-97) between consecutive beads,
 *     as Interact_Membrane_Beads (parallel/beadbox.h:185-196): the force on
 *     bead m is S(r_m - r_{m-1}) + S(r_m - r_{m+1}), S(dr) = k (rest - d) dr/d.
 *   bending (no counterpart in the reference): E = kappa sum_j (1 - cos phi_j),
 *     phi_j the angle between the bonds u = r_j - r_{j-1} and w = r_{j+1} - r_j.
 *     With c = u.w / (|u||w|), dc/du = w/(|u||w|) - c u/|u|^2 and
 *     dc/dw = u/(|u||w|) - c w/|w|^2, bead m receives
 *       kappa dc_{m-1}/dw + kappa (dc_m/du - dc_m/dw) - kappa dc_{m+1}/du. */
SPP_HD void spp_ring_forces(const SppConsts* k, const float* px, const float* py, float* fx,
                            float* fy) {
  float bx[4], by[4], ib[4], b2[4];
  for (int q = 0; q < 4; ++q) {
    bx[q] = spp_min_image_f(px[q + 1] - px[q], k->L, k->L2);
    by[q] = spp_min_image_f(py[q + 1] - py[q], k->L, k->L2);
    b2[q] = fmaf(bx[q], bx[q], by[q] * by[q]);
    ib[q] = spp_rsqrtf(b2[q]);
  }
  float gx = 0.0f, gy = 0.0f;
  /* bonds (m-1, m) and (m, m+1): S(b_1) - S(b_2) with S(b) = k (rest - |b|) b / |b| */
  {
    const float t1 = k->k_bond * (k->bond_rest * ib[1] - 1.0f);
    const float t2 = k->k_bond * (k->bond_rest * ib[2] - 1.0f);
    gx = gx + t1 * bx[1];
    gy = gy + t1 * by[1];
    gx = gx - t2 * bx[2];
    gy = gy - t2 * by[2];
  }
  if (k->kappa != 0.0f) {
    /* angle j = m + q - 1 for q = 0, 1, 2 uses u = b_q, w = b_{q+1} */
    for (int q = 0; q < 3; ++q) {
      const float iuw = ib[q] * ib[q + 1];
      const float c = (bx[q] * bx[q + 1] + by[q] * by[q + 1]) * iuw;
      const float cu = c * (ib[q] * ib[q]);
      const float cw = c * (ib[q + 1] * ib[q + 1]);
      /* dc/du and dc/dw */
      const float dux = bx[q + 1] * iuw - cu * bx[q];
      const float duy = by[q + 1] * iuw - cu * by[q];
      const float dwx = bx[q] * iuw - cw * bx[q + 1];
      const float dwy = by[q] * iuw - cw * by[q + 1];
      if (q == 0) {
        gx = gx + k->kappa * dwx;
        gy = gy + k->kappa * dwy;
      } else if (q == 1) {
        gx = gx + k->kappa * (dux - dwx);
        gy = gy + k->kappa * (duy - dwy);
      } else {
        gx = gx - k->kappa * dux;
        gy = gy - k->kappa * duy;
      }
    }
  }
  *fx = gx;
  *fy = gy;
}

/* Id of the ring bead at offset o (-2..2) from bead id along its ring. */
SPP_HD uint32_t spp_ring_neighbor(const SppConsts* k, uint32_t id, int o) {
  const uint32_t M = (uint32_t)k->ring_size;
  const uint32_t ring = id / M, m = id % M;
  const uint32_t mm = (uint32_t)(((int)m + o + (int)M) % (int)M);
  return ring * M + mm;
}

/* Velocity and angular velocity of a body of SPP_MODEL_BEADS
 * (ActiveBrownianChain::Move_Runge_Kutta2_*, shared/particle.h:917-962, with
 * m_parallel = m_perpendicular = mu as for nb = 1): swimmers move at
 * v0 (cos, sin) + mu F and turn at k_perp torque0; membrane beads (F0 = 0)
 * move at mu F and do not turn. */
SPP_HD void spp_bead_velocity(const SppConsts* k, int swimmer, const SppAccF* a, float rfx,
                              float rfy, float ci, float si, float* vx, float* vy, float* om) {
  const float Fx = a->fx + rfx;
  const float Fy = a->fy + rfy;
  if (swimmer) {
    *vx = k->v0 * ci + k->mu * Fx;
    *vy = k->v0 * si + k->mu * Fy;
    *om = k->ang_drift;
  } else {
    *vx = k->mu * Fx;
    *vy = k->mu * Fy;
    *om = 0.0f;
  }
}

/* ------------------------------------------------------------------ */
/* cells                                                               */
/* ------------------------------------------------------------------ */
/* Cell coordinate along one axis for D cells over [-L, L).
 * SPP_BIN_GEOMETRIC: floor((x + L) * D / 2L); SPP_BIN_REFERENCE:
 * (int)((int)(x + L) * D / 2L), the reference's integer truncation
 * (serial/box.h:116-117).  Clamped to [0, D). */
SPP_HD int spp_cell_coord(float x, float L, float L2, int D, int rule) {
  int c;
  if (rule == SPP_BIN_REFERENCE) {
    int ix = (int)(x + L);
    c = (int)((float)(ix * D) / L2);
  } else {
    c = (int)floorf(((x + L) * (float)D) / L2);
  }
  if (c < 0) c = 0;
  if (c >= D) c = D - 1;
  return c;
}

/* Morton (Z-order) key of a cell, 16 bits per axis. */
SPP_HD uint32_t spp_morton_spread(uint32_t v) {
  v &= 0x0000ffffu;
  v = (v | (v << 8)) & 0x00ff00ffu;
  v = (v | (v << 4)) & 0x0f0f0f0fu;
  v = (v | (v << 2)) & 0x33333333u;
  v = (v | (v << 1)) & 0x55555555u;
  return v;
}
SPP_HD uint32_t spp_morton(uint32_t cx, uint32_t cy) {
  return spp_morton_spread(cx) | (spp_morton_spread(cy) << 1);
}

#endif /* SPP_PHYSICS_H */
