/*
 * ORACLE -- test infrastructure only.  Nothing in the product links this
 * file; tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg call it
 * as the checker.
 *
 * FP64 CPU restatement of the reference's per-step particle update
 * (hamidallaei/SPP), with the reference's single global GSL stream replaced
 * by the Philox counter stream of spp_gb300/csrc/spp_fp32.h (the same draws
 * the GPU uses, mapped to doubles here).
 *
 * What is restated, and from where:
 *   - min-image / wrap            shared/c2dvector.h:67-73 (Periodic_Transform)
 *   - half-shell pair traversal   serial/box.h:322-338, shared/cell.h:112-128
 *                                 (every pair once, Newton's third law)
 *   - R12_Repulsive_Truncated     shared/force-fields.h:14-39
 *   - VicsekParticle              shared/particle.h:145-189
 *   - VicsekParticle2             shared/particle.h:193-250
 *   - ContinuousParticle (Euler)  shared/particle.h:254-378
 *   - RepulsiveParticle           Reset :559-564, Noise_Gen :566-569,
 *                                 Move :571-587, RK2 :589-631, RK4 :633-726,
 *                                 Interact :728-757
 *   - polarization                parallel/node.h:1565-1591
 * Configured extensions that the reference does not have (no reference
 * oracle; this file is their specification): the arg-of-vector-sum Vicsek
 * rule, harmonic repulsion k(1 - d/r_rep), the 1/n_i-normalised alignment,
 * RK2/RK4 for the continuous model.
 *
 * Parity pin: oracle/ref_harness.cpp runs the reference's own particle.h
 * code on the same inputs and Philox draws; tests/test_oracle_pin.py checks
 * this file against it.
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include "../include/spp.h"
#include "../spp_gb300/csrc/spp_fp32.h"

/* ------------------------------------------------------------------ */
/* noise (doubles from the same Philox bits the kernels use)           */
/* ------------------------------------------------------------------ */
static double orc_normal(const SppParams* p, int pid, int64_t step) {
  spp_u32x4 d = spp_draw(p->seed, p->system_id, (uint32_t)pid, (uint32_t)step, SPP_RNG_ROT_NOISE);
  double u1 = spp_u01_open0_d(d.v[0]);
  double u2 = spp_u01_d(d.v[1]);
  return sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
}
static double orc_uniform_pm_pi(const SppParams* p, int pid, int64_t step) {
  spp_u32x4 d = spp_draw(p->seed, p->system_id, (uint32_t)pid, (uint32_t)step, SPP_RNG_VICSEK);
  double u = spp_u01_d(d.v[0]);
  return -M_PI * (1.0 - u) + M_PI * u; /* gsl_ran_flat(r, -pi, pi): a (1-u) + b u */
}

/* Set for a closed box (SPP_BOUNDARY_WALLS) for the duration of a run: the
 * reference built without PERIODIC_BOUNDARY_CONDITION skips every
 * Periodic_Transform. */
static __thread int g_closed = 0;

/* Cutoff-event recorder (parity tests): while on, every pair evaluation of
 * the alignment predicate whose distance lies within `window` of the
 * alignment radius is recorded as (stage, i, j, inside, d), with i < j and
 * `stage` counting the force evaluations since orc64_watch() (one per
 * Euler step, two per RK2 step, four per RK4 step).  The FP32 mirror
 * records the same events from its own arithmetic (orc32_watch), so a test
 * can find the pairs on which the two precisions took different sides of
 * the hard cutoff. */
static __thread struct {
  int32_t *stage, *pi, *pj;
  int8_t* inside;
  double* dist;
  int64_t cap, cnt;
  double r, window;
  int32_t cur;
  int on;
} g_w;

void orc64_watch(int32_t* stage, int32_t* pi, int32_t* pj, int8_t* inside, double* dist, int64_t cap,
                 double r, double window) {
  g_w.stage = stage; g_w.pi = pi; g_w.pj = pj; g_w.inside = inside; g_w.dist = dist;
  g_w.cap = cap; g_w.cnt = 0; g_w.r = r; g_w.window = window; g_w.cur = 0;
  g_w.on = stage != NULL;
}
int64_t orc64_watch_count(void) { return g_w.cnt; }

static inline void watch_pair(int i, int j, double d, int inside) {
  if (!g_w.on || fabs(d - g_w.r) >= g_w.window) return;
  if (g_w.cnt < g_w.cap) {
    g_w.stage[g_w.cnt] = g_w.cur;
    g_w.pi[g_w.cnt] = i < j ? i : j;
    g_w.pj[g_w.cnt] = i < j ? j : i;
    g_w.inside[g_w.cnt] = (int8_t)inside;
    g_w.dist[g_w.cnt] = d;
  }
  g_w.cnt++;
}

/* Periodic_Transform, shared/c2dvector.h:67-73 */
static inline double pt(double x, double L) {
  if (g_closed) return x;
  double L2 = 2.0 * L;
  return x - L2 * (double)(int)floor(x / L2 + 0.5);
}
/* theta wrap, shared/particle.h:599 */
static inline double wrap_angle(double th) {
  return th - floor(th / (2 * M_PI) + 0.5) * 2 * M_PI;
}

/* ------------------------------------------------------------------ */
/* cell list (geometric binning, width >= cutoff)                      */
/* ------------------------------------------------------------------ */
typedef struct {
  int D;
  int* head;
  int* next;
} ocells;

static void cells_build(ocells* c, int n, const double* x, const double* y, double L, double rcut) {
  int D = (int)floor(2.0 * L / rcut);
  if (D < 3) D = 1; /* brute force */
  c->D = D;
  c->head = (int*)malloc(sizeof(int) * (size_t)D * D);
  c->next = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  for (int k = 0; k < D * D; ++k) c->head[k] = -1;
  for (int i = n - 1; i >= 0; --i) {
    int cx = (int)floor((x[i] + L) * D / (2.0 * L));
    int cy = (int)floor((y[i] + L) * D / (2.0 * L));
    if (cx < 0) cx = 0; if (cx >= D) cx = D - 1;
    if (cy < 0) cy = 0; if (cy >= D) cy = D - 1;
    int k = cx * D + cy;
    c->next[i] = c->head[k];
    c->head[k] = i;
  }
}
static void cells_free(ocells* c) { free(c->head); free(c->next); }

/* Visit every unordered pair once (half shell: self, right, up, up-right,
 * down-right; serial/box.h:330-338). */
typedef void (*pair_fn)(void* ctx, int i, int j);
static void cells_for_pairs(const ocells* c, int n, pair_fn fn, void* ctx) {
  int D = c->D;
  if (D == 1) {
    for (int i = 0; i < n; ++i)
      for (int j = i + 1; j < n; ++j) fn(ctx, i, j);
    return;
  }
  static const int off[4][2] = {{1, 0}, {0, 1}, {1, 1}, {1, -1}};
  for (int cx = 0; cx < D; ++cx)
    for (int cy = 0; cy < D; ++cy) {
      int k = cx * D + cy;
      for (int i = c->head[k]; i >= 0; i = c->next[i])
        for (int j = c->next[i]; j >= 0; j = c->next[j]) fn(ctx, i, j);
      for (int o = 0; o < 4; ++o) {
        int nx = (cx + off[o][0] + D) % D, ny = (cy + off[o][1] + D) % D;
        int kk = nx * D + ny;
        for (int i = c->head[k]; i >= 0; i = c->next[i])
          for (int j = c->head[kk]; j >= 0; j = c->next[j]) fn(ctx, i, j);
      }
    }
}

/* ------------------------------------------------------------------ */
/* state                                                               */
/* ------------------------------------------------------------------ */
typedef struct {
  const SppParams* p;
  int n;
  double *x, *y, *xu, *yu, *th;   /* r (wrapped), r_original, theta */
  double *vx, *vy;                /* heading */
  double *fx, *fy, *tq;           /* force, torque accumulators */
  int* nb;                        /* neighbor_size */
  double *avx, *avy, *ath;        /* Vicsek averages */
  double *tho, *xo, *yo, *dth;    /* theta_old, r_old, dtheta */
  double *k1f_x, *k1f_y, *k1t, *k2f_x, *k2f_y, *k2t, *k3f_x, *k3f_y, *k3t;
  double* wtq;                    /* wall torque of RepulsiveParticle (added after the alignment normalisation) */
  int* tflag;                     /* RTPChain::tumble_flag */
  double* telapsed;               /* RTPChain::tumble_elapesed_time */
} ostate;

static double* dalloc(int n) { return (double*)calloc((size_t)(n > 0 ? n : 1), sizeof(double)); }

static void state_alloc(ostate* s, const SppParams* p) {
  int n = p->n;
  memset(s, 0, sizeof(*s));
  s->p = p; s->n = n;
  s->x = dalloc(n); s->y = dalloc(n); s->xu = dalloc(n); s->yu = dalloc(n); s->th = dalloc(n);
  s->vx = dalloc(n); s->vy = dalloc(n); s->fx = dalloc(n); s->fy = dalloc(n); s->tq = dalloc(n);
  s->nb = (int*)calloc((size_t)(n > 0 ? n : 1), sizeof(int));
  s->avx = dalloc(n); s->avy = dalloc(n); s->ath = dalloc(n);
  s->tho = dalloc(n); s->xo = dalloc(n); s->yo = dalloc(n); s->dth = dalloc(n);
  s->k1f_x = dalloc(n); s->k1f_y = dalloc(n); s->k1t = dalloc(n);
  s->k2f_x = dalloc(n); s->k2f_y = dalloc(n); s->k2t = dalloc(n);
  s->k3f_x = dalloc(n); s->k3f_y = dalloc(n); s->k3t = dalloc(n);
  s->wtq = dalloc(n);
  s->tflag = (int*)calloc((size_t)(n > 0 ? n : 1), sizeof(int));
  s->telapsed = dalloc(n);
}
static void state_free(ostate* s) {
  free(s->tflag);
  free(s->wtq);
  free(s->telapsed);
  double* arr[] = {s->x, s->y, s->xu, s->yu, s->th, s->vx, s->vy, s->fx, s->fy, s->tq,
                   s->avx, s->avy, s->ath, s->tho, s->xo, s->yo, s->dth,
                   s->k1f_x, s->k1f_y, s->k1t, s->k2f_x, s->k2f_y, s->k2t, s->k3f_x, s->k3f_y, s->k3t};
  for (size_t k = 0; k < sizeof(arr) / sizeof(arr[0]); ++k) free(arr[k]);
  free(s->nb);
}

static int chain_nb(const SppParams* p) {
  return p->model == SPP_MODEL_BEADS && p->chain_beads > 1 ? p->chain_beads : 1;
}

static double interaction_radius(const SppParams* p) {
  double r = p->model == SPP_MODEL_BEADS ? 0.0 : p->r_align;
  if (p->force_law != SPP_FORCE_NONE && p->r_rep > r) r = p->r_rep;
  if (p->model == SPP_MODEL_VICSEK_REF_VECTOR && p->r_push > r) r = p->r_push;
  /* two chains interact while some bead pair is within r_chain: centres up
   * to (nb - 1) separation + r_chain apart */
  if (chain_nb(p) > 1 && p->force_law != SPP_FORCE_NONE) {
    double reach = (chain_nb(p) - 1) * p->bead_separation + p->r_chain;
    if (reach > r) r = reach;
  }
  return r;
}

/* ActiveBrownianChain::Set_nb, shared/particle.h:856-876: m_parallel,
 * m_perpendicular, k_perpendicular of a body of nb beads. */
static void chain_mobility(int nb, double separation, double sigma_p, double* mpar, double* mperp,
                           double* kperp) {
  if (nb == 1) { *mpar = 0.5; *mperp = 0.5; *kperp = 1; return; }
  double aspect_ratio = 1 / ((separation * (nb - 1) / sigma_p) + 1);
  double e2 = 1 - aspect_ratio * aspect_ratio;
  double e = sqrt(e2);
  double L = log((1 + e) / (1 - e));
  *mpar = 1.0;
  *mperp = 0.5 * (2 * e + (3 * e2 - 1) * L) / ((1 + e2) * L - 2 * e);
  *kperp = 6 / (1 + aspect_ratio * aspect_ratio) / sigma_p / sigma_p;
}

/* ------------------------------------------------------------------ */
/* pair interactions                                                   */
/* ------------------------------------------------------------------ */
/* R12_Repulsive_Truncated, shared/force-fields.h:14-39 */
static void r12_trunc(double dx, double dy, double d, double rc, double sigma, double A,
                      double* Fx, double* Fy) {
  double q = sigma / d, q2 = q * q, q4 = q2 * q2, q8 = q4 * q4, q13 = q8 * q4 * q;
  double c = sigma / rc, c2 = c * c, c4 = c2 * c2, c8 = c4 * c4, c13 = c8 * c4 * c;
  double strength = A * (q13 - c13);
  *Fx = strength * dx / d;
  *Fy = strength * dy / d;
}

/* RepulsiveParticle::Interact, shared/particle.h:728-757 (and the harmonic /
 * 1/n_i variants of the configured model). */
static void abp_pair(void* ctx, int i, int j) {
  ostate* s = (ostate*)ctx;
  const SppParams* p = s->p;
  double dx = pt(s->x[i] - s->x[j], p->L), dy = pt(s->y[i] - s->y[j], p->L);
  double d2 = dx * dx + dy * dy;
  double d = sqrt(d2);
  if (p->force_law != SPP_FORCE_NONE && d < p->r_rep && d > 0) {
    double Fx, Fy;
    if (p->force_law == SPP_FORCE_R12_TRUNC) {
      r12_trunc(dx, dy, d, p->r_rep, p->sigma_rep, p->k_rep, &Fx, &Fy);
    } else {
      double mag = p->k_rep * (1.0 - d / p->r_rep);
      Fx = mag * dx / d;
      Fy = mag * dy / d;
    }
    s->fx[i] += Fx; s->fy[i] += Fy;
    s->fx[j] -= Fx; s->fy[j] -= Fy;
  }
  watch_pair(i, j, d, d < p->r_align);
  if (d < p->r_align) {
    s->nb[i]++; s->nb[j]++;
    double t = sin(s->th[j] - s->th[i]);
    if (p->align_mode == SPP_ALIGN_REFERENCE) t = p->g * t / (M_PI * p->r_align * p->r_align);
    s->tq[i] += t;
    s->tq[j] -= t;
  }
}

/* ContinuousParticle::Interact, shared/particle.h:296-338 */
static void cont_pair(void* ctx, int i, int j) {
  ostate* s = (ostate*)ctx;
  const SppParams* p = s->p;
  double dx = pt(s->x[i] - s->x[j], p->L), dy = pt(s->y[i] - s->y[j], p->L);
  double d2 = dx * dx + dy * dy;
  watch_pair(i, j, sqrt(d2), d2 < p->r_align * p->r_align);
  if (d2 < p->r_align * p->r_align) {
    s->nb[i]++; s->nb[j]++;
    double d = sqrt(d2);
    double ti = (1 - p->alpha) * sin(s->th[j] - s->th[i]) / M_PI;
    s->tq[i] += ti;
    s->tq[j] -= ti;
    if (p->alpha != 0.0 && d > 0) {
      s->tq[i] -= p->alpha * (dx * s->vy[i] - dy * s->vx[i]) / (M_PI * d);
      s->tq[j] += p->alpha * (dx * s->vy[j] - dy * s->vx[j]) / (M_PI * d);
    }
  }
}

/* VicsekParticle::Interact, shared/particle.h:171-188 */
static void vicsek_angle_pair(void* ctx, int i, int j) {
  ostate* s = (ostate*)ctx;
  const SppParams* p = s->p;
  double dx = pt(s->x[i] - s->x[j], p->L), dy = pt(s->y[i] - s->y[j], p->L);
  double d2 = dx * dx + dy * dy;
  if (d2 < p->r_align * p->r_align) {
    s->nb[i]++; s->nb[j]++;
    s->ath[i] += s->th[j];
    s->ath[j] += s->th[i];
  }
}

/* VicsekParticle2::Interact, shared/particle.h:221-246 */
static void vicsek_vector_pair(void* ctx, int i, int j) {
  ostate* s = (ostate*)ctx;
  const SppParams* p = s->p;
  double dx = pt(s->x[i] - s->x[j], p->L), dy = pt(s->y[i] - s->y[j], p->L);
  double d2 = dx * dx + dy * dy;
  double d = sqrt(d2);
  if (d2 < p->r_align * p->r_align) {
    s->nb[i]++; s->nb[j]++;
    s->avx[i] += s->vx[j]; s->avy[i] += s->vy[j];
    s->avx[j] += s->vx[i]; s->avy[j] += s->vy[i];
    if (d < p->r_push && d > 0) {
      double fa = p->beta_push / (1 + exp(d / p->r_push - 2));
      double ex = dx / d, ey = dy / d;
      s->avx[i] += ex * fa; s->avy[i] += ey * fa;
      s->avx[j] -= ex * fa; s->avy[j] -= ey * fa;
    }
  }
}

/* arg(sum e^{i theta_j}) over |r_ij| < r, self included (configured rule) */
static void vicsek_sum_pair(void* ctx, int i, int j) {
  ostate* s = (ostate*)ctx;
  const SppParams* p = s->p;
  double dx = pt(s->x[i] - s->x[j], p->L), dy = pt(s->y[i] - s->y[j], p->L);
  double d2 = dx * dx + dy * dy;
  if (d2 < p->r_align * p->r_align) {
    s->avx[i] += s->vx[j]; s->avy[i] += s->vy[j];
    s->avx[j] += s->vx[i]; s->avy[j] += s->vy[i];
  }
}

static void interact_all(ostate* s, pair_fn fn) {
  ocells c;
  cells_build(&c, s->n, s->x, s->y, s->p->L, interaction_radius(s->p));
  cells_for_pairs(&c, s->n, fn, s);
  cells_free(&c);
}

/* ------------------------------------------------------------------ */
/* RepulsiveParticle moves                                             */
/* ------------------------------------------------------------------ */
static void abp_reset(ostate* s) {
  /* RepulsiveParticle::Reset, particle.h:559-564: f = v (self propulsion). */
  for (int i = 0; i < s->n; ++i) {
    s->nb[i] = 1; s->tq[i] = 0;
    s->fx[i] = s->p->v0 * s->vx[i];
    s->fy[i] = s->p->v0 * s->vy[i];
  }
}
static double abp_torque(const ostate* s, int i) {
  const SppParams* p = s->p;
  if (p->model == SPP_MODEL_CONTINUOUS) return p->g * s->tq[i];
  if (p->align_mode == SPP_ALIGN_MEAN) return p->g * s->tq[i] / s->nb[i] + s->wtq[i];
  return s->tq[i] + s->wtq[i];
}
static void set_v(ostate* s, int i) { s->vx[i] = cos(s->th[i]); s->vy[i] = sin(s->th[i]); }

/* Walls of a closed box: Box::Init_Topology (parallel/box.h:97-101) plus
 * the extra segments, each through Wall::Init (shared/wall.h:27-41). */
typedef struct { double x1, y1, x2, y2, dx, dy, len, theta; } owall;

static int box_walls(const SppParams* p, owall* w) {
  double seg[SPP_MAX_WALLS][4] = {{-p->L, -p->L, -p->L, p->L}, {-p->L, p->L, p->L, p->L},
                                  {p->L, p->L, p->L, -p->L}, {p->L, -p->L, -p->L, -p->L}};
  int nw = 4;
  for (int e = 0; e < p->n_walls && nw < SPP_MAX_WALLS; ++e, ++nw)
    for (int c = 0; c < 4; ++c) seg[nw][c] = p->walls[e][c];
  for (int e = 0; e < nw; ++e) {
    w[e].x1 = seg[e][0]; w[e].y1 = seg[e][1]; w[e].x2 = seg[e][2]; w[e].y2 = seg[e][3];
    double dx = w[e].x2 - w[e].x1, dy = w[e].y2 - w[e].y1;
    w[e].len = sqrt(dx * dx + dy * dy);
    w[e].dx = dx / w[e].len; w[e].dy = dy / w[e].len;
    double th = atan(w[e].dy / w[e].dx);
    if (w[e].dx < 0.) th += M_PI;
    th -= 2 * M_PI * (int)(th / M_PI);
    w[e].theta = th;
  }
  return nw;
}

/* Wall::Interact (shared/wall.h:192-265) of the walls w[0..nw) on one
 * particle at (x, y) with heading theta (v = (vx, vy)): RepulsiveParticle
 * force and torque into *fx, *fy, *wtq; ContinuousParticle torque into
 * *ctq (before the factor g of Move). */
static void wall_terms64(const SppParams* p, const owall* w, int nw, double x, double y, double th,
                         double vx, double vy, double* fx, double* fy, double* wtq, double* ctq) {
  for (int e = 0; e < nw; ++e) {
    double r1x = pt(x - w[e].x1, p->L), r1y = pt(y - w[e].y1, p->L);
    double proj = r1x * w[e].dx + r1y * w[e].dy;
    if (p->model == SPP_MODEL_CONTINUOUS) {
      double drx = r1x - w[e].dx * proj, dry = r1y - w[e].dy * proj;
      double d2 = drx * drx + dry * dry;
      if (d2 < 1) *ctq += p->g_w_cont * ((vx * dry - vy * drx) / (2 * M_PI * d2));
      continue;
    }
    /* Distance_Vector, wall.h:127-148 */
    double drx, dry;
    if (proj < w[e].len && proj > 0) {
      drx = r1x - w[e].dx * proj; dry = r1y - w[e].dy * proj;
    } else {
      double r2x = pt(x - w[e].x2, p->L), r2y = pt(y - w[e].y2, p->L);
      double d21 = r1x * r1x + r1y * r1y, d22 = r2x * r2x + r2y * r2y;
      if (d22 < d21) { drx = r2x; dry = r2y; } else { drx = r1x; dry = r1y; }
    }
    double d2 = drx * drx + dry * dry;
    double d = sqrt(d2);
    if (d < p->r_c_w) {
      drx /= d; dry /= d;
      double rc2 = p->r_c_w * p->r_c_w;
      double mag = p->A_w * (exp(-d / p->sigma_w) * (1. / d2 + 1. / (p->sigma_w * d)) -
                             exp(-p->r_c_w / p->sigma_w) * (1. / rc2 + 1. / (p->sigma_w * p->r_c_w)));
      *fx += drx * mag; *fy += dry * mag;
    }
    if (d < p->r_f_w && proj < w[e].len && proj > 0.) {
      double sx = cos(th), sy = sin(th);
      if (drx * sx + dry * sy < 0.) {
        double dtheta = th - w[e].theta;
        double t = p->g_w * sin(dtheta) / M_PI;
        dtheta -= 2 * M_PI * ((int)(dtheta / (2 * M_PI)));
        if (dtheta < 0.) dtheta += 2 * M_PI;
        if (dtheta > M_PI / 2 && dtheta < 3 * M_PI / 2) t *= -1.;
        *wtq -= t;
      }
    }
  }
}

/* Wall::Interact(VicsekParticle*), shared/wall.h:163-190, of the walls
 * w[0..nw): where the particle's foot lies inside a segment and its distance
 * is below 1, the wall counts as a neighbour and adds the particle's own
 * heading relative to the wall's direction, folded to [-pi/2, pi/2], to the
 * angle sum (as the reference writes it). */
static void vicsek_walls64(const SppParams* p, const owall* w, int nw, double x, double y, double th,
                           int* nb, double* ath) {
  for (int e = 0; e < nw; ++e) {
    double r1x = pt(x - w[e].x1, p->L), r1y = pt(y - w[e].y1, p->L);
    double proj = r1x * w[e].dx + r1y * w[e].dy;
    if (!(proj < w[e].len && proj > 0)) continue;
    double drx = r1x - w[e].dx * proj, dry = r1y - w[e].dy * proj;
    double dth = th - w[e].theta;
    dth -= 2 * M_PI * (int)(dth / M_PI);
    if (dth > M_PI / 2 || dth < -M_PI / 2) {
      dth += M_PI;
      dth -= 2 * M_PI * (int)(dth / M_PI);
    }
    if (drx * drx + dry * dry < 1) {
      (*nb)++;
      *ath += dth;
    }
  }
}

/* The walls of a closed box on every particle after the pair sums
 * (parallel/box.h:296-302). */
static void walls_interact(ostate* s) {
  const SppParams* p = s->p;
  owall w[SPP_MAX_WALLS];
  const int nw = box_walls(p, w);
  for (int i = 0; i < s->n; ++i) {
    s->wtq[i] = 0.0;
    wall_terms64(p, w, nw, s->x[i], s->y[i], s->th[i], s->vx[i], s->vy[i], &s->fx[i], &s->fy[i],
                 &s->wtq[i], &s->tq[i]);
  }
}

/* The circular box: Box::Interact, parallel/box.h:285-294 (CIRCULAR_BOX
 * without PERIODIC_BOUNDARY_CONDITION): beyond r = L - 1 the torque
 * 40 g (v_y x - v_x y) / (2 pi r (L - r)) is added with the pair terms --
 * to the continuous model's torque sum, which Move multiplies by g, and
 * after the alignment normalisation of the repulsive model, where the
 * walls' torques go as well. */
static void circle_interact(ostate* s) {
  const SppParams* p = s->p;
  for (int i = 0; i < s->n; ++i) {
    s->wtq[i] = 0.0;
    const double r = sqrt(s->x[i] * s->x[i] + s->y[i] * s->y[i]);
    if (r > p->L - 1) {
      const double t = 40 * p->g * (s->vy[i] * s->x[i] - s->vx[i] * s->y[i]) / (2 * M_PI * r * (p->L - r));
      if (p->model == SPP_MODEL_CONTINUOUS) s->tq[i] += t;
      else s->wtq[i] += t;
    }
  }
}

/* One particle against the segments p->walls[0 .. n_walls) alone (the
 * box walls are segments like these), for the pin against the reference's
 * Wall::Interact. */
void orc64_wall_terms(const SppParams* p, double x, double y, double th, double* out4) {
  owall w[SPP_MAX_WALLS];
  SppParams q = *p;
  q.L = 1e9;                /* box_walls puts its 4 box walls far away: skip them */
  box_walls(&q, w);
  const int nw = p->n_walls;
  for (int e = 0; e < nw; ++e) w[e] = w[e + 4];
  out4[0] = out4[1] = out4[2] = out4[3] = 0.0;
  g_closed = 1;
  if (p->model == SPP_MODEL_VICSEK_REF_ANGLE) {
    /* {count, angle sum, 0, 0} */
    int nb = 0;
    vicsek_walls64(p, w, nw, x, y, th, &nb, &out4[1]);
    out4[0] = nb;
  } else {
    wall_terms64(p, w, nw, x, y, th, cos(th), sin(th), &out4[0], &out4[1], &out4[2], &out4[3]);
  }
  g_closed = 0;
}

static void abp_stage_forces(ostate* s) {
  abp_reset(s);
  interact_all(s, s->p->model == SPP_MODEL_CONTINUOUS ? cont_pair : abp_pair);
  if (s->p->boundary == SPP_BOUNDARY_WALLS) walls_interact(s);
  if (s->p->boundary == SPP_BOUNDARY_CIRCLE) circle_interact(s);
  g_w.cur++;
}

static void abp_step(ostate* s, int64_t step) {
  const SppParams* p = s->p;
  double dt = p->dt, half_dt = 0.5 * dt, dt6 = dt / 6;
  double sigma = sqrt(2 * p->Dr * dt);
  int n = s->n;
  if (p->integrator == SPP_INT_EULER) {
    /* RepulsiveParticle::Move, particle.h:571-587 */
    abp_stage_forces(s);
    for (int i = 0; i < n; ++i) {
      s->dth[i] = sigma * orc_normal(p, i, step);
      s->th[i] += dt * abp_torque(s, i);
      s->th[i] += s->dth[i];
      set_v(s, i);
      s->xu[i] += s->fx[i] * dt; s->yu[i] += s->fy[i] * dt;
      s->x[i] = pt(s->xu[i], p->L); s->y[i] = pt(s->yu[i], p->L);
    }
    return;
  }
  if (p->integrator == SPP_INT_RK2) {
    abp_stage_forces(s);
    for (int i = 0; i < n; ++i) { /* Move_Runge_Kutta2_1, particle.h:589-611 */
      s->dth[i] = sigma * orc_normal(p, i, step);
      s->tho[i] = s->th[i]; s->xo[i] = s->xu[i]; s->yo[i] = s->yu[i];
      s->th[i] += half_dt * abp_torque(s, i);
      s->th[i] += s->dth[i] / 2;
      s->th[i] = wrap_angle(s->th[i]);
      set_v(s, i);
      s->x[i] += s->fx[i] * half_dt; s->y[i] += s->fy[i] * half_dt;
      s->x[i] = pt(s->x[i], p->L); s->y[i] = pt(s->y[i], p->L);
    }
    abp_stage_forces(s);
    for (int i = 0; i < n; ++i) { /* Move_Runge_Kutta2_2, particle.h:613-631 */
      s->th[i] = s->tho[i] + dt * abp_torque(s, i);
      s->th[i] += s->dth[i];
      s->th[i] = wrap_angle(s->th[i]);
      set_v(s, i);
      s->xu[i] = s->xo[i] + s->fx[i] * dt; s->yu[i] = s->yo[i] + s->fy[i] * dt;
      s->x[i] = pt(s->xu[i], p->L); s->y[i] = pt(s->yu[i], p->L);
    }
    return;
  }
  /* RK4, particle.h:633-726 */
  abp_stage_forces(s);
  for (int i = 0; i < n; ++i) {
    s->dth[i] = sigma * orc_normal(p, i, step);
    s->tho[i] = s->th[i]; s->xo[i] = s->xu[i]; s->yo[i] = s->yu[i];
    double t = abp_torque(s, i);
    s->th[i] += half_dt * t;
    s->th[i] += s->dth[i] / 2;
    s->th[i] = wrap_angle(s->th[i]);
    set_v(s, i);
    s->x[i] += s->fx[i] * half_dt; s->y[i] += s->fy[i] * half_dt;
    s->x[i] = pt(s->x[i], p->L); s->y[i] = pt(s->y[i], p->L);
    s->k1f_x[i] = s->fx[i]; s->k1f_y[i] = s->fy[i]; s->k1t[i] = t;
  }
  abp_stage_forces(s);
  for (int i = 0; i < n; ++i) {
    double t = abp_torque(s, i);
    s->th[i] = s->tho[i] + half_dt * t;
    s->th[i] += s->dth[i] / 2;
    s->th[i] = wrap_angle(s->th[i]);
    set_v(s, i);
    s->xu[i] = s->xo[i] + s->fx[i] * half_dt; s->yu[i] = s->yo[i] + s->fy[i] * half_dt;
    s->x[i] = pt(s->xu[i], p->L); s->y[i] = pt(s->yu[i], p->L);
    s->k2f_x[i] = s->fx[i]; s->k2f_y[i] = s->fy[i]; s->k2t[i] = t;
  }
  abp_stage_forces(s);
  for (int i = 0; i < n; ++i) {
    double t = abp_torque(s, i);
    s->th[i] = s->tho[i] + dt * t;
    s->th[i] += s->dth[i];
    s->th[i] = wrap_angle(s->th[i]);
    set_v(s, i);
    s->xu[i] = s->xo[i] + s->fx[i] * dt; s->yu[i] = s->yo[i] + s->fy[i] * dt;
    s->x[i] = pt(s->xu[i], p->L); s->y[i] = pt(s->yu[i], p->L);
    s->k3f_x[i] = s->fx[i]; s->k3f_y[i] = s->fy[i]; s->k3t[i] = t;
  }
  abp_stage_forces(s);
  for (int i = 0; i < n; ++i) {
    double t = abp_torque(s, i);
    s->th[i] = s->tho[i] + (s->k1t[i] + s->k2t[i] * 2 + s->k3t[i] * 2 + t) * dt6;
    s->th[i] += s->dth[i];
    s->th[i] = wrap_angle(s->th[i]);
    set_v(s, i);
    s->xu[i] = s->xo[i] + (s->k1f_x[i] + s->k2f_x[i] * 2 + s->k3f_x[i] * 2 + s->fx[i]) * dt6;
    s->yu[i] = s->yo[i] + (s->k1f_y[i] + s->k2f_y[i] * 2 + s->k3f_y[i] * 2 + s->fy[i]) * dt6;
    s->x[i] = pt(s->xu[i], p->L); s->y[i] = pt(s->yu[i], p->L);
  }
}

/* ------------------------------------------------------------------ */
/* ActiveBrownianChain (nb = 1) bodies + ring membranes                 */
/* ------------------------------------------------------------------ */
/* ActiveBrownianChain::Interact for two single-bead bodies, shared/
 * particle.h:964-984 (R12 with the membrane sigma/cutoff), or the harmonic
 * law; no alignment. */
static void bead_pair(void* ctx, int i, int j) {
  ostate* s = (ostate*)ctx;
  const SppParams* p = s->p;
  double dx = pt(s->x[i] - s->x[j], p->L), dy = pt(s->y[i] - s->y[j], p->L);
  double d = sqrt(dx * dx + dy * dy);
  if (p->force_law != SPP_FORCE_NONE && d < p->r_rep && d > 0) {
    double Fx, Fy;
    if (p->force_law == SPP_FORCE_R12_TRUNC) {
      r12_trunc(dx, dy, d, p->r_rep, p->sigma_rep, p->k_rep, &Fx, &Fy);
    } else {
      double mag = p->k_rep * (1.0 - d / p->r_rep);
      Fx = mag * dx / d;
      Fy = mag * dy / d;
    }
    s->fx[i] += Fx; s->fy[i] += Fy;
    s->fx[j] -= Fx; s->fy[j] -= Fy;
  }
}

static int n_beads(const SppParams* p) { return p->n_rings * p->ring_size; }

/* Beads of body i: membrane beads have one, swimmers chain_beads. */
static int body_nb(const SppParams* p, int i) { return i < n_beads(p) ? 1 : chain_nb(p); }

/* ActiveBrownianChain::Interact, shared/particle.h:964-1012, for bodies of
 * which at least one is a chain: every bead pair at s_i = v_i separation
 * ((1 - nb_i)/2 + a), s_j likewise, within r_chain exchanges the R12 force
 * (sigma_chain, r_chain) on dr = dr0 + s_i - s_j, with the lever-arm
 * torques s_i x F on i and -s_j x F on j. */
static void chain_pair(void* ctx, int i, int j) {
  ostate* s = (ostate*)ctx;
  const SppParams* p = s->p;
  int nbi = body_nb(p, i), nbj = body_nb(p, j);
  if (nbi == 1 && nbj == 1) { bead_pair(ctx, i, j); return; }
  if (p->force_law == SPP_FORCE_NONE) return;
  double dx0 = pt(s->x[i] - s->x[j], p->L), dy0 = pt(s->y[i] - s->y[j], p->L);
  for (int a = 0; a < nbi; ++a)
    for (int b = 0; b < nbj; ++b) {
      double oa = p->bead_separation * ((1 - nbi) / 2.0 + a);
      double ob = p->bead_separation * ((1 - nbj) / 2.0 + b);
      double six = s->vx[i] * oa, siy = s->vy[i] * oa;
      double sjx = s->vx[j] * ob, sjy = s->vy[j] * ob;
      double dx = dx0 + six - sjx, dy = dy0 + siy - sjy;
      double d = sqrt(dx * dx + dy * dy);
      if (d < p->r_chain && d > 0) {
        double Fx, Fy;
        r12_trunc(dx, dy, d, p->r_chain, p->sigma_chain, p->k_rep, &Fx, &Fy);
        s->fx[i] += Fx; s->fy[i] += Fy;
        s->fx[j] -= Fx; s->fy[j] -= Fy;
        s->tq[i] += six * Fy - siy * Fx;
        s->tq[j] += -sjx * Fy + sjy * Fx;
      }
    }
}

/* Mobilities of body i: the configured mu / k_perp for single beads, the
 * Set_nb values for chains. */
static void body_mobility(const SppParams* p, int i, double* mpar, double* mperp, double* kperp) {
  if (body_nb(p, i) > 1) {
    chain_mobility(body_nb(p, i), p->bead_separation, p->sigma_chain, mpar, mperp, kperp);
  } else {
    *mpar = p->mu; *mperp = p->mu; *kperp = p->k_perp;
  }
}

/* ActiveBrownianChain::Reset, particle.h:878-883: torque = torque0, f = F0 v
 * with F0 = v0 / m_parallel for swimmers (speed v0 = m_parallel F0) and 0
 * for membrane beads. */
static void bead_reset(ostate* s) {
  const SppParams* p = s->p;
  int nm = n_beads(p);
  for (int i = 0; i < s->n; ++i) {
    double mpar, mperp, kperp;
    body_mobility(p, i, &mpar, &mperp, &kperp);
    double F0 = i < nm ? 0.0 : p->v0 / mpar;
    s->tq[i] = p->torque0;
    s->fx[i] = F0 * s->vx[i];
    s->fy[i] = F0 * s->vy[i];
  }
}

/* Interact_Membrane_Beads, parallel/beadbox.h:185-196, per ring: Spring
 * (force-fields.h:87-97) between i and (i+1) % M; then the bending forces of
 * E = kappa sum_j (1 - cos phi_j) (no counterpart in the reference). */
static void ring_forces(ostate* s) {
  const SppParams* p = s->p;
  int M = p->ring_size;
  for (int r = 0; r < p->n_rings; ++r) {
    int base = r * M;
    for (int m = 0; m < M; ++m) {
      int a = base + m, b = base + (m + 1) % M;
      double dx = pt(s->x[a] - s->x[b], p->L), dy = pt(s->y[a] - s->y[b], p->L);
      double d = sqrt(dx * dx + dy * dy);
      double Fx = p->k_bond * (p->bond_rest - d) * dx / d;
      double Fy = p->k_bond * (p->bond_rest - d) * dy / d;
      s->fx[a] += Fx; s->fy[a] += Fy;
      s->fx[b] -= Fx; s->fy[b] -= Fy;
    }
    if (p->kappa_bend == 0.0) continue;
    for (int m = 0; m < M; ++m) {
      int jm = base + (m + M - 1) % M, j = base + m, jp = base + (m + 1) % M;
      double ux = pt(s->x[j] - s->x[jm], p->L), uy = pt(s->y[j] - s->y[jm], p->L);
      double wx = pt(s->x[jp] - s->x[j], p->L), wy = pt(s->y[jp] - s->y[j], p->L);
      double lu = sqrt(ux * ux + uy * uy), lw = sqrt(wx * wx + wy * wy);
      double c = (ux * wx + uy * wy) / (lu * lw);
      double dux = wx / (lu * lw) - c * ux / (lu * lu), duy = wy / (lu * lw) - c * uy / (lu * lu);
      double dwx = ux / (lu * lw) - c * wx / (lw * lw), dwy = uy / (lu * lw) - c * wy / (lw * lw);
      double kp = p->kappa_bend;
      s->fx[jm] -= kp * dux; s->fy[jm] -= kp * duy;
      s->fx[j] += kp * (dux - dwx); s->fy[j] += kp * (duy - dwy);
      s->fx[jp] += kp * dwx; s->fy[jp] += kp * dwy;
    }
  }
}

static void bead_stage_forces(ostate* s) {
  bead_reset(s);
  ring_forces(s);
  interact_all(s, chain_nb(s->p) > 1 ? chain_pair : bead_pair);
}

/* Moves of ActiveBrownianChain (particle.h:898-962) with m_parallel =
 * m_perpendicular = mu: dr = mu f h, dtheta = k_perp torque h (+ noise for
 * swimmers).  RK4 follows RepulsiveParticle's scheme (:633-726) with these
 * rates (no reference counterpart for beads).  Membrane beads keep their
 * heading (F0 = 0 makes it irrelevant to their motion). */
/* RTPChain::Noise_Gen (shared/particle.h:1085-1103): a running swimmer
 * starts a tumble of random sign with probability lambda dt; a tumble lasts
 * while its elapsed time, accumulated in steps of dt, is < t_tumble. */
static double tumble_noise(ostate* s, int i, int64_t step) {
  const SppParams* p = s->p;
  if (s->tflag[i] == 0) {
    double u = spp_u01_d(spp_draw(p->seed, p->system_id, (uint32_t)i, (uint32_t)step, SPP_RNG_TUMBLE).v[0]);
    if (u < p->tumble_rate * p->dt) {
      double u2 = spp_u01_d(spp_draw(p->seed, p->system_id, (uint32_t)i, (uint32_t)step, SPP_RNG_TUMBLE_SIGN).v[0]);
      s->tflag[i] = 2 * (int)(unsigned long)(u2 * 2.0) - 1;
      s->telapsed[i] += p->dt;
    }
  } else {
    if (s->telapsed[i] < p->tumble_time) {
      s->telapsed[i] += p->dt;
    } else {
      s->telapsed[i] = 0;
      s->tflag[i] = 0;
    }
  }
  double mpar, mperp, kperp;
  body_mobility(p, i, &mpar, &mperp, &kperp);
  return kperp * p->dt * s->tflag[i] * p->tumble_torque;
}

static void bead_step(ostate* s, int64_t step) {
  const SppParams* p = s->p;
  double dt = p->dt, half_dt = 0.5 * dt, dt6 = dt / 6;
  double sigma = sqrt(2 * p->Dr * dt);
  int n = s->n, nm = n_beads(p);
  int nst = p->integrator == SPP_INT_RK4 ? 4 : (p->integrator == SPP_INT_RK2 ? 2 : 1);
  for (int stage = 0; stage < nst; ++stage) {
    bead_stage_forces(s);
    for (int i = 0; i < n; ++i) {
      int swim = i >= nm;
      double mpar, mperp, kperp;
      body_mobility(p, i, &mpar, &mperp, &kperp);
      double om = swim ? kperp * s->tq[i] : 0.0;
      if (stage == 0) {
        if (!swim) s->dth[i] = 0.0;
        else if (p->rot_noise == SPP_NOISE_TUMBLE) s->dth[i] = tumble_noise(s, i, step);
        else s->dth[i] = sigma * orc_normal(p, i, step);
        s->tho[i] = s->th[i]; s->xo[i] = s->xu[i]; s->yo[i] = s->yu[i];
      }
      /* m_perp f + (m_par - m_perp) (f . w) w, w the heading the forces
       * were evaluated at; Move() (Euler) turns first and projects on the
       * new heading (particle.h:898-915) */
      double wx = s->vx[i], wy = s->vy[i];
      if (nst == 1 && swim) {
        double tn = s->tho[i] + dt * om + s->dth[i];
        wx = cos(tn); wy = sin(tn);
      }
      double fw = s->fx[i] * wx + s->fy[i] * wy;
      double vx = mperp * s->fx[i] + (mpar - mperp) * fw * wx;
      double vy = mperp * s->fy[i] + (mpar - mperp) * fw * wy;
      double h, frac;
      if (nst == 1) { h = dt; frac = 1; }
      else if (nst == 2) { h = stage == 0 ? half_dt : dt; frac = stage == 0 ? 0.5 : 1.0; }
      else {
        if (stage == 0) { s->k1f_x[i] = vx; s->k1f_y[i] = vy; s->k1t[i] = om; }
        else if (stage == 1) { s->k2f_x[i] = vx; s->k2f_y[i] = vy; s->k2t[i] = om; }
        else if (stage == 2) { s->k3f_x[i] = vx; s->k3f_y[i] = vy; s->k3t[i] = om; }
        else {
          vx = s->k1f_x[i] + s->k2f_x[i] * 2 + s->k3f_x[i] * 2 + vx;
          vy = s->k1f_y[i] + s->k2f_y[i] * 2 + s->k3f_y[i] * 2 + vy;
          om = s->k1t[i] + s->k2t[i] * 2 + s->k3t[i] * 2 + om;
        }
        h = stage < 2 ? half_dt : (stage == 2 ? dt : dt6);
        frac = stage < 2 ? 0.5 : 1.0;
      }
      if (swim) {
        s->th[i] = s->tho[i] + h * om + frac * s->dth[i];
        if (nst > 1) s->th[i] = wrap_angle(s->th[i]);
      }
      double nxu = s->xo[i] + vx * h, nyu = s->yo[i] + vy * h;
      if (stage == nst - 1) { s->xu[i] = nxu; s->yu[i] = nyu; }
      s->x[i] = pt(nxu, p->L);
      s->y[i] = pt(nyu, p->L);
    }
    for (int i = 0; i < n; ++i) set_v(s, i);
  }
}

/* ContinuousParticle::Move (Euler), shared/particle.h:268-293 */
static void cont_euler_step(ostate* s, int64_t step) {
  const SppParams* p = s->p;
  double dt = p->dt, sigma = sqrt(2 * p->Dr * dt);
  for (int i = 0; i < s->n; ++i) { s->nb[i] = 1; s->tq[i] = 0; }
  interact_all(s, cont_pair);
  if (p->boundary == SPP_BOUNDARY_WALLS) walls_interact(s);
  if (p->boundary == SPP_BOUNDARY_CIRCLE) circle_interact(s);
  g_w.cur++;
  for (int i = 0; i < s->n; ++i) {
    double torque = p->g * s->tq[i] + sigma * orc_normal(p, i, step);
    s->th[i] += torque * dt;
    set_v(s, i);
    s->xu[i] += s->vx[i] * (p->v0 * dt); s->yu[i] += s->vy[i] * (p->v0 * dt);
    s->x[i] = pt(s->xu[i], p->L); s->y[i] = pt(s->yu[i], p->L);
  }
}

/* ------------------------------------------------------------------ */
/* Vicsek models                                                       */
/* ------------------------------------------------------------------ */
static void vicsek_move_common(ostate* s, int i) {
  const SppParams* p = s->p;
  set_v(s, i);
  s->xu[i] += s->vx[i] * (p->dt * p->v0); s->yu[i] += s->vy[i] * (p->dt * p->v0);
  s->x[i] = pt(s->x[i] + s->vx[i] * (p->dt * p->v0), p->L);
  s->y[i] = pt(s->y[i] + s->vy[i] * (p->dt * p->v0), p->L);
}

static void vicsek_step(ostate* s, int64_t step) {
  const SppParams* p = s->p;
  int n = s->n;
  for (int i = 0; i < n; ++i) { s->nb[i] = 0; s->avx[i] = s->avy[i] = s->ath[i] = 0; }
  if (p->model == SPP_MODEL_VICSEK) {
    for (int i = 0; i < n; ++i) { s->avx[i] = s->vx[i]; s->avy[i] = s->vy[i]; } /* self term */
    interact_all(s, vicsek_sum_pair);
    for (int i = 0; i < n; ++i) {
      double th = atan2(s->avy[i], s->avx[i]) + p->eta * orc_uniform_pm_pi(p, i, step);
      s->th[i] = wrap_angle(th);
      vicsek_move_common(s, i);
    }
  } else if (p->model == SPP_MODEL_VICSEK_REF_ANGLE) {
    interact_all(s, vicsek_angle_pair);
    if (p->boundary == SPP_BOUNDARY_WALLS) {
      owall w[SPP_MAX_WALLS];
      const int nw = box_walls(p, w);
      for (int i = 0; i < n; ++i) vicsek_walls64(p, w, nw, s->x[i], s->y[i], s->th[i], &s->nb[i], &s->ath[i]);
    }
    for (int i = 0; i < n; ++i) { /* VicsekParticle::Move, particle.h:148-163 */
      double avg = s->nb[i] > 0 ? s->ath[i] / s->nb[i] : s->th[i];
      s->th[i] = avg + p->eta * orc_uniform_pm_pi(p, i, step);
      vicsek_move_common(s, i);
    }
  } else {
    interact_all(s, vicsek_vector_pair);
    for (int i = 0; i < n; ++i) { /* VicsekParticle2::Move, particle.h:198-213 */
      if (s->nb[i] == 0) { s->avx[i] = s->vx[i]; s->avy[i] = s->vy[i]; }
      double ra = orc_uniform_pm_pi(p, i, step);
      s->avx[i] += s->nb[i] * p->eta * cos(ra);
      s->avy[i] += s->nb[i] * p->eta * sin(ra);
      s->th[i] = atan2(s->avy[i], s->avx[i]);
      vicsek_move_common(s, i);
    }
  }
}

/* ------------------------------------------------------------------ */
/* exported                                                            */
/* ------------------------------------------------------------------ */
/* Runs nsteps steps starting at absolute step index step0.
 * x,y: wrapped positions; xu,yu: unwrapped (r_original); th: headings. */
int orc64_run(const SppParams* p, int nsteps, int64_t step0, double* x, double* y, double* th,
              double* xu, double* yu) {
  ostate s;
  state_alloc(&s, p);
  int n = p->n;
  memcpy(s.x, x, sizeof(double) * n); memcpy(s.y, y, sizeof(double) * n);
  memcpy(s.xu, xu, sizeof(double) * n); memcpy(s.yu, yu, sizeof(double) * n);
  memcpy(s.th, th, sizeof(double) * n);
  for (int i = 0; i < n; ++i) set_v(&s, i);
  int rc = 0;
  g_closed = p->boundary == SPP_BOUNDARY_WALLS || p->boundary == SPP_BOUNDARY_CIRCLE;
  for (int k = 0; k < nsteps; ++k) {
    int64_t step = step0 + k;
    switch (p->model) {
      case SPP_MODEL_VICSEK:
      case SPP_MODEL_VICSEK_REF_ANGLE:
      case SPP_MODEL_VICSEK_REF_VECTOR: vicsek_step(&s, step); break;
      case SPP_MODEL_ABP: abp_step(&s, step); break;
      case SPP_MODEL_BEADS: bead_step(&s, step); break;
      case SPP_MODEL_CONTINUOUS:
        if (p->integrator == SPP_INT_EULER) cont_euler_step(&s, step);
        else abp_step(&s, step);
        break;
      default: rc = SPP_ERR_UNSUPPORTED; k = nsteps; break;
    }
  }
  memcpy(x, s.x, sizeof(double) * n); memcpy(y, s.y, sizeof(double) * n);
  memcpy(xu, s.xu, sizeof(double) * n); memcpy(yu, s.yu, sizeof(double) * n);
  memcpy(th, s.th, sizeof(double) * n);
  g_closed = 0;
  state_free(&s);
  return rc;
}

/* Unique pairs (i<j) with sqrt(d2) < r, the reference's predicate
 * (shared/cell.h:84-86). Returns the total count; writes up to cap. */
typedef struct { const double *x, *y; double L, r; int32_t *pi, *pj; int64_t cap, cnt; } pairctx;
static void pair_collect(void* ctx, int i, int j) {
  pairctx* c = (pairctx*)ctx;
  double dx = pt(c->x[i] - c->x[j], c->L), dy = pt(c->y[i] - c->y[j], c->L);
  if (sqrt(dx * dx + dy * dy) < c->r) {
    if (c->cnt < c->cap) {
      c->pi[c->cnt] = i < j ? i : j;
      c->pj[c->cnt] = i < j ? j : i;
    }
    c->cnt++;
  }
}
int64_t orc64_pairs(int n, const double* x, const double* y, double L, double r, int32_t* pi,
                    int32_t* pj, int64_t cap) {
  ocells c;
  cells_build(&c, n, x, y, L, r);
  pairctx ctx = {x, y, L, r, pi, pj, cap, 0};
  cells_for_pairs(&c, n, pair_collect, &ctx);
  cells_free(&c);
  return ctx.cnt;
}

/* Box::Update_Cells binning (serial/box.h:116-117) and the geometric rule. */
void orc_cells(int n, const double* x, const double* y, double L, int D, int rule, int32_t* cx,
               int32_t* cy) {
  for (int i = 0; i < n; ++i) {
    int a, b;
    if (rule == SPP_BIN_REFERENCE) {
      a = (int)((int)(x[i] + L) * D / (2.0 * L));
      b = (int)((int)(y[i] + L) * D / (2.0 * L));
    } else {
      a = (int)floor((x[i] + L) * D / (2.0 * L));
      b = (int)floor((y[i] + L) * D / (2.0 * L));
    }
    if (a >= D) a = D - 1; if (a < 0) a = 0;
    if (b >= D) b = D - 1; if (b < 0) b = 0;
    cx[i] = a; cy[i] = b;
  }
}

/* Polarization |(1/N) sum v_i| (parallel/node.h:1565-1591). */
double orc_polarization(int n, const double* th, double* px, double* py) {
  double sx = 0, sy = 0;
  for (int i = 0; i < n; ++i) { sx += cos(th[i]); sy += sin(th[i]); }
  sx /= n; sy /= n;
  if (px) *px = sx;
  if (py) *py = sy;
  return sqrt(sx * sx + sy * sy);
}

/* ------------------------------------------------------------------ */
/* Lyapunov spectrum                                                   */
/* ------------------------------------------------------------------ */
/* Modified Gram-Schmidt on K vectors of length len (VectorSet::
 * Renormalize(us), shared/vector-set.h:118-127: each vector loses its
 * projections on the already orthonormalised ones, then is normalised);
 * log of each norm added to log_stretch[a] (when not NULL) after dividing by
 * scale. */
static void mgs(int K, size_t len, double* V, double* log_stretch, double scale) {
  for (int a = 0; a < K; ++a) {
    double* va = V + (size_t)a * len;
    for (int b = 0; b < a; ++b) {
      const double* vb = V + (size_t)b * len;
      double dot = 0;
      for (size_t e = 0; e < len; ++e) dot += vb[e] * va[e];
      for (size_t e = 0; e < len; ++e) va[e] -= dot * vb[e];
    }
    double nn = 0;
    for (size_t e = 0; e < len; ++e) nn += va[e] * va[e];
    double nrm = sqrt(nn);
    for (size_t e = 0; e < len; ++e) va[e] /= nrm;
    if (log_stretch) log_stretch[a] += log(nrm / scale);
  }
}

/* The clone method's renormalisation on its own: K deviation vectors
 * [K][3][n] are orthonormalised in place and log(|R_aa| / scale) is added
 * to log_stretch[a], where R_aa is what LyapunovBox's growth ratio
 * (parallel/lyapunovbox.h:177-181) measures times the amplitude. */
int orc64_gram_schmidt(int K, int n, double* V, double* log_stretch, double scale) {
  if (K < 1 || n < 1 || !V) return SPP_ERR_INVALID;
  mgs(K, (size_t)3 * n, V, log_stretch, scale);
  return SPP_OK;
}

typedef struct {
  ostate* s;
  const double* U;  /* stage tangent input [K][3][n] */
  double* T;        /* theta slope sums [K][n] */
  int K;
} tctx;

/* sum_j cos(th_j - th_i) (u_j - u_i) over pairs within the alignment radius */
static void tangent_pair(void* ctx, int i, int j) {
  tctx* c = (tctx*)ctx;
  ostate* s = c->s;
  const SppParams* p = s->p;
  double dx = pt(s->x[i] - s->x[j], p->L), dy = pt(s->y[i] - s->y[j], p->L);
  if (dx * dx + dy * dy < p->r_align * p->r_align) {
    double cij = cos(s->th[j] - s->th[i]);
    int n = s->n;
    for (int v = 0; v < c->K; ++v) {
      double ui = c->U[(size_t)(v * 3 + 2) * n + i], uj = c->U[(size_t)(v * 3 + 2) * n + j];
      c->T[(size_t)v * n + i] += cij * (uj - ui);
      c->T[(size_t)v * n + j] += cij * (ui - uj);
    }
  }
}

/* Tangent-space estimator in FP64: continuous model (alpha = 0), RK2/RK4
 * base steps (abp_step's RK schemes) with the tangent vectors advanced by
 * the derivative of each stage; MGS every renorm_every steps and at the end.
 * V is [K][x|y|theta][n] (orthonormal on entry). */
int orc64_lyap_tangent(const SppParams* p, int nsteps, int renorm_every, int K, double* x, double* y,
                       double* th, double* xu, double* yu, double* V, double* log_stretch) {
  if (p->model != SPP_MODEL_CONTINUOUS || p->alpha != 0.0 || p->integrator == SPP_INT_EULER)
    return SPP_ERR_UNSUPPORTED;
  ostate s;
  state_alloc(&s, p);
  int n = p->n;
  memcpy(s.x, x, sizeof(double) * n); memcpy(s.y, y, sizeof(double) * n);
  memcpy(s.xu, xu, sizeof(double) * n); memcpy(s.yu, yu, sizeof(double) * n);
  memcpy(s.th, th, sizeof(double) * n);
  for (int i = 0; i < n; ++i) set_v(&s, i);
  size_t len = (size_t)K * 3 * n;
  double *U = malloc(sizeof(double) * len), *ACC = malloc(sizeof(double) * len);
  double *T = malloc(sizeof(double) * (size_t)K * n), *SL = malloc(sizeof(double) * len);
  int nst = p->integrator == SPP_INT_RK4 ? 4 : 2;
  double dt = p->dt, gp = p->g * (1 - p->alpha) / M_PI;
  double sigma = sqrt(2 * p->Dr * dt);
  for (int st = 0; st < nsteps; ++st) {
    for (int i = 0; i < n; ++i) {
      s.tho[i] = s.th[i]; s.xo[i] = s.xu[i]; s.yo[i] = s.yu[i];
      s.dth[i] = sigma * orc_normal(p, i, st);
    }
    memcpy(U, V, sizeof(double) * len);
    for (int stage = 0; stage < nst; ++stage) {
      /* tangent slopes at this stage state */
      memset(T, 0, sizeof(double) * (size_t)K * n);
      tctx c = {&s, U, T, K};
      ocells cl;
      cells_build(&cl, n, s.x, s.y, p->L, p->r_align);
      cells_for_pairs(&cl, n, tangent_pair, &c);
      cells_free(&cl);
      for (int v = 0; v < K; ++v)
        for (int i = 0; i < n; ++i) {
          double ut = U[(size_t)(v * 3 + 2) * n + i];
          SL[(size_t)(v * 3 + 0) * n + i] = -p->v0 * sin(s.th[i]) * ut;
          SL[(size_t)(v * 3 + 1) * n + i] = p->v0 * cos(s.th[i]) * ut;
          SL[(size_t)(v * 3 + 2) * n + i] = gp * T[(size_t)v * n + i];
        }
      /* base stage (forces at the same state) */
      abp_stage_forces(&s);
      double h, hw, frac;
      if (nst == 2) { h = stage == 0 ? 0.5 * dt : dt; hw = h; frac = stage == 0 ? 0.5 : 1.0; }
      else { h = stage < 2 ? 0.5 * dt : dt; hw = stage == 3 ? dt / 6 : h; frac = stage < 2 ? 0.5 : 1.0; }
      for (int i = 0; i < n; ++i) {
        double t = abp_torque(&s, i), fx = s.fx[i], fy = s.fy[i];
        if (nst == 4) {
          if (stage == 0) { s.k1f_x[i] = fx; s.k1f_y[i] = fy; s.k1t[i] = t; }
          else if (stage == 1) { s.k2f_x[i] = fx; s.k2f_y[i] = fy; s.k2t[i] = t; }
          else if (stage == 2) { s.k3f_x[i] = fx; s.k3f_y[i] = fy; s.k3t[i] = t; }
          else {
            t = s.k1t[i] + s.k2t[i] * 2 + s.k3t[i] * 2 + t;
            fx = s.k1f_x[i] + s.k2f_x[i] * 2 + s.k3f_x[i] * 2 + fx;
            fy = s.k1f_y[i] + s.k2f_y[i] * 2 + s.k3f_y[i] * 2 + fy;
          }
        }
        s.th[i] = wrap_angle(s.tho[i] + hw * t + frac * s.dth[i]);
        double nxu = s.xo[i] + fx * hw, nyu = s.yo[i] + fy * hw;
        if (stage == nst - 1) { s.xu[i] = nxu; s.yu[i] = nyu; }
        s.x[i] = pt(nxu, p->L); s.y[i] = pt(nyu, p->L);
      }
      for (int i = 0; i < n; ++i) set_v(&s, i);
      /* tangent stage update */
      for (size_t e = 0; e < len; ++e) {
        double sl = SL[e];
        if (nst == 2) {
          if (stage == 0) U[e] = V[e] + 0.5 * dt * sl;
          else V[e] = V[e] + dt * sl;
        } else {
          if (stage == 0) { ACC[e] = sl; U[e] = V[e] + 0.5 * dt * sl; }
          else if (stage == 1) { ACC[e] += 2 * sl; U[e] = V[e] + 0.5 * dt * sl; }
          else if (stage == 2) { ACC[e] += 2 * sl; U[e] = V[e] + dt * sl; }
          else V[e] = V[e] + dt / 6 * (ACC[e] + sl);
        }
      }
    }
    if (renorm_every > 0 && ((st + 1) % renorm_every == 0 || st + 1 == nsteps))
      mgs(K, (size_t)3 * n, V, log_stretch, 1.0);
  }
  memcpy(x, s.x, sizeof(double) * n); memcpy(y, s.y, sizeof(double) * n);
  memcpy(xu, s.xu, sizeof(double) * n); memcpy(yu, s.yu, sizeof(double) * n);
  memcpy(th, s.th, sizeof(double) * n);
  free(U); free(ACC); free(T); free(SL);
  state_free(&s);
  return SPP_OK;
}

/* Benettin clone method of LyapunovBox::Evolution_Reorthonormalize
 * (parallel/lyapunovbox.h:128-194): per interval of tau steps, each
 * direction u_a (orthonormal, [K][3][n]) seeds a clone base + eps u_a
 * (Add_Deviation, :46-67); the clones and the base evolve with the full
 * dynamics; the differences (State_Hyper_Vector::operator-, min image and
 * wrapped angle) are Gram-Schmidt'ed into the next directions, and
 * log(|projection| / eps) (the ratio of :177-183) is summed per direction. */
/* One system of an interval of the clone method: the base (a < 0) or
 * clone a, evolved tau steps on its own thread (orc64_run keeps its state
 * in thread-local storage). */
#define ORC_CLONE_MAX 16
typedef struct {
  const SppParams* p;
  int tau;
  int64_t step;
  double *x, *y, *th, *xu, *yu;
  int rc;
} clone_job;

static void* clone_thread(void* arg) {
  clone_job* j = (clone_job*)arg;
  j->rc = orc64_run(j->p, j->tau, j->step, j->x, j->y, j->th, j->xu, j->yu);
  return NULL;
}

int orc64_lyap_clone(const SppParams* p, int n_intervals, int tau, int K, double eps, double* x,
                     double* y, double* th, double* xu, double* yu, double* V, double* log_stretch) {
  int n = p->n;
  size_t len = (size_t)3 * n;
  /* system 0 is the base trajectory, 1..K the clones base + eps u_a */
  double* buf = malloc(sizeof(double) * (size_t)5 * n * (size_t)(K + 1));
  clone_job job[ORC_CLONE_MAX + 1];
  pthread_t tid[ORC_CLONE_MAX + 1];
  int started[ORC_CLONE_MAX + 1];
  int64_t step = 0;
  int rc = SPP_OK;
  if (K > ORC_CLONE_MAX) rc = SPP_ERR_INVALID;
  for (int it = 0; it < n_intervals && rc == SPP_OK; ++it) {
    for (int a = 0; a <= K; ++a) {
      double* q = buf + (size_t)5 * n * a;
      clone_job* j = &job[a];
      j->p = p; j->tau = tau; j->step = step;
      j->x = q; j->y = q + n; j->th = q + 2 * n; j->xu = q + 3 * n; j->yu = q + 4 * n;
      const double* u = a == 0 ? NULL : V + (size_t)(a - 1) * len;
      for (int i = 0; i < n; ++i) {
        const double ux = u ? eps * u[i] : 0.0, uy = u ? eps * u[n + i] : 0.0;
        const double ut = u ? eps * u[2 * n + i] : 0.0;
        j->x[i] = u ? pt(x[i] + ux, p->L) : x[i];
        j->y[i] = u ? pt(y[i] + uy, p->L) : y[i];
        j->th[i] = th[i] + ut;
        j->xu[i] = xu[i] + ux;
        j->yu[i] = yu[i] + uy;
      }
    }
    for (int a = 0; a <= K; ++a) {
      started[a] = pthread_create(&tid[a], NULL, clone_thread, &job[a]) == 0;
      if (!started[a]) clone_thread(&job[a]);   /* no thread: run it here */
    }
    for (int a = 0; a <= K; ++a)
      if (started[a]) pthread_join(tid[a], NULL);
    for (int a = 0; a <= K; ++a)
      if (job[a].rc != SPP_OK) rc = job[a].rc;
    if (rc != SPP_OK) break;
    const clone_job* b = &job[0];
    for (int a = 0; a < K; ++a) {
      const clone_job* c = &job[a + 1];
      double* w = V + (size_t)a * len;
      for (int i = 0; i < n; ++i) {
        double dth = c->th[i] - b->th[i];
        w[i] = pt(c->x[i] - b->x[i], p->L);
        w[n + i] = pt(c->y[i] - b->y[i], p->L);
        w[2 * n + i] = dth - 2 * M_PI * ceil((dth - M_PI) / (2 * M_PI));
      }
    }
    mgs(K, len, V, log_stretch, eps);
    memcpy(x, b->x, sizeof(double) * n); memcpy(y, b->y, sizeof(double) * n);
    memcpy(th, b->th, sizeof(double) * n); memcpy(xu, b->xu, sizeof(double) * n);
    memcpy(yu, b->yu, sizeof(double) * n);
    step += tau;
  }
  free(buf);
  return rc;
}
