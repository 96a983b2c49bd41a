/*
 * ORACLE -- test infrastructure only (tests/, smoke() and bench.py's CPU
 * baseline call it as the checker; the product never links it).
 *
 * CPU execution of the kernels' FP32 arithmetic.  The per-pair and
 * per-particle formulas come from spp_gb300/csrc/spp_physics.h, the header
 * the kernels compile; everything around them is restated here in the
 * simplest serial form: a plain cell list rebuilt every stage, particles in
 * id order, no Verlet list, no reordering, no graphs.  The neighbour sums
 * are FP32 in ascending particle id (Verlet models, matching the kernels'
 * id-sorted lists) or order-independent fixed point (Vicsek models), so the
 * GPU must reproduce these bits exactly; any difference is a fault in
 * binning, lists, reordering or the rebuild trigger.  Its physics is checked independently against the FP64
 * restatement (spp_oracle64.c), which is itself pinned to the reference
 * (ref_harness.cpp).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "../include/spp.h"
#include "../spp_gb300/csrc/spp_physics.h"

typedef struct {
  int D;
  int* head;
  int* next;
} mcells;

static void mcells_build(mcells* c, int n, const float* x, const float* y, const SppConsts* k,
                         double rcut) {
  int D = (int)floor(2.0 * (double)k->L / (rcut * 1.001));
  if (D < 3) D = 1;
  c->D = D;
  c->head = (int*)malloc(sizeof(int) * (size_t)D * D);
  c->next = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  for (int q = 0; q < D * D; ++q) c->head[q] = -1;
  for (int i = n - 1; i >= 0; --i) {
    int cx = spp_cell_coord(x[i], k->L, k->L2, D, SPP_BIN_GEOMETRIC);
    int cy = spp_cell_coord(y[i], k->L, k->L2, D, SPP_BIN_GEOMETRIC);
    c->next[i] = c->head[cx * D + cy];
    c->head[cx * D + cy] = i;
  }
}
static void mcells_free(mcells* c) { free(c->head); free(c->next); }

/* Calls visit(j) for every candidate j of particle i (i itself included). */
#define FOR_CANDIDATES(c, k, xi, yi, n, j, ...)                                      \
  do {                                                                               \
    if ((c)->D == 1) {                                                               \
      for (int j = 0; j < (n); ++j) { __VA_ARGS__ }                                         \
    } else {                                                                         \
      int _cx = spp_cell_coord(xi, (k)->L, (k)->L2, (c)->D, SPP_BIN_GEOMETRIC);      \
      int _cy = spp_cell_coord(yi, (k)->L, (k)->L2, (c)->D, SPP_BIN_GEOMETRIC);      \
      for (int _ox = -1; _ox <= 1; ++_ox)                                            \
        for (int _oy = -1; _oy <= 1; ++_oy) {                                        \
          int _nx = (_cx + _ox + (c)->D) % (c)->D, _ny = (_cy + _oy + (c)->D) % (c)->D; \
          for (int j = (c)->head[_nx * (c)->D + _ny]; j >= 0; j = (c)->next[j]) { __VA_ARGS__ } \
        }                                                                            \
    }                                                                                \
  } while (0)

/* Cutoff-event recorder, the FP32 counterpart of orc64_watch: pair
 * evaluations whose separation lies within `window` of the alignment radius
 * are recorded as (stage, i, j, inside, d) with the kernels' own predicate
 * (d2 < ral2 in FP32, d2 from spp_sep); stage counts the force evaluations
 * since orc32_watch(). */
static struct {
  int32_t *stage, *pi, *pj;
  int8_t* inside;
  double* dist;
  int64_t cap, cnt;
  double r, window;
  int32_t cur;
  int on;
} g_w32;

void orc32_watch(int32_t* stage, int32_t* pi, int32_t* pj, int8_t* inside, double* dist, int64_t cap,
                 double r, double window) {
  g_w32.stage = stage; g_w32.pi = pi; g_w32.pj = pj; g_w32.inside = inside; g_w32.dist = dist;
  g_w32.cap = cap; g_w32.cnt = 0; g_w32.r = r; g_w32.window = window; g_w32.cur = 0;
  g_w32.on = stage != NULL;
}
int64_t orc32_watch_count(void) { return g_w32.cnt; }

static void watch32(const SppConsts* k, int i, int j, float xi, float yi, float xj, float yj) {
  float dx, dy;
  const float d2 = spp_sep(k, xi, yi, xj, yj, &dx, &dy);
  const double d = sqrt((double)d2);
  if (fabs(d - g_w32.r) >= g_w32.window) return;
  if (g_w32.cnt < g_w32.cap) {
    g_w32.stage[g_w32.cnt] = g_w32.cur;
    g_w32.pi[g_w32.cnt] = i;
    g_w32.pj[g_w32.cnt] = j;
    g_w32.inside[g_w32.cnt] = (int8_t)(d2 < k->ral2);
    g_w32.dist[g_w32.cnt] = d;
  }
  g_w32.cnt++;
}

static double mirror_rcut(const SppParams* p) { return spp_interaction_range(p); }

static int cmp_int(const void* a, const void* b) {
  int x = *(const int*)a, y = *(const int*)b;
  return (x > y) - (x < y);
}

/* Sums received by every particle from the state (x, y, c, s), neighbours
 * taken in ascending particle id (the order of the kernels' sorted lists). */
static int abp_accumulate(const SppConsts* k, int n, const float* x, const float* y, const float* c,
                          const float* s, double rcut, SppAccF* acc) {
  mcells cl;
  mcells_build(&cl, n, x, y, k, rcut);
  int ovf = 0;
  int cap = 64;
  int* cand = (int*)malloc(sizeof(int) * cap);
  for (int i = 0; i < n; ++i) {
    SppAccF a;
    spp_accf_zero(&a);
    int m = 0;
    FOR_CANDIDATES(&cl, k, x[i], y[i], n, j, {
      if (j != i) {
        if (m == cap) { cap *= 2; cand = (int*)realloc(cand, sizeof(int) * cap); }
        cand[m++] = j;
      }
    });
    qsort(cand, (size_t)m, sizeof(int), cmp_int);
    if (g_w32.on)
      for (int q = 0; q < m; ++q)
        if (cand[q] > i) watch32(k, i, cand[q], x[i], y[i], x[cand[q]], y[cand[q]]);
    if (k->lanes > 1) {
      /* the kernels' lane split: lane r sums the neighbours with id % 4 == r
       * in id order, then (p0 + p1) + (p2 + p3) */
      SppAccF part[SPP_GATHER_LANES];
      for (int r = 0; r < SPP_GATHER_LANES; ++r) spp_accf_zero(&part[r]);
      for (int q = 0; q < m; ++q) {
        int j = cand[q];
        spp_pair_abp(k, &part[j & 3], x[i], y[i], c[i], s[i], x[j], y[j], c[j], s[j]);
      }
      a.fx = spp_lane_sum4(part[0].fx, part[1].fx, part[2].fx, part[3].fx);
      a.fy = spp_lane_sum4(part[0].fy, part[1].fy, part[2].fy, part[3].fy);
      a.tq = spp_lane_sum4(part[0].tq, part[1].tq, part[2].tq, part[3].tq);
      a.ss = spp_lane_sum4(part[0].ss, part[1].ss, part[2].ss, part[3].ss);
      a.sc = spp_lane_sum4(part[0].sc, part[1].sc, part[2].sc, part[3].sc);
      a.cnt = part[0].cnt + part[1].cnt + part[2].cnt + part[3].cnt;
      a.ovf = part[0].ovf | part[1].ovf | part[2].ovf | part[3].ovf;
      ovf |= a.ovf;
      acc[i] = a;
      continue;
    }
    const int chain = spp_pair_kind(k) == SPP_KIND_CHAIN;
    const int nbi = chain && i >= k->n_beads ? k->chain_nb : 1;
    for (int q = 0; q < m; ++q) {
      int j = cand[q];
      if (chain) {
        const int nbj = j >= k->n_beads ? k->chain_nb : 1;
        spp_pair_chain(k, k->force_law, 1, &a, nbi, nbj, x[i], y[i], c[i], s[i], x[j], y[j], c[j], s[j]);
      } else {
        spp_pair_abp(k, &a, x[i], y[i], c[i], s[i], x[j], y[j], c[j], s[j]);
      }
    }
    ovf |= a.ovf;
    acc[i] = a;
  }
  free(cand);
  mcells_free(&cl);
  g_w32.cur++;
  return ovf;
}

/* Velocity, angular velocity and noise of body i from its received sums
 * (ABP/continuous: spp_abp_forces; beads: ring forces + spp_bead_velocity). */
static void body_rates(const SppConsts* k, int i, const SppAccF* a, const float* cx,
                       const float* cy, float ci, float si, uint32_t step, const float* tdth,
                       float th0, int euler, float* fx, float* fy, float* tau, float* dth) {
  if (k->model == SPP_MODEL_BEADS) {
    int bead = i < k->n_beads;
    float rfx = 0.0f, rfy = 0.0f;
    if (bead) {
      float px[5], py[5];
      for (int o = -2; o <= 2; ++o) {
        uint32_t j = spp_ring_neighbor(k, (uint32_t)i, o);
        px[o + 2] = cx[j];
        py[o + 2] = cy[j];
      }
      spp_ring_forces(k, px, py, &rfx, &rfy);
    }
    *dth = bead ? 0.0f : (tdth ? tdth[i] : spp_rot_noise(k, (uint32_t)i, step));
    if (!bead && k->chain_nb > 1) {
      spp_chain_velocity(k, a, ci, si, ci, si, fx, fy, tau);
      if (euler) { /* Move() projects on the heading after the turn */
        float wc, ws;
        spp_sincosf(spp_euler_theta(k, th0, *tau, *dth), &ws, &wc);
        spp_chain_velocity(k, a, ci, si, wc, ws, fx, fy, tau);
      }
    } else {
      spp_bead_velocity(k, !bead, a, rfx, rfy, ci, si, fx, fy, tau);
    }
  } else {
    spp_abp_forces(k, k->closed, a, cx[i], cy[i], ci, si, fx, fy, tau);
    *dth = spp_rot_noise(k, (uint32_t)i, step);
  }
}

static int abp_run32(const SppParams* p, const SppConsts* k, int nsteps, int64_t step0, float* x,
                     float* y, float* th, int32_t* ix, int32_t* iy) {
  int n = p->n;
  double rcut = mirror_rcut(p);
  float* c = (float*)malloc(sizeof(float) * n);
  float* s = (float*)malloc(sizeof(float) * n);
  float *hx = (float*)malloc(sizeof(float) * n), *hy = (float*)malloc(sizeof(float) * n);
  float *hc = (float*)malloc(sizeof(float) * n), *hs = (float*)malloc(sizeof(float) * n);
  float *kx = (float*)malloc(sizeof(float) * n), *ky = (float*)malloc(sizeof(float) * n);
  float* kt = (float*)malloc(sizeof(float) * n);
  SppAccF* acc = (SppAccF*)malloc(sizeof(SppAccF) * (n > 0 ? n : 1));
  /* run and tumble: the swimmers' states (all running at the start of the
   * call) and the step's dtheta, drawn once per step as the kernels do */
  int32_t* tstate = k->tumble ? (int32_t*)calloc((size_t)(n > 0 ? n : 1), sizeof(int32_t)) : NULL;
  float* tdth = k->tumble ? (float*)malloc(sizeof(float) * (n > 0 ? n : 1)) : NULL;
  int rc = SPP_OK;
  for (int i = 0; i < n; ++i) spp_sincosf(th[i], &s[i], &c[i]);
  for (int st = 0; st < nsteps && rc == SPP_OK; ++st) {
    uint32_t step = (uint32_t)(step0 + st);
    if (k->tumble)
      for (int i = 0; i < n; ++i)
        tdth[i] = i < k->n_beads ? 0.0f : spp_tumble_noise(k, (uint32_t)i, step, &tstate[i]);
    if (p->integrator == SPP_INT_EULER) {
      /* every body's rates from the state at the start of the step (ring
       * forces read the neighbours' old positions), then all moves */
      if (abp_accumulate(k, n, x, y, c, s, rcut, acc)) rc = SPP_ERR_OVERFLOW;
      for (int i = 0; i < n; ++i) {
        float fx, fy, tau, dth;
        body_rates(k, i, &acc[i], x, y, c[i], s[i], step, tdth, th[i], 1, &fx, &fy, &tau, &dth);
        int gx = ix[i], gy = iy[i];
        float nt, ncs, nsn;
        spp_euler_update(x[i], y[i], th[i], fx, fy, tau, dth, k, &hx[i], &hy[i], &nt, &ncs, &nsn,
                         &gx, &gy, k->closed);
        kx[i] = nt; hc[i] = ncs; hs[i] = nsn;
        ix[i] = gx; iy[i] = gy;
      }
      memcpy(x, hx, sizeof(float) * n); memcpy(y, hy, sizeof(float) * n);
      memcpy(th, kx, sizeof(float) * n); memcpy(c, hc, sizeof(float) * n); memcpy(s, hs, sizeof(float) * n);
      continue;
    }
    int nst = p->integrator == SPP_INT_RK4 ? 4 : 2;
    for (int stage = 0; stage < nst; ++stage) {
      const float *cx = stage == 0 ? x : hx, *cy = stage == 0 ? y : hy;
      const float *cc = stage == 0 ? c : hc, *cs = stage == 0 ? s : hs;
      if (abp_accumulate(k, n, cx, cy, cc, cs, rcut, acc)) rc = SPP_ERR_OVERFLOW;
      int last = stage == nst - 1;
      float* nx = (float*)malloc(sizeof(float) * n);
      float* ny = (float*)malloc(sizeof(float) * n);
      float* nc = (float*)malloc(sizeof(float) * n);
      float* ns = (float*)malloc(sizeof(float) * n);
      for (int i = 0; i < n; ++i) {
        float fx, fy, tau, dth;
        body_rates(k, i, &acc[i], cx, cy, cc[i], cs[i], step, tdth, th[i], 0, &fx, &fy, &tau, &dth);
        float h, frac;
        if (nst == 2) {
          h = stage == 0 ? k->half_dt : k->dt;
          frac = stage == 0 ? 0.5f : 1.0f;
        } else {
          if (stage == 0) { kx[i] = fx; ky[i] = fy; kt[i] = tau; }
          else if (stage < 3) { kx[i] = kx[i] + 2.0f * fx; ky[i] = ky[i] + 2.0f * fy; kt[i] = kt[i] + 2.0f * tau; }
          else { fx = kx[i] + fx; fy = ky[i] + fy; tau = kt[i] + tau; }
          h = stage < 2 ? k->half_dt : (stage == 2 ? k->dt : k->dt6);
          frac = stage < 2 ? 0.5f : 1.0f;
        }
        float tnew;
        int gx = ix[i], gy = iy[i];
        spp_stage_update(h, frac, x[i], y[i], th[i], fx, fy, tau, dth, k, &nx[i], &ny[i], &tnew,
                         &nc[i], &ns[i], &gx, &gy, k->closed);
        if (last) { th[i] = tnew; ix[i] = gx; iy[i] = gy; }
      }
      if (last) {
        memcpy(x, nx, sizeof(float) * n); memcpy(y, ny, sizeof(float) * n);
        memcpy(c, nc, sizeof(float) * n); memcpy(s, ns, sizeof(float) * n);
      } else {
        memcpy(hx, nx, sizeof(float) * n); memcpy(hy, ny, sizeof(float) * n);
        memcpy(hc, nc, sizeof(float) * n); memcpy(hs, ns, sizeof(float) * n);
      }
      free(nx); free(ny); free(nc); free(ns);
    }
  }
  free(c); free(s); free(hx); free(hy); free(hc); free(hs); free(kx); free(ky); free(kt); free(acc);
  free(tstate); free(tdth);
  return rc;
}

static int vicsek_run32(const SppParams* p, const SppConsts* k, int nsteps, int64_t step0, float* x,
                        float* y, float* th, int32_t* ix, int32_t* iy) {
  int n = p->n;
  double rcut = mirror_rcut(p);
  float* c = (float*)malloc(sizeof(float) * n);
  float* s = (float*)malloc(sizeof(float) * n);
  float *nx = (float*)malloc(sizeof(float) * n), *ny = (float*)malloc(sizeof(float) * n);
  float *nt = (float*)malloc(sizeof(float) * n), *nc = (float*)malloc(sizeof(float) * n);
  float* ns = (float*)malloc(sizeof(float) * n);
  int rc = SPP_OK;
  for (int i = 0; i < n; ++i) spp_sincosf(th[i], &s[i], &c[i]);
  for (int st = 0; st < nsteps; ++st) {
    uint32_t step = (uint32_t)(step0 + st);
    mcells cl;
    mcells_build(&cl, n, x, y, k, rcut);
    for (int i = 0; i < n; ++i) {
      SppAcc a;
      spp_acc_zero(&a);
      FOR_CANDIDATES(&cl, k, x[i], y[i], n, j, {
        spp_pair_vicsek(k, &a, x[i], y[i], x[j], y[j], c[j], s[j], th[j], j == i);
      });
      if (k->closed && k->model == SPP_MODEL_VICSEK_REF_ANGLE) spp_vicsek_walls(k, &a, x[i], y[i], th[i]);
      if (a.ovf) rc = SPP_ERR_OVERFLOW;
      spp_u32x4 d = spp_draw(k->seed, k->system, (uint32_t)i, step, SPP_RNG_VICSEK);
      int gx = ix[i], gy = iy[i];
      spp_vicsek_update(k, &a, x[i], y[i], th[i], c[i], s[i], d.v[0], &nx[i], &ny[i], &nt[i], &nc[i],
                        &ns[i], &gx, &gy);
      ix[i] = gx; iy[i] = gy;
    }
    mcells_free(&cl);
    memcpy(x, nx, sizeof(float) * n); memcpy(y, ny, sizeof(float) * n);
    memcpy(th, nt, sizeof(float) * n); memcpy(c, nc, sizeof(float) * n);
    memcpy(s, ns, sizeof(float) * n);
  }
  free(c); free(s); free(nx); free(ny); free(nt); free(nc); free(ns);
  return rc;
}

/* Runs nsteps from absolute step step0.  x, y wrapped in [-L, L); ix, iy
 * box-crossing counts (unwrapped = x + 2L ix). */
int orc32_run(const SppParams* p, int nsteps, int64_t step0, float* x, float* y, float* th,
              int32_t* ix, int32_t* iy) {
  SppConsts k;
  spp_consts_from_params(&k, p);
  switch (p->model) {
    case SPP_MODEL_VICSEK:
    case SPP_MODEL_VICSEK_REF_ANGLE:
    case SPP_MODEL_VICSEK_REF_VECTOR:
      return vicsek_run32(p, &k, nsteps, step0, x, y, th, ix, iy);
    case SPP_MODEL_ABP:
    case SPP_MODEL_CONTINUOUS:
    case SPP_MODEL_BEADS:
      return abp_run32(p, &k, nsteps, step0, x, y, th, ix, iy);
    default:
      return SPP_ERR_UNSUPPORTED;
  }
}

/* Unique pairs (i<j) under the kernels' FP32 predicate d2 < (float)(r*r). */
int64_t orc32_pairs(const SppParams* p, const float* x, const float* y, double r, int32_t* pi,
                    int32_t* pj, int64_t cap) {
  SppConsts k;
  spp_consts_from_params(&k, p);
  int n = p->n;
  float r2 = (float)(r * r);
  mcells cl;
  mcells_build(&cl, n, x, y, &k, r);
  int64_t cnt = 0;
  for (int i = 0; i < n; ++i) {
    FOR_CANDIDATES(&cl, &k, x[i], y[i], n, j, {
      if (j > i) {
        float dx, dy;
        float d2 = spp_sep(&k, x[i], y[i], x[j], y[j], &dx, &dy);
        if (d2 < r2) {
          if (cnt < cap) { pi[cnt] = i; pj[cnt] = j; }
          cnt++;
        }
      }
    });
  }
  mcells_free(&cl);
  return cnt;
}

/* Cell coordinates with the kernels' FP32 formula (spp_cell_coord). */
void orc32_cells(const SppParams* p, const float* x, const float* y, int D, int rule, int32_t* cx,
                 int32_t* cy) {
  SppConsts k;
  spp_consts_from_params(&k, p);
  for (int i = 0; i < p->n; ++i) {
    cx[i] = spp_cell_coord(x[i], k.L, k.L2, D, rule);
    cy[i] = spp_cell_coord(y[i], k.L, k.L2, D, rule);
  }
}

/* Exposed primitives of spp_fp32.h, for the CPU tests of the arithmetic. */
void orc32_fx_sum(int n, const float* x, int32_t* hi, int32_t* lo, float* value) {
  spp_fx a = {0, 0};
  for (int i = 0; i < n; ++i) spp_fx_add(&a, x[i]);
  *hi = a.hi;
  *lo = a.lo;
  *value = spp_fx_value(a);
}
float orc32_rsqrt(float x) { return spp_rsqrtf(x); }
void orc32_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  spp_u32x4 o = spp_philox4x32_10(ctr[0], ctr[1], ctr[2], ctr[3], key[0], key[1]);
  memcpy(out, o.v, sizeof(o.v));
}
/* The kernels' draw from precomputed round keys (key = the 64-bit seed). */
void orc32_philox_ks(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t ks[20];
  spp_philox_round_keys((uint64_t)key[0] | ((uint64_t)key[1] << 32), ks);
  spp_u32x4 o = spp_philox4x32_10_ks(ctr[0], ctr[1], ctr[2], ctr[3], ks);
  memcpy(out, o.v, sizeof(o.v));
}
void orc32_math(int fn, int n, const float* a, const float* b, float* out) {
  for (int i = 0; i < n; ++i) {
    switch (fn) {
      case 0: out[i] = spp_sinf(a[i]); break;
      case 1: out[i] = spp_cosf(a[i]); break;
      case 2: out[i] = spp_atan2f(a[i], b[i]); break;
      case 3: out[i] = spp_logf(a[i]); break;
      case 4: out[i] = spp_expf(a[i]); break;
      case 5: out[i] = spp_wrap_angle_f(a[i]); break;
      default: out[i] = 0; break;
    }
  }
}

/* ------------------------------------------------------------------ */
/* tangent dynamics + FP64 renormalisation, as the kernels compute them  */
/* ------------------------------------------------------------------ */
/* Cholesky-QR pass with the reduction order of k_gram / k_chol / k_apply:
 * SPP_GRAM_BLOCKS x SPP_GRAM_THREADS threads stride over the elements, a
 * shuffle-down tree per warp, warps summed in order, blocks summed in order. */
static int mirror_cholqr_pass(int K, int len, float* V, double* log_stretch, int accumulate) {
  const int NE = K * (K + 1) / 2;
  const int stride = SPP_GRAM_BLOCKS * SPP_GRAM_THREADS;
  static double part[SPP_GRAM_BLOCKS][SPP_GRAM_ENTRIES];
  double thr[SPP_GRAM_THREADS][SPP_GRAM_ENTRIES];
  for (int b = 0; b < SPP_GRAM_BLOCKS; ++b) {
    for (int t = 0; t < SPP_GRAM_THREADS; ++t) {
      for (int q = 0; q < NE; ++q) thr[t][q] = 0.0;
      for (int e = b * SPP_GRAM_THREADS + t; e < len; e += stride) {
        double v[SPP_LYAP_MAX];
        for (int a = 0; a < K; ++a) v[a] = (double)V[(size_t)a * len + e];
        for (int a = 0; a < K; ++a)
          for (int c = 0; c <= a; ++c) thr[t][a * (a + 1) / 2 + c] = thr[t][a * (a + 1) / 2 + c] + v[a] * v[c];
      }
    }
    double warp_part[SPP_GRAM_THREADS / 32][SPP_GRAM_ENTRIES];
    for (int w = 0; w < SPP_GRAM_THREADS / 32; ++w) {
      for (int q = 0; q < NE; ++q) {
        double x[32];
        for (int l = 0; l < 32; ++l) x[l] = thr[w * 32 + l][q];
        for (int o = 16; o > 0; o >>= 1) {
          double y[32];
          for (int l = 0; l < 32; ++l) y[l] = x[l] + (l + o < 32 ? x[l + o] : x[l]);
          memcpy(x, y, sizeof(x));
        }
        warp_part[w][q] = x[0];
      }
    }
    for (int q = 0; q < NE; ++q) {
      double x = 0.0;
      for (int w = 0; w < SPP_GRAM_THREADS / 32; ++w) x = x + warp_part[w][q];
      part[b][q] = x;
    }
  }
  double G[SPP_GRAM_ENTRIES];
  for (int q = 0; q < NE; ++q) {
    double x = 0.0;
    for (int b = 0; b < SPP_GRAM_BLOCKS; ++b) x = x + part[b][q];
    G[q] = x;
  }
  double rinv[SPP_LYAP_MAX * SPP_LYAP_MAX], lr[SPP_LYAP_MAX];
  if (spp_cholesky_inverse(K, G, rinv, lr)) return 1;
  if (accumulate)
    for (int a = 0; a < K; ++a) log_stretch[a] = log_stretch[a] + lr[a];
  for (int e = 0; e < len; ++e) {
    double v[SPP_LYAP_MAX];
    for (int a = 0; a < K; ++a) v[a] = (double)V[(size_t)a * len + e];
    for (int a = 0; a < K; ++a) {
      double x = 0.0;
      for (int c = 0; c <= a; ++c) x = x + v[c] * rinv[c * SPP_LYAP_MAX + a];
      V[(size_t)a * len + e] = (float)x;
    }
  }
  return 0;
}

int orc32_renormalize(int K, int n, float* V, double* log_stretch, int accumulate) {
  for (int pass = 0; pass < 2; ++pass)
    if (mirror_cholqr_pass(K, 3 * n, V, log_stretch, accumulate)) return SPP_ERR_NUMERIC;
  return SPP_OK;
}

/* The kernels' initial tangent vectors: N(0,1) from the tangent stream,
 * then orthonormalised. */
int orc32_lyap_init(const SppParams* p, int K, uint64_t seed, float* V) {
  int n = p->n;
  for (int e = 0; e < K * 3 * n; ++e) {
    int id = e % n, vc = e / n;
    spp_u32x4 r = spp_draw(seed, p->system_id, (uint32_t)id, (uint32_t)vc, SPP_RNG_TANGENT);
    V[e] = spp_normal_f(r.v[0], r.v[1]);
  }
  double dummy[SPP_LYAP_MAX] = {0};
  return orc32_renormalize(K, n, V, dummy, 0);
}

/* Base (continuous model, RK2/RK4) and tangent steps; renormalisation after
 * every renorm_every steps and at the end (renorm_every <= 0: never). */
int orc32_lyap_run(const SppParams* p, int nsteps, int64_t step0, int renorm_every, int K, float* x,
                   float* y, float* th, int32_t* ix, int32_t* iy, float* V, double* log_stretch) {
  SppConsts k;
  spp_consts_from_params(&k, p);
  const int n = p->n;
  const int nst = p->integrator == SPP_INT_RK4 ? 4 : 2;
  const double rcut = mirror_rcut(p);
  float *c = malloc(sizeof(float) * n), *s = malloc(sizeof(float) * n);
  float *hx = malloc(sizeof(float) * n), *hy = malloc(sizeof(float) * n);
  float *hc = malloc(sizeof(float) * n), *hs = malloc(sizeof(float) * n);
  float *kx = malloc(sizeof(float) * n), *ky = malloc(sizeof(float) * n), *kt = malloc(sizeof(float) * n);
  float *nx = malloc(sizeof(float) * n), *ny = malloc(sizeof(float) * n);
  float *nc = malloc(sizeof(float) * n), *ns = malloc(sizeof(float) * n);
  size_t len = (size_t)K * 3 * n;
  float *ua = malloc(sizeof(float) * len), *ub = malloc(sizeof(float) * len);
  float *acc = malloc(sizeof(float) * len);
  SppAccF* A = malloc(sizeof(SppAccF) * n);
  int* cand = malloc(sizeof(int) * 64);
  int cap = 64;
  int rc = SPP_OK;
  for (int i = 0; i < n; ++i) spp_sincosf(th[i], &s[i], &c[i]);
  for (int st = 0; st < nsteps && rc == SPP_OK; ++st) {
    uint32_t step = (uint32_t)(step0 + st);
    for (int stage = 0; stage < nst; ++stage) {
      const float *cx = stage == 0 ? x : hx, *cy = stage == 0 ? y : hy;
      const float *cc = stage == 0 ? c : hc, *cs = stage == 0 ? s : hs;
      const float* uin = stage == 0 ? V : ((stage & 1) ? ua : ub);
      float* uout = (stage & 1) ? ub : ua;
      int last = stage == nst - 1;
      mcells cl;
      mcells_build(&cl, n, cx, cy, &k, rcut);
      /* tangent slopes need the neighbour list at this stage state, in id order */
      float* slopes = malloc(sizeof(float) * len);
      for (int i = 0; i < n; ++i) {
        int m = 0;
        FOR_CANDIDATES(&cl, &k, cx[i], cy[i], n, j, {
          if (j != i) {
            if (m == cap) { cap *= 2; cand = realloc(cand, sizeof(int) * cap); }
            cand[m++] = j;
          }
        });
        qsort(cand, (size_t)m, sizeof(int), cmp_int);
        /* one lane (k.lanes == 1) or the kernels' four: neighbours with
         * id % 4 == r in lane r, lane sums combined as (p0 + p1) + (p2 + p3) */
        const int L = k.lanes;
        SppAccF part[SPP_GATHER_LANES];
        float tpart[SPP_GATHER_LANES][SPP_LYAP_MAX];
        for (int r = 0; r < L; ++r) {
          spp_accf_zero(&part[r]);
          for (int v = 0; v < K; ++v) tpart[r][v] = 0.0f;
        }
        for (int q = 0; q < m; ++q) {
          int j = cand[q];
          const int r = L > 1 ? (j & 3) : 0;
          spp_pair_abp(&k, &part[r], cx[i], cy[i], cc[i], cs[i], cx[j], cy[j], cc[j], cs[j]);
          float dx, dy;
          float d2 = spp_sep(&k, cx[i], cy[i], cx[j], cy[j], &dx, &dy);
          if (d2 < k.ral2) {
            float cij = spp_tangent_coupling(cc[i], cs[i], cc[j], cs[j]);
            for (int v = 0; v < K; ++v)
              tpart[r][v] = tpart[r][v] + cij * (uin[(size_t)(v * 3 + 2) * n + j] - uin[(size_t)(v * 3 + 2) * n + i]);
          }
        }
        SppAccF a = part[0];
        float tacc[SPP_LYAP_MAX];
        for (int v = 0; v < K; ++v) tacc[v] = tpart[0][v];
        if (L > 1) {
          a.fx = spp_lane_sum4(part[0].fx, part[1].fx, part[2].fx, part[3].fx);
          a.fy = spp_lane_sum4(part[0].fy, part[1].fy, part[2].fy, part[3].fy);
          a.tq = spp_lane_sum4(part[0].tq, part[1].tq, part[2].tq, part[3].tq);
          a.ss = spp_lane_sum4(part[0].ss, part[1].ss, part[2].ss, part[3].ss);
          a.sc = spp_lane_sum4(part[0].sc, part[1].sc, part[2].sc, part[3].sc);
          a.cnt = part[0].cnt + part[1].cnt + part[2].cnt + part[3].cnt;
          a.ovf = part[0].ovf | part[1].ovf | part[2].ovf | part[3].ovf;
          for (int v = 0; v < K; ++v) tacc[v] = spp_lane_sum4(tpart[0][v], tpart[1][v], tpart[2][v], tpart[3][v]);
        }
        A[i] = a;
        const float gp = k.g * k.one_minus_alpha_over_pi;
        for (int v = 0; v < K; ++v) {
          float ui = uin[(size_t)(v * 3 + 2) * n + i];
          slopes[(size_t)(v * 3 + 0) * n + i] = -k.v0 * cs[i] * ui;
          slopes[(size_t)(v * 3 + 1) * n + i] = k.v0 * cc[i] * ui;
          slopes[(size_t)(v * 3 + 2) * n + i] = gp * tacc[v];
        }
      }
      mcells_free(&cl);
      /* base stage update */
      for (int i = 0; i < n; ++i) {
        float fx, fy, tau;
        spp_abp_forces(&k, k.closed, &A[i], cx[i], cy[i], cc[i], cs[i], &fx, &fy, &tau);
        float dth = spp_rot_noise(&k, (uint32_t)i, step);
        float h, frac;
        if (nst == 2) {
          h = stage == 0 ? k.half_dt : k.dt;
          frac = stage == 0 ? 0.5f : 1.0f;
        } else {
          if (stage == 0) { kx[i] = fx; ky[i] = fy; kt[i] = tau; }
          else if (stage < 3) { kx[i] = kx[i] + 2.0f * fx; ky[i] = ky[i] + 2.0f * fy; kt[i] = kt[i] + 2.0f * tau; }
          else { fx = kx[i] + fx; fy = ky[i] + fy; tau = kt[i] + tau; }
          h = stage < 2 ? k.half_dt : (stage == 2 ? k.dt : k.dt6);
          frac = stage < 2 ? 0.5f : 1.0f;
        }
        float tnew;
        int gx = ix[i], gy = iy[i];
        spp_stage_update(h, frac, x[i], y[i], th[i], fx, fy, tau, dth, &k, &nx[i], &ny[i], &tnew,
                         &nc[i], &ns[i], &gx, &gy, k.closed);
        if (last) { th[i] = tnew; ix[i] = gx; iy[i] = gy; }
      }
      /* tangent stage update */
      for (size_t e = 0; e < len; ++e) {
        float t0 = V[e];
        float a = stage == 0 ? 0.0f : acc[e];
        float uo = 0.0f;
        spp_tangent_stage_update(&k, stage, nst, slopes[e], &t0, &a, &uo);
        if (last) V[e] = t0;
        else uout[e] = uo;
        if (nst == 4 && stage < 3) acc[e] = a;
      }
      free(slopes);
      if (last) {
        memcpy(x, nx, sizeof(float) * n); memcpy(y, ny, sizeof(float) * n);
        memcpy(c, nc, sizeof(float) * n); memcpy(s, ns, sizeof(float) * n);
      } else {
        memcpy(hx, nx, sizeof(float) * n); memcpy(hy, ny, sizeof(float) * n);
        memcpy(hc, nc, sizeof(float) * n); memcpy(hs, ns, sizeof(float) * n);
      }
    }
    if (renorm_every > 0 && ((st + 1) % renorm_every == 0 || st + 1 == nsteps))
      if (orc32_renormalize(K, n, V, log_stretch, 1)) rc = SPP_ERR_NUMERIC;
  }
  free(c); free(s); free(hx); free(hy); free(hc); free(hs); free(kx); free(ky); free(kt);
  free(nx); free(ny); free(nc); free(ns); free(ua); free(ub); free(acc); free(A); free(cand);
  return rc;
}

/* ---------------------------------------------------------------- */
/* pair histograms of the observables (spp_radial_distribution,      */
/* spp_pair_distribution), all ordered pairs, same FP32 expressions  */
/* ---------------------------------------------------------------- */
void orc32_radial(const float* x, const float* y, int n, double L, double r_max, int nbins,
                  uint64_t* counts, int closed) {
  const float Lf = (float)L, L2 = (float)(2.0 * L);
  const float rm = (float)r_max, r2max = rm * rm, dr = rm / (float)nbins;
  for (int b = 0; b < nbins; ++b) counts[b] = 0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      if (j == i) continue;
      const float dx = closed ? x[i] - x[j] : spp_min_image_f(x[i] - x[j], Lf, L2);
      const float dy = closed ? y[i] - y[j] : spp_min_image_f(y[i] - y[j], Lf, L2);
      const float d2 = fmaf(dx, dx, dy * dy);
      if (d2 < r2max) {
        int b = (int)(sqrtf(d2) / dr);
        b = b < nbins ? b : nbins - 1;
        counts[b]++;
      }
    }
}

void orc32_pair_distribution(const float* x, const float* y, const float* c, const float* s, int n,
                             double lx, double ly, int gx, int gy, uint64_t* counts) {
  const float lxf = (float)lx, lyf = (float)ly;
  for (int b = 0; b < gx * gy; ++b) counts[b] = 0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      if (j == i) continue;
      const float dx = x[j] - x[i];
      const float dy = y[j] - y[i];
      const float ty = c[i] * dx + s[i] * dy;
      const float tx = s[i] * dx - c[i] * dy;
      if (fabsf(tx) < lxf && fabsf(ty) < lyf) {
        int bx = (int)((float)gx * ((tx / lxf) + 1.0f) / 2.0f);
        int by = (int)((float)gy * ((ty / lyf) + 1.0f) / 2.0f);
        bx = bx < gx ? bx : gx - 1;
        by = by < gy ? by : gy - 1;
        counts[(size_t)bx * gy + by]++;
      }
    }
}

/* The kernels' run-and-tumble constants for p (spp_consts_from_params). */
int32_t orc32_tumble_steps(const SppParams* p) {
  SppConsts k;
  spp_consts_from_params(&k, p);
  return k.tumble_steps;
}

/* The kernels' FP32 wall terms (spp_wall_terms) for one particle at (x, y)
 * with heading (cos th, sin th) from spp_sincosf, for the segments
 * p->walls[0 .. n_walls) alone: out3 = {fx, fy, torque}. */
void orc32_wall_terms(const SppParams* p, float x, float y, float th, float* out3) {
  SppConsts k;
  spp_consts_from_params(&k, p);
  for (int e = 0; e < p->n_walls; ++e) {   /* drop the 4 box walls */
    k.wall_x1[e] = k.wall_x1[e + 4]; k.wall_y1[e] = k.wall_y1[e + 4];
    k.wall_x2[e] = k.wall_x2[e + 4]; k.wall_y2[e] = k.wall_y2[e + 4];
    k.wall_ex[e] = k.wall_ex[e + 4]; k.wall_ey[e] = k.wall_ey[e + 4];
    k.wall_len[e] = k.wall_len[e + 4];
  }
  k.n_walls = p->n_walls;
  for (int e = 0; e < p->n_walls; ++e) k.wall_theta[e] = k.wall_theta[e + 4];
  if (p->model == SPP_MODEL_VICSEK_REF_ANGLE) {
    /* {count, angle sum, 0}: the neighbours and angle sum the walls add */
    SppAcc a;
    spp_acc_zero(&a);
    spp_vicsek_walls(&k, &a, x, y, th);
    out3[0] = (float)a.cnt;
    out3[1] = spp_fx_value(a.at);
    out3[2] = 0.0f;
    return;
  }
  float s, c;
  spp_sincosf(th, &s, &c);
  spp_wall_terms(&k, x, y, c, s, &out3[0], &out3[1], &out3[2]);
}

/* The circle torque of one particle (FP32, the kernels' spp_circle_torque). */
float orc32_circle_torque(const SppParams* p, float x, float y, float th) {
  SppConsts k;
  spp_consts_from_params(&k, p);
  float s, c;
  spp_sincosf(th, &s, &c);
  return spp_circle_torque(&k, x, y, c, s);
}
