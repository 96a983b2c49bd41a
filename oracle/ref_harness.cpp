/*
 * ORACLE -- test infrastructure only.  Built by oracle/build.py into
 * oracle/_ref/libspp_ref.so from the reference's own headers, which are
 * included from the reference checkout (never copied); that library exists
 * only where the reference is present.
 *
 * Drives the reference's particle classes (shared/particle.h) through the
 * reference's step sequence (serial/box.h:458-506: Interact over every pair
 * once, then Move*() on every particle, per Runge-Kutta stage), with the
 * GSL calls answered by the Philox shim in oracle/refshim/gsl.  It stands in
 * for Box because box.h/node.h need MPI and Boost and do not compile as
 * shipped (set-up.h assigns the const globals of parameters.h:81,83;
 * parameters.h:50 fixes Particle to ActiveBrownianChain).  Neither header is
 * included here, so no reference file needs patching: particle.h,
 * c2dvector.h, parameters.h, force-fields.h, wall.h, vector-set.h and
 * state-hyper-vector.h compile unmodified.
 *
 * Pair enumeration uses a cell list of width >= the largest cutoff; pairs
 * are visited in a different order than the reference's cell traversal,
 * which changes FP64 sums only in the last bits.
 */
#include "particle.h"   /* shared/particle.h of the reference */
#include "wall.h"       /* shared/wall.h of the reference */
#include "vector-set.h" /* shared/vector-set.h and state-hyper-vector.h of the reference */
#include <fstream>
#include <sstream>
#include "statistics.h" /* analyze/statistics.h of the reference (Boost: oracle/refshim) */
#include "../include/spp.h"
#include <vector>
#include <cmath>

namespace {

void set_box(double L) {
  Lx = L; Ly = L; Lx2 = 2 * L; Ly2 = 2 * L;
}
void set_dt(double d) {
  dt = d; half_dt = d / 2; dt_over_6 = d / 6;
}

template <class P>
void interact_all(std::vector<P>& ps, double L, double rcut) {
  int n = (int)ps.size();
  int D = (int)std::floor(2 * L / rcut);
  if (D < 3) {
    for (int i = 0; i < n; ++i)
      for (int j = i + 1; j < n; ++j) ps[i].Interact(ps[j]);
    return;
  }
  std::vector<int> head((size_t)D * D, -1), next(n, -1);
  for (int i = n - 1; i >= 0; --i) {
    int cx = (int)std::floor((ps[i].r.x + L) * D / (2 * L));
    int cy = (int)std::floor((ps[i].r.y + L) * D / (2 * L));
    cx = cx < 0 ? 0 : (cx >= D ? D - 1 : cx);
    cy = cy < 0 ? 0 : (cy >= D ? D - 1 : cy);
    next[i] = head[cx * D + cy];
    head[cx * D + cy] = i;
  }
  static const int off[4][2] = {{1, 0}, {0, 1}, {1, 1}, {1, -1}};
  for (int cx = 0; cx < D; ++cx)
    for (int cy = 0; cy < D; ++cy) {
      int k = cx * D + cy;
      for (int i = head[k]; i >= 0; i = next[i])
        for (int j = next[i]; j >= 0; j = next[j]) ps[i].Interact(ps[j]);
      for (int o = 0; o < 4; ++o) {
        int kk = ((cx + off[o][0] + D) % D) * D + (cy + off[o][1] + D) % D;
        for (int i = head[k]; i >= 0; i = next[i])
          for (int j = head[kk]; j >= 0; j = next[j]) ps[i].Interact(ps[j]);
      }
    }
}

template <class P>
void load(std::vector<P>& ps, const double* x, const double* y, const double* th, const double* xu,
          const double* yu) {
  for (size_t i = 0; i < ps.size(); ++i) {
    ps[i].r.x = x[i]; ps[i].r.y = y[i];
    ps[i].r_original.x = xu[i]; ps[i].r_original.y = yu[i];
    ps[i].theta = th[i];
    ps[i].v.x = std::cos(th[i]); ps[i].v.y = std::sin(th[i]);
    ps[i].Reset();
  }
}
template <class P>
void store(const std::vector<P>& ps, double* x, double* y, double* th, double* xu, double* yu) {
  for (size_t i = 0; i < ps.size(); ++i) {
    x[i] = ps[i].r.x; y[i] = ps[i].r.y; th[i] = ps[i].theta;
    xu[i] = ps[i].r_original.x; yu[i] = ps[i].r_original.y;
  }
}

/* Move functions that draw noise are called with the draw context set to
 * (particle id, step), so the shim hands each particle the Philox draw the
 * kernels use for it. */
template <class P, class F>
void move_all(std::vector<P>& ps, const SppParams* p, int64_t step, F move) {
  for (size_t i = 0; i < ps.size(); ++i) {
    shim_set_context(p->seed, p->system_id, (uint32_t)i, (uint32_t)step);
    move(ps[i]);
  }
}

/* Vicsek-family Move() advances r but not r_original; track it for output. */
template <class P>
void vicsek_steps(const SppParams* p, int nsteps, int64_t step0, double* x, double* y, double* th,
                  double* xu, double* yu) {
  std::vector<P> ps(p->n);
  load(ps, x, y, th, xu, yu);
  BasicDynamicParticle::noise_amplitude = p->eta;
  BasicDynamicParticle::speed = p->v0;
  for (int k = 0; k < nsteps; ++k) {
    for (auto& q : ps) q.Reset();
    interact_all(ps, p->L, 1.0);
    move_all(ps, p, step0 + k, [&](P& q) {
      q.Move();
      q.r_original.x += q.v.x * (p->dt * p->v0);
      q.r_original.y += q.v.y * (p->dt * p->v0);
    });
  }
  store(ps, x, y, th, xu, yu);
}

/* Interact_Membrane_Beads (parallel/beadbox.h:185-196), restated per ring
 * with the reference's Spring(). */
template <class P>
void ring_springs(std::vector<P>& ps, const SppParams* p) {
  const int M = p->ring_size;
  for (int r = 0; r < p->n_rings; ++r)
    for (int m = 0; m < M; ++m) {
      const int a = r * M + m, b = r * M + (m + 1) % M;
      C2DVector dr = ps[a].r - ps[b].r;
      dr.Periodic_Transform();
      Real d = std::sqrt(dr.Square());
      C2DVector f = Spring(dr, d, p->bond_rest, p->k_bond);
      ps[a].f += f;
      ps[b].f -= f;
    }
}

template <class P>
int chain_steps(const SppParams* p, int nsteps, int64_t step0, double* x, double* y, double* th,
                double* xu, double* yu) {
  const int nm = p->n_rings * p->ring_size;
  std::vector<P> ps(p->n);
  ActiveBrownianChain::sigma_m = p->sigma_rep;
  ActiveBrownianChain::repulsion_radius_m = p->r_rep;
  ActiveBrownianChain::A_p = p->k_rep;
  ActiveBrownianChain::torque0 = p->torque0;
  /* chain statics (particle.h:1050-1054), read by Set_nb and Interact */
  ActiveBrownianChain::sigma_p = p->sigma_chain;
  ActiveBrownianChain::repulsion_radius = p->r_chain;
  ActiveBrownianChain::separation = p->bead_separation;
  BasicDynamicParticle::Set_Dr(p->Dr);
  const int nb = p->chain_beads > 1 ? p->chain_beads : 1;
  double rcut = p->r_rep;
  if (nb > 1 && (nb - 1) * p->bead_separation + p->r_chain > rcut)
    rcut = (nb - 1) * p->bead_separation + p->r_chain;
  for (int i = 0; i < p->n; ++i) {
    ps[i].Set_nb(i < nm ? 1 : nb);
    /* speed v0 = m_parallel F0 */
    ps[i].Set_F0(i < nm ? 0.0 : (nb > 1 ? p->v0 / ps[i].m_parallel : p->v0 / p->mu));
  }
  load(ps, x, y, th, xu, yu);
  for (int k = 0; k < nsteps; ++k) {
    int64_t step = step0 + k;
    if (p->integrator == SPP_INT_EULER) {
      ring_springs(ps, p);
      interact_all(ps, p->L, rcut);
      move_all(ps, p, step, [](P& q) { q.Move(); });
    } else {
      ring_springs(ps, p);
      interact_all(ps, p->L, rcut);
      move_all(ps, p, step, [](P& q) { q.Move_Runge_Kutta2_1(); });
      ring_springs(ps, p);
      interact_all(ps, p->L, rcut);
      move_all(ps, p, step, [](P& q) { q.Move_Runge_Kutta2_2(); });
    }
  }
  store(ps, x, y, th, xu, yu);
  return SPP_OK;
}

}  // namespace

extern "C" int ref_run(const SppParams* p, int nsteps, int64_t step0, double* x, double* y,
                       double* th, double* xu, double* yu) {
  set_box(p->L);
  set_dt(p->dt);
  switch (p->model) {
    case SPP_MODEL_VICSEK_REF_ANGLE:
      if (p->r_align != 1.0) return SPP_ERR_UNSUPPORTED;  /* particle.h:179 tests d2 < 1 */
      vicsek_steps<VicsekParticle>(p, nsteps, step0, x, y, th, xu, yu);
      return SPP_OK;
    case SPP_MODEL_VICSEK_REF_VECTOR:
      if (p->r_align != 1.0) return SPP_ERR_UNSUPPORTED;  /* particle.h:231 */
      VicsekParticle2::beta = p->beta_push;
      VicsekParticle2::rc = p->r_push;
      vicsek_steps<VicsekParticle2>(p, nsteps, step0, x, y, th, xu, yu);
      return SPP_OK;
    case SPP_MODEL_CONTINUOUS: {
      if (p->r_align != 1.0 || p->integrator != SPP_INT_EULER) return SPP_ERR_UNSUPPORTED;
      std::vector<ContinuousParticle> ps(p->n);
      ContinuousParticle::Set_g(p->g);
      ContinuousParticle::Set_alpha(p->alpha);
      ContinuousParticle::Kamp = 0;
      BasicDynamicParticle::Set_Dr(p->Dr);
      BasicDynamicParticle::speed = p->v0;
      load(ps, x, y, th, xu, yu);
      for (int k = 0; k < nsteps; ++k) {
        interact_all(ps, p->L, 1.0);
        move_all(ps, p, step0 + k, [&](ContinuousParticle& q) {
          C2DVector before = q.r;
          q.Move();
          C2DVector dr = q.r - before;
          dr.Periodic_Transform();
          q.r_original += dr;
        });
      }
      store(ps, x, y, th, xu, yu);
      return SPP_OK;
    }
    case SPP_MODEL_ABP: {
      /* RepulsiveParticle: R12 force, reference alignment normalisation, f = v (unit speed). */
      if (p->force_law != SPP_FORCE_R12_TRUNC || p->align_mode != SPP_ALIGN_REFERENCE ||
          p->v0 != 1.0)
        return SPP_ERR_UNSUPPORTED;
      std::vector<RepulsiveParticle> ps(p->n);
      RepulsiveParticle::Set_repulsion_radius(p->r_rep);
      RepulsiveParticle::Set_alignment_radius(p->r_align);
      RepulsiveParticle::Set_sigma_p(p->sigma_rep);
      RepulsiveParticle::Set_A_p(p->k_rep);
      RepulsiveParticle::Set_g(p->g);
      BasicDynamicParticle::Set_Dr(p->Dr);
      load(ps, x, y, th, xu, yu);
      double rcut = std::max(p->r_rep, p->r_align);
      for (int k = 0; k < nsteps; ++k) {
        int64_t step = step0 + k;
        if (p->integrator == SPP_INT_EULER) {
          interact_all(ps, p->L, rcut);
          move_all(ps, p, step, [](RepulsiveParticle& q) { q.Move(); });
        } else if (p->integrator == SPP_INT_RK2) {
          interact_all(ps, p->L, rcut);
          move_all(ps, p, step, [](RepulsiveParticle& q) { q.Move_Runge_Kutta2_1(); });
          interact_all(ps, p->L, rcut);
          move_all(ps, p, step, [](RepulsiveParticle& q) { q.Move_Runge_Kutta2_2(); });
        } else {
          interact_all(ps, p->L, rcut);
          move_all(ps, p, step, [](RepulsiveParticle& q) { q.Move_Runge_Kutta4_1(); });
          interact_all(ps, p->L, rcut);
          move_all(ps, p, step, [](RepulsiveParticle& q) { q.Move_Runge_Kutta4_2(); });
          interact_all(ps, p->L, rcut);
          move_all(ps, p, step, [](RepulsiveParticle& q) { q.Move_Runge_Kutta4_3(); });
          interact_all(ps, p->L, rcut);
          move_all(ps, p, step, [](RepulsiveParticle& q) { q.Move_Runge_Kutta4_4(); });
        }
      }
      store(ps, x, y, th, xu, yu);
      return SPP_OK;
    }
    case SPP_MODEL_BEADS: {
      /* ActiveBrownianChain with nb = 1 (mobilities 0.5, 0.5, 1 from Set_nb,
       * particle.h:856-864), or its run-and-tumble subclass RTPChain
       * (:1061-1108); no bending, no RK4 in the reference. */
      if (p->force_law != SPP_FORCE_R12_TRUNC || p->kappa_bend != 0.0 || p->mu != 0.5 ||
          p->k_perp != 1.0 || p->integrator == SPP_INT_RK4)
        return SPP_ERR_UNSUPPORTED;
      if (p->rot_noise == SPP_NOISE_TUMBLE) {
        RTPChain::lambda = p->tumble_rate;
        RTPChain::t_tumble = p->tumble_time;
        RTPChain::torque_tumble = p->tumble_torque;
        return chain_steps<RTPChain>(p, nsteps, step0, x, y, th, xu, yu);
      }
      return chain_steps<ActiveBrownianChain>(p, nsteps, step0, x, y, th, xu, yu);
    }
    default:
      return SPP_ERR_UNSUPPORTED;
  }
}

/* The reference's force law, for a direct check of the restatement. */
extern "C" void ref_r12_truncated(double dx, double dy, double cutoff, double sigma, double A,
                                  double* fx, double* fy) {
  C2DVector dr;
  dr.x = dx; dr.y = dy;
  Real d = std::sqrt(dr.Square());
  C2DVector f = R12_Repulsive_Truncated(dr, d, cutoff, sigma, A);
  *fx = f.x; *fy = f.y;
}
extern "C" void ref_spring(double dx, double dy, double sigma, double A, double* fx, double* fy) {
  C2DVector dr;
  dr.x = dx; dr.y = dy;
  Real d = std::sqrt(dr.Square());
  C2DVector f = Spring(dr, d, sigma, A);
  *fx = f.x; *fy = f.y;
}

/* The reference's walls (Wall::Init, Wall::Interact, shared/wall.h) on one
 * particle, for the segments p->walls[0 .. p->n_walls) alone.  out4 =
 * {f.x, f.y, torque} of a RepulsiveParticle, {0, 0, 0, torque} of a
 * ContinuousParticle, or {neighbour count, angle sum} of a VicsekParticle.  The harness is built with the reference's
 * PERIODIC_BOUNDARY_CONDITION, so the box is set 1e9 wide here: then the
 * Periodic_Transform calls of Wall change nothing, as in the reference's
 * closed-box build. */
extern "C" void ref_wall_terms(const SppParams* p, double x, double y, double th, double* out4) {
  set_box(1e9);
  out4[0] = out4[1] = out4[2] = out4[3] = 0.0;
  if (p->model == SPP_MODEL_VICSEK_REF_ANGLE) {
    /* {neighbor_size, average_theta} the walls add to a reset VicsekParticle */
    VicsekParticle q;
    q.r.x = x; q.r.y = y; q.theta = th;
    q.v.x = std::cos(th); q.v.y = std::sin(th);
    q.Reset();
    for (int e = 0; e < p->n_walls; ++e) {
      Wall w;
      w.Init(p->walls[e][0], p->walls[e][1], p->walls[e][2], p->walls[e][3]);
      w.Interact(&q);
    }
    out4[0] = q.neighbor_size;
    out4[1] = q.average_theta;
    return;
  }
  if (p->model == SPP_MODEL_CONTINUOUS) {
    ContinuousParticle::gw = p->g_w_cont;
    ContinuousParticle q;
    q.r.x = x; q.r.y = y; q.theta = th;
    q.v.x = std::cos(th); q.v.y = std::sin(th);
    q.torque = 0;
    for (int e = 0; e < p->n_walls; ++e) {
      Wall w;
      w.Init(p->walls[e][0], p->walls[e][1], p->walls[e][2], p->walls[e][3]);
      w.Interact(&q);
    }
    out4[3] = q.torque;
  } else {
    RepulsiveParticle::r_c_w = p->r_c_w;
    RepulsiveParticle::r_f_w = p->r_f_w;
    RepulsiveParticle::sigma_w = p->sigma_w;
    RepulsiveParticle::A_w = p->A_w;
    RepulsiveParticle::g_w = p->g_w;
    RepulsiveParticle q;
    q.r.x = x; q.r.y = y; q.theta = th;
    q.v.x = std::cos(th); q.v.y = std::sin(th);
    q.f.x = 0; q.f.y = 0; q.torque = 0;
    for (int e = 0; e < p->n_walls; ++e) {
      Wall w;
      w.Init(p->walls[e][0], p->walls[e][1], p->walls[e][2], p->walls[e][3]);
      w.Interact(&q);
    }
    out4[0] = q.f.x; out4[1] = q.f.y; out4[2] = q.torque;
  }
}

/* The renormalisation of the reference's Benettin clone method on K
 * deviation vectors of n particles, stored [K][3][n] (x, y, theta blocks):
 * VectorSet::Renormalize(us) (shared/vector-set.h:118-127) writes the
 * orthonormal directions to U, and ratio[a] is the growth ratio that
 * LyapunovBox::Evolution_Reorthonormalize takes from them
 * (parallel/lyapunovbox.h:177-181: the deviation projected on its
 * orthonormalised direction, |.| / amplitude; restated here with the
 * reference's own State_Hyper_Vector operators, since lyapunovbox.h needs
 * Box and MPI).  The reference keeps its base trajectory in v[0], which
 * Renormalize skips, so the K deviations sit in v[1..K]. */
extern "C" int ref_vectorset_renormalize(int K, int n, double L, double amplitude, const double* V,
                                         double* U, double* ratio) {
  if (K < 1 || n < 1) return 1;
  set_box(L);
  C2DVector::Init_Rand(1);
  VectorSet::direction_num = K + 1;
  VectorSet::particle_num = n;
  VectorSet::amplitude = amplitude;
  VectorSet vs, us;
  for (int a = 0; a < K; ++a) {
    const double* v = V + (size_t)a * 3 * n;
    BasicParticle0* q = vs.v[a + 1].particle;
    for (int i = 0; i < n; ++i) {
      q[i].r.x = v[i];
      q[i].r.y = v[n + i];
      q[i].theta = v[2 * n + i];
    }
  }
  vs.Renormalize(us);
  for (int a = 0; a < K; ++a) {
    const BasicParticle0* q = us.v[a + 1].particle;
    double* u = U + (size_t)a * 3 * n;
    for (int i = 0; i < n; ++i) {
      u[i] = q[i].r.x;
      u[n + i] = q[i].r.y;
      u[2 * n + i] = q[i].theta;
    }
    State_Hyper_Vector proj = us.v[a + 1] * (vs.v[a + 1] * us.v[a + 1]);
    ratio[a] = proj.Magnitude() / VectorSet::amplitude;
  }
  return 0;
}

/* The order-parameter judges of the reference's analysis on a polarization
 * series p[0..T): Stat<double>::Compute with Find_Correlation_Length
 * (analyze/statistics.h:35-82) on P and on P^4, then the combination of
 * Compute_Order_Parameters (analyze/analyze.h:121-146): <P>, its error,
 * sigma2 = variance * area and G = 1 - <P^4> / (3 <P^2>), the reference's
 * form.  The reference forms P^4 as |v|^2 |v|^2 from the mean heading
 * vector v; from a series of P it is (P P)(P P).  out: mean, mean_square,
 * variance, std, min, max, corr_len, error, sigma2, p4_mean, G. */
extern "C" int ref_order_parameters(const double* series, int T, double area, double* out) {
  if (T < 2) return 1;
  Stat<double> p, p4;
  for (int i = 0; i < T; ++i) {
    const double s2 = series[i] * series[i];
    p.Add_Data(series[i]);
    p4.Add_Data(s2 * s2);
  }
  p.Compute();
  p4.Compute();
  const double v[11] = {p.mean, p.mean_square, p.variance, p.std, p.min, p.max, p.corr_len,
                        p.error, p.variance * area, p4.mean, 1 - (p4.mean / (3 * p.mean_square))};
  for (int q = 0; q < 11; ++q) out[q] = v[q];
  return 0;
}

/* The record bytes that the reference's frame writer emits per particle
 * (operator<<(ostream&, Box*), parallel/box.h:476-502, calls Write on each):
 * kind 0 through RepulsiveParticle::Write (shared/particle.h:759-764:
 * r_original, then theta), kind 1 through ActiveBrownianChain::Write with
 * F0 = 0 (a membrane bead, :1038-1039: r_original only), kind 2 with F0 = 1
 * (a swimmer, :1040-1045).  Returns the byte count, or -1 if cap is short. */
extern "C" long ref_write_records(int kind, int n, const double* xu, const double* yu,
                                  const double* th, unsigned char* out, long cap) {
  std::ostringstream os(std::ios::binary);
  for (int i = 0; i < n; ++i) {
    if (kind == 0) {
      RepulsiveParticle q;
      q.r_original.x = xu[i];
      q.r_original.y = yu[i];
      q.theta = th[i];
      q.Write(os);
    } else {
      ActiveBrownianChain q;
      q.Set_F0(kind == 1 ? 0.0 : 1.0);
      q.r_original.x = xu[i];
      q.r_original.y = yu[i];
      q.theta = th[i];
      q.Write(os);
    }
  }
  const std::string b = os.str();
  if ((long)b.size() > cap) return -1;
  for (size_t k = 0; k < b.size(); ++k) out[k] = (unsigned char)b[k];
  return (long)b.size();
}
