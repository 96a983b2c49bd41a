// spp_box.hpp -- header-only C++ adapter that keeps the reference's Box calling
// shape (parallel/box.h:15-58, serial/box.h:15-61) on top of the C ABI in
// spp.h, so driver code such as parallel/repulsive-vicsek.cpp:27-105 (an
// equilibrium loop of Multi_Step(cell_update_period) calls followed by
// out_file << box) keeps its structure:
//
//   spp::Box box(params);                 // Box(Lx, Ly, phi) + Init(node, rho)
//   box.Init(x, y, theta);                // Positioning_Particles / Sync
//   for (...) box.Multi_Step(steps);      // Multi_Step(cell_update_period)
//   box.Save_Polarization(pol_file);      // parallel/box.h:467-473
//   out_file << box;                      // parallel/box.h:476-502 (.bin frame)
//
// Errors throw spp::Error (status + message) where the reference prints and
// calls exit(0) (shared/cell.h:45-49, parallel/box.h:224-228).
#ifndef SPP_BOX_HPP
#define SPP_BOX_HPP

#include <cmath>
#include <cstdint>
#include <ostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "spp.h"

namespace spp {

class Error : public std::runtime_error {
 public:
  Error(int status, const std::string& where)
      : std::runtime_error(where + ": " + spp_status_string(status) + " " + spp_last_error()),
        status_(status) {}
  int status() const { return status_; }

 private:
  int status_;
};

inline void check(int status, const char* where) {
  if (status != SPP_OK) throw Error(status, where);
}

// State_Hyper_Vector counterpart (shared/state-hyper-vector.h:6-41): positions,
// headings, box-crossing counters and the Philox step counter, which is what
// makes Load() reproduce the noise (the reference copies the GSL state).
struct State {
  std::vector<float> x, y, theta;
  std::vector<int32_t> img_x, img_y;
  int64_t step = 0;
};

// Chooses p's launch shape (threads per particle, Verlet skin) by timing the
// candidates on the device from the state (x, y, theta); call before
// constructing the Box.  The reference fixes both from compile-time globals
// (shared/parameters.h:80-99).
inline SppTuneReport Autotune(SppParams& p, const std::vector<float>& x, const std::vector<float>& y,
                              const std::vector<float>& theta, int trial_steps = 200,
                              int what = SPP_TUNE_LANES | SPP_TUNE_SKIN) {
  if ((int64_t)x.size() != p.n || (int64_t)y.size() != p.n || (int64_t)theta.size() != p.n)
    throw Error(SPP_ERR_INVALID, "Autotune: state arrays must hold n values");
  SppTuneReport r;
  check(spp_autotune(&p, x.data(), y.data(), theta.data(), trial_steps, what, &r), "spp_autotune");
  return r;
}

class Box {
 public:
  explicit Box(const SppParams& p) : p_(p), t(0.0), polarization(0.0) {
    check(spp_create(&p_, &sys_), "spp_create");
    N = p_.n;
  }
  ~Box() { spp_destroy(sys_); }
  Box(const Box&) = delete;
  Box& operator=(const Box&) = delete;

  // Box::Init / Positioning_Particles: place the particles, bin them and build
  // the neighbour list.
  void Init(const std::vector<float>& x, const std::vector<float>& y,
            const std::vector<float>& theta, double t0 = 0.0) {
    step0_ = (int64_t)std::llround(t0 / p_.dt);
    check(spp_upload_state(sys_, x.data(), y.data(), theta.data(), nullptr, nullptr, N, step0_),
          "spp_upload_state");
    t = t0;
  }

  // Box::Sync / Update_Cells / Update_Neighbor_List: re-bin from the current state.
  void Sync() { Load(Save()); }
  void Update_Cells() { Sync(); }

  // Box::One_Step (parallel/box.h:354-391).
  void One_Step() { Multi_Step(1); }

  // Box::Multi_Step(steps) (parallel/box.h:394-439).  Neighbour lists are
  // rebuilt on the device when displacements require it, not after a fixed
  // number of steps, so the cell-update interval of Multi_Step(steps,
  // interval) has no effect beyond the step count.
  void Multi_Step(int steps) {
    check(spp_step(sys_, steps), "spp_step");
    t += p_.dt * steps;
  }
  void Multi_Step(int steps, int /*interval*/) { Multi_Step(steps); }

  // Box::Save / Box::Load (parallel/box.h:222-267).
  State Save() {
    State s;
    s.x.resize(N); s.y.resize(N); s.theta.resize(N); s.img_x.resize(N); s.img_y.resize(N);
    check(spp_download_state(sys_, s.x.data(), s.y.data(), s.theta.data(), s.img_x.data(),
                             s.img_y.data(), N),
          "spp_download_state");
    SppObservables o;
    check(spp_observables(sys_, &o), "spp_observables");
    s.step = step0_ + o.step;
    return s;
  }
  void Load(const State& s) {
    check(spp_upload_state(sys_, s.x.data(), s.y.data(), s.theta.data(), s.img_x.data(),
                           s.img_y.data(), N, s.step),
          "spp_upload_state");
    step0_ = s.step;
    t = s.step * p_.dt;
  }

  // Node::Compute_Polarization (parallel/node.h:1565-1591).
  double Compute_Polarization() {
    SppObservables o;
    check(spp_observables(sys_, &o), "spp_observables");
    polarization = o.polarization;
    return polarization;
  }

  // Box::Save_Polarization (parallel/box.h:467-473): "t<TAB>P" per line.
  void Save_Polarization(std::ostream& os) {
    os << t << "\t" << Compute_Polarization() << "\n";
  }

  // operator<<(ostream&, Box*) (parallel/box.h:476-502): t, Lx, Ly as
  // doubles (Lx = Ly = the half-width L), nb, Ns, Nm as int32, then the Nm
  // membrane beads (the first n_rings x ring_size particles of a bead model)
  // as (x, y) float32 (C2DVector::write, shared/c2dvector.h:175-184) and the
  // Ns swimmers as (x, y, theta) float32 (RepulsiveParticle::Write, shared/
  // particle.h:759-764); x, y are the unwrapped positions r_original.
  friend std::ostream& operator<<(std::ostream& os, Box& box) {
    State s = box.Save();
    double L = box.p_.L;
    // the first swimmer's chain length (particle[Nm].nb)
    int32_t nb = box.p_.model == SPP_MODEL_BEADS && box.p_.chain_beads > 1 ? box.p_.chain_beads : 1;
    int32_t Nm = box.p_.model == SPP_MODEL_BEADS ? box.p_.n_rings * box.p_.ring_size : 0;
    int32_t Ns = box.N - Nm;
    os.write(reinterpret_cast<const char*>(&box.t), sizeof(double));
    os.write(reinterpret_cast<const char*>(&L), sizeof(double));
    os.write(reinterpret_cast<const char*>(&L), sizeof(double));
    os.write(reinterpret_cast<const char*>(&nb), sizeof(int32_t));
    os.write(reinterpret_cast<const char*>(&Ns), sizeof(int32_t));
    os.write(reinterpret_cast<const char*>(&Nm), sizeof(int32_t));
    for (int i = 0; i < box.N; ++i) {
      float rec[3] = {(float)(s.x[i] + 2.0 * L * s.img_x[i]), (float)(s.y[i] + 2.0 * L * s.img_y[i]),
                      s.theta[i]};
      os.write(reinterpret_cast<const char*>(rec), (i < Nm ? 2 : 3) * sizeof(float));
    }
    return os;
  }

  SppSystem* handle() { return sys_; }
  const SppParams& params() const { return p_; }

  int N;
  double t;
  double polarization;

 private:
  SppParams p_;
  SppSystem* sys_ = nullptr;
  int64_t step0_ = 0;
};

}  // namespace spp

#endif  // SPP_BOX_HPP
