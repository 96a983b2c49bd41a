/*
 * tune.cu -- spp_autotune: the launch shape of a Verlet-list system, chosen
 * by timing its candidates on the device.
 *
 * The reference sizes its cells and lists from compile-time globals
 * (cell_update_interval, lx_min and the Verlet radius of
 * shared/parameters.h:80-99) whatever the system's size or density.  Here
 * two choices are left to measurement, per (model, N, density):
 *   - threads per particle in the neighbour sums (gather_lanes 1 or 4): four
 *     lanes fill the GPU when the system is small or its lists are long, one
 *     lane wastes fewer instructions on large, uniform systems;
 *   - the Verlet skin: a wider skin means longer lists in every stage and
 *     fewer rebuilds.
 * Only the public entry points are used: each candidate is a fresh system,
 * stepped untimed (graph capture, list growth), then timed with CUDA events
 * by spp_time_steps.
 */
#include <string>
#include "spp_internal.cuh"

namespace {

int tune_fail(int status, const std::string& m) {
  spp_internal_set_error(m.c_str());
  return status;
}

/* One candidate: create, upload, trial untimed steps (they capture every
 * step graph the timed run replays, and grow the list), then trial timed
 * steps.  A list regrowth inside the timed window (the overflowed steps are
 * re-run after the timing events) is timed again, up to three times. */
void tune_one(const SppParams& q, const float* x, const float* y, const float* th, int trial,
              SppTuneCandidate* c) {
  c->gather_lanes = q.gather_lanes;
  c->skin = q.skin;
  c->ms_per_step = 0.0;
  c->late_rebuilds = 0;
  SppSystem* s = nullptr;
  int rc = spp_create(&q, &s);
  if (rc == SPP_OK) rc = spp_upload_state(s, x, y, th, nullptr, nullptr, q.n, 0);
  if (rc == SPP_OK) rc = spp_step(s, trial);
  SppObservables o;
  if (rc == SPP_OK) rc = spp_observables(s, &o);
  double ms = 0.0;
  for (int attempt = 0; rc == SPP_OK && attempt < 3; ++attempt) {
    const int32_t cap0 = o.list_capacity;
    rc = spp_time_steps(s, trial, &ms);
    if (rc == SPP_OK) rc = spp_observables(s, &o);
    if (rc == SPP_OK && o.list_capacity == cap0) break;
  }
  if (rc == SPP_OK) {
    c->ms_per_step = ms / trial;
    c->late_rebuilds = o.late_rebuilds;
  }
  c->status = rc;
  if (s) spp_destroy(s);
}

}  // namespace

extern "C" int spp_autotune(SppParams* p, const float* x, const float* y, const float* theta,
                            int trial_steps, int what, SppTuneReport* report) {
  if (!p || !x || !y || !theta || !report)
    return tune_fail(SPP_ERR_INVALID, "spp_autotune: NULL argument");
  if (trial_steps < 1 || trial_steps > 1000000)
    return tune_fail(SPP_ERR_INVALID, "spp_autotune: trial_steps must be in [1, 1000000]");
  if (what < 1 || (what & ~(SPP_TUNE_LANES | SPP_TUNE_SKIN)) != 0)
    return tune_fail(SPP_ERR_INVALID, "spp_autotune: what must combine SPP_TUNE_LANES and SPP_TUNE_SKIN");
  if (p->model != SPP_MODEL_ABP && p->model != SPP_MODEL_CONTINUOUS && p->model != SPP_MODEL_BEADS)
    return tune_fail(SPP_ERR_UNSUPPORTED,
                     "spp_autotune: the Verlet-list models (ABP, continuous, beads) have a launch shape to tune");
  const bool lane_model = p->model == SPP_MODEL_ABP || p->model == SPP_MODEL_CONTINUOUS ||
                          (p->model == SPP_MODEL_BEADS && p->chain_beads <= 1);
  int lanes[2] = {p->gather_lanes, 0};
  int n_lanes = 1;
  if ((what & SPP_TUNE_LANES) && lane_model) {
    lanes[0] = 1;
    lanes[1] = 4;
    n_lanes = 2;
  }
  /* the caller's skin first, so that equal times keep it */
  static const double skin_factor[4] = {1.0, 0.5, 1.5, 2.0};
  const int n_skin = (what & SPP_TUNE_SKIN) ? 4 : 1;

  SppTuneReport r = {};
  r.best = -1;
  int first_bad = SPP_OK;
  std::string first_msg;
  for (int a = 0; a < n_lanes; ++a) {
    for (int b = 0; b < n_skin; ++b) {
      SppParams q = *p;
      q.gather_lanes = lanes[a];
      q.skin = p->skin * skin_factor[b];
      SppTuneCandidate* c = &r.c[r.n_candidates++];
      tune_one(q, x, y, theta, trial_steps, c);
      if (c->status != SPP_OK && first_bad == SPP_OK) {
        first_bad = c->status;
        first_msg = spp_last_error();
      }
      if (c->status == SPP_OK && c->late_rebuilds == 0 &&
          (r.best < 0 || c->ms_per_step < r.c[r.best].ms_per_step))
        r.best = r.n_candidates - 1;
    }
  }
  *report = r;
  if (r.best < 0) {
    if (first_bad != SPP_OK) return tune_fail(first_bad, "spp_autotune: no candidate ran: " + first_msg);
    return tune_fail(SPP_ERR_INVALID,
                     "spp_autotune: every candidate missed list rebuilds (the step outruns the skin)");
  }
  p->gather_lanes = r.c[r.best].gather_lanes;
  p->skin = r.c[r.best].skin;
  return SPP_OK;
}
