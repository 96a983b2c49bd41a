/*
 * api.cu -- the C ABI of include/spp.h.
 *
 * One SppSystem owns the device buffers of one periodic box and launches on
 * one CUDA stream.  spp_step() replays CUDA graphs of whole steps:
 *   ABP / continuous:  [stage kernel] x stages  ->  IF(rebuild) { zero counts,
 *                      bin_count, scan x3, scatter, build_list }
 *   Vicsek (dt = 1):   zero counts, bin_count, scan x3, scatter, step kernel
 * The IF condition is set on the device by the last stage kernel
 * (cudaGraphSetConditional), so a replay of many steps never returns to the
 * host.  This is the GB300 counterpart of Box::Multi_Step (parallel/box.h:
 * 394-439), whose per-step MPI barriers and fixed-period Quick_Update_Cells
 * disappear.
 */
#include <cstdio>
#include <cstring>
#include <cmath>
#include <string>
#include <vector>
#include "spp_internal.cuh"
#include "spp_lyap.cuh"

namespace {

thread_local std::string g_err;

int fail(int status, const std::string& msg) {
  g_err = msg;
  return status;
}

#define CUDA_TRY(expr)                                                                      \
  do {                                                                                      \
    cudaError_t _e = (expr);                                                                \
    if (_e != cudaSuccess)                                                                  \
      return fail(SPP_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e));       \
  } while (0)

constexpr int GRAPH_CHUNK = 32;

struct GraphEntry {
  int nsteps;
  cudaGraph_t graph;
  cudaGraphExec_t exec;
};

}  // namespace

void spp_internal_set_error(const char* msg) { g_err = msg ? msg : ""; }

struct SppSystem {
  SppParams p;
  SppConsts k;
  DevState d;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;   /* used only while capturing conditional bodies */
  /* the tangent stages of a Lyapunov run, forked off `stream` so that each
   * runs beside the base stage of the same Runge-Kutta stage */
  cudaStream_t tan_stream = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  bool own_stream = false;
  bool uses_list = false;        /* Verlet list models (ABP, continuous) */
  int nstages = 1;
  int per_step_kernels = 0;
  int per_rebuild_kernels = 0;
  int64_t host_launches = 0;
  int64_t graph_kernels = 0;
  int64_t direct_rebuilds = 0;
  int64_t regrowths = 0;         /* neighbour-list regrowths after an overflow */
  /* frame marked for spp_ring_motion: unwrapped positions and headings by
   * particle id, and the step counter at the mark (-1: none) */
  double2* mark_xy = nullptr;
  float* mark_th = nullptr;
  int64_t mark_step = -1;
  int64_t target_step = 0;       /* step the caller has asked to reach */
  int64_t step0 = 0;
  bool uploaded = false;
  bool use_graphs = true;
  bool small_vicsek = false;     /* whole steps in one block (k_vicsek_small) */
  float* stage_x = nullptr;      /* staging for uploads/downloads */
  float* stage_y = nullptr;
  float* stage_t = nullptr;
  int2* stage_img = nullptr;
  std::vector<GraphEntry> graphs;
  /* tangent-space (Lyapunov) estimator */
  LyapState lyap;
  bool lyap_on = false;
  int64_t lyap_steps = 0;        /* steps since spp_lyap_init */
  int lyap_renorm_every = 10;
  std::vector<GraphEntry> lyap_graphs;  /* keyed by steps per renormalisation chunk */
};

namespace {

void free_graphs(SppSystem* s) {
  for (auto& g : s->graphs) {
    cudaGraphExecDestroy(g.exec);
    cudaGraphDestroy(g.graph);
  }
  s->graphs.clear();
}

template <class T>
int dalloc(T** ptr, size_t count) {
  *ptr = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc((void**)ptr, count * sizeof(T));
  if (e != cudaSuccess) {
    *ptr = nullptr;
    return fail(SPP_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  return SPP_OK;
}

void free_lyap(SppSystem* s) {
  LyapState& L = s->lyap;
  void* ptrs[] = {L.t0, L.ua, L.ub, L.acc, L.uslot, L.partial, L.rinv, L.log_stretch, L.error};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  memset(&L, 0, sizeof(L));
  for (auto& g : s->lyap_graphs) {
    cudaGraphExecDestroy(g.exec);
    cudaGraphDestroy(g.graph);
  }
  s->lyap_graphs.clear();
  s->lyap_on = false;
}

void free_dev(SppSystem* s) {
  if (s->mark_xy) cudaFree(s->mark_xy);
  if (s->mark_th) cudaFree(s->mark_th);
  s->mark_xy = nullptr;
  s->mark_th = nullptr;
  s->mark_step = -1;
  DevState& d = s->d;
  void* ptrs[] = {d.pos, d.half, d.half2, d.theta, d.img, d.id, d.inv, d.kacc, d.dth, d.ref, d.pos_alt,
                  d.theta_alt, d.img_alt, d.id_alt, d.key, d.rank, d.cell_count, d.cell_start,
                  d.scan_tmp, d.nbr, d.nn, d.long_q, d.nn_lanes, d.tumble, d.ctl, d.red, s->stage_x, s->stage_y, s->stage_t,
                  s->stage_img};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  memset(&s->d, 0, sizeof(s->d));
  s->stage_x = s->stage_y = s->stage_t = nullptr;
  s->stage_img = nullptr;
}

double interaction_radius(const SppParams& p) { return spp_interaction_range(&p); }

int validate(const SppParams* p) {
  if (!p) return fail(SPP_ERR_INVALID, "params is NULL");
  if (p->struct_size != sizeof(SppParams))
    return fail(SPP_ERR_INVALID, "SppParams.struct_size does not match this library");
  if (p->n < 1) return fail(SPP_ERR_INVALID, "n must be >= 1");
  if (!(p->L > 0) || !(p->dt > 0)) return fail(SPP_ERR_INVALID, "L and dt must be > 0");
  if (!(p->r_align > 0)) return fail(SPP_ERR_INVALID, "r_align must be > 0");
  if (p->Dr < 0 || p->skin < 0) return fail(SPP_ERR_INVALID, "Dr and skin must be >= 0");
  if (p->rot_noise != SPP_NOISE_GAUSSIAN && p->rot_noise != SPP_NOISE_TUMBLE)
    return fail(SPP_ERR_INVALID, "rot_noise must be SPP_NOISE_GAUSSIAN or SPP_NOISE_TUMBLE");
  if (p->rot_noise == SPP_NOISE_TUMBLE) {
    if (p->model != SPP_MODEL_BEADS)
      return fail(SPP_ERR_UNSUPPORTED, "run and tumble is built for SPP_MODEL_BEADS swimmers (RTPChain)");
    if (!(p->tumble_rate >= 0) || !std::isfinite(p->tumble_rate) || !std::isfinite(p->tumble_time) ||
        !std::isfinite(p->tumble_torque) || p->tumble_time / p->dt > 2.0e9)
      return fail(SPP_ERR_INVALID, "tumble_rate >= 0, finite tumble_time / tumble_torque, "
                                   "tumble_time / dt < 2e9");
  }
  if (p->chain_beads < 0 || p->chain_beads > SPP_MAX_CHAIN_BEADS)
    return fail(SPP_ERR_INVALID, "chain_beads must be 0 .. SPP_MAX_CHAIN_BEADS (0 and 1: single beads)");
  if (p->chain_beads > 1) {
    if (p->model != SPP_MODEL_BEADS)
      return fail(SPP_ERR_UNSUPPORTED, "multi-bead swimmers are built for SPP_MODEL_BEADS (ActiveBrownianChain)");
    if (p->force_law != SPP_FORCE_R12_TRUNC && p->force_law != SPP_FORCE_NONE)
      return fail(SPP_ERR_INVALID, "chains interact by R12_Repulsive_Truncated (SPP_FORCE_R12_TRUNC) or not at all");
    if (!(p->bead_separation > 0) || !(p->sigma_chain > 0) || !(p->r_chain > 0) ||
        !std::isfinite(p->bead_separation) || !std::isfinite(p->sigma_chain) || !std::isfinite(p->r_chain))
      return fail(SPP_ERR_INVALID, "bead_separation, sigma_chain and r_chain must be finite and > 0");
  }
  if (p->gather_lanes != 0 && p->gather_lanes != 1 && p->gather_lanes != SPP_GATHER_LANES)
    return fail(SPP_ERR_INVALID, "gather_lanes must be 0 (automatic), 1 or 4");
  if (p->gather_lanes == SPP_GATHER_LANES && p->model != SPP_MODEL_ABP && p->model != SPP_MODEL_CONTINUOUS &&
      !(p->model == SPP_MODEL_BEADS && p->chain_beads <= 1))
    return fail(SPP_ERR_UNSUPPORTED,
                "gather_lanes = 4 is built for SPP_MODEL_ABP, SPP_MODEL_CONTINUOUS and single-bead SPP_MODEL_BEADS");
  if (p->boundary != SPP_BOUNDARY_PERIODIC && p->boundary != SPP_BOUNDARY_WALLS &&
      p->boundary != SPP_BOUNDARY_CIRCLE)
    return fail(SPP_ERR_INVALID, "boundary must be SPP_BOUNDARY_PERIODIC, _WALLS or _CIRCLE");
  if (p->boundary == SPP_BOUNDARY_CIRCLE) {
    if (p->model != SPP_MODEL_ABP && p->model != SPP_MODEL_CONTINUOUS)
      return fail(SPP_ERR_UNSUPPORTED, "the circular box is built for SPP_MODEL_ABP and SPP_MODEL_CONTINUOUS "
                                       "(the particles with a torque, parallel/box.h:285-294)");
    if (p->n_walls != 0) return fail(SPP_ERR_INVALID, "the circular box has no wall segments (n_walls = 0)");
  }
  if (p->boundary == SPP_BOUNDARY_WALLS) {
    if (p->model != SPP_MODEL_ABP && p->model != SPP_MODEL_CONTINUOUS &&
        p->model != SPP_MODEL_VICSEK_REF_ANGLE && p->model != SPP_MODEL_VICSEK_REF_VECTOR)
      return fail(SPP_ERR_UNSUPPORTED, "walls are built for SPP_MODEL_ABP, SPP_MODEL_CONTINUOUS, "
                                       "SPP_MODEL_VICSEK_REF_ANGLE and SPP_MODEL_VICSEK_REF_VECTOR "
                                       "(the reference's Wall::Interact overloads)");
    if (p->n_walls < 0 || p->n_walls > SPP_MAX_WALLS - 4)
      return fail(SPP_ERR_INVALID, "n_walls must be 0 .. SPP_MAX_WALLS - 4 (the box has 4 walls)");
    for (int w = 0; w < p->n_walls; ++w) {
      const double* q = p->walls[w];
      if (!std::isfinite(q[0]) || !std::isfinite(q[1]) || !std::isfinite(q[2]) || !std::isfinite(q[3]) ||
          (q[0] == q[2] && q[1] == q[3]))
        return fail(SPP_ERR_INVALID, "wall " + std::to_string(w) + ": finite end points, nonzero length");
    }
    const double wp[6] = {p->A_w, p->sigma_w, p->r_c_w, p->r_f_w, p->g_w, p->g_w_cont};
    for (double v : wp)
      if (!std::isfinite(v)) return fail(SPP_ERR_INVALID, "wall parameters must be finite");
    if (p->r_c_w > 0 && !(p->sigma_w > 0))
      return fail(SPP_ERR_INVALID, "wall repulsion (r_c_w > 0) needs sigma_w > 0");
  }
  switch (p->model) {
    case SPP_MODEL_VICSEK:
    case SPP_MODEL_VICSEK_REF_ANGLE:
    case SPP_MODEL_VICSEK_REF_VECTOR:
      break;
    case SPP_MODEL_BEADS:
      if (p->n_rings < 0 || (p->n_rings > 0 && p->ring_size < 3) ||
          (int64_t)p->n_rings * p->ring_size > p->n)
        return fail(SPP_ERR_INVALID, "membrane rings: need ring_size >= 3 and n_rings*ring_size <= n");
      /* fall through */
    case SPP_MODEL_ABP:
    case SPP_MODEL_CONTINUOUS:
      if (p->integrator != SPP_INT_EULER && p->integrator != SPP_INT_RK2 &&
          p->integrator != SPP_INT_RK4)
        return fail(SPP_ERR_INVALID, "integrator must be SPP_INT_EULER, _RK2 or _RK4");
      if (!(p->skin > 0)) return fail(SPP_ERR_INVALID, "the Verlet-list models need skin > 0");
      if (p->model == SPP_MODEL_CONTINUOUS && p->force_law != SPP_FORCE_NONE)
        return fail(SPP_ERR_UNSUPPORTED, "ContinuousParticle has no pair repulsion (shared/particle.h:296-338): "
                                         "force_law must be SPP_FORCE_NONE");
      if (p->model != SPP_MODEL_CONTINUOUS && p->force_law != SPP_FORCE_NONE &&
          p->force_law != SPP_FORCE_HARMONIC && p->force_law != SPP_FORCE_R12_TRUNC)
        return fail(SPP_ERR_INVALID, "unknown force law");
      /* a harmonic pair term is bounded by k_rep; the fixed-point sums take
       * terms below 2^16 */
      if (p->force_law == SPP_FORCE_HARMONIC && !(std::fabs(p->k_rep) < 65536.0))
        return fail(SPP_ERR_INVALID, "|k_rep| must be < 65536");
      break;
    default:
      return fail(SPP_ERR_UNSUPPORTED, "model not built into this library");
  }
  return SPP_OK;
}

int enqueue_rebuild(SppSystem* s, cudaStream_t st, int64_t* launches) {
  CUDA_TRY(cudaMemsetAsync(s->d.cell_count, 0, sizeof(uint32_t) * s->d.n_keys, st));
  launch_bin_count(s->k, s->d, st, launches);
  launch_scan(s->d, st, launches);
  launch_scatter(s->d, st, launches);
  launch_build_list(s->k, s->d, s->uses_list ? 1 : 0, st, launches);
  CUDA_TRY(cudaGetLastError());
  return SPP_OK;
}

/* One step of the model, enqueued on st (stream or capture). */
int enqueue_step(SppSystem* s, cudaStream_t st, bool capture, int64_t* launches) {
  if (!s->uses_list && s->small_vicsek) {
    if (launch_vicsek_small(s->k, s->d, 1, st, launches) != 0)
      return fail(SPP_ERR_CUDA, "k_vicsek_small: cluster launch refused (shared memory or cluster shape)");
    CUDA_TRY(cudaGetLastError());
    return SPP_OK;
  }
  if (!s->uses_list) {
    CUDA_TRY(cudaMemsetAsync(s->d.cell_count, 0, sizeof(uint32_t) * s->d.n_keys, st));
    launch_bin_count(s->k, s->d, st, launches);
    launch_scan(s->d, st, launches);
    launch_scatter(s->d, st, launches);
    launch_vicsek_step(s->k, s->d, st, launches);
    CUDA_TRY(cudaGetLastError());
    return SPP_OK;
  }
  cudaGraphConditionalHandle handle = 0;
  if (capture) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t g;
    CUDA_TRY(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, nullptr, nullptr, nullptr));
    CUDA_TRY(cudaGraphConditionalHandleCreate(&handle, g, 0, cudaGraphCondAssignDefault));
  }
  for (int stage = 0; stage < s->nstages; ++stage)
    launch_abp_stage(s->k, s->d, stage, s->nstages, handle, capture ? 1 : 0, st, launches);
  CUDA_TRY(cudaGetLastError());
  if (!capture) return SPP_OK;
  /* IF(rebuild) node whose body holds the rebuild kernels. */
  cudaStreamCaptureStatus cs;
  cudaGraph_t g;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  CUDA_TRY(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &ndeps));
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = handle;
  cp.conditional.type = cudaGraphCondTypeIf;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  CUDA_TRY(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  CUDA_TRY(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1,
                                               cudaStreamSetCaptureDependencies));
  CUDA_TRY(cudaStreamBeginCaptureToGraph(s->side, body, nullptr, nullptr, 0,
                                         cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_rebuild(s, s->side, nullptr);
  cudaGraph_t body_out = body;
  cudaError_t e = cudaStreamEndCapture(s->side, &body_out);
  if (rc != SPP_OK) return rc;
  if (e != cudaSuccess) return fail(SPP_ERR_CUDA, std::string("capture rebuild body: ") +
                                                      cudaGetErrorString(e));
  return SPP_OK;
}

int get_graph(SppSystem* s, int nsteps, cudaGraphExec_t* out) {
  for (auto& g : s->graphs)
    if (g.nsteps == nsteps) { *out = g.exec; return SPP_OK; }
  cudaGraph_t graph = nullptr;
  CUDA_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  int rc = SPP_OK;
  for (int i = 0; i < nsteps && rc == SPP_OK; ++i) rc = enqueue_step(s, s->stream, true, nullptr);
  cudaError_t e = cudaStreamEndCapture(s->stream, &graph);
  if (rc != SPP_OK) { if (graph) cudaGraphDestroy(graph); return rc; }
  if (e != cudaSuccess) return fail(SPP_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  cudaGraphExec_t exec;
  e = cudaGraphInstantiate(&exec, graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    return fail(SPP_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  }
  s->graphs.push_back({nsteps, graph, exec});
  *out = exec;
  return SPP_OK;
}

int run_steps(SppSystem* s, int64_t nsteps) {
  if (s->small_vicsek) {
    /* one launch per call runs every step */
    while (nsteps > 0) {
      const int chunk = nsteps > (1 << 20) ? (1 << 20) : (int)nsteps;
      if (launch_vicsek_small(s->k, s->d, chunk, s->stream, &s->host_launches) != 0)
        return fail(SPP_ERR_CUDA, "k_vicsek_small: cluster launch refused (shared memory or cluster shape)");
      CUDA_TRY(cudaGetLastError());
      nsteps -= chunk;
    }
    return SPP_OK;
  }
  if (!s->use_graphs) {
    for (int64_t i = 0; i < nsteps; ++i) {
      int rc = enqueue_step(s, s->stream, false, &s->host_launches);
      if (rc != SPP_OK) return rc;
      if (s->uses_list) {
        Ctl c;
        CUDA_TRY(cudaMemcpyAsync(&c, s->d.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s->stream));
        CUDA_TRY(cudaStreamSynchronize(s->stream));
        if (c.need_rebuild) {
          rc = enqueue_rebuild(s, s->stream, &s->host_launches);
          if (rc != SPP_OK) return rc;
          s->direct_rebuilds++;
        }
      }
    }
    return SPP_OK;
  }
  while (nsteps > 0) {
    int chunk = nsteps >= GRAPH_CHUNK ? GRAPH_CHUNK : (int)nsteps;
    cudaGraphExec_t exec;
    int rc = get_graph(s, chunk, &exec);
    if (rc != SPP_OK) return rc;
    CUDA_TRY(cudaGraphLaunch(exec, s->stream));
    s->graph_kernels += (int64_t)chunk * s->per_step_kernels;
    nsteps -= chunk;
  }
  return SPP_OK;
}

int read_ctl(SppSystem* s, Ctl* c) {
  CUDA_TRY(cudaMemcpyAsync(c, s->d.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return SPP_OK;
}

int list_capacity_for(const SppParams& p, double rlist) {
  double area = 4.0 * p.L * p.L;
  double expected = (double)p.n / area * M_PI * rlist * rlist;
  int cap = (int)std::ceil(expected * 2.0 + 8.0);
  if (cap < 16) cap = 16;
  return (cap + 3) & ~3;
}

int alloc_list(SppSystem* s, int cap) {
  if (s->d.nbr) cudaFree(s->d.nbr);
  s->d.nbr = nullptr;
  s->d.cap = cap;
  return dalloc(&s->d.nbr, (size_t)cap * s->d.n);
}

int enqueue_lyap_step(SppSystem* s, cudaStream_t st, bool capture, int64_t* launches);
int launch_lyap_chunks(SppSystem* s, int64_t nsteps);

/* Base + tangent steps with direct launches (recovery path): the rebuild is
 * decided on the host after each step, renormalisation every
 * lyap_renorm_every steps and at the end.  Extra renormalisation points
 * leave the summed log-stretches unchanged (the stretches multiply). */
int run_lyap_direct(SppSystem* s, int64_t nsteps) {
  for (int64_t i = 0; i < nsteps; ++i) {
    int rc = enqueue_lyap_step(s, s->stream, false, &s->host_launches);
    if (rc != SPP_OK) return rc;
    Ctl c;
    CUDA_TRY(cudaMemcpyAsync(&c, s->d.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (c.frozen) return SPP_OK;  /* the caller grows the list and comes back */
    if (c.need_rebuild) {
      rc = enqueue_rebuild(s, s->stream, &s->host_launches);
      if (rc != SPP_OK) return rc;
      s->direct_rebuilds++;
    }
    if ((i + 1) % s->lyap_renorm_every == 0 || i + 1 == nsteps)
      launch_renormalize(s->lyap, 1, s->stream, &s->host_launches);
  }
  return SPP_OK;
}

/* Grows the neighbour list after an overflow and finishes the steps the
 * frozen kernels skipped.  A system whose density keeps growing (flocks
 * without repulsion) may overflow again after some progress; recovery goes
 * on while the steps advance and gives up after 8 overflows in a row at the
 * same step. */
int recover(SppSystem* s) {
  int64_t last_frozen_step = -1;
  for (int stalls = 0; stalls < 8;) {
    Ctl c;
    int rc = read_ctl(s, &c);
    if (rc != SPP_OK) return rc;
    if (c.bad_index)
      return fail(SPP_ERR_BOUNDS, "a kernel met an index out of range and skipped the access "
                                  "(SPP_CHECKED build); the state is not reliable");
    if (c.fx_overflow)
      return fail(SPP_ERR_OVERFLOW, "a pair term exceeded the fixed-point range (overlapping "
                                    "particles under an R12 force?); the state is not reliable");
    if (!c.frozen) {
      if ((int64_t)c.step >= s->target_step) return SPP_OK;
      if (s->lyap_on && s->use_graphs) rc = launch_lyap_chunks(s, s->target_step - (int64_t)c.step);
      else if (s->lyap_on) rc = run_lyap_direct(s, s->target_step - (int64_t)c.step);
      else rc = run_steps(s, s->target_step - (int64_t)c.step);
      if (rc != SPP_OK) return rc;
      continue;
    }
    if ((int64_t)c.step <= last_frozen_step) ++stalls;
    else stalls = 0;
    last_frozen_step = (int64_t)c.step;
    /* densities that grew once tend to keep growing (flocking): grow by at
     * least half the current capacity, so that a long run regrows rarely */
    int64_t need = (int64_t)c.list_need * 3 / 2 + 8;
    if (need < (int64_t)s->d.cap * 3 / 2 + 4) need = (int64_t)s->d.cap * 3 / 2 + 4;
    if (need > (int64_t)s->d.n + 4) need = (int64_t)s->d.n + 4;
    int cap = (int)((need + 3) & ~(int64_t)3);
    free_graphs(s);
    for (auto& g : s->lyap_graphs) {
      cudaGraphExecDestroy(g.exec);
      cudaGraphDestroy(g.graph);
    }
    s->lyap_graphs.clear();
    rc = alloc_list(s, cap);
    if (rc != SPP_OK) return rc;
    s->regrowths++;
    CUDA_TRY(cudaMemsetAsync(&s->d.ctl->frozen, 0, sizeof(uint32_t), s->stream));
    CUDA_TRY(cudaMemsetAsync(&s->d.ctl->list_need, 0, sizeof(uint32_t), s->stream));
    rc = enqueue_rebuild(s, s->stream, &s->host_launches);
    if (rc != SPP_OK) return rc;
    s->direct_rebuilds++;
  }
  return fail(SPP_ERR_OVERFLOW, "neighbour list kept overflowing");
}

/* One step of base + tangent dynamics: each base stage is followed by the
 * tangent stage evaluated on the same stage state. */
int enqueue_lyap_step(SppSystem* s, cudaStream_t st, bool capture, int64_t* launches) {
  cudaGraphConditionalHandle handle = 0;
  if (capture) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t g;
    CUDA_TRY(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, nullptr, nullptr, nullptr));
    CUDA_TRY(cudaGraphConditionalHandleCreate(&handle, g, 0, cudaGraphCondAssignDefault));
  }
  const DevState& d = s->d;
  /* Base and tangent stage s both read the stage input that stage s - 1
   * wrote and write buffers the other does not touch, so they run side by
   * side (the tangent stage on tan_stream); both finish before stage s + 1,
   * whose base stage overwrites a buffer that a tangent stage of this step
   * has read (RK2: the start state; RK4: half), and before the rebuild that
   * reorders the slots. */
  const bool fork = s->tan_stream != nullptr;
  for (int stage = 0; stage < s->nstages; ++stage) {
    const float4* cur;
    if (s->nstages == 2) cur = stage == 0 ? d.pos : d.half;
    else {
      const float4* bufs[3] = {d.pos, d.half, d.half2};
      static const int cur_sel[4] = {0, 1, 2, 1};
      cur = bufs[cur_sel[stage]];
    }
    cudaStream_t ts = st;
    if (fork) {
      CUDA_TRY(cudaEventRecord(s->ev_fork, st));
      CUDA_TRY(cudaStreamWaitEvent(s->tan_stream, s->ev_fork, 0));
      ts = s->tan_stream;
    }
    launch_abp_stage(s->k, d, stage, s->nstages, handle, capture ? 1 : 0, st, launches);
    launch_tangent_stage(s->k, d, s->lyap, stage, s->nstages, cur, ts, launches);
    if (fork) {
      CUDA_TRY(cudaEventRecord(s->ev_join, s->tan_stream));
      CUDA_TRY(cudaStreamWaitEvent(st, s->ev_join, 0));
    }
  }
  CUDA_TRY(cudaGetLastError());
  if (!capture) return SPP_OK;
  cudaStreamCaptureStatus cs;
  cudaGraph_t g;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  CUDA_TRY(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &ndeps));
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = handle;
  cp.conditional.type = cudaGraphCondTypeIf;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  CUDA_TRY(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  CUDA_TRY(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1,
                                               cudaStreamSetCaptureDependencies));
  CUDA_TRY(cudaStreamBeginCaptureToGraph(s->side, body, nullptr, nullptr, 0,
                                         cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_rebuild(s, s->side, nullptr);
  cudaGraph_t body_out = body;
  cudaError_t e = cudaStreamEndCapture(s->side, &body_out);
  if (rc != SPP_OK) return rc;
  if (e != cudaSuccess) return fail(SPP_ERR_CUDA, std::string("capture rebuild body: ") +
                                                      cudaGetErrorString(e));
  return SPP_OK;
}

/* Graph of `chunk` base+tangent steps followed by the FP64 renormalisation. */
int get_lyap_graph(SppSystem* s, int chunk, cudaGraphExec_t* out) {
  for (auto& g : s->lyap_graphs)
    if (g.nsteps == chunk) { *out = g.exec; return SPP_OK; }
  cudaGraph_t graph = nullptr;
  CUDA_TRY(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  int rc = SPP_OK;
  for (int i = 0; i < chunk && rc == SPP_OK; ++i) rc = enqueue_lyap_step(s, s->stream, true, nullptr);
  if (rc == SPP_OK) launch_renormalize(s->lyap, 1, s->stream, nullptr);
  cudaError_t e = cudaStreamEndCapture(s->stream, &graph);
  if (rc != SPP_OK) { if (graph) cudaGraphDestroy(graph); return rc; }
  if (e != cudaSuccess) return fail(SPP_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  cudaGraphExec_t exec;
  e = cudaGraphInstantiate(&exec, graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    return fail(SPP_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  }
  s->lyap_graphs.push_back({chunk, graph, exec});
  *out = exec;
  return SPP_OK;
}

/* Graphs of renorm_every base + tangent steps, each closed by the FP64
 * renormalisation.  Also the recovery path after a list overflow: the steps
 * the frozen kernels skipped are run again the same way (the chunk ends of
 * the re-run are extra renormalisation points, which leave the summed
 * log-stretches unchanged). */
int launch_lyap_chunks(SppSystem* s, int64_t nsteps) {
  const int every = s->lyap_renorm_every > 0 ? s->lyap_renorm_every : 10;
  int64_t left = nsteps;
  while (left > 0) {
    int chunk = left >= every ? every : (int)left;
    cudaGraphExec_t exec;
    int rc = get_lyap_graph(s, chunk, &exec);
    if (rc != SPP_OK) return rc;
    CUDA_TRY(cudaGraphLaunch(exec, s->stream));
    s->graph_kernels += (int64_t)chunk * (2 * s->nstages + 1) + 6;  /* stages x (base, tangent) + gather; renormalisation */
    left -= chunk;
  }
  return SPP_OK;
}

}  // namespace

/* Internal view of a system for the observables (observables.cu). */
int spp_internal_view(SppSystem* s, DevState* d, SppConsts* k, cudaStream_t* st) {
  if (!s) return fail(SPP_ERR_INVALID, "system is NULL");
  if (!s->uploaded) return fail(SPP_ERR_INVALID, "no state uploaded");
  *d = s->d;
  *k = s->k;
  *st = s->stream;
  return SPP_OK;
}

void spp_internal_count_launches(SppSystem* s, int n) {
  if (s) s->host_launches += n;
}

int spp_internal_mark(SppSystem* s, double2** xy, float** th, int64_t** step) {
  if (!s->mark_xy) {
    int rc = dalloc(&s->mark_xy, (size_t)s->p.n);
    if (rc == SPP_OK) rc = dalloc(&s->mark_th, (size_t)s->p.n);
    if (rc != SPP_OK) return rc;
  }
  *xy = s->mark_xy;
  *th = s->mark_th;
  *step = &s->mark_step;
  return SPP_OK;
}

double spp_internal_dt(SppSystem* s) { return s->p.dt; }

int64_t spp_internal_step(SppSystem* s) {
  Ctl c;
  if (read_ctl(s, &c) != SPP_OK) return -1;
  return (int64_t)c.step;
}

extern "C" {

int spp_abi_version(void) { return SPP_ABI_VERSION; }

const char* spp_status_string(int st) {
  switch (st) {
    case SPP_OK: return "SPP_OK";
    case SPP_ERR_INVALID: return "SPP_ERR_INVALID";
    case SPP_ERR_ALLOC: return "SPP_ERR_ALLOC";
    case SPP_ERR_CUDA: return "SPP_ERR_CUDA";
    case SPP_ERR_OVERFLOW: return "SPP_ERR_OVERFLOW";
    case SPP_ERR_TIMEOUT: return "SPP_ERR_TIMEOUT";
    case SPP_ERR_UNSUPPORTED: return "SPP_ERR_UNSUPPORTED";
    case SPP_ERR_NUMERIC: return "SPP_ERR_NUMERIC";
    case SPP_ERR_BOUNDS: return "SPP_ERR_BOUNDS";
    default: return "SPP_ERR_UNKNOWN";
  }
}

const char* spp_last_error(void) { return g_err.c_str(); }

int spp_params_init(SppParams* p, int model) {
  if (!p) return fail(SPP_ERR_INVALID, "params is NULL");
  memset(p, 0, sizeof(*p));
  p->struct_size = sizeof(SppParams);
  p->model = model;
  p->seed = 10;                   /* shared/parameters.h:60 */
  p->L = 64.0;                    /* Lx_int, parameters.h:68 */
  p->dt = 1.0 / 1024;             /* parameters.h:77 */
  p->v0 = 1.0;                    /* speed, parameters.h:89 */
  p->g = 1.0;
  p->r_align = 1.0;
  p->sigma_rep = 1.0;
  p->beta_push = 2.5;             /* VicsekParticle2::beta, particle.h:249 */
  p->r_push = 0.127;              /* VicsekParticle2::rc, particle.h:250 */
  p->mu = 0.5;                    /* m_parallel = m_perpendicular for nb = 1, particle.h:861-863 */
  p->k_perp = 1.0;
  p->bond_rest = 1.0;
  p->integrator = SPP_INT_EULER;
  p->force_law = SPP_FORCE_NONE;
  p->align_mode = SPP_ALIGN_REFERENCE;
  /* RTPChain statics, particle.h:1106-1108 (used with SPP_NOISE_TUMBLE) */
  p->rot_noise = SPP_NOISE_GAUSSIAN;
  p->tumble_rate = 0.1;
  p->tumble_time = 10 * 0.1;
  p->tumble_torque = 1.0;
  /* walls: RepulsiveParticle's wall statics are never assigned in the
   * reference (particle.h:781-785: zero), ContinuousParticle::gw = 20
   * (particle.h:378) */
  p->boundary = SPP_BOUNDARY_PERIODIC;
  p->g_w_cont = 20.0;
  /* ActiveBrownianChain statics, particle.h:1049-1054 (used with chain_beads > 1) */
  p->chain_beads = 1;
  p->bead_separation = 1.0;
  p->sigma_chain = 1.0;
  p->r_chain = 1.1;
  switch (model) {
    case SPP_MODEL_ABP:           /* RepulsiveParticle statics, particle.h:774-786 */
      p->integrator = SPP_INT_RK2;
      p->force_law = SPP_FORCE_R12_TRUNC;
      p->k_rep = 2.0; p->sigma_rep = 1.0; p->r_align = 1.1; p->r_rep = 1.2;
      p->skin = 0.3;
      break;
    case SPP_MODEL_CONTINUOUS:    /* ContinuousParticle statics, particle.h:373-378 */
      p->g = 4.0; p->alpha = 0.5; p->skin = 0.3;
      break;
    case SPP_MODEL_BEADS:         /* ActiveBrownianChain statics, particle.h:1049-1056 */
      p->integrator = SPP_INT_RK2;
      p->force_law = SPP_FORCE_R12_TRUNC;
      p->k_rep = 1.0; p->sigma_rep = 0.5; p->r_rep = 0.55; p->skin = 0.3;
      break;
    case SPP_MODEL_VICSEK:
    case SPP_MODEL_VICSEK_REF_ANGLE:
    case SPP_MODEL_VICSEK_REF_VECTOR:
      break;
    default:
      return fail(SPP_ERR_UNSUPPORTED, "unknown model");
  }
  return SPP_OK;
}

int spp_chain_mobility(int nb, double separation, double sigma, double* out3) {
  if (!out3) return fail(SPP_ERR_INVALID, "out is NULL");
  if (nb < 1 || nb > SPP_MAX_CHAIN_BEADS) return fail(SPP_ERR_INVALID, "nb must be 1 .. SPP_MAX_CHAIN_BEADS");
  if (nb > 1 && (!(separation > 0) || !(sigma > 0)))
    return fail(SPP_ERR_INVALID, "separation and sigma must be > 0");
  spp_chain_mobility_d(nb, separation, sigma, out3);
  return SPP_OK;
}

int spp_create(const SppParams* p, SppSystem** out) {
  if (!out) return fail(SPP_ERR_INVALID, "out is NULL");
  *out = nullptr;
  int rc = validate(p);
  if (rc != SPP_OK) return rc;
  SppSystem* s = new SppSystem();
  s->p = *p;
  spp_consts_from_params(&s->k, p);
  prepare_abp_stage();
  s->uses_list = (p->model == SPP_MODEL_ABP || p->model == SPP_MODEL_CONTINUOUS ||
                  p->model == SPP_MODEL_BEADS);
  s->nstages = p->integrator == SPP_INT_RK4 ? 4 : (p->integrator == SPP_INT_RK2 ? 2 : 1);
  if (!s->uses_list) s->nstages = 1;
  const char* env = getenv("SPP_NO_GRAPHS");
  s->use_graphs = !(env && env[0] == '1');
  double rcell = s->uses_list ? (double)interaction_radius(*p) + p->skin : interaction_radius(*p);
  int D = (int)std::floor(2.0 * p->L / (rcell * 1.001));
  if (D < 3) {
    delete s;
    return fail(SPP_ERR_INVALID, "box too small for the cell list: 2L / r_cell < 3");
  }
  if (D > 65535) {
    delete s;
    return fail(SPP_ERR_INVALID, "too many cells per side (> 65535)");
  }
  int bits = 0;
  while ((1 << bits) < D) ++bits;
  DevState& d = s->d;
  memset(&d, 0, sizeof(d));
  d.n = p->n;
  d.D = D;
  d.morton_bits = bits;
  d.n_keys = 1u << (2 * bits);
  {
    const char* sv = getenv("SPP_VICSEK_SMALL");
    s->small_vicsek = !s->uses_list && !(sv && sv[0] == '0') && vicsek_small_fits(s->k, d);
  }
  int cap = p->list_capacity > 0 ? p->list_capacity : list_capacity_for(*p, rcell);
  if (!s->uses_list) cap = 0;
  size_t n = (size_t)p->n;
  uint32_t nscan = (d.n_keys + 4095) / 4096;
  if (nscan > 4096) {
    delete s;
    return fail(SPP_ERR_INVALID, "cell grid too large for the scan");
  }
  rc = SPP_OK;
  rc = rc ? rc : dalloc(&d.pos, n);
  rc = rc ? rc : dalloc(&d.half, s->uses_list ? n : 1);
  rc = rc ? rc : dalloc(&d.half2, s->nstages > 2 ? n : 1);
  rc = rc ? rc : dalloc(&d.theta, n);
  rc = rc ? rc : dalloc(&d.img, n);
  rc = rc ? rc : dalloc(&d.id, n);
  if (p->model == SPP_MODEL_BEADS) rc = rc ? rc : dalloc(&d.inv, n);
  if (s->k.tumble) rc = rc ? rc : dalloc(&d.tumble, n);
  rc = rc ? rc : dalloc(&d.kacc, s->nstages > 2 ? n : 1);
  rc = rc ? rc : dalloc(&d.dth, s->nstages > 1 ? n : 1);
  rc = rc ? rc : dalloc(&d.ref, n);
  rc = rc ? rc : dalloc(&d.pos_alt, n);
  rc = rc ? rc : dalloc(&d.theta_alt, n);
  rc = rc ? rc : dalloc(&d.img_alt, n);
  rc = rc ? rc : dalloc(&d.id_alt, n);
  rc = rc ? rc : dalloc(&d.key, n);
  rc = rc ? rc : dalloc(&d.rank, n);
  rc = rc ? rc : dalloc(&d.cell_count, d.n_keys);
  rc = rc ? rc : dalloc(&d.cell_start, d.n_keys);
  rc = rc ? rc : dalloc(&d.scan_tmp, nscan);
  rc = rc ? rc : dalloc(&d.nn, n);
  rc = rc ? rc : dalloc(&d.long_q, n);
  if (s->k.lanes > 1) rc = rc ? rc : dalloc(&d.nn_lanes, n);
  rc = rc ? rc : dalloc(&d.ctl, 1);
  rc = rc ? rc : dalloc(&d.red, 4);
  rc = rc ? rc : dalloc(&s->stage_x, n);
  rc = rc ? rc : dalloc(&s->stage_y, n);
  rc = rc ? rc : dalloc(&s->stage_t, n);
  rc = rc ? rc : dalloc(&s->stage_img, n);
  if (rc == SPP_OK && s->uses_list) rc = alloc_list(s, cap);
  if (rc != SPP_OK) {
    free_dev(s);
    delete s;
    return rc;
  }
  cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMemset(d.ctl, 0, sizeof(Ctl));
  if (e != cudaSuccess) {
    free_dev(s);
    delete s;
    return fail(SPP_ERR_CUDA, std::string("stream/ctl setup: ") + cudaGetErrorString(e));
  }
  s->own_stream = true;
  s->per_rebuild_kernels = 7;   /* bin_count, scan x3, scatter, build_list, sort_long */
  s->per_step_kernels = s->uses_list ? (s->nstages == 1 ? 2 : s->nstages) : 6;
  *out = s;
  return SPP_OK;
}

int spp_destroy(SppSystem* s) {
  if (!s) return SPP_OK;
  if (s->stream) cudaStreamSynchronize(s->stream);
  free_graphs(s);
  free_lyap(s);
  free_dev(s);
  if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
  if (s->side) cudaStreamDestroy(s->side);
  if (s->tan_stream) cudaStreamDestroy(s->tan_stream);
  if (s->ev_fork) cudaEventDestroy(s->ev_fork);
  if (s->ev_join) cudaEventDestroy(s->ev_join);
  delete s;
  return SPP_OK;
}

int spp_set_stream(SppSystem* s, void* stream) {
  if (!s) return fail(SPP_ERR_INVALID, "system is NULL");
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  free_graphs(s);
  if (s->own_stream) cudaStreamDestroy(s->stream);
  if (stream) {
    s->stream = (cudaStream_t)stream;
    s->own_stream = false;
  } else {
    CUDA_TRY(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    s->own_stream = true;
  }
  return SPP_OK;
}

int spp_upload_state(SppSystem* s, const float* x, const float* y, const float* theta,
                     const int32_t* img_x, const int32_t* img_y, int n, int64_t step0) {
  if (!s || !x || !y || !theta) return fail(SPP_ERR_INVALID, "NULL argument");
  if (n != s->p.n) return fail(SPP_ERR_INVALID, "n differs from the system's particle count");
  if (step0 < 0 || step0 > 0xffffffffLL) return fail(SPP_ERR_INVALID, "step0 out of range");
  /* the inputs are checked on the device, where they are placed
   * (k_init_state); the upload is refused, and the system left without a
   * state, if any value is non-finite or any position lies outside [-L, L) */
  s->uploaded = false;
  size_t bytes = sizeof(float) * (size_t)n;
  CUDA_TRY(cudaMemcpyAsync(s->stage_x, x, bytes, cudaMemcpyHostToDevice, s->stream));
  CUDA_TRY(cudaMemcpyAsync(s->stage_y, y, bytes, cudaMemcpyHostToDevice, s->stream));
  CUDA_TRY(cudaMemcpyAsync(s->stage_t, theta, bytes, cudaMemcpyHostToDevice, s->stream));
  int32_t* img_dev = nullptr;
  if (img_x || img_y) {
    img_dev = reinterpret_cast<int32_t*>(s->stage_img);  /* 2n int32: x counters, then y counters */
    if (img_x) CUDA_TRY(cudaMemcpyAsync(img_dev, img_x, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s->stream));
    else CUDA_TRY(cudaMemsetAsync(img_dev, 0, sizeof(int32_t) * n, s->stream));
    if (img_y) CUDA_TRY(cudaMemcpyAsync(img_dev + n, img_y, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s->stream));
    else CUDA_TRY(cudaMemsetAsync(img_dev + n, 0, sizeof(int32_t) * n, s->stream));
  }
  Ctl c;
  memset(&c, 0, sizeof(c));
  c.step = (uint32_t)step0;
  c.bad_nonfinite = 0xffffffffu;
  c.bad_range = 0xffffffffu;
  CUDA_TRY(cudaMemcpyAsync(s->d.ctl, &c, sizeof(Ctl), cudaMemcpyHostToDevice, s->stream));
  /* every swimmer starts running (RTPChain::RTPChain, particle.h:1078-1083) */
  if (s->d.tumble) CUDA_TRY(cudaMemsetAsync(s->d.tumble, 0, sizeof(int32_t) * (size_t)n, s->stream));
  launch_init_state(s->k, s->d, s->stage_x, s->stage_y, s->stage_t, img_dev, s->stream);
  s->host_launches++;
  int rc = enqueue_rebuild(s, s->stream, &s->host_launches);
  if (rc != SPP_OK) return rc;
  s->direct_rebuilds++;
  rc = read_ctl(s, &c);
  if (rc != SPP_OK) return rc;
  if (c.bad_nonfinite != 0xffffffffu)
    return fail(SPP_ERR_NUMERIC, "non-finite input at particle " + std::to_string(c.bad_nonfinite));
  if (c.bad_range != 0xffffffffu)
    return fail(SPP_ERR_INVALID, "position outside [-L, L) at particle " + std::to_string(c.bad_range));
  s->step0 = step0;
  s->target_step = step0;
  s->uploaded = true;
  s->mark_step = -1;   /* a new state: no frame marked */
  return recover(s);
}

int spp_download_state(SppSystem* s, float* x, float* y, float* theta, int32_t* img_x,
                       int32_t* img_y, int n) {
  if (!s || !x || !y || !theta) return fail(SPP_ERR_INVALID, "NULL argument");
  if (n != s->p.n) return fail(SPP_ERR_INVALID, "n differs from the system's particle count");
  if (!s->uploaded) return fail(SPP_ERR_INVALID, "no state uploaded");
  int rc = spp_sync(s);
  if (rc != SPP_OK) return rc;
  int32_t* img_dev = reinterpret_cast<int32_t*>(s->stage_img);  /* 2n int32: x, then y */
  launch_gather_state(s->k, s->d, s->stage_x, s->stage_y, s->stage_t, img_dev, s->stream);
  s->host_launches++;
  size_t bytes = sizeof(float) * (size_t)n;
  CUDA_TRY(cudaMemcpyAsync(x, s->stage_x, bytes, cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaMemcpyAsync(y, s->stage_y, bytes, cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaMemcpyAsync(theta, s->stage_t, bytes, cudaMemcpyDeviceToHost, s->stream));
  if (img_x) CUDA_TRY(cudaMemcpyAsync(img_x, img_dev, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s->stream));
  if (img_y) CUDA_TRY(cudaMemcpyAsync(img_y, img_dev + n, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return SPP_OK;
}

int spp_download_tumble(SppSystem* s, int32_t* state, int n) {
  if (!s || !state) return fail(SPP_ERR_INVALID, "NULL argument");
  if (n != s->p.n) return fail(SPP_ERR_INVALID, "n differs from the system's particle count");
  if (!s->uploaded) return fail(SPP_ERR_INVALID, "no state uploaded");
  if (!s->d.tumble) return fail(SPP_ERR_INVALID, "the system has no run-and-tumble state "
                                                 "(rot_noise is not SPP_NOISE_TUMBLE)");
  int rc = spp_sync(s);
  if (rc != SPP_OK) return rc;
  CUDA_TRY(cudaMemcpyAsync(state, s->d.tumble, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost,
                           s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return SPP_OK;
}

int spp_upload_tumble(SppSystem* s, const int32_t* state, int n) {
  if (!s || !state) return fail(SPP_ERR_INVALID, "NULL argument");
  if (n != s->p.n) return fail(SPP_ERR_INVALID, "n differs from the system's particle count");
  if (!s->uploaded) return fail(SPP_ERR_INVALID, "upload the state (spp_upload_state) first");
  if (!s->d.tumble) return fail(SPP_ERR_INVALID, "the system has no run-and-tumble state "
                                                 "(rot_noise is not SPP_NOISE_TUMBLE)");
  /* 0 (running) or +-c with 1 <= c <= the tumble length in steps; membrane
   * beads never tumble */
  const int32_t cmax = s->k.tumble_steps;
  for (int i = 0; i < n; ++i) {
    const int32_t v = state[i];
    if (v < -cmax || v > cmax || (v != 0 && i < s->k.n_beads))
      return fail(SPP_ERR_INVALID, "tumble state of particle " + std::to_string(i) + " out of range");
  }
  int rc = spp_sync(s);
  if (rc != SPP_OK) return rc;
  CUDA_TRY(cudaMemcpyAsync(s->d.tumble, state, sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice,
                           s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return SPP_OK;
}

int spp_step(SppSystem* s, int nsteps) {
  if (!s) return fail(SPP_ERR_INVALID, "system is NULL");
  if (nsteps < 0) return fail(SPP_ERR_INVALID, "nsteps < 0");
  if (!s->uploaded) return fail(SPP_ERR_INVALID, "no state uploaded");
  if (s->target_step + nsteps > 0xffffffffLL) return fail(SPP_ERR_INVALID, "step counter overflow");
  s->target_step += nsteps;
  return run_steps(s, nsteps);
}

int spp_sync(SppSystem* s) {
  if (!s) return fail(SPP_ERR_INVALID, "system is NULL");
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  CUDA_TRY(cudaGetLastError());
  return recover(s);
}

int spp_observables(SppSystem* s, SppObservables* o) {
  if (!s || !o) return fail(SPP_ERR_INVALID, "NULL argument");
  int rc = spp_sync(s);
  if (rc != SPP_OK) return rc;
  CUDA_TRY(cudaMemsetAsync(s->d.red, 0, 2 * sizeof(double), s->stream));
  launch_polarization(s->d, s->stream);
  s->host_launches++;
  long long sums[2];
  CUDA_TRY(cudaMemcpyAsync(sums, s->d.red, sizeof(sums), cudaMemcpyDeviceToHost, s->stream));
  Ctl c;
  CUDA_TRY(cudaMemcpyAsync(&c, s->d.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  const double inv = 1.0 / 134217728.0; /* fixed-point units of 2^-27 */
  memset(o, 0, sizeof(*o));
  o->step = (int64_t)c.step - s->step0;
  o->t = (double)o->step * s->p.dt;
  o->px = (double)sums[0] * inv / s->p.n;
  o->py = (double)sums[1] * inv / s->p.n;
  o->polarization = std::sqrt(o->px * o->px + o->py * o->py);
  o->n_rebuilds = c.n_rebuilds;
  o->n = s->p.n;
  o->list_capacity = s->d.cap;
  o->max_neighbors = (int32_t)c.max_nn;
  o->cells_per_side = s->d.D;
  o->late_rebuilds = c.late_rebuilds;
  o->list_regrowths = s->regrowths;
  o->bulk_timeouts = c.bulk_timeouts;
  return SPP_OK;
}

int spp_pairs(SppSystem* s, double r, int32_t* pi, int32_t* pj, int cap, int64_t* n_pairs) {
  if (!s || !n_pairs || (cap > 0 && (!pi || !pj))) return fail(SPP_ERR_INVALID, "NULL argument");
  if (!s->uploaded) return fail(SPP_ERR_INVALID, "no state uploaded");
  double width = 2.0 * s->p.L / s->d.D;
  if (!(r > 0) || r > width) return fail(SPP_ERR_INVALID, "r must be in (0, cell width]");
  int rc = spp_sync(s);
  if (rc != SPP_OK) return rc;
  rc = enqueue_rebuild(s, s->stream, &s->host_launches);  /* bin the current positions */
  if (rc != SPP_OK) return rc;
  s->direct_rebuilds++;
  unsigned long long* counter = nullptr;
  int32_t *dpi = nullptr, *dpj = nullptr;
  rc = dalloc(&counter, 1);
  if (rc == SPP_OK) rc = dalloc(&dpi, cap > 0 ? cap : 1);
  if (rc == SPP_OK) rc = dalloc(&dpj, cap > 0 ? cap : 1);
  if (rc == SPP_OK) {
    cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s->stream);
    launch_pairs_count(s->k, s->d, (float)(r * r), counter, dpi, dpj, cap, s->stream);
    s->host_launches++;
    unsigned long long total = 0;
    cudaMemcpyAsync(&total, counter, sizeof(total), cudaMemcpyDeviceToHost, s->stream);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess && cap > 0) {
      size_t m = total < (unsigned long long)cap ? (size_t)total : (size_t)cap;
      e = cudaMemcpy(pi, dpi, m * sizeof(int32_t), cudaMemcpyDeviceToHost);
      if (e == cudaSuccess) e = cudaMemcpy(pj, dpj, m * sizeof(int32_t), cudaMemcpyDeviceToHost);
    }
    if (e != cudaSuccess) rc = fail(SPP_ERR_CUDA, std::string("pairs: ") + cudaGetErrorString(e));
    *n_pairs = (int64_t)total;
  }
  if (counter) cudaFree(counter);
  if (dpi) cudaFree(dpi);
  if (dpj) cudaFree(dpj);
  return rc;
}

int spp_cells(SppSystem* s, int D, int rule, int32_t* cell_x, int32_t* cell_y, int n) {
  if (!s || !cell_x || !cell_y) return fail(SPP_ERR_INVALID, "NULL argument");
  if (n != s->p.n || D < 1 || (rule != SPP_BIN_GEOMETRIC && rule != SPP_BIN_REFERENCE))
    return fail(SPP_ERR_INVALID, "bad n, D or rule");
  if (!s->uploaded) return fail(SPP_ERR_INVALID, "no state uploaded");
  int rc = spp_sync(s);
  if (rc != SPP_OK) return rc;
  int32_t *dx = nullptr, *dy = nullptr;
  rc = dalloc(&dx, (size_t)n);
  if (rc == SPP_OK) rc = dalloc(&dy, (size_t)n);
  if (rc == SPP_OK) {
    launch_cells(s->k, s->d, D, rule, dx, dy, s->stream);
    s->host_launches++;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) e = cudaMemcpy(cell_x, dx, sizeof(int32_t) * n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(cell_y, dy, sizeof(int32_t) * n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = fail(SPP_ERR_CUDA, std::string("cells: ") + cudaGetErrorString(e));
  }
  if (dx) cudaFree(dx);
  if (dy) cudaFree(dy);
  return rc;
}

int spp_profile(SppSystem* s, int nsteps, SppProfile* out) {
  if (!s || !out || nsteps < 0) return fail(SPP_ERR_INVALID, "bad argument");
  if (!s->uploaded) return fail(SPP_ERR_INVALID, "no state uploaded");
  int rc = spp_sync(s);
  if (rc != SPP_OK) return rc;
  memset(out, 0, sizeof(*out));
  const int per_step = s->uses_list ? s->nstages : 1;
  const int nev = 2 * (nsteps * per_step + nsteps) + 2;
  std::vector<cudaEvent_t> ev;
  ev.reserve((size_t)nev);
  auto mk = [&]() -> cudaEvent_t {
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    ev.push_back(e);
    return e;
  };
  struct Span { cudaEvent_t a, b; int kind; };
  std::vector<Span> spans;
  cudaEvent_t first = mk();
  CUDA_TRY(cudaEventRecord(first, s->stream));
  for (int i = 0; i < nsteps && rc == SPP_OK; ++i) {
    if (s->uses_list) {
      for (int stage = 0; stage < s->nstages; ++stage) {
        cudaEvent_t a = mk(), b = mk();
        cudaEventRecord(a, s->stream);
        launch_abp_stage(s->k, s->d, stage, s->nstages, 0, 0, s->stream, &s->host_launches);
        cudaEventRecord(b, s->stream);
        spans.push_back({a, b, 0});
      }
      Ctl c;
      rc = read_ctl(s, &c);
      if (rc == SPP_OK && c.need_rebuild) {
        cudaEvent_t a = mk(), b = mk();
        cudaEventRecord(a, s->stream);
        rc = enqueue_rebuild(s, s->stream, &s->host_launches);
        cudaEventRecord(b, s->stream);
        spans.push_back({a, b, 1});
        s->direct_rebuilds++;
      }
    } else {
      cudaEvent_t a = mk(), b = mk();
      cudaEventRecord(a, s->stream);
      rc = enqueue_step(s, s->stream, false, &s->host_launches);
      cudaEventRecord(b, s->stream);
      spans.push_back({a, b, 0});
    }
    s->target_step += 1;
  }
  cudaEvent_t last = mk();
  cudaEventRecord(last, s->stream);
  cudaError_t e = cudaStreamSynchronize(s->stream);
  if (rc == SPP_OK && e != cudaSuccess) rc = fail(SPP_ERR_CUDA, cudaGetErrorString(e));
  if (rc == SPP_OK) {
    for (auto& sp : spans) {
      float ms = 0;
      cudaEventElapsedTime(&ms, sp.a, sp.b);
      if (sp.kind == 0) { out->stage_ms += ms; out->stage_launches++; }
      else { out->rebuild_ms += ms; out->rebuilds++; }
    }
    float tot = 0;
    cudaEventElapsedTime(&tot, first, last);
    out->total_ms = tot;
    out->steps = nsteps;
  }
  for (auto x : ev) cudaEventDestroy(x);
  return rc;
}

int spp_lyap_init(SppSystem* s, int K, uint64_t seed) {
  if (!s) return fail(SPP_ERR_INVALID, "system is NULL");
  if (!s->uploaded) return fail(SPP_ERR_INVALID, "no state uploaded");
  if (K < 1 || K > SPP_LYAP_MAX) return fail(SPP_ERR_INVALID, "need 1 <= K <= 8 tangent vectors");
  if (s->p.model != SPP_MODEL_CONTINUOUS || s->p.alpha != 0.0 || s->p.force_law != SPP_FORCE_NONE ||
      s->p.boundary != SPP_BOUNDARY_PERIODIC)
    return fail(SPP_ERR_UNSUPPORTED,
                "the tangent dynamics is built for the periodic continuous model with alpha = 0 and no repulsion");
  if (s->nstages < 2) return fail(SPP_ERR_UNSUPPORTED, "tangent dynamics needs RK2 or RK4");
  int rc = spp_sync(s);
  if (rc != SPP_OK) return rc;
  free_lyap(s);
  LyapState& L = s->lyap;
  L.K = K;
  L.n = s->p.n;
  size_t len = (size_t)K * 3 * s->p.n;
  rc = dalloc(&L.t0, len);
  rc = rc ? rc : dalloc(&L.ua, len);
  rc = rc ? rc : dalloc(&L.ub, len);
  rc = rc ? rc : dalloc(&L.acc, len);
  rc = rc ? rc : dalloc(&L.uslot, 2 * tangent_slot_floats(K, s->p.n));
  rc = rc ? rc : dalloc(&L.partial, (size_t)SPP_GRAM_BLOCKS * SPP_GRAM_ENTRIES);
  rc = rc ? rc : dalloc(&L.rinv, (size_t)SPP_LYAP_MAX * SPP_LYAP_MAX);
  rc = rc ? rc : dalloc(&L.log_stretch, SPP_LYAP_MAX);
  rc = rc ? rc : dalloc(&L.error, 1);
  if (rc != SPP_OK) { free_lyap(s); return rc; }
  CUDA_TRY(cudaMemsetAsync(L.log_stretch, 0, sizeof(double) * SPP_LYAP_MAX, s->stream));
  CUDA_TRY(cudaMemsetAsync(L.error, 0, sizeof(uint32_t), s->stream));
  CUDA_TRY(cudaMemsetAsync(L.uslot, 0, 2 * sizeof(float) * tangent_slot_floats(K, s->p.n), s->stream));
  launch_tangent_init(L, seed, s->p.system_id, s->stream);
  launch_renormalize(L, 0, s->stream, &s->host_launches);
  s->host_launches += 1;
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  uint32_t err = 0;
  CUDA_TRY(cudaMemcpy(&err, L.error, sizeof(err), cudaMemcpyDeviceToHost));
  if (err) { free_lyap(s); return fail(SPP_ERR_NUMERIC, "initial tangent vectors are dependent"); }
  if (!s->tan_stream) {
    /* all three or none: without them the tangent stages run on the base stream */
    cudaStream_t ts = nullptr;
    cudaEvent_t ef = nullptr, ej = nullptr;
    if (cudaStreamCreateWithFlags(&ts, cudaStreamNonBlocking) == cudaSuccess &&
        cudaEventCreateWithFlags(&ef, cudaEventDisableTiming) == cudaSuccess &&
        cudaEventCreateWithFlags(&ej, cudaEventDisableTiming) == cudaSuccess) {
      s->tan_stream = ts;
      s->ev_fork = ef;
      s->ev_join = ej;
    } else {
      cudaGetLastError();
      if (ts) cudaStreamDestroy(ts);
      if (ef) cudaEventDestroy(ef);
      if (ej) cudaEventDestroy(ej);
    }
  }
  s->lyap_on = true;
  s->lyap_steps = 0;
  return SPP_OK;
}

int spp_lyap_set_vectors(SppSystem* s, const float* v, int K) {
  if (!s || !v) return fail(SPP_ERR_INVALID, "NULL argument");
  if (!s->lyap_on || K != s->lyap.K) return fail(SPP_ERR_INVALID, "spp_lyap_init with this K first");
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  CUDA_TRY(cudaMemcpy(s->lyap.t0, v, sizeof(float) * (size_t)K * 3 * s->p.n, cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemset(s->lyap.log_stretch, 0, sizeof(double) * SPP_LYAP_MAX));
  s->lyap_steps = 0;
  return SPP_OK;
}

int spp_lyap_step(SppSystem* s, int nsteps, int renorm_every) {
  if (!s) return fail(SPP_ERR_INVALID, "system is NULL");
  if (!s->lyap_on) return fail(SPP_ERR_INVALID, "spp_lyap_init first");
  if (nsteps < 0 || renorm_every < 1) return fail(SPP_ERR_INVALID, "need nsteps >= 0, renorm_every >= 1");
  s->target_step += nsteps;
  s->lyap_renorm_every = renorm_every;
  s->lyap_steps += nsteps;
  if (!s->use_graphs) {
    int rc = run_lyap_direct(s, nsteps);
    return rc != SPP_OK ? rc : recover(s);
  }
  return launch_lyap_chunks(s, nsteps);
}

int spp_lyap_exponents(SppSystem* s, double* lambda, int K, double* elapsed) {
  if (!s || !lambda) return fail(SPP_ERR_INVALID, "NULL argument");
  if (!s->lyap_on || K > s->lyap.K) return fail(SPP_ERR_INVALID, "spp_lyap_init first / K too large");
  int rc = spp_sync(s);
  if (rc != SPP_OK) return rc;
  Ctl c;
  rc = read_ctl(s, &c);
  if (rc != SPP_OK) return rc;
  (void)c;
  double ls[SPP_LYAP_MAX];
  uint32_t err = 0;
  CUDA_TRY(cudaMemcpy(ls, s->lyap.log_stretch, sizeof(ls), cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(&err, s->lyap.error, sizeof(err), cudaMemcpyDeviceToHost));
  if (err) return fail(SPP_ERR_NUMERIC, "tangent vectors became dependent");
  const double T = (double)s->lyap_steps * s->p.dt;
  for (int a = 0; a < K; ++a) lambda[a] = T > 0 ? ls[a] / T : 0.0;
  if (elapsed) *elapsed = T;
  return SPP_OK;
}

int spp_lyap_vectors(SppSystem* s, float* v, int K) {
  if (!s || !v) return fail(SPP_ERR_INVALID, "NULL argument");
  if (!s->lyap_on || K != s->lyap.K) return fail(SPP_ERR_INVALID, "spp_lyap_init with this K first");
  int rc = spp_sync(s);
  if (rc != SPP_OK) return rc;
  CUDA_TRY(cudaMemcpy(v, s->lyap.t0, sizeof(float) * (size_t)K * 3 * s->p.n, cudaMemcpyDeviceToHost));
  return SPP_OK;
}

int spp_time_steps(SppSystem* s, int nsteps, double* ms) {
  if (!s || !ms) return fail(SPP_ERR_INVALID, "NULL argument");
  cudaEvent_t a, b;
  CUDA_TRY(cudaEventCreate(&a));
  CUDA_TRY(cudaEventCreate(&b));
  cudaEventRecord(a, s->stream);
  int rc = spp_step(s, nsteps);
  /* A list overflow freezes the stage kernels; recover() then regrows the
   * list and runs the skipped steps.  The end event follows that recovery,
   * so every requested step lies inside the timed interval. */
  if (rc == SPP_OK) rc = spp_sync(s);
  cudaEventRecord(b, s->stream);
  cudaError_t e = cudaEventSynchronize(b);
  float t = 0;
  if (rc == SPP_OK && e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc != SPP_OK) return rc;
  if (e != cudaSuccess) return fail(SPP_ERR_CUDA, cudaGetErrorString(e));
  *ms = t;
  return SPP_OK;
}

int64_t spp_kernel_launches(SppSystem* s) {
  if (!s) return 0;
  Ctl c;
  if (read_ctl(s, &c) != SPP_OK) return -1;
  int64_t graph_rebuilds = (int64_t)c.n_rebuilds - s->direct_rebuilds;
  if (graph_rebuilds < 0) graph_rebuilds = 0;
  return s->host_launches + s->graph_kernels + graph_rebuilds * s->per_rebuild_kernels;
}

void* spp_stream(SppSystem* s) { return s ? (void*)s->stream : nullptr; }

}  // extern "C"
