/*
 * batch.cu -- many independent Vicsek systems in one set of launches.
 *
 * The reference runs a parameter sweep as a task farm: serial/mpi-main.cpp:
 * 157-176 hands noise values round-robin to MPI ranks, each rank running
 * whole independent boxes one after another.  Here every system of the
 * sweep lives in one set of device arrays, indexed by a per-system offset
 * table (particle range, cell range, constants, activity, step count), and
 * each phase of a step is ONE launch over all particles of all systems:
 *   zero counts | k_batch_bin | scan (global) | k_batch_scatter |
 *   k_batch_step | k_batch_finish
 * Small systems (1k particles) that alone could not fill the GPU share it
 * with the large ones; the step loop is captured in CUDA graphs.  Retired or
 * finished systems stay in place and are copied through without work.
 *
 * Per-system observables are accumulated on the device every step: the
 * polarization P = |sum (cos, sin)| / N (exact fixed-point sums), its first
 * four moments over a start-up window, and its mean over a stationary
 * window -- the inputs and targets of the sweep surrogate.
 */
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include "spp_internal.cuh"
#include "spp_batch.cuh"

namespace {

/* Compact particle index t -> (system, slot). */
__device__ __forceinline__ int act_slot(const DevBatch& b, int t, int* s) {
  *s = (int)b.act_sys[t];
  return t + b.sact[*s].a_corr;
}

/* Keys are compact cell indices: a system's D x D row-major grid starts at
 * its a_coff, so the scan runs over the cells of active systems only and a
 * system's cell starts, plus its a_corr, are slots of its own particle range. */
__global__ void __launch_bounds__(SPP_BLOCK) k_batch_bin(DevBatch b) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= b.n_act) return;
  int s;
  const int i = act_slot(b, t, &s);
  const BatchSys& S = b.sys[s];
  const float4 p = b.pos[i];
  const int cx = spp_cell_coord(p.x, S.k.L, S.k.L2, (int)S.D, SPP_BIN_GEOMETRIC);
  const int cy = spp_cell_coord(p.y, S.k.L, S.k.L2, (int)S.D, SPP_BIN_GEOMETRIC);
  const uint32_t key = b.sact[s].a_coff + (uint32_t)cy * S.D + (uint32_t)cx;
  const unsigned mask = __activemask();
  const unsigned peers = __match_any_sync(mask, key);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(&b.cell_count[key], (uint32_t)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  b.key[t] = key;
  b.rank[t] = base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
}

/* Exact fixed-point parts (hi, lo) of a heading's cos and sin, split as the
 * alignment sums split every term (spp_fx_add).  The scatter computes them
 * once per particle and step, so the neighbour loop of the vector-sum rule
 * adds integers only; the sums, being exact, do not depend on the order in
 * which the candidates are visited. */
__device__ __forceinline__ int4 fx_parts(float c, float s) {
  spp_fx a = {0, 0}, b = {0, 0};
  spp_fx_add(&a, c);
  spp_fx_add(&b, s);
  return make_int4(a.hi, a.lo, b.hi, b.lo);
}

__global__ void __launch_bounds__(SPP_BLOCK) k_batch_scatter(DevBatch b) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= b.n_act) return;
  int s;
  const int i = act_slot(b, t, &s);
  const uint32_t dst = b.cell_start[b.key[t]] + b.rank[t] + (uint32_t)b.sact[s].a_corr;
  const float4 p = b.pos[i];
  b.pos_alt[dst] = p;
  b.fx_alt[dst] = fx_parts(p.z, p.w);
  b.theta_alt[dst] = b.theta[i];
  b.img_alt[dst] = b.img[i];
  b.id_alt[dst] = b.id[i];
}

#ifndef SPP_BATCH_UNROLL
#define SPP_BATCH_UNROLL 2       /* candidates whose loads are issued together */
#endif
#ifndef SPP_BATCH_MIN_BLOCKS
#define SPP_BATCH_MIN_BLOCKS 6   /* resident 256-thread blocks per SM the step kernel is built for */
#endif

/* Models of the batch step kernel: one rule for all systems of the batch
 * (the common case), or any mix (runtime dispatch per system). */
constexpr int BATCH_MIXED = -1;

/* One candidate j of particle i (cell-ordered slot i, position p); q and f
 * are candidate j's position record and fixed-point heading parts. */
template <int MODEL>
__device__ __forceinline__ void visit(const DevBatch& b, const SppConsts& k, int interior, float4 p, int i,
                                      uint32_t j, float4 q, int4 f, SppAcc* a) {
  const int model = MODEL == BATCH_MIXED ? k.model : MODEL;
  if (model == SPP_MODEL_VICSEK) {
    float dx, dy, d2;
    if (interior) {
      dx = p.x - q.x;
      dy = p.y - q.y;
      d2 = fmaf(dx, dx, dy * dy);
    } else {
      d2 = spp_sep(&k, p.x, p.y, q.x, q.y, &dx, &dy);
    }
    if (d2 < k.ral2) {
      a->ax.hi += f.x;
      a->ax.lo += f.y;
      a->ay.hi += f.z;
      a->ay.lo += f.w;
      a->cnt += 1;
    }
  } else {
    const float thj = model == SPP_MODEL_VICSEK_REF_ANGLE ? b.theta_alt[j] : 0.0f;
    spp_pair_vicsek(&k, a, p.x, p.y, q.x, q.y, q.z, q.w, thj, (int)j == i);
  }
}

/* Walks a lane's candidate sequence t = 0 .. T-1 (T the warp's longest):
 * segments of lengths l0, l01 - l0, lt - l01 starting at slots m0, m1 + l0,
 * m2 + l01; SPP_BATCH_UNROLL candidates per trip with their loads first. */
template <int MODEL>
__device__ __forceinline__ void walk(const DevBatch& b, const SppConsts& k, int interior, float4 p, int i, int T,
                                     int lt, int l0, int l01, uint32_t m0, uint32_t m1, uint32_t m2,
                                     SppAcc* a) {
  const int vec = MODEL == BATCH_MIXED ? (k.model == SPP_MODEL_VICSEK) : (MODEL == SPP_MODEL_VICSEK);
  for (int t0 = 0; t0 < T; t0 += SPP_BATCH_UNROLL) {
    float4 q[SPP_BATCH_UNROLL];
    int4 f[SPP_BATCH_UNROLL];
    uint32_t j[SPP_BATCH_UNROLL];
#pragma unroll
    for (int u = 0; u < SPP_BATCH_UNROLL; ++u) {
      const int t = t0 + u;
      j[u] = (uint32_t)t + (t < l0 ? m0 : (t < l01 ? m1 : m2));
      q[u] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      f[u] = make_int4(0, 0, 0, 0);
      if (t < lt) {
        if (MODEL == SPP_MODEL_VICSEK) {  /* the vector rule needs the position only */
          const float2 xy = __ldg(reinterpret_cast<const float2*>(b.pos_alt + j[u]));
          q[u] = make_float4(xy.x, xy.y, 0.0f, 0.0f);
        } else {
          q[u] = __ldg(b.pos_alt + j[u]);
        }
        if (vec) f[u] = __ldg(b.fx_alt + j[u]);
      }
    }
#pragma unroll
    for (int u = 0; u < SPP_BATCH_UNROLL; ++u)
      if (t0 + u < lt) visit<MODEL>(b, k, interior, p, i, j[u], q[u], f[u], a);
  }
}

/* Segments of the candidate sequence of a particle in cell (cx, cy): for each
 * of the rows cy-1, cy, cy+1 the columns [cx-1, cx+1] clipped to the grid
 * (wrap = 0), or the one column the periodic wrap adds (wrap = 1: column D-1
 * for cx = 0, column 0 for cx = D-1, none otherwise). */
__device__ __forceinline__ void segments(const DevBatch& b, const BatchSys* S, SysAct A, int cx, int cy,
                                         int wrap, uint32_t* m0, uint32_t* m1, uint32_t* m2, int* l0, int* l01,
                                         int* lt) {
  const int D = (int)S->D;
  int ca, cb;
  if (!wrap) {
    ca = cx > 0 ? cx - 1 : 0;
    cb = cx < D - 1 ? cx + 1 : D - 1;
  } else {
    ca = cb = cx == 0 ? D - 1 : 0;
  }
  const int none = wrap && cx != 0 && cx != D - 1;
  uint32_t lo[3], hi[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    int ny = cy + r - 1;
    ny = ny < 0 ? ny + D : (ny >= D ? ny - D : ny);
    const uint32_t row = A.a_coff + (uint32_t)ny * (uint32_t)D;
    lo[r] = hi[r] = 0;
    if (!none) {
      lo[r] = b.cell_start[row + (uint32_t)ca] + (uint32_t)A.a_corr;
      hi[r] = b.cell_start[row + (uint32_t)cb] + b.cell_count[row + (uint32_t)cb] + (uint32_t)A.a_corr;
    }
  }
  *m0 = lo[0];
  *l0 = (int)(hi[0] - lo[0]);
  *l01 = *l0 + (int)(hi[1] - lo[1]);
  *lt = *l01 + (int)(hi[2] - lo[2]);
  *m1 = lo[1] - (uint32_t)*l0;   /* slot = t + m1 for l0 <= t < l01 (wraps as unsigned) */
  *m2 = lo[2] - (uint32_t)*l01;
}

/* One Vicsek step of every active system (VicsekParticle{,2}::Interact/Move,
 * shared/particle.h:145-247, or the arg-sum rule), from the cell-ordered
 * copy back into the primary arrays; per-system heading sums for P.
 *
 * Candidates: the 3x3 cells around a particle are, per grid row, one run of
 * consecutive keys (row-major keys), i.e. one contiguous range of the
 * cell-ordered arrays; a lane walks its three row ranges as one flattened
 * sequence, and the warp runs the longest lane's count, so lanes diverge only
 * in the length of their sequences.  The cell that the periodic wrap adds to
 * a row (a particle in the first or last column) is walked in a second pass,
 * entered only by warps that have such a lane.  A warp whose particles all
 * sit in interior cells (no wrap in any candidate) takes plain differences
 * instead of minimum images: for such pairs the two are the same number. */
template <int MODEL>
__global__ void __launch_bounds__(SPP_BLOCK, SPP_BATCH_MIN_BLOCKS) k_batch_step(DevBatch b) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  long long ux = 0, uy = 0;
  int s = -1, i = -1;
  int active = 0;
  const BatchSys* S = nullptr;
  SysAct A = {0u, 0};
  float4 p = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (t < b.n_act) {
    i = act_slot(b, t, &s);
    S = &b.sys[s];
    A = b.sact[s];
    active = (int)S->active;
    p = b.pos_alt[i];
  }
  int cx = 0, cy = 0, interior = 1, edge = 0;
  uint32_t m0 = 0, m1 = 0, m2 = 0;
  int l0 = 0, l01 = 0, lt = 0;
  if (active) {
    const int D = (int)S->D;
    cx = spp_cell_coord(p.x, S->k.L, S->k.L2, D, SPP_BIN_GEOMETRIC);
    cy = spp_cell_coord(p.y, S->k.L, S->k.L2, D, SPP_BIN_GEOMETRIC);
    /* |dx|, |dy| < 2 cell widths <= L for D >= 4: no image is ever nearer */
    interior = (D >= 4 && cx >= 1 && cx <= D - 2 && cy >= 1 && cy <= D - 2);
    edge = (cx == 0 || cx == D - 1);
    segments(b, S, A, cx, cy, 0, &m0, &m1, &m2, &l0, &l01, &lt);
  }
  const int all_interior = __all_sync(0xffffffffu, interior);
  const int any_edge = __any_sync(0xffffffffu, edge);
  const int T = (int)__reduce_max_sync(0xffffffffu, (unsigned)lt);
  SppAcc a;
  spp_acc_zero(&a);
  if (active) walk<MODEL>(b, S->k, all_interior, p, i, T, lt, l0, l01, m0, m1, m2, &a);
  if (any_edge) {
    lt = 0;
    if (active) segments(b, S, A, cx, cy, 1, &m0, &m1, &m2, &l0, &l01, &lt);
    const int WT = (int)__reduce_max_sync(0xffffffffu, (unsigned)lt);
    if (active) walk<MODEL>(b, S->k, 0, p, i, WT, lt, l0, l01, m0, m1, m2, &a);
  }
  if (active) {
    const SppConsts& k = S->k;
    if (a.ovf) atomicOr(&b.ctl->fx_overflow, 1u);
    const float th0 = b.theta_alt[i];
    const uint32_t id = b.id_alt[i];
    const spp_u32x4 r = spp_draw(k.seed, k.system, id, S->steps, SPP_RNG_VICSEK);
    float x, y, c, sn, t;
    int gx = 0, gy = 0;
    spp_vicsek_update(&k, &a, p.x, p.y, th0, p.z, p.w, r.v[0], &x, &y, &t, &c, &sn, &gx, &gy);
    const int2 g = b.img_alt[i];
    b.pos[i] = make_float4(x, y, c, sn);
    b.theta[i] = t;
    b.img[i] = make_int2(g.x + gx, g.y + gy);
    b.id[i] = id;
    spp_fx hx = {0, 0}, hy = {0, 0};
    spp_fx_add(&hx, c);
    spp_fx_add(&hy, sn);
    ux = spp_fx_units(hx);
    uy = spp_fx_units(hy);
  } else {
    if (i >= 0) {  /* finished since the compact space was built: copied through */
      b.pos[i] = p;
      b.theta[i] = b.theta_alt[i];
      b.img[i] = b.img_alt[i];
      b.id[i] = b.id_alt[i];
    }
    s = -1;  /* no contribution */
  }
  /* heading sums: one atomic per group of lanes of the same system (a tree
   * when the whole warp is one system, the common case) */
  const unsigned peers = __match_any_sync(0xffffffffu, s);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(peers) - 1;
  long long sx = ux, sy = uy;
  if (peers == 0xffffffffu) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sx += __shfl_down_sync(0xffffffffu, sx, o);
      sy += __shfl_down_sync(0xffffffffu, sy, o);
    }
  } else {
    for (int o = 1; o < 32; ++o) {
      const int src = (lane + o) & 31;
      const long long vx = __shfl_sync(0xffffffffu, ux, src);
      const long long vy = __shfl_sync(0xffffffffu, uy, src);
      if (lane == leader && ((peers >> src) & 1u)) { sx += vx; sy += vy; }
    }
  }
  if (lane == leader && s >= 0) {
    atomicAdd(reinterpret_cast<unsigned long long*>(&b.stats[s].sx), (unsigned long long)sx);
    atomicAdd(reinterpret_cast<unsigned long long*>(&b.stats[s].sy), (unsigned long long)sy);
  }
}

/* Per system: P of the step just taken, moment sums, step counter, and the
 * stop at max_steps. */
__global__ void k_batch_finish(DevBatch b) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= b.n_sys) return;
  BatchSys& S = b.sys[s];
  BatchStats& T = b.stats[s];
  if (!S.active) return;
  const double inv = 7.450580596923828125e-09;  /* 2^-27 */
  const double px = (double)T.sx * inv / S.n, py = (double)T.sy * inv / S.n;
  const double P = sqrt(px * px + py * py);
  T.sx = 0;
  T.sy = 0;
  const uint32_t t = S.steps + 1u;  /* steps completed after this one */
  if ((int)t <= b.window) {
    const double P2 = P * P;
    T.w1 += P;
    T.w2 += P2;
    T.w3 += P2 * P;
    T.w4 += P2 * P2;
  }
  if ((int)t > b.stationary_from) {
    T.s1 += P;
    T.s2 += P * P;
    T.s4 += (P * P) * (P * P);
    T.ns += 1;
  }
  T.p_last = P;
  S.steps = t;
  if (b.max_steps > 0 && (int)t >= b.max_steps) S.active = 0u;
}

__global__ void k_batch_flags(DevBatch b) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < b.n_sys) b.flags[s] = b.sys[s].active;
}

__global__ void k_batch_init(DevBatch b, const float* x, const float* y, const float* th) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.n_total) return;
  float s, c;
  spp_sincosf(th[i], &s, &c);
  b.pos[i] = make_float4(x[i], y[i], c, s);
  b.theta[i] = th[i];
  b.img[i] = make_int2(0, 0);
  b.id[i] = (uint32_t)i - b.sys[b.sys_of[i]].p_off;
}

__global__ void k_batch_gather(DevBatch b, float* x, float* y, float* th, int2* img) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b.n_total) return;
  const BatchSys& S = b.sys[b.sys_of[i]];
  const uint32_t dst = S.p_off + b.id[i];
  const float4 p = b.pos[i];
  x[dst] = p.x;
  y[dst] = p.y;
  th[dst] = b.theta[i];
  img[dst] = b.img[i];
}

__global__ void k_batch_set_active(DevBatch b, const int32_t* idx, int count, uint32_t value) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < count) {
    const int s = idx[q];
    if (s >= 0 && s < b.n_sys) {
      /* a system that reached max_steps stays finished */
      const int finished = b.max_steps > 0 && (int)b.sys[s].steps >= b.max_steps;
      b.sys[s].active = (value && !finished) ? 1u : 0u;
    }
  }
}

int bfail(int status, const std::string& m) {
  spp_internal_set_error(m.c_str());
  return status;
}

#define BCUDA(expr)                                                                     \
  do {                                                                                  \
    cudaError_t _e = (expr);                                                            \
    if (_e != cudaSuccess) return bfail(SPP_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

inline int nblocks(int n) { return (n + SPP_BLOCK - 1) / SPP_BLOCK; }

}  // namespace

struct SppBatch {
  DevBatch d;
  std::vector<BatchSys> host_sys;
  uint32_t n_keys = 0;
  cudaStream_t stream = nullptr;
  float *stage_x = nullptr, *stage_y = nullptr, *stage_t = nullptr;
  int2* stage_img = nullptr;
  std::vector<std::pair<int, cudaGraphExec_t>> graphs;
  std::vector<cudaGraph_t> graph_defs;
  int64_t launches = 0;
  bool uploaded = false;
  int model = -1;  /* the one model of all systems, or -1 for a mix */
  std::vector<uint32_t> act_flags;  /* the active set the compact launch space was built for */
  bool act_valid = false;
};

namespace {

template <class T>
int balloc(T** p, size_t count) {
  *p = nullptr;
  cudaError_t e = cudaMalloc((void**)p, (count ? count : 1) * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    return bfail(SPP_ERR_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  return SPP_OK;
}

void batch_free(SppBatch* b) {
  for (auto& g : b->graphs) cudaGraphExecDestroy(g.second);
  for (auto g : b->graph_defs) cudaGraphDestroy(g);
  b->graphs.clear();
  b->graph_defs.clear();
  DevBatch& d = b->d;
  void* ptrs[] = {d.sys, d.stats, d.sys_of, d.pos, d.pos_alt, d.theta, d.theta_alt, d.img,
                  d.img_alt, d.id, d.id_alt, d.key, d.rank, d.cell_count, d.cell_start, d.fx_alt,
                  d.scan_tmp, d.ctl, d.act_sys, d.sact, d.flags, b->stage_x, b->stage_y, b->stage_t,
                  b->stage_img};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  memset(&b->d, 0, sizeof(b->d));
  if (b->stream) cudaStreamDestroy(b->stream);
  b->stream = nullptr;
}

int enqueue_batch_step(SppBatch* b, cudaStream_t st) {
  const DevBatch& d = b->d;
  BCUDA(cudaMemsetAsync(d.cell_count, 0, sizeof(uint32_t) * (size_t)d.n_act_keys, st));
  const int nb = nblocks(d.n_act);
  k_batch_bin<<<nb, SPP_BLOCK, 0, st>>>(d);
  launch_scan_u32(d.cell_count, (uint32_t)d.n_act_keys, d.scan_tmp, d.cell_start, st, nullptr);
  k_batch_scatter<<<nb, SPP_BLOCK, 0, st>>>(d);
  switch (b->model) {
    case SPP_MODEL_VICSEK: k_batch_step<SPP_MODEL_VICSEK><<<nb, SPP_BLOCK, 0, st>>>(d); break;
    case SPP_MODEL_VICSEK_REF_ANGLE: k_batch_step<SPP_MODEL_VICSEK_REF_ANGLE><<<nb, SPP_BLOCK, 0, st>>>(d); break;
    case SPP_MODEL_VICSEK_REF_VECTOR: k_batch_step<SPP_MODEL_VICSEK_REF_VECTOR><<<nb, SPP_BLOCK, 0, st>>>(d); break;
    default: k_batch_step<BATCH_MIXED><<<nb, SPP_BLOCK, 0, st>>>(d); break;
  }
  k_batch_finish<<<nblocks(d.n_sys), SPP_BLOCK, 0, st>>>(d);
  BCUDA(cudaGetLastError());
  return SPP_OK;
}

constexpr int BATCH_GRAPH_CHUNK = 32;

void batch_drop_graphs(SppBatch* b) {
  for (auto& g : b->graphs) cudaGraphExecDestroy(g.second);
  for (auto g : b->graph_defs) cudaGraphDestroy(g);
  b->graphs.clear();
  b->graph_defs.clear();
}

/* Reads the active flags and, when the set of active systems changed since
 * the compact launch space was built, rebuilds it (and the step graphs,
 * whose launch sizes depend on it). */
int batch_refresh_active(SppBatch* b) {
  DevBatch& d = b->d;
  const int ns = d.n_sys;
  k_batch_flags<<<nblocks(ns), SPP_BLOCK, 0, b->stream>>>(d);
  b->launches += 1;
  std::vector<uint32_t> flags((size_t)ns);
  BCUDA(cudaMemcpyAsync(flags.data(), d.flags, sizeof(uint32_t) * ns, cudaMemcpyDeviceToHost, b->stream));
  BCUDA(cudaStreamSynchronize(b->stream));
  if (b->act_valid && flags == b->act_flags) return SPP_OK;
  std::vector<SysAct> sact((size_t)ns);
  std::vector<uint32_t> act_sys;
  act_sys.reserve((size_t)d.n_total);
  uint32_t a_poff = 0, a_coff = 0;
  for (int s = 0; s < ns; ++s) {
    const BatchSys& S = b->host_sys[(size_t)s];
    sact[(size_t)s] = {0u, 0};
    if (!flags[(size_t)s]) continue;
    sact[(size_t)s] = {a_coff, (int32_t)S.p_off - (int32_t)a_poff};
    act_sys.insert(act_sys.end(), S.n, (uint32_t)s);
    a_poff += S.n;
    a_coff += S.D * S.D;
  }
  BCUDA(cudaMemcpyAsync(d.sact, sact.data(), sizeof(SysAct) * ns, cudaMemcpyHostToDevice, b->stream));
  if (a_poff)
    BCUDA(cudaMemcpyAsync(d.act_sys, act_sys.data(), sizeof(uint32_t) * a_poff, cudaMemcpyHostToDevice,
                          b->stream));
  BCUDA(cudaStreamSynchronize(b->stream));
  batch_drop_graphs(b);
  d.n_act = (int)a_poff;
  d.n_act_keys = (int)a_coff;
  b->act_flags = flags;
  b->act_valid = true;
  return SPP_OK;
}

int batch_graph(SppBatch* b, int nsteps, cudaGraphExec_t* out) {
  for (auto& g : b->graphs)
    if (g.first == nsteps) { *out = g.second; return SPP_OK; }
  cudaGraph_t graph = nullptr;
  BCUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  int rc = SPP_OK;
  for (int i = 0; i < nsteps && rc == SPP_OK; ++i) rc = enqueue_batch_step(b, b->stream);
  cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
  if (rc != SPP_OK) { if (graph) cudaGraphDestroy(graph); return rc; }
  if (e != cudaSuccess) return bfail(SPP_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
  cudaGraphExec_t exec;
  e = cudaGraphInstantiate(&exec, graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    return bfail(SPP_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
  }
  b->graphs.push_back({nsteps, exec});
  b->graph_defs.push_back(graph);
  *out = exec;
  return SPP_OK;
}

int batch_step_enqueue(SppBatch* b, int nsteps) {
  if (b->d.n_act == 0) return SPP_OK;  /* nothing active */
  while (nsteps > 0) {
    int chunk = nsteps >= BATCH_GRAPH_CHUNK ? BATCH_GRAPH_CHUNK : nsteps;
    cudaGraphExec_t exec;
    int rc = batch_graph(b, chunk, &exec);
    if (rc != SPP_OK) return rc;
    BCUDA(cudaGraphLaunch(exec, b->stream));
    b->launches += (int64_t)chunk * 7;
    nsteps -= chunk;
  }
  return SPP_OK;
}


}  // namespace

extern "C" {

int spp_batch_create(const SppParams* systems, int n_systems, SppBatch** out) {
  if (!systems || !out || n_systems < 1) return bfail(SPP_ERR_INVALID, "bad arguments");
  *out = nullptr;
  SppBatch* b = new SppBatch();
  b->host_sys.resize((size_t)n_systems);
  uint64_t p_off = 0, c_off = 0;
  for (int s = 0; s < n_systems; ++s) {
    const SppParams& p = systems[s];
    if (p.struct_size != sizeof(SppParams) || p.n < 1 || !(p.L > 0) || !(p.r_align > 0) ||
        (p.model != SPP_MODEL_VICSEK && p.model != SPP_MODEL_VICSEK_REF_ANGLE &&
         p.model != SPP_MODEL_VICSEK_REF_VECTOR) || p.boundary != SPP_BOUNDARY_PERIODIC) {
      delete b;
      return bfail(SPP_ERR_INVALID, "system " + std::to_string(s) +
                                        ": batches hold periodic Vicsek-family systems with n >= 1, L > 0");
    }
    double rc = p.r_align;
    if (p.model == SPP_MODEL_VICSEK_REF_VECTOR && p.r_push > rc) rc = p.r_push;
    int D = (int)std::floor(2.0 * p.L / (rc * 1.001));
    if (D < 3) {
      delete b;
      return bfail(SPP_ERR_INVALID, "system " + std::to_string(s) + ": box too small (2L/r < 3)");
    }
    b->model = s == 0 ? p.model : (b->model == p.model ? b->model : -1);
    BatchSys& S = b->host_sys[(size_t)s];
    memset(&S, 0, sizeof(S));
    spp_consts_from_params(&S.k, &p);
    S.p_off = (uint32_t)p_off;
    S.n = (uint32_t)p.n;
    S.c_off = (uint32_t)c_off;
    S.D = (uint32_t)D;
    S.active = 1u;
    S.steps = 0u;
    p_off += (uint64_t)p.n;
    c_off += (uint64_t)D * (uint64_t)D;
  }
  if (p_off > 0x7fffffffULL || c_off > scan_max_elements()) {
    delete b;
    return bfail(SPP_ERR_INVALID, "batch too large (particles or cells)");
  }
  DevBatch& d = b->d;
  memset(&d, 0, sizeof(d));
  d.n_total = (int)p_off;
  d.n_sys = n_systems;
  b->n_keys = (uint32_t)c_off;
  d.window = 500;
  d.stationary_from = 0;
  d.max_steps = 0;
  size_t n = (size_t)p_off;
  int rc = SPP_OK;
  rc = rc ? rc : balloc(&d.sys, (size_t)n_systems);
  rc = rc ? rc : balloc(&d.stats, (size_t)n_systems);
  rc = rc ? rc : balloc(&d.sys_of, n);
  rc = rc ? rc : balloc(&d.pos, n);
  rc = rc ? rc : balloc(&d.pos_alt, n);
  rc = rc ? rc : balloc(&d.theta, n);
  rc = rc ? rc : balloc(&d.theta_alt, n);
  rc = rc ? rc : balloc(&d.img, n);
  rc = rc ? rc : balloc(&d.img_alt, n);
  rc = rc ? rc : balloc(&d.fx_alt, n);
  rc = rc ? rc : balloc(&d.id, n);
  rc = rc ? rc : balloc(&d.id_alt, n);
  rc = rc ? rc : balloc(&d.key, n);
  rc = rc ? rc : balloc(&d.rank, n);
  rc = rc ? rc : balloc(&d.cell_count, (size_t)c_off);
  rc = rc ? rc : balloc(&d.cell_start, (size_t)c_off);
  rc = rc ? rc : balloc(&d.scan_tmp, ((size_t)c_off + 4095) / 4096 + 1);
  rc = rc ? rc : balloc(&d.ctl, 1);
  rc = rc ? rc : balloc(&d.act_sys, n);
  rc = rc ? rc : balloc(&d.sact, (size_t)n_systems);
  rc = rc ? rc : balloc(&d.flags, (size_t)n_systems);
  rc = rc ? rc : balloc(&b->stage_x, n);
  rc = rc ? rc : balloc(&b->stage_y, n);
  rc = rc ? rc : balloc(&b->stage_t, n);
  rc = rc ? rc : balloc(&b->stage_img, n);
  if (rc != SPP_OK) {
    batch_free(b);
    delete b;
    return rc;
  }
  std::vector<uint32_t> sys_of(n);
  for (int s = 0; s < n_systems; ++s)
    for (uint32_t q = 0; q < b->host_sys[s].n; ++q) sys_of[b->host_sys[s].p_off + q] = (uint32_t)s;
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMemcpy(d.sys, b->host_sys.data(), sizeof(BatchSys) * n_systems, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d.sys_of, sys_of.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(d.stats, 0, sizeof(BatchStats) * n_systems);
  if (e == cudaSuccess) e = cudaMemset(d.ctl, 0, sizeof(Ctl));
  if (e != cudaSuccess) {
    batch_free(b);
    delete b;
    return bfail(SPP_ERR_CUDA, std::string("batch setup: ") + cudaGetErrorString(e));
  }
  *out = b;
  return SPP_OK;
}

int spp_batch_destroy(SppBatch* b) {
  if (!b) return SPP_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  batch_free(b);
  delete b;
  return SPP_OK;
}

int spp_batch_set_windows(SppBatch* b, int window_steps, int stationary_from, int max_steps) {
  if (!b || window_steps < 0 || stationary_from < 0 || max_steps < 0)
    return bfail(SPP_ERR_INVALID, "bad arguments");
  BCUDA(cudaStreamSynchronize(b->stream));
  for (auto& g : b->graphs) cudaGraphExecDestroy(g.second);
  for (auto g : b->graph_defs) cudaGraphDestroy(g);
  b->graphs.clear();
  b->graph_defs.clear();
  b->d.window = window_steps;
  b->d.stationary_from = stationary_from;
  b->d.max_steps = max_steps;
  return SPP_OK;
}

int spp_batch_upload(SppBatch* b, const float* x, const float* y, const float* theta, int total_n) {
  if (!b || !x || !y || !theta) return bfail(SPP_ERR_INVALID, "NULL argument");
  if (total_n != b->d.n_total) return bfail(SPP_ERR_INVALID, "total_n differs from the batch size");
  for (const BatchSys& S : b->host_sys) {
    const float L = S.k.L;
    for (uint32_t q = 0; q < S.n; ++q) {
      const uint32_t i = S.p_off + q;
      if (!std::isfinite(x[i]) || !std::isfinite(y[i]) || !std::isfinite(theta[i]))
        return bfail(SPP_ERR_NUMERIC, "non-finite input at particle " + std::to_string(i));
      if (x[i] < -L || x[i] >= L || y[i] < -L || y[i] >= L)
        return bfail(SPP_ERR_INVALID, "position outside its system's box at particle " + std::to_string(i));
    }
  }
  size_t bytes = sizeof(float) * (size_t)total_n;
  BCUDA(cudaMemcpyAsync(b->stage_x, x, bytes, cudaMemcpyHostToDevice, b->stream));
  BCUDA(cudaMemcpyAsync(b->stage_y, y, bytes, cudaMemcpyHostToDevice, b->stream));
  BCUDA(cudaMemcpyAsync(b->stage_t, theta, bytes, cudaMemcpyHostToDevice, b->stream));
  /* reset per-system counters and statistics */
  for (auto& S : b->host_sys) { S.active = 1u; S.steps = 0u; }
  BCUDA(cudaMemcpyAsync(b->d.sys, b->host_sys.data(), sizeof(BatchSys) * b->host_sys.size(),
                        cudaMemcpyHostToDevice, b->stream));
  BCUDA(cudaMemsetAsync(b->d.stats, 0, sizeof(BatchStats) * b->host_sys.size(), b->stream));
  k_batch_init<<<nblocks(b->d.n_total), SPP_BLOCK, 0, b->stream>>>(b->d, b->stage_x, b->stage_y,
                                                                      b->stage_t);
  b->launches += 1;
  BCUDA(cudaStreamSynchronize(b->stream));
  b->uploaded = true;
  return SPP_OK;
}

int spp_batch_step(SppBatch* b, int nsteps) {
  if (!b || nsteps < 0) return bfail(SPP_ERR_INVALID, "bad arguments");
  if (!b->uploaded) return bfail(SPP_ERR_INVALID, "no state uploaded");
  int rc = batch_refresh_active(b);
  if (rc != SPP_OK) return rc;
  return batch_step_enqueue(b, nsteps);
}

int spp_batch_poll(SppBatch* b, SppSweepStats* out, int n_systems) {
  if (!b || !out || n_systems != b->d.n_sys) return bfail(SPP_ERR_INVALID, "bad arguments");
  BCUDA(cudaStreamSynchronize(b->stream));
  std::vector<BatchSys> sys((size_t)n_systems);
  std::vector<BatchStats> st((size_t)n_systems);
  Ctl c;
  BCUDA(cudaMemcpy(sys.data(), b->d.sys, sizeof(BatchSys) * n_systems, cudaMemcpyDeviceToHost));
  BCUDA(cudaMemcpy(st.data(), b->d.stats, sizeof(BatchStats) * n_systems, cudaMemcpyDeviceToHost));
  BCUDA(cudaMemcpy(&c, b->d.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
  if (c.fx_overflow) return bfail(SPP_ERR_OVERFLOW, "fixed-point range exceeded");
  for (int s = 0; s < n_systems; ++s) {
    SppSweepStats& o = out[s];
    memset(&o, 0, sizeof(o));
    const BatchStats& T = st[(size_t)s];
    const int64_t nw = (int64_t)(sys[s].steps < (uint32_t)b->d.window ? sys[s].steps : (uint32_t)b->d.window);
    o.steps = sys[s].steps;
    o.active = (int32_t)sys[s].active;
    o.p_last = T.p_last;
    o.window_steps = nw;
    if (nw > 0) {
      const double m1 = T.w1 / nw, m2 = T.w2 / nw, m3 = T.w3 / nw, m4 = T.w4 / nw;
      const double var = m2 - m1 * m1;
      o.p_mean = m1;
      o.p_var = var;
      const double c4 = m4 - 4 * m3 * m1 + 6 * m2 * m1 * m1 - 3 * m1 * m1 * m1 * m1;
      o.p_kurt = var > 0 ? c4 / (var * var) : 0.0;
    }
    o.stationary_steps = T.ns;
    if (T.ns > 0) {
      o.p_stationary = T.s1 / T.ns;
      o.p2_stationary = T.s2 / T.ns;
      o.p4_stationary = T.s4 / T.ns;
      if (o.p2_stationary > 0) {
        o.binder = 1.0 - o.p4_stationary / (3.0 * o.p2_stationary * o.p2_stationary);
        o.binder_reference = 1.0 - o.p4_stationary / (3.0 * o.p2_stationary);
      }
    }
  }
  return SPP_OK;
}

static int batch_set_active(SppBatch* b, const int32_t* systems, int count, uint32_t value) {
  if (!b || (count > 0 && !systems) || count < 0) return bfail(SPP_ERR_INVALID, "bad arguments");
  if (count == 0) return SPP_OK;
  int32_t* d_idx = nullptr;
  int rc = balloc(&d_idx, (size_t)count);
  if (rc != SPP_OK) return rc;
  BCUDA(cudaMemcpyAsync(d_idx, systems, sizeof(int32_t) * count, cudaMemcpyHostToDevice, b->stream));
  k_batch_set_active<<<nblocks(count), SPP_BLOCK, 0, b->stream>>>(b->d, d_idx, count, value);
  b->launches += 1;
  cudaError_t e = cudaStreamSynchronize(b->stream);
  cudaFree(d_idx);
  if (e != cudaSuccess) return bfail(SPP_ERR_CUDA, cudaGetErrorString(e));
  return SPP_OK;
}

int spp_batch_retire(SppBatch* b, const int32_t* systems, int count) {
  return batch_set_active(b, systems, count, 0u);
}

int spp_batch_resume(SppBatch* b, const int32_t* systems, int count) {
  return batch_set_active(b, systems, count, 1u);
}

int spp_batch_download(SppBatch* b, float* x, float* y, float* theta, int32_t* img_x,
                       int32_t* img_y, int total_n) {
  if (!b || !x || !y || !theta || total_n != b->d.n_total) return bfail(SPP_ERR_INVALID, "bad arguments");
  k_batch_gather<<<nblocks(total_n), SPP_BLOCK, 0, b->stream>>>(b->d, b->stage_x, b->stage_y,
                                                                  b->stage_t, b->stage_img);
  b->launches += 1;
  size_t bytes = sizeof(float) * (size_t)total_n;
  BCUDA(cudaMemcpyAsync(x, b->stage_x, bytes, cudaMemcpyDeviceToHost, b->stream));
  BCUDA(cudaMemcpyAsync(y, b->stage_y, bytes, cudaMemcpyDeviceToHost, b->stream));
  BCUDA(cudaMemcpyAsync(theta, b->stage_t, bytes, cudaMemcpyDeviceToHost, b->stream));
  std::vector<int2> img;
  if (img_x || img_y) {
    img.resize((size_t)total_n);
    BCUDA(cudaMemcpyAsync(img.data(), b->stage_img, sizeof(int2) * (size_t)total_n,
                          cudaMemcpyDeviceToHost, b->stream));
  }
  BCUDA(cudaStreamSynchronize(b->stream));
  for (int i = 0; i < (int)img.size(); ++i) {
    if (img_x) img_x[i] = img[i].x;
    if (img_y) img_y[i] = img[i].y;
  }
  return SPP_OK;
}

int64_t spp_batch_kernel_launches(SppBatch* b) { return b ? b->launches : 0; }

int spp_batch_time_steps(SppBatch* b, int nsteps, double* ms) {
  if (!b || !ms) return bfail(SPP_ERR_INVALID, "NULL argument");
  if (!b->uploaded || nsteps < 0) return bfail(SPP_ERR_INVALID, "no state uploaded or bad step count");
  int rc = batch_refresh_active(b);
  if (rc != SPP_OK) return rc;
  if (b->d.n_act > 0) {  /* capture outside the timed region */
    cudaGraphExec_t exec;
    rc = batch_graph(b, nsteps >= BATCH_GRAPH_CHUNK ? BATCH_GRAPH_CHUNK : nsteps, &exec);
    if (rc == SPP_OK && nsteps % BATCH_GRAPH_CHUNK && nsteps > BATCH_GRAPH_CHUNK)
      rc = batch_graph(b, nsteps % BATCH_GRAPH_CHUNK, &exec);
    if (rc != SPP_OK) return rc;
  }
  cudaEvent_t e0, e1;
  BCUDA(cudaEventCreate(&e0));
  BCUDA(cudaEventCreate(&e1));
  cudaEventRecord(e0, b->stream);
  rc = batch_step_enqueue(b, nsteps);
  cudaEventRecord(e1, b->stream);
  cudaError_t e = cudaEventSynchronize(e1);
  float t = 0;
  if (rc == SPP_OK && e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != SPP_OK) return rc;
  if (e != cudaSuccess) return bfail(SPP_ERR_CUDA, cudaGetErrorString(e));
  *ms = t;
  return SPP_OK;
}

}  // extern "C"
