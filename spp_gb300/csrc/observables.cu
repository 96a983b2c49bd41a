/*
 * observables.cu -- order parameters and pair statistics of a system.
 *
 * The reference computes these offline, from frames saved to disk:
 *   Compute_Order_Parameters  analyze/analyze.h:121-146  (<P>, sigma^2, error, G)
 *   Stat::Compute             analyze/statistics.h:35-54
 *   Stat::Find_Correlation_Length analyze/statistics.h:68-82
 *   Pair_Distribution         analyze/analyze.h:365-424  (body-frame histogram)
 * Here the frames come from the device: the polarization series is recorded
 * every `every` steps with the exact fixed-point heading sums, and the pair
 * histograms are built by a counting sort of the current positions into
 * cells at least as wide as the histogram's range, one thread per particle
 * walking its 3 x 3 cells, with per-block shared-memory histograms flushed
 * by integer atomics (the counts do not depend on the visiting order).  A
 * radial g(r) is project-defined: the reference has only the body-frame
 * histogram.
 */
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include "spp_internal.cuh"

namespace {

int ofail(int status, const std::string& msg) {
  spp_internal_set_error(msg.c_str());
  return status;
}

#define OCUDA(expr)                                                                        \
  do {                                                                                     \
    cudaError_t _e = (expr);                                                               \
    if (_e != cudaSuccess) return ofail(SPP_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

/* ---------------------------------------------------------------- */
/* a counting sort of the current positions into a D x D row-major grid */
/* ---------------------------------------------------------------- */
struct Grid {
  int n, D;
  int closed;             /* a closed box: plain differences, no minimum image */
  float L, L2;
  const float4* pos;
  uint32_t *count, *start, *key, *rank, *tmp;
  float4* sorted;
};

__global__ void __launch_bounds__(SPP_BLOCK) k_obs_bin(Grid g) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  const float4 p = g.pos[i];
  const int cx = spp_cell_coord(p.x, g.L, g.L2, g.D, SPP_BIN_GEOMETRIC);
  const int cy = spp_cell_coord(p.y, g.L, g.L2, g.D, SPP_BIN_GEOMETRIC);
  const uint32_t key = (uint32_t)cy * (uint32_t)g.D + (uint32_t)cx;
  g.key[i] = key;
  g.rank[i] = atomicAdd(&g.count[key], 1u);
}

__global__ void __launch_bounds__(SPP_BLOCK) k_obs_scatter(Grid g) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  g.sorted[g.start[g.key[i]] + g.rank[i]] = g.pos[i];
}

/* Radial histogram: ordered pairs within r_max, minimum image (plain
 * differences in a closed box). */
__global__ void __launch_bounds__(SPP_BLOCK) k_obs_radial(Grid g, float r2max, float dr, int nbins,
                                                          unsigned long long* counts) {
  extern __shared__ uint32_t hist[];
  for (int b = threadIdx.x; b < nbins; b += blockDim.x) hist[b] = 0u;
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < g.n) {
    const float4 p = g.sorted[i];
    const int cx = spp_cell_coord(p.x, g.L, g.L2, g.D, SPP_BIN_GEOMETRIC);
    const int cy = spp_cell_coord(p.y, g.L, g.L2, g.D, SPP_BIN_GEOMETRIC);
    for (int oy = -1; oy <= 1; ++oy) {
      int ny = cy + oy;
      ny = ny < 0 ? ny + g.D : (ny >= g.D ? ny - g.D : ny);
      for (int ox = -1; ox <= 1; ++ox) {
        int nx = cx + ox;
        nx = nx < 0 ? nx + g.D : (nx >= g.D ? nx - g.D : nx);
        const uint32_t c = (uint32_t)ny * (uint32_t)g.D + (uint32_t)nx;
        const uint32_t s0 = g.start[c], s1 = s0 + g.count[c];
        for (uint32_t j = s0; j < s1; ++j) {
          if ((int)j == i) continue;
          const float4 q = g.sorted[j];
          const float dx = g.closed ? p.x - q.x : spp_min_image_f(p.x - q.x, g.L, g.L2);
          const float dy = g.closed ? p.y - q.y : spp_min_image_f(p.y - q.y, g.L, g.L2);
          const float d2 = fmaf(dx, dx, dy * dy);
          if (d2 < r2max) {
            int b = (int)(sqrtf(d2) / dr);
            b = b < nbins ? b : nbins - 1;
            atomicAdd(&hist[b], 1u);
          }
        }
      }
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < nbins; b += blockDim.x)
    if (hist[b]) atomicAdd(&counts[b], (unsigned long long)hist[b]);
}

/* Body-frame histogram of Pair_Distribution: plain differences, heading of
 * the first particle of the pair. */
__global__ void __launch_bounds__(SPP_BLOCK) k_obs_pairdist(Grid g, float lx, float ly, int gx, int gy,
                                                            unsigned long long* counts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  const float4 p = g.sorted[i];
  const int cx = spp_cell_coord(p.x, g.L, g.L2, g.D, SPP_BIN_GEOMETRIC);
  const int cy = spp_cell_coord(p.y, g.L, g.L2, g.D, SPP_BIN_GEOMETRIC);
  for (int oy = -1; oy <= 1; ++oy) {
    int ny = cy + oy;
    if (ny < 0 || ny >= g.D) continue;  /* across the boundary the plain difference exceeds the range */
    for (int ox = -1; ox <= 1; ++ox) {
      int nx = cx + ox;
      if (nx < 0 || nx >= g.D) continue;
      const uint32_t c = (uint32_t)ny * (uint32_t)g.D + (uint32_t)nx;
      const uint32_t s0 = g.start[c], s1 = s0 + g.count[c];
      for (uint32_t j = s0; j < s1; ++j) {
        if ((int)j == i) continue;
        const float4 q = g.sorted[j];
        const float dx = q.x - p.x;
        const float dy = q.y - p.y;
        const float ty = p.z * dx + p.w * dy;
        const float tx = p.w * dx - p.z * dy;
        if (fabsf(tx) < lx && fabsf(ty) < ly) {
          int bx = (int)((float)gx * ((tx / lx) + 1.0f) / 2.0f);
          int by = (int)((float)gy * ((ty / ly) + 1.0f) / 2.0f);
          bx = bx < gx ? bx : gx - 1;
          by = by < gy ? by : gy - 1;
          atomicAdd(&counts[(size_t)bx * gy + by], 1ull);
        }
      }
    }
  }
}

/* Per ring: sums of x, y, x^2, y^2, xy of the unwrapped positions of its
 * beads (block 2r) and of its swimmers (block 2r + 1), in FP64 with a fixed
 * reduction tree.  Slot of particle id q: inv[q]. */
__global__ void __launch_bounds__(SPP_BLOCK) k_obs_ring_sums(DevState d, SppConsts k, int n_rings, int ring_size,
                                                             int sw_per_ring, double* sums) {
  __shared__ double red[5][SPP_BLOCK];
  const int ring = blockIdx.x >> 1, part = blockIdx.x & 1;
  const int first = part == 0 ? ring * ring_size : n_rings * ring_size + ring * sw_per_ring;
  const int count = part == 0 ? ring_size : sw_per_ring;
  double a[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int q = threadIdx.x; q < count; q += blockDim.x) {
    const uint32_t slot = d.inv[first + q];
    const float4 p = d.pos[slot];
    const int2 g = d.img[slot];
    const double x = (double)p.x + (double)k.L2 * (double)g.x;
    const double y = (double)p.y + (double)k.L2 * (double)g.y;
    a[0] += x;
    a[1] += y;
    a[2] += x * x;
    a[3] += y * y;
    a[4] += x * y;
  }
  for (int c = 0; c < 5; ++c) red[c][threadIdx.x] = a[c];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int c = 0; c < 5; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 5) sums[(size_t)blockIdx.x * 5 + threadIdx.x] = red[threadIdx.x][0];
}

/* Positions (unwrapped, FP64) and headings of every particle, by id: the
 * frame spp_ring_motion measures from (Save_Particles_Positions,
 * parallel/beadbox.h:315-322). */
__global__ void __launch_bounds__(SPP_BLOCK) k_obs_mark(DevState d, SppConsts k, double2* xy, float* th) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  const uint32_t id = d.id[i];
  const float4 p = d.pos[i];
  const int2 g = d.img[i];
  xy[id] = make_double2((double)p.x + (double)k.L2 * (double)g.x, (double)p.y + (double)k.L2 * (double)g.y);
  th[id] = d.theta[i];
}

/* Per ring, sums over its beads (block 2r) and its swimmers (block 2r + 1)
 * of x, y, x^2, y^2, xy, v_x, v_y, x v_y - y v_x and (swimmers) the spin,
 * with v = (r - r_marked) / elapsed and the spin the heading change folded
 * to [-pi, pi) as beadbox.h:354-356 folds it, over elapsed; FP64, fixed
 * reduction tree. */
constexpr int MOTION_SUMS = 9;
__global__ void __launch_bounds__(SPP_BLOCK) k_obs_ring_motion(DevState d, SppConsts k, int n_rings, int ring_size,
                                                               int sw_per_ring, const double2* mxy,
                                                               const float* mth, double inv_elapsed,
                                                               double* sums) {
  __shared__ double red[MOTION_SUMS][SPP_BLOCK];
  const int ring = blockIdx.x >> 1, part = blockIdx.x & 1;
  const int first = part == 0 ? ring * ring_size : n_rings * ring_size + ring * sw_per_ring;
  const int count = part == 0 ? ring_size : sw_per_ring;
  double a[MOTION_SUMS];
  for (int c = 0; c < MOTION_SUMS; ++c) a[c] = 0.0;
  const double two_pi = 6.283185307179586476925286766559;
  for (int q = threadIdx.x; q < count; q += blockDim.x) {
    const uint32_t id = (uint32_t)(first + q);
    const uint32_t slot = d.inv[id];
    const float4 p = d.pos[slot];
    const int2 g = d.img[slot];
    const double x = (double)p.x + (double)k.L2 * (double)g.x;
    const double y = (double)p.y + (double)k.L2 * (double)g.y;
    const double2 m = mxy[id];
    const double vx = (x - m.x) * inv_elapsed, vy = (y - m.y) * inv_elapsed;
    a[0] += x;
    a[1] += y;
    a[2] += x * x;
    a[3] += y * y;
    a[4] += x * y;
    a[5] += vx;
    a[6] += vy;
    a[7] += x * vy - y * vx;
    if (part == 1) {
      double dth = (double)d.theta[slot] - (double)mth[id];
      dth -= two_pi * floor(dth / two_pi);
      dth -= two_pi * floor(dth / (0.5 * two_pi));
      a[8] += dth * inv_elapsed;
    }
  }
  for (int c = 0; c < MOTION_SUMS; ++c) red[c][threadIdx.x] = a[c];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int c = 0; c < MOTION_SUMS; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < MOTION_SUMS) sums[(size_t)blockIdx.x * MOTION_SUMS + threadIdx.x] = red[threadIdx.x][0];
}

/* The reference's formulas (beadbox.h:402-428) from the five sums of n points. */
void shape_from_sums(const double* m, int n, double* cm_x, double* cm_y, double* xx, double* yy, double* xy,
                     double* l1, double* l2, double* rg, double* delta) {
  *cm_x = m[0] / n;
  *cm_y = m[1] / n;
  *xx = (m[2] / n) - *cm_x * *cm_x;
  *yy = (m[3] / n) - *cm_y * *cm_y;
  *xy = (m[4] / n) - *cm_x * *cm_y;
  const double root = std::sqrt((*xx - *yy) * (*xx - *yy) + 4 * *xy * *xy);
  *l1 = 0.5 * (*xx + *yy) + 0.5 * root;
  *l2 = 0.5 * (*xx + *yy) - 0.5 * root;
  *rg = std::sqrt(*xx + *yy);
  const double dl = (*l1 - *l2) / (*l1 + *l2);
  *delta = dl * dl;
}

inline int nblk(int n) { return (n + SPP_BLOCK - 1) / SPP_BLOCK; }

/* Sorts the system's current positions into a grid of cells at least `range`
 * wide; the caller frees the grid with grid_free. */
int grid_build(SppSystem* s, double range, Grid* g, cudaStream_t* st) {
  DevState d;
  SppConsts k;
  int rc = spp_sync(s);
  if (rc != SPP_OK) return rc;
  rc = spp_internal_view(s, &d, &k, st);
  if (rc != SPP_OK) return rc;
  memset(g, 0, sizeof(*g));
  const int D = (int)std::floor(2.0 * (double)k.L / (range * 1.001));
  if (!(range > 0) || D < 3) return ofail(SPP_ERR_INVALID, "range must be in (0, 2L/3]");
  if ((double)D * D > 4.0e8) return ofail(SPP_ERR_INVALID, "range too small for the box (too many cells)");
  g->n = d.n;
  g->D = D;
  g->L = k.L;
  g->L2 = k.L2;
  g->closed = k.closed;
  g->pos = d.pos;
  const size_t nc = (size_t)D * D, n = (size_t)d.n;
  cudaError_t e = cudaMalloc((void**)&g->count, sizeof(uint32_t) * nc);
  if (e == cudaSuccess) e = cudaMalloc((void**)&g->start, sizeof(uint32_t) * nc);
  if (e == cudaSuccess) e = cudaMalloc((void**)&g->tmp, sizeof(uint32_t) * (nc / 4096 + 2));
  if (e == cudaSuccess) e = cudaMalloc((void**)&g->key, sizeof(uint32_t) * n);
  if (e == cudaSuccess) e = cudaMalloc((void**)&g->rank, sizeof(uint32_t) * n);
  if (e == cudaSuccess) e = cudaMalloc((void**)&g->sorted, sizeof(float4) * n);
  if (e != cudaSuccess) return ofail(SPP_ERR_ALLOC, std::string("grid: ") + cudaGetErrorString(e));
  OCUDA(cudaMemsetAsync(g->count, 0, sizeof(uint32_t) * nc, *st));
  k_obs_bin<<<nblk(g->n), SPP_BLOCK, 0, *st>>>(*g);
  launch_scan_u32(g->count, (uint32_t)nc, g->tmp, g->start, *st, nullptr);
  k_obs_scatter<<<nblk(g->n), SPP_BLOCK, 0, *st>>>(*g);
  OCUDA(cudaGetLastError());
  spp_internal_count_launches(s, 5);
  return SPP_OK;
}

void grid_free(Grid* g) {
  void* ptrs[] = {g->count, g->start, g->tmp, g->key, g->rank, g->sorted};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  memset(g, 0, sizeof(*g));
}

/* Autocorrelation length as Stat::Find_Correlation_Length computes it: the
 * first lag tau < T/2 at which the normalised autocorrelation, each term
 * divided by (T - tau) before it is added, falls below 0.01 (T/2 - 1 when
 * none does; 0 when the series is constant). */
double correlation_length(const double* x, int T, double mean, double variance) {
  double corr_len = 0.0;
  for (int tau = 0; tau < T / 2; ++tau) {
    double c = 0.0;
    for (int i = 0; i < T - tau; ++i) c += (x[i] - mean) * (x[i + tau] - mean) / (double)(T - tau);
    c /= variance;
    corr_len = (double)tau;
    if (c < 0.01) break;
  }
  return corr_len;
}

}  // namespace

extern "C" {

int spp_order_parameters(const double* p, int T, double area, SppOrderStats* out) {
  if (!p || !out || T < 2) return ofail(SPP_ERR_INVALID, "need a series of at least 2 samples");
  memset(out, 0, sizeof(*out));
  double mn = p[0], mx = p[0], sum = 0.0, sq = 0.0, sum4 = 0.0;
  for (int i = 0; i < T; ++i) {
    if (!std::isfinite(p[i])) return ofail(SPP_ERR_NUMERIC, "non-finite sample");
    mn = p[i] < mn ? p[i] : mn;
    mx = p[i] > mx ? p[i] : mx;
    sum += p[i];
    sq += p[i] * p[i];
    const double p2 = p[i] * p[i];
    sum4 += p2 * p2;
  }
  out->samples = T;
  out->min = mn;
  out->max = mx;
  out->mean = sum / T;
  out->mean_square = sq / T;
  out->variance = out->mean_square - out->mean * out->mean;
  out->std = std::sqrt(out->variance);
  out->corr_len = correlation_length(p, T, out->mean, out->variance);
  out->error = std::sqrt(out->variance * out->corr_len / T);
  out->sigma2 = out->variance * area;
  out->p4_mean = sum4 / T;
  if (out->mean_square > 0) {
    out->binder = 1.0 - out->p4_mean / (3.0 * out->mean_square * out->mean_square);
    out->binder_reference = 1.0 - out->p4_mean / (3.0 * out->mean_square);
  }
  return SPP_OK;
}

int spp_polarization_series(SppSystem* s, int nframes, int every, double* p, double* px, double* py) {
  if (!s || !p || nframes < 1 || every < 1) return ofail(SPP_ERR_INVALID, "bad arguments");
  DevState d;
  SppConsts k;
  cudaStream_t st;
  int rc = spp_internal_view(s, &d, &k, &st);
  if (rc != SPP_OK) return rc;
  unsigned long long* sums = nullptr;
  OCUDA(cudaMalloc((void**)&sums, sizeof(unsigned long long) * 2 * (size_t)nframes));
  std::vector<long long> host(2 * (size_t)nframes);
  cudaError_t e = cudaMemsetAsync(sums, 0, sizeof(unsigned long long) * 2 * (size_t)nframes, st);
  /* the Verlet-list models may freeze on a full neighbour list; their frames
   * wait for the steps (re-run by spp_sync) before P is read.  The Vicsek
   * models have no list: their frames queue up without host round trips. */
  const bool listed = k.model == SPP_MODEL_ABP || k.model == SPP_MODEL_CONTINUOUS || k.model == SPP_MODEL_BEADS;
  for (int f = 0; f < nframes && rc == SPP_OK && e == cudaSuccess; ++f) {
    rc = spp_step(s, every);
    if (rc == SPP_OK && listed) rc = spp_sync(s);
    if (rc == SPP_OK) {
      rc = spp_internal_view(s, &d, &k, &st);
      launch_polarization_into(d, sums + 2 * (size_t)f, st);
      spp_internal_count_launches(s, 1);
      e = cudaGetLastError();
    }
  }
  if (rc == SPP_OK && e == cudaSuccess)
    e = cudaMemcpyAsync(host.data(), sums, sizeof(long long) * host.size(), cudaMemcpyDeviceToHost, st);
  if (rc == SPP_OK && e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (rc == SPP_OK && e == cudaSuccess && !listed) rc = spp_sync(s);   /* device-side status */
  cudaFree(sums);
  if (rc != SPP_OK) return rc;
  if (e != cudaSuccess) return ofail(SPP_ERR_CUDA, cudaGetErrorString(e));
  const double inv = 1.0 / 134217728.0; /* fixed-point units of 2^-27 */
  for (int f = 0; f < nframes; ++f) {
    const double ax = (double)host[2 * (size_t)f] * inv / d.n;
    const double ay = (double)host[2 * (size_t)f + 1] * inv / d.n;
    p[f] = std::sqrt(ax * ax + ay * ay);
    if (px) px[f] = ax;
    if (py) py[f] = ay;
  }
  return SPP_OK;
}

int spp_radial_distribution(SppSystem* s, double r_max, int nbins, uint64_t* counts) {
  if (!s || !counts || nbins < 1 || nbins > 4096) return ofail(SPP_ERR_INVALID, "bad arguments");
  Grid g;
  cudaStream_t st;
  int rc = grid_build(s, r_max, &g, &st);
  if (rc != SPP_OK) { grid_free(&g); return rc; }
  unsigned long long* dc = nullptr;
  cudaError_t e = cudaMalloc((void**)&dc, sizeof(unsigned long long) * nbins);
  if (e == cudaSuccess) e = cudaMemsetAsync(dc, 0, sizeof(unsigned long long) * nbins, st);
  if (e == cudaSuccess) {
    const float rm = (float)r_max;
    k_obs_radial<<<nblk(g.n), SPP_BLOCK, sizeof(uint32_t) * nbins, st>>>(g, rm * rm, rm / (float)nbins, nbins, dc);
    spp_internal_count_launches(s, 1);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(counts, dc, sizeof(uint64_t) * nbins, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (dc) cudaFree(dc);
  grid_free(&g);
  if (e != cudaSuccess) return ofail(SPP_ERR_CUDA, std::string("radial distribution: ") + cudaGetErrorString(e));
  return SPP_OK;
}

int spp_pair_distribution(SppSystem* s, double lx, double ly, int gx, int gy, uint64_t* counts) {
  if (!s || !counts || gx < 1 || gy < 1 || (int64_t)gx * gy > 65536 || !(lx > 0) || !(ly > 0))
    return ofail(SPP_ERR_INVALID, "bad arguments");
  Grid g;
  cudaStream_t st;
  int rc = grid_build(s, std::sqrt(lx * lx + ly * ly), &g, &st);
  if (rc != SPP_OK) { grid_free(&g); return rc; }
  const size_t nb = (size_t)gx * gy;
  unsigned long long* dc = nullptr;
  cudaError_t e = cudaMalloc((void**)&dc, sizeof(unsigned long long) * nb);
  if (e == cudaSuccess) e = cudaMemsetAsync(dc, 0, sizeof(unsigned long long) * nb, st);
  if (e == cudaSuccess) {
    k_obs_pairdist<<<nblk(g.n), SPP_BLOCK, 0, st>>>(g, (float)lx, (float)ly, gx, gy, dc);
    spp_internal_count_launches(s, 1);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(counts, dc, sizeof(uint64_t) * nb, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (dc) cudaFree(dc);
  grid_free(&g);
  if (e != cudaSuccess) return ofail(SPP_ERR_CUDA, std::string("pair distribution: ") + cudaGetErrorString(e));
  return SPP_OK;
}

int spp_ring_shapes(SppSystem* s, SppRingShape* out, int n_rings) {
  if (!s || !out) return ofail(SPP_ERR_INVALID, "NULL argument");
  int rc = spp_sync(s);
  if (rc != SPP_OK) return rc;
  DevState d;
  SppConsts k;
  cudaStream_t st;
  rc = spp_internal_view(s, &d, &k, &st);
  if (rc != SPP_OK) return rc;
  if (k.model != SPP_MODEL_BEADS || k.n_beads <= 0 || k.ring_size <= 0)
    return ofail(SPP_ERR_INVALID, "ring shapes need a bead model with rings");
  const int nr = k.n_beads / k.ring_size;
  if (n_rings != nr) return ofail(SPP_ERR_INVALID, "n_rings differs from the system's ring count");
  const int sw = (d.n - k.n_beads) / nr;
  double* sums = nullptr;
  OCUDA(cudaMalloc((void**)&sums, sizeof(double) * 10 * (size_t)nr));
  k_obs_ring_sums<<<2 * nr, SPP_BLOCK, 0, st>>>(d, k, nr, k.ring_size, sw, sums);
  spp_internal_count_launches(s, 1);
  std::vector<double> h(10 * (size_t)nr);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), sums, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(sums);
  if (e != cudaSuccess) return ofail(SPP_ERR_CUDA, std::string("ring shapes: ") + cudaGetErrorString(e));
  for (int r = 0; r < nr; ++r) {
    SppRingShape& o = out[r];
    memset(&o, 0, sizeof(o));
    shape_from_sums(&h[10 * (size_t)r], k.ring_size, &o.mb_cm_x, &o.mb_cm_y, &o.mb_xx, &o.mb_yy, &o.mb_xy,
                    &o.mb_lambda1, &o.mb_lambda2, &o.mb_Rg, &o.mb_Delta);
    if (sw > 0)
      shape_from_sums(&h[10 * (size_t)r + 5], sw, &o.sw_cm_x, &o.sw_cm_y, &o.sw_xx, &o.sw_yy, &o.sw_xy,
                      &o.sw_lambda1, &o.sw_lambda2, &o.sw_Rg, &o.sw_Delta);
  }
  return SPP_OK;
}

int spp_ring_motion_mark(SppSystem* s) {
  if (!s) return ofail(SPP_ERR_INVALID, "NULL argument");
  int rc = spp_sync(s);
  if (rc != SPP_OK) return rc;
  DevState d;
  SppConsts k;
  cudaStream_t st;
  rc = spp_internal_view(s, &d, &k, &st);
  if (rc != SPP_OK) return rc;
  double2* xy;
  float* th;
  int64_t* step;
  rc = spp_internal_mark(s, &xy, &th, &step);
  if (rc != SPP_OK) return rc;
  k_obs_mark<<<nblk(d.n), SPP_BLOCK, 0, st>>>(d, k, xy, th);
  spp_internal_count_launches(s, 1);
  OCUDA(cudaGetLastError());
  const int64_t now = spp_internal_step(s);   /* waits for the stream */
  if (now < 0) return ofail(SPP_ERR_CUDA, "ring motion: reading the step counter failed");
  *step = now;
  return SPP_OK;
}

int spp_ring_motion(SppSystem* s, SppRingMotion* out, int n_rings) {
  if (!s || !out) return ofail(SPP_ERR_INVALID, "NULL argument");
  int rc = spp_sync(s);
  if (rc != SPP_OK) return rc;
  DevState d;
  SppConsts k;
  cudaStream_t st;
  rc = spp_internal_view(s, &d, &k, &st);
  if (rc != SPP_OK) return rc;
  if (k.model != SPP_MODEL_BEADS || k.n_beads <= 0 || k.ring_size <= 0)
    return ofail(SPP_ERR_INVALID, "ring motion needs a bead model with rings");
  const int nr = k.n_beads / k.ring_size;
  if (n_rings != nr) return ofail(SPP_ERR_INVALID, "n_rings differs from the system's ring count");
  double2* xy;
  float* th;
  int64_t* mark;
  rc = spp_internal_mark(s, &xy, &th, &mark);
  if (rc != SPP_OK) return rc;
  if (*mark < 0) return ofail(SPP_ERR_INVALID, "no frame marked: call spp_ring_motion_mark first");
  const int64_t now = spp_internal_step(s);
  if (now < 0) return ofail(SPP_ERR_CUDA, "ring motion: reading the step counter failed");
  if (now <= *mark) return ofail(SPP_ERR_INVALID, "no step taken since the marked frame");
  const double elapsed = (double)(now - *mark) * spp_internal_dt(s);
  const int sw = (d.n - k.n_beads) / nr;
  double* sums = nullptr;
  OCUDA(cudaMalloc((void**)&sums, sizeof(double) * 2 * MOTION_SUMS * (size_t)nr));
  k_obs_ring_motion<<<2 * nr, SPP_BLOCK, 0, st>>>(d, k, nr, k.ring_size, sw, xy, th, 1.0 / elapsed, sums);
  spp_internal_count_launches(s, 1);
  std::vector<double> h(2 * MOTION_SUMS * (size_t)nr);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), sums, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(sums);
  if (e != cudaSuccess) return ofail(SPP_ERR_CUDA, std::string("ring motion: ") + cudaGetErrorString(e));
  for (int r = 0; r < nr; ++r) {
    /* Compute_All_Variables, parallel/beadbox.h:385-428 */
    const double* m = &h[2 * MOTION_SUMS * (size_t)r];
    const double* w = m + MOTION_SUMS;
    const double Nm = k.ring_size, Ns = sw;
    SppRingMotion& o = out[r];
    memset(&o, 0, sizeof(o));
    const double mcx = m[0] / Nm, mcy = m[1] / Nm;
    o.mb_v_cm_x = m[5] / Nm;
    o.mb_v_cm_y = m[6] / Nm;
    const double mxx = m[2] / Nm - mcx * mcx, myy = m[3] / Nm - mcy * mcy;
    o.mb_l = m[7] / Nm - mcx * o.mb_v_cm_y + mcy * o.mb_v_cm_x;
    o.mb_omega = o.mb_l / (mxx + myy);
    if (sw > 0) {
      const double scx = w[0] / Ns, scy = w[1] / Ns;
      o.sw_v_cm_x = w[5] / Ns;
      o.sw_v_cm_y = w[6] / Ns;
      const double sxx = w[2] / Ns - scx * scx, syy = w[3] / Ns - scy * scy;
      o.sw_l = w[7] / Ns - scx * o.mb_v_cm_y + scy * o.mb_v_cm_x - mcx * o.sw_v_cm_y + mcy * o.sw_v_cm_x +
               mcx * o.mb_v_cm_y - mcy * o.mb_v_cm_x;
      o.sw_spin = w[8] / Ns;
      const double dcx = mcx - scx, dcy = mcy - scy;
      o.sw_omega = o.sw_l / (sxx + syy + dcx * dcx + dcy * dcy);
    }
  }
  /* the current frame becomes the marked one (Save_Particles_Positions at
   * the end of Compute_All_Variables) */
  k_obs_mark<<<nblk(d.n), SPP_BLOCK, 0, st>>>(d, k, xy, th);
  spp_internal_count_launches(s, 1);
  OCUDA(cudaGetLastError());
  OCUDA(cudaStreamSynchronize(st));
  *mark = now;
  return SPP_OK;
}

}  // extern "C"
