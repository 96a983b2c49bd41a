/*
 * kernels_cells.cu -- cell binning and neighbour lists on sm_103a.
 *
 * Replaces Box::Update_Cells (serial/box.h:107-134, parallel/node.h:710-911)
 * and Box::Update_Neighbor_List (serial/box.h:137-179, shared/cell.h:74-103).
 * The reference pushes particle ids into a vector<int> per cell and keeps a
 * half Verlet list per particle, rebuilt every cell_update_period steps.
 * Here:
 *   1. bin_count: one thread per particle computes its cell's Morton key and
 *      takes a slot in that cell with one atomicAdd per group of lanes
 *      sharing the key (__match_any_sync warp aggregation).
 *   2. scan: exclusive prefix sum of the per-key counts (three passes).
 *   3. scatter: every particle's state moves to its cell-ordered slot, so
 *      that spatial neighbours are neighbours in memory (Morton order keeps
 *      2-D tiles of cells contiguous).
 *   4. build_list: one thread per particle scans the 3x3 cells around it and
 *      records every particle within r_list = r_cut + skin (full list: each
 *      pair appears in both particles' lists, so the force kernels gather
 *      without atomics), column-major nbr[slot * n + i], each list sorted by
 *      particle id so that the force kernels sum in a reproducible order.
 * Order inside a cell depends on atomic arrival order and is therefore not
 * deterministic; the sorted lists (Verlet models) and the order-independent
 * fixed-point sums (Vicsek models) keep the physics deterministic.
 */
#include "spp_internal.cuh"

namespace {

__device__ __forceinline__ uint32_t cell_key(const SppConsts& k, const DevState& d, float x, float y,
                                             int* cx, int* cy) {
  *cx = spp_cell_coord(x, k.L, k.L2, d.D, SPP_BIN_GEOMETRIC);
  *cy = spp_cell_coord(y, k.L, k.L2, d.D, SPP_BIN_GEOMETRIC);
  return spp_morton((uint32_t)*cx, (uint32_t)*cy);
}

__global__ void __launch_bounds__(SPP_BLOCK) k_bin_count(SppConsts k, DevState d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) d.ctl->long_n = 0u;   /* the long-list queue of this rebuild (k_build_list) */
  if (i >= d.n) return;
  float4 p = d.pos[i];
  int cx, cy;
  uint32_t key = cell_key(k, d, p.x, p.y, &cx, &cy);
  if (!spp_index_ok(d.ctl, key, d.n_keys)) key = 0u;
  unsigned mask = __activemask();
  unsigned peers = __match_any_sync(mask, key);
  int lane = threadIdx.x & 31;
  int leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(&d.cell_count[key], (uint32_t)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  d.key[i] = key;
  d.rank[i] = base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
}

/* ---- exclusive scan of cell_count into cell_start ---------------------- */
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_PER_THREAD = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_PER_THREAD;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v) {
  __shared__ uint32_t warp_sums[32];
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int nwarps = (int)(blockDim.x >> 5);
  uint32_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < nwarps ? warp_sums[lane] : 0u;
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    warp_sums[lane] = wi - w; /* exclusive prefix of the warp sums */
  }
  __syncthreads();
  return incl - v + warp_sums[warp];
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const uint32_t* __restrict__ in,
                                                              uint32_t n, uint32_t* block_sums) {
  uint32_t base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_PER_THREAD;
  uint32_t s = 0;
#pragma unroll
  for (int q = 0; q < SCAN_PER_THREAD; ++q)
    if (base + q < n) s += in[base + q];
  s = __reduce_add_sync(0xffffffffu, s);
  __shared__ uint32_t ws[SCAN_THREADS / 32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    uint32_t t = ws[threadIdx.x];
    t = __reduce_add_sync(0xffffffffu, t);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = t;
  }
}

/* Exclusive scan of at most SCAN_TILE block sums, in place (one block). */
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_top(uint32_t* sums, uint32_t nb) {
  uint32_t v[SCAN_PER_THREAD];
  uint32_t base = threadIdx.x * SCAN_PER_THREAD;
  uint32_t local = 0;
#pragma unroll
  for (int q = 0; q < SCAN_PER_THREAD; ++q) {
    v[q] = (base + q < nb) ? sums[base + q] : 0u;
    local += v[q];
  }
  uint32_t excl = block_exclusive_scan(local);
#pragma unroll
  for (int q = 0; q < SCAN_PER_THREAD; ++q) {
    if (base + q < nb) sums[base + q] = excl;
    excl += v[q];
  }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(const uint32_t* __restrict__ in,
                                                             uint32_t n,
                                                             const uint32_t* __restrict__ block_offs,
                                                             uint32_t* __restrict__ out) {
  uint32_t base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_PER_THREAD;
  uint32_t v[SCAN_PER_THREAD];
  uint32_t local = 0;
#pragma unroll
  for (int q = 0; q < SCAN_PER_THREAD; ++q) {
    v[q] = (base + q < n) ? in[base + q] : 0u;
    local += v[q];
  }
  uint32_t excl = block_exclusive_scan(local) + block_offs[blockIdx.x];
#pragma unroll
  for (int q = 0; q < SCAN_PER_THREAD; ++q) {
    if (base + q < n) out[base + q] = excl;
    excl += v[q];
  }
}

__global__ void __launch_bounds__(SPP_BLOCK) k_scatter(DevState d) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  const uint32_t key = d.key[i];
  if (!spp_index_ok(d.ctl, key, d.n_keys)) return;
  uint32_t dst = d.cell_start[key] + d.rank[i];
  if (!spp_index_ok(d.ctl, dst, d.n)) return;
  d.pos_alt[dst] = d.pos[i];
  d.theta_alt[dst] = d.theta[i];
  d.img_alt[dst] = d.img[i];
  d.id_alt[dst] = d.id[i];
}

/* Verlet list from the cell-ordered copy (alt), then the copy moves back
 * into the primary arrays. with_list == 0 only copies (no list).  The copy
 * always completes, even when some list overflows: the overflow only sets
 * the frozen flag, which stops the stage kernels until the host has grown
 * the list and rebuilt it.
 * Accepted neighbours are collected as (id << 32 | slot) keys in a per-thread
 * array, insertion-sorted there (lists hold ~5 entries at unit density) and
 * written once; lists longer than the array fall back to sorting in place. */
#ifndef SPP_LIST_LOCAL
#define SPP_LIST_LOCAL 12
#endif
/* keys kept in shared memory per thread (column threadIdx.x of a
 * [LIST_LOCAL][SPP_BLOCK] array: conflict-free); entries up to LIST_TAIL
 * are inserted in order in global memory, a list longer than that is
 * finished by k_sort_long */
constexpr int LIST_LOCAL = SPP_LIST_LOCAL;
#ifndef SPP_LIST_TAIL
#define SPP_LIST_TAIL 16
#endif
constexpr int LIST_TAIL = SPP_LIST_TAIL;

/* spp_list_order with the lane count known at compile time */
template <int LANES>
__device__ __forceinline__ uint32_t list_order(uint32_t id) {
  return LANES == 1 ? id : ((id & 3u) << 30) | (id >> 2);
}

/* SPP_LIST_ROWS 1: the 3 x 3 cells are visited row by row with the three
 * cells' ranges of a row loaded together (three dependent round trips per
 * particle instead of nine) and walked as one sequence, two candidates per
 * trip with both loads in flight; Morton keys built from per-axis spreads,
 * candidates read as (x, y) only, and the minimum image skipped for
 * particles far from the box edges (where it changes no separation within
 * the list radius, and a candidate across the edge is rejected either way).
 * Measured at the 1M workload 600 steps in (whole rebuild, us): 151.7 with
 * the cell-by-cell walk, 148.4 with rows one candidate per trip, 139.6 with
 * rows two per trip (40 registers; 141.9 when held to 32). */
#ifndef SPP_LIST_ROWS
#define SPP_LIST_ROWS 1
#endif
/* 1: the row walk loads both candidates' ids with their positions
 * (rebuild 139.6 -> 136.8 us at the 1M workload) */
#ifndef SPP_LIST_IDS_EARLY
#define SPP_LIST_IDS_EARLY 1
#endif
/* blocks per SM the list build is compiled for (0: the compiler's choice) */
#ifndef SPP_LIST_MIN_BLOCKS
#define SPP_LIST_MIN_BLOCKS 0
#endif
#if SPP_LIST_MIN_BLOCKS > 0
#define SPP_LIST_BOUNDS __launch_bounds__(SPP_BLOCK, SPP_LIST_MIN_BLOCKS)
#else
#define SPP_LIST_BOUNDS __launch_bounds__(SPP_BLOCK)
#endif

template <int LANES>
__global__ void SPP_LIST_BOUNDS k_build_list(SppConsts k, DevState d, int with_list) {
  __shared__ unsigned long long skeys[LIST_LOCAL][SPP_BLOCK];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t cnt = 0;
  unsigned long long lane_cnt = 0;   /* neighbours per id % 4, 16 bits each */
  if (i < d.n) {
    float4 p = d.pos_alt[i];
    if (with_list) {
#define keys(q) skeys[(q)][threadIdx.x]
      int cx, cy;
      cell_key(k, d, p.x, p.y, &cx, &cy);
      const int D = d.D;
      const uint32_t cap = (uint32_t)d.cap;
      /* one candidate j (cell-ordered slot) */
      auto visit = [&](uint32_t j, uint32_t idj, float dx, float dy, float d2) {
        if (d2 < k.rlist2) {
          const unsigned long long key =
              ((unsigned long long)list_order<LANES>(idj) << 32) | (unsigned long long)j;
          if (LANES > 1) lane_cnt += 1ull << (16 * (idj & 3u));
          if (cnt < (uint32_t)LIST_LOCAL) {
            /* the order words are unique, so comparing them orders the keys */
            const uint32_t ko = (uint32_t)(key >> 32);
            int pos = (int)cnt;
            while (pos > 0 && (uint32_t)(keys(pos - 1) >> 32) > ko) {
              keys(pos) = keys(pos - 1);
              --pos;
            }
            keys(pos) = key;
          } else if (cnt < cap && cnt < (uint32_t)LIST_TAIL) {
            /* a longer list: the first LIST_LOCAL keys are still local;
             * keep the next ones sorted in place in global memory */
            int pos = (int)cnt;
            while (pos > LIST_LOCAL) {
              const int32_t prev = d.nbr[(size_t)(pos - 1) * d.n + i];
              if (list_order<LANES>(d.id_alt[prev]) < (uint32_t)(key >> 32)) break;
              d.nbr[(size_t)pos * d.n + i] = prev;
              --pos;
            }
            if (pos == LIST_LOCAL && keys(LIST_LOCAL - 1) > key) {
              /* belongs among the local keys: swap with the local maximum */
              unsigned long long moved = keys(LIST_LOCAL - 1);
              int lp = LIST_LOCAL - 1;
              while (lp > 0 && keys(lp - 1) > key) {
                keys(lp) = keys(lp - 1);
                --lp;
              }
              keys(lp) = key;
              d.nbr[(size_t)pos * d.n + i] = (int32_t)(uint32_t)moved;
            } else {
              d.nbr[(size_t)pos * d.n + i] = (int32_t)j;
            }
          } else if (cnt < cap) {
            /* a long list: the rest is appended unsorted and k_sort_long
             * orders the whole list */
            d.nbr[(size_t)cnt * d.n + i] = (int32_t)j;
          }
          ++cnt;
        }
      };
#if SPP_LIST_ROWS
      const int wrap = !(k.closed || (fabsf(p.x) < k.interior && fabsf(p.y) < k.interior));
      uint32_t mx[3];
#pragma unroll
      for (int o = 0; o < 3; ++o) {
        int nx = cx + o - 1;
        nx = nx < 0 ? nx + D : (nx >= D ? nx - D : nx);
        mx[o] = spp_morton_spread((uint32_t)nx);
      }
      for (int oy = -1; oy <= 1; ++oy) {
        int ny = cy + oy;
        ny = ny < 0 ? ny + D : (ny >= D ? ny - D : ny);
        const uint32_t my = spp_morton_spread((uint32_t)ny) << 1;
        uint32_t s0[3], c[3];
#pragma unroll
        for (int o = 0; o < 3; ++o) {
          const uint32_t kk = mx[o] | my;
          s0[o] = 0u;
          c[o] = 0u;
          if (!spp_index_ok(d.ctl, kk, d.n_keys)) continue;
          s0[o] = d.cell_start[kk];
          c[o] = d.cell_count[kk];
          if (!spp_index_ok(d.ctl, (long long)s0[o] + c[o], (long long)d.n + 1)) c[o] = 0u;
        }
        /* the row's three ranges as one sequence, two candidates per trip
         * with both loads in flight */
        const uint32_t c01 = c[0] + c[1], total = c01 + c[2];
        auto slot_of = [&](uint32_t t) {
          return t < c[0] ? s0[0] + t : (t < c01 ? s0[1] + (t - c[0]) : s0[2] + (t - c01));
        };
        for (uint32_t t = 0; t < total; t += 2) {
          const uint32_t ja = slot_of(t);
          const uint32_t jb = t + 1 < total ? slot_of(t + 1) : ja;
          const float2 qa = reinterpret_cast<const float2*>(d.pos_alt)[2 * (size_t)ja];
          const float2 qb = reinterpret_cast<const float2*>(d.pos_alt)[2 * (size_t)jb];
#if SPP_LIST_IDS_EARLY
          /* both ids with the positions: an accepted candidate's key does not
           * wait on a second load */
          const uint32_t ida = d.id_alt[ja], idb = d.id_alt[jb];
#endif
          float dxa, dya, dxb, dyb;
          const float d2a = wrap ? spp_pair_sep(&k, 1, p.x, p.y, qa.x, qa.y, &dxa, &dya)
                                 : spp_pair_sep(&k, 0, p.x, p.y, qa.x, qa.y, &dxa, &dya);
          const float d2b = wrap ? spp_pair_sep(&k, 1, p.x, p.y, qb.x, qb.y, &dxb, &dyb)
                                 : spp_pair_sep(&k, 0, p.x, p.y, qb.x, qb.y, &dxb, &dyb);
#if SPP_LIST_IDS_EARLY
          if ((int)ja != i) visit(ja, ida, dxa, dya, d2a);
          if (t + 1 < total && (int)jb != i) visit(jb, idb, dxb, dyb, d2b);
#else
          if ((int)ja != i && d2a < k.rlist2) visit(ja, d.id_alt[ja], dxa, dya, d2a);
          if (t + 1 < total && (int)jb != i && d2b < k.rlist2) visit(jb, d.id_alt[jb], dxb, dyb, d2b);
#endif
        }
      }
#else
      for (int oy = -1; oy <= 1; ++oy) {
        int ny = cy + oy;
        ny = ny < 0 ? ny + D : (ny >= D ? ny - D : ny);
        for (int ox = -1; ox <= 1; ++ox) {
          int nx = cx + ox;
          nx = nx < 0 ? nx + D : (nx >= D ? nx - D : nx);
          uint32_t kk = spp_morton((uint32_t)nx, (uint32_t)ny);
          if (!spp_index_ok(d.ctl, kk, d.n_keys)) continue;
          uint32_t s0 = d.cell_start[kk], c = d.cell_count[kk];
          if (!spp_index_ok(d.ctl, (long long)s0 + c, (long long)d.n + 1)) continue;
          for (uint32_t j = s0; j < s0 + c; ++j) {
            if ((int)j == i) continue;
            float4 q = d.pos_alt[j];
            float dx, dy;
            float d2 = spp_sep(&k, p.x, p.y, q.x, q.y, &dx, &dy);
            if (d2 < k.rlist2) visit(j, d.id_alt[j], dx, dy, d2);
          }
        }
      }
#endif
      const uint32_t nloc = cnt < (uint32_t)LIST_LOCAL ? cnt : (uint32_t)LIST_LOCAL;
      const uint32_t nw = nloc < cap ? nloc : cap;
      for (uint32_t q = 0; q < nw; ++q) d.nbr[(size_t)q * d.n + i] = (int32_t)(uint32_t)keys(q);
      d.nn[i] = (int32_t)(cnt < cap ? cnt : cap);
      if (LANES > 1) d.nn_lanes[i] = lane_cnt;   /* meaningful when the list fits */
      if (cnt > (uint32_t)LIST_TAIL && cap > (uint32_t)LIST_TAIL)
        d.long_q[atomicAdd(&d.ctl->long_n, 1u)] = i;
      d.ref[i] = make_float2(p.x, p.y);
#undef keys
    }
    d.pos[i] = p;
    d.theta[i] = d.theta_alt[i];
    d.img[i] = d.img_alt[i];
    d.id[i] = d.id_alt[i];
    if (d.inv) d.inv[d.id_alt[i]] = (uint32_t)i;
  }
  if (with_list) {
    uint32_t m = __reduce_max_sync(0xffffffffu, cnt);
    if ((threadIdx.x & 31) == 0 && m > 0) {
      atomicMax(&d.ctl->max_nn, m);
      if (m > (uint32_t)d.cap) {
        atomicMax(&d.ctl->list_need, m);
        atomicExch(&d.ctl->frozen, 1u);
      }
    }
  }
  if (i == 0) atomicAdd(&d.ctl->n_rebuilds, 1u);
}

/* Sorts the list of particle i (m entries, m <= 32 R) by (id, slot): one
 * warp, R keys per lane, element e = r * 32 + lane, a bitonic network
 * (partners across lanes by shuffle, across r in registers).  Ids are
 * unique, so the order is the one the insertion sort of short lists gives. */
template <int R>
__device__ __forceinline__ void warp_sort_list(const SppConsts& k, const DevState& d, int i, int m) {
  const int lane = threadIdx.x & 31;
  unsigned long long key[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int q = r * 32 + lane;
    if (q < m) {
      int32_t j = d.nbr[(size_t)q * d.n + i];
      if (!spp_index_ok(d.ctl, j, d.n)) j = i;
      key[r] = ((unsigned long long)spp_list_order(&k, d.id_alt[j]) << 32) | (unsigned long long)(uint32_t)j;
    } else {
      key[r] = ~0ull;
    }
  }
#pragma unroll
  for (int size = 2; size <= 32 * R; size <<= 1) {
#pragma unroll
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      if (stride >= 32) {
        const int rs = stride >> 5;
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int rp = r ^ rs;
          if (rp > r) {
            const bool up = ((r * 32 + lane) & size) == 0;
            const unsigned long long a = key[r], b = key[rp];
            if (up ? (a > b) : (a < b)) {
              key[r] = b;
              key[rp] = a;
            }
          }
        }
      } else {
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const unsigned long long other = __shfl_xor_sync(0xffffffffu, key[r], stride);
          const bool up = ((r * 32 + lane) & size) == 0;
          const bool lower = (lane & stride) == 0;
          const bool keep_min = (up == lower);
          const unsigned long long lo = key[r] < other ? key[r] : other;
          const unsigned long long hi = key[r] < other ? other : key[r];
          key[r] = keep_min ? lo : hi;
        }
      }
    }
  }
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int q = r * 32 + lane;
    if (q < m) d.nbr[(size_t)q * d.n + i] = (int32_t)(uint32_t)key[r];
  }
}

/* Lists longer than LIST_LOCAL, queued by k_build_list: one warp per list
 * (grid-stride over the queue).  Lists beyond 512 entries, which only
 * extreme densities produce, are insertion-sorted by one lane. */
__global__ void __launch_bounds__(SPP_BLOCK) k_sort_long(SppConsts k, DevState d) {
  const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
  const uint32_t total = d.ctl->long_n;
  for (uint32_t w = (uint32_t)warp; w < total; w += (uint32_t)nwarps) {
    const int i = d.long_q[w];
    if (!spp_index_ok(d.ctl, i, d.n)) continue;
    const int m = d.nn[i];
    if (m <= 32) warp_sort_list<1>(k, d, i, m);
    else if (m <= 64) warp_sort_list<2>(k, d, i, m);
    else if (m <= 128) warp_sort_list<4>(k, d, i, m);
    else if (m <= 256) warp_sort_list<8>(k, d, i, m);
    else if (m <= 512) warp_sort_list<16>(k, d, i, m);
    else if ((threadIdx.x & 31) == 0) {
      for (int q = 1; q < m; ++q) {
        const int32_t j = d.nbr[(size_t)q * d.n + i];
        const uint32_t oj = spp_list_order(&k, d.id_alt[j]);
        int pos = q;
        while (pos > 0) {
          const int32_t prev = d.nbr[(size_t)(pos - 1) * d.n + i];
          if (spp_list_order(&k, d.id_alt[prev]) < oj) break;
          d.nbr[(size_t)pos * d.n + i] = prev;
          --pos;
        }
        d.nbr[(size_t)pos * d.n + i] = j;
      }
    }
  }
}

/* Unique pairs (by particle id) within r, through the cell list. */
__global__ void __launch_bounds__(SPP_BLOCK) k_pairs(SppConsts k, DevState d, float r2,
                                                     unsigned long long* counter, int32_t* pi,
                                                     int32_t* pj, long long cap) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  float4 p = d.pos[i];
  uint32_t idi = d.id[i];
  int cx, cy;
  cell_key(k, d, p.x, p.y, &cx, &cy);
  const int D = d.D;
  for (int oy = -1; oy <= 1; ++oy) {
    int ny = (cy + oy + D) % D;
    for (int ox = -1; ox <= 1; ++ox) {
      int nx = (cx + ox + D) % D;
      uint32_t kk = spp_morton((uint32_t)nx, (uint32_t)ny);
      uint32_t s0 = d.cell_start[kk], c = d.cell_count[kk];
      for (uint32_t j = s0; j < s0 + c; ++j) {
        uint32_t idj = d.id[j];
        if (idj <= idi) continue;
        float4 q = d.pos[j];
        float dx, dy;
        if (spp_sep(&k, p.x, p.y, q.x, q.y, &dx, &dy) < r2) {
          unsigned long long slot = atomicAdd(counter, 1ull);
          if ((long long)slot < cap) {
            pi[slot] = (int32_t)idi;
            pj[slot] = (int32_t)idj;
          }
        }
      }
    }
  }
}

__global__ void k_cells(SppConsts k, DevState d, int D, int rule, int32_t* cx, int32_t* cy) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  float4 p = d.pos[i];
  uint32_t id = d.id[i];
  cx[id] = spp_cell_coord(p.x, k.L, k.L2, D, rule);
  cy[id] = spp_cell_coord(p.y, k.L, k.L2, D, rule);
}

/* Places the uploaded state (particle-id order) and checks it: the smallest
 * index with a non-finite value and the smallest with a position outside
 * [-L, L) go to the control block, which the host reads before it accepts
 * the upload.  Invalid values stay bounded in what follows: cell
 * coordinates are clamped, and comparisons with NaN are false. */
__global__ void k_init_state(SppConsts k, DevState d, const float* __restrict__ x, const float* __restrict__ y,
                             const float* __restrict__ th, const int32_t* __restrict__ img_xy) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  const float xi = x[i], yi = y[i], ti = th[i];
  if (!isfinite(xi) || !isfinite(yi) || !isfinite(ti)) atomicMin(&d.ctl->bad_nonfinite, (uint32_t)i);
  else if (!k.closed && !(xi >= -k.L && xi < k.L && yi >= -k.L && yi < k.L))
    atomicMin(&d.ctl->bad_range, (uint32_t)i);  /* a closed box has no wrap to undo: any finite position */
  float s, c;
  spp_sincosf(ti, &s, &c);
  d.pos[i] = make_float4(xi, yi, c, s);
  d.theta[i] = ti;
  d.img[i] = img_xy ? make_int2(img_xy[i], img_xy[d.n + i]) : make_int2(0, 0);
  d.id[i] = (uint32_t)i;
}

__global__ void k_gather_state(DevState d, float* x, float* y, float* th, int32_t* img_xy) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= d.n) return;
  uint32_t id = d.id[i];
  float4 p = d.pos[i];
  x[id] = p.x;
  y[id] = p.y;
  th[id] = d.theta[i];
  const int2 g = d.img[i];
  img_xy[id] = g.x;
  img_xy[d.n + id] = g.y;
}

inline int blocks_for(int n, int b = SPP_BLOCK) { return (n + b - 1) / b; }

}  // namespace

void launch_bin_count(const SppConsts& k, const DevState& d, cudaStream_t s, int64_t* launches) {
  if (d.n == 0) return;
  k_bin_count<<<blocks_for(d.n), SPP_BLOCK, 0, s>>>(k, d);
  if (launches) *launches += 1;
}

void launch_scan_u32(const uint32_t* in, uint32_t n, uint32_t* block_tmp, uint32_t* out,
                     cudaStream_t s, int64_t* launches) {
  uint32_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  k_scan_reduce<<<nb, SCAN_THREADS, 0, s>>>(in, n, block_tmp);
  k_scan_top<<<1, SCAN_THREADS, 0, s>>>(block_tmp, nb);
  k_scan_apply<<<nb, SCAN_THREADS, 0, s>>>(in, n, block_tmp, out);
  if (launches) *launches += 3;
}

uint32_t scan_max_elements() { return (uint32_t)SCAN_TILE * (uint32_t)SCAN_TILE; }

void launch_scan(const DevState& d, cudaStream_t s, int64_t* launches) {
  launch_scan_u32(d.cell_count, d.n_keys, d.scan_tmp, d.cell_start, s, launches);
}

void launch_scatter(const DevState& d, cudaStream_t s, int64_t* launches) {
  if (d.n == 0) return;
  k_scatter<<<blocks_for(d.n), SPP_BLOCK, 0, s>>>(d);
  if (launches) *launches += 1;
}

void launch_build_list(const SppConsts& k, const DevState& d, int with_list, cudaStream_t s,
                       int64_t* launches) {
  if (d.n == 0) return;
  if (with_list && k.lanes == SPP_GATHER_LANES)
    k_build_list<SPP_GATHER_LANES><<<blocks_for(d.n), SPP_BLOCK, 0, s>>>(k, d, with_list);
  else
    k_build_list<1><<<blocks_for(d.n), SPP_BLOCK, 0, s>>>(k, d, with_list);
  if (launches) *launches += 1;
  if (with_list) {
    /* 8 warps per block, 8 blocks per SM of a 152-SM part, looping over
     * the queue */
    int nb = (d.n + 7) / 8;
    if (nb > 1216) nb = 1216;
    k_sort_long<<<nb, SPP_BLOCK, 0, s>>>(k, d);
    if (launches) *launches += 1;
  }
}

void launch_pairs_count(const SppConsts& k, const DevState& d, float r2, unsigned long long* counter,
                        int32_t* pi, int32_t* pj, long long cap, cudaStream_t s) {
  if (d.n == 0) return;
  k_pairs<<<blocks_for(d.n), SPP_BLOCK, 0, s>>>(k, d, r2, counter, pi, pj, cap);
}

void launch_cells(const SppConsts& k, const DevState& d, int D, int rule, int32_t* cx, int32_t* cy,
                  cudaStream_t s) {
  if (d.n == 0) return;
  k_cells<<<blocks_for(d.n), SPP_BLOCK, 0, s>>>(k, d, D, rule, cx, cy);
}

void launch_init_state(const SppConsts& k, const DevState& d, const float* x, const float* y,
                       const float* th, const int32_t* img_xy, cudaStream_t s) {
  if (d.n == 0) return;
  k_init_state<<<blocks_for(d.n), SPP_BLOCK, 0, s>>>(k, d, x, y, th, img_xy);
}

void launch_gather_state(const SppConsts& k, const DevState& d, float* x, float* y, float* th,
                         int32_t* img_xy, cudaStream_t s) {
  (void)k;
  if (d.n == 0) return;
  k_gather_state<<<blocks_for(d.n), SPP_BLOCK, 0, s>>>(d, x, y, th, img_xy);
}
