/*
 * noalloc.cu -- neighbour-pair search that allocates no memory.
 *
 * spp_pairs() works on a system handle whose cell list lives in buffers the
 * library allocated with cudaMalloc.  Some callers cannot allocate: code that
 * runs while another component owns the device's memory budget (a host
 * framework with its own pool, a fixed-footprint embedded deployment), or a
 * latency-critical loop in which cudaMalloc/cudaFree would synchronise the
 * device.  spp_pairs_noalloc() serves them: the caller passes its own device
 * buffers for the positions and the results, and all scratch (cell counts,
 * cell starts, per-particle keys, ranks and the cell-ordered copy) lives in
 * the file-scope array below, which exists once per GPU that loads this
 * library, for the life of the process.
 *
 * Shared state: every call uses the same scratch array and leaves its
 * contents behind; each call clears what must start at zero.  Calls that
 * overlap on the GPU (different streams, or different host threads without
 * ordering) race on it and must be serialised by the caller.
 */
#include <cuda.h>   /* CUcontext and CUresult types only: the two driver entry points below
                       come from the runtime (cudaGetDriverEntryPointByVersion) */
#include <cmath>
#include <mutex>
#include <string>
#include "spp_internal.cuh"

namespace {

constexpr int NA_MAX_N = SPP_NOALLOC_MAX_N;
constexpr int NA_MAX_SIDE = SPP_NOALLOC_MAX_CELLS_PER_SIDE;
constexpr int NA_MAX_KEYS = NA_MAX_SIDE * NA_MAX_SIDE;  /* Morton keys of 8 + 8 bits */
constexpr int NA_SCAN_THREADS = 1024;

/* Layout of the scratch array (all offsets multiples of 256 bytes). */
struct NaScratch {
  unsigned long long count_pairs;         /* pairs found (all, even beyond cap) */
  unsigned long long pad0[31];
  uint32_t cell_count[NA_MAX_KEYS];
  uint32_t cell_start[NA_MAX_KEYS];
  uint32_t key[NA_MAX_N];
  uint32_t rank[NA_MAX_N];
  uint32_t perm[NA_MAX_N];                /* cell-ordered slot -> particle index */
  float2 sorted[NA_MAX_N];                /* cell-ordered positions */
};

static __device__ __align__(256) NaScratch g_na_scratch;

/* Host-side device addresses of g_na_scratch, one per CUDA context.  Each
 * context that loads this library holds its own copy of the array, and a
 * context created after cudaDeviceReset may place it elsewhere, so the
 * address is keyed by the context's unique id (cuCtxGetId: ids are never
 * reused within a process), not by the device ordinal.  The table is read
 * and written under g_na_mu. */
constexpr int NA_MAX_CONTEXTS = 64;
struct NaEntry {
  unsigned long long ctx_id;
  NaScratch* ptr;
};
std::mutex g_na_mu;
NaEntry g_na_cache[NA_MAX_CONTEXTS];
int g_na_used = 0;
int g_na_next = 0;   /* slot replaced next once the table is full */

typedef CUresult(CUDAAPI* NaCtxGetCurrent)(CUcontext*);
typedef CUresult(CUDAAPI* NaCtxGetId)(CUcontext, unsigned long long*);

/* Unique id of the calling thread's current context; false if there is none
 * (the runtime has not made one current on this thread yet) or the driver
 * does not offer the entry points. */
bool na_current_context(unsigned long long* id) {
  static std::once_flag once;
  static NaCtxGetCurrent get_current = nullptr;
  static NaCtxGetId get_id = nullptr;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<NaCtxGetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<NaCtxGetId>(f);
    cudaGetLastError();
  });
  if (!get_current || !get_id) return false;
  CUcontext c = nullptr;
  if (get_current(&c) != CUDA_SUCCESS || !c) return false;
  return get_id(c, id) == CUDA_SUCCESS;
}

NaScratch* na_lookup(unsigned long long id) {
  std::lock_guard<std::mutex> g(g_na_mu);
  for (int i = 0; i < g_na_used; ++i)
    if (g_na_cache[i].ctx_id == id) return g_na_cache[i].ptr;
  return nullptr;
}

void na_remember(unsigned long long id, NaScratch* ptr) {
  std::lock_guard<std::mutex> g(g_na_mu);
  for (int i = 0; i < g_na_used; ++i)
    if (g_na_cache[i].ctx_id == id) { g_na_cache[i].ptr = ptr; return; }
  if (g_na_used < NA_MAX_CONTEXTS) {
    g_na_cache[g_na_used++] = {id, ptr};
  } else {
    g_na_cache[g_na_next] = {id, ptr};
    g_na_next = (g_na_next + 1) % NA_MAX_CONTEXTS;
  }
}

__global__ void k_na_clear(NaScratch* s, int n_keys) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_keys) s->cell_count[i] = 0u;
  if (i == 0) s->count_pairs = 0ull;
}

__global__ void k_na_count(NaScratch* s, const float* __restrict__ x, const float* __restrict__ y,
                           int n, float L, float L2, int D) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int cx = spp_cell_coord(x[i], L, L2, D, SPP_BIN_GEOMETRIC);
  const int cy = spp_cell_coord(y[i], L, L2, D, SPP_BIN_GEOMETRIC);
  const uint32_t key = spp_morton((uint32_t)cx, (uint32_t)cy);
  const unsigned mask = __activemask();
  const unsigned peers = __match_any_sync(mask, key);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(&s->cell_count[key], (uint32_t)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  s->key[i] = key;
  s->rank[i] = base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
}

/* Exclusive scan of n_keys <= 65536 counts in one block: each thread sums a
 * contiguous run, the block scans the run totals, each thread writes its run. */
__global__ void __launch_bounds__(NA_SCAN_THREADS) k_na_scan(NaScratch* s, int n_keys) {
  __shared__ uint32_t warp_sums[32];
  const int per = (n_keys + NA_SCAN_THREADS - 1) / NA_SCAN_THREADS;
  const int b0 = threadIdx.x * per;
  uint32_t local = 0;
  for (int q = 0; q < per; ++q)
    if (b0 + q < n_keys) local += s->cell_count[b0 + q];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = local;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = warp_sums[lane];
    uint32_t wi = w;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    warp_sums[lane] = wi - w;
  }
  __syncthreads();
  uint32_t run = incl - local + warp_sums[warp];
  for (int q = 0; q < per; ++q) {
    if (b0 + q < n_keys) {
      s->cell_start[b0 + q] = run;
      run += s->cell_count[b0 + q];
    }
  }
}

__global__ void k_na_scatter(NaScratch* s, const float* __restrict__ x, const float* __restrict__ y,
                             int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t dst = s->cell_start[s->key[i]] + s->rank[i];
  s->perm[dst] = (uint32_t)i;
  s->sorted[dst] = make_float2(x[i], y[i]);
}

/* One thread per cell-ordered slot; pairs (i < j by particle index) within r
 * under the kernels' FP32 predicate. */
__global__ void k_na_pairs(NaScratch* s, SppConsts k, int n, int D, float r2, int32_t* pi,
                           int32_t* pj, long long cap) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const uint32_t i = s->perm[t];
  const float2 p = s->sorted[t];
  const int cx = spp_cell_coord(p.x, k.L, k.L2, D, SPP_BIN_GEOMETRIC);
  const int cy = spp_cell_coord(p.y, k.L, k.L2, D, SPP_BIN_GEOMETRIC);
  for (int oy = -1; oy <= 1; ++oy) {
    const int ny = (cy + oy + D) % D;
    for (int ox = -1; ox <= 1; ++ox) {
      const int nx = (cx + ox + D) % D;
      const uint32_t kk = spp_morton((uint32_t)nx, (uint32_t)ny);
      const uint32_t s0 = s->cell_start[kk], c = s->cell_count[kk];
      for (uint32_t u = s0; u < s0 + c; ++u) {
        const uint32_t j = s->perm[u];
        if (j <= i) continue;
        const float2 q = s->sorted[u];
        float dx, dy;
        if (spp_sep(&k, p.x, p.y, q.x, q.y, &dx, &dy) < r2) {
          const unsigned long long slot = atomicAdd(&s->count_pairs, 1ull);
          if ((long long)slot < cap) {
            pi[slot] = (int32_t)i;
            pj[slot] = (int32_t)j;
          }
        }
      }
    }
  }
}

__global__ void k_na_publish(const NaScratch* s, int64_t* count_out) {
  *count_out = (int64_t)s->count_pairs;
}

int na_fail(int status, const std::string& m) {
  spp_internal_set_error(m.c_str());
  return status;
}

}  // namespace

extern "C" int spp_pairs_noalloc(const float* x, const float* y, int n, double L, double r,
                                 int32_t* pi, int32_t* pj, int64_t cap, int64_t* count,
                                 void* stream) {
  if (!x || !y || !count || (cap > 0 && (!pi || !pj)) || cap < 0)
    return na_fail(SPP_ERR_INVALID, "spp_pairs_noalloc: NULL or negative argument");
  if (n < 1 || n > NA_MAX_N)
    return na_fail(SPP_ERR_INVALID, "spp_pairs_noalloc: n must be in [1, " +
                                        std::to_string(NA_MAX_N) + "], got " + std::to_string(n));
  if (!(L > 0) || !(r > 0))
    return na_fail(SPP_ERR_INVALID, "spp_pairs_noalloc: L and r must be > 0");
  int D = (int)std::floor(2.0 * L / (r * 1.001));
  if (D > NA_MAX_SIDE) D = NA_MAX_SIDE;  /* wider cells only add candidates */
  if (D < 3)
    return na_fail(SPP_ERR_INVALID, "spp_pairs_noalloc: box too small for the cell grid (2L/r < 3)");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  /* The scratch array's device address in the current context: known from an
   * earlier call in this context, else looked up now with cudaGetSymbolAddress
   * (which makes the device's primary context current if the thread has none;
   * no allocation is involved).  The lookup may load this library's device
   * code, which a stream capture must not see: inside a capture only an
   * address found earlier in the same context is used. */
  unsigned long long ctx = 0;
  bool have_ctx = na_current_context(&ctx);
  NaScratch* s = have_ctx ? na_lookup(ctx) : nullptr;
  cudaError_t e;
  if (!s) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
      cudaGetLastError();
      cs = cudaStreamCaptureStatusActive;   /* cannot tell: treat as capturing */
    }
    if (cs != cudaStreamCaptureStatusNone)
      return na_fail(SPP_ERR_INVALID, "spp_pairs_noalloc: the first call in a CUDA context sets up the "
                                      "scratch address and must come before any stream capture");
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_na_scratch);
    if (e != cudaSuccess)
      return na_fail(SPP_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    s = reinterpret_cast<NaScratch*>(p);
    if (!have_ctx) have_ctx = na_current_context(&ctx);
    if (have_ctx) na_remember(ctx, s);
  }
  int bits = 0;
  while ((1 << bits) < D) ++bits;
  const int n_keys = 1 << (2 * bits);
  SppParams p;
  spp_params_init(&p, SPP_MODEL_VICSEK);
  p.n = n;
  p.L = L;
  SppConsts k;
  spp_consts_from_params(&k, &p);
  const int B = 256;
  k_na_clear<<<(n_keys + B - 1) / B, B, 0, st>>>(s, n_keys);
  k_na_count<<<(n + B - 1) / B, B, 0, st>>>(s, x, y, n, k.L, k.L2, D);
  k_na_scan<<<1, NA_SCAN_THREADS, 0, st>>>(s, n_keys);
  k_na_scatter<<<(n + B - 1) / B, B, 0, st>>>(s, x, y, n);
  k_na_pairs<<<(n + B - 1) / B, B, 0, st>>>(s, k, n, D, (float)(r * r), pi, pj, (long long)cap);
  k_na_publish<<<1, 1, 0, st>>>(s, count);
  e = cudaGetLastError();
  if (e != cudaSuccess) return na_fail(SPP_ERR_CUDA, cudaGetErrorString(e));
  return SPP_OK;
}
