/*
 * kernels_lyap.cu -- tangent dynamics and FP64 renormalisation on sm_103a.
 *
 * The reference estimates Lyapunov exponents with k finite perturbations of
 * the full dynamics (Benettin clones, parallel/lyapunovbox.h:128-194): each
 * clone is a whole copy of the system, evolved and differenced against the
 * base run, then Gram-Schmidt renormalised (shared/vector-set.h:118-127).
 * Here the k tangent vectors are advanced by the linearised integrator next
 * to the base trajectory:
 *   k_tangent_stage: after each base stage, one thread per (particle,
 *     vector) gathers cos(th_j - th_i) of its neighbours (same id-sorted
 *     list, FP32 sums in id order) and advances its vector through the JVP
 *     of that stage.
 *     Tangent vectors are stored by particle id, [k][x|y|th][n], so the
 *     cell reordering at list rebuilds does not touch them.
 *   Renormalisation every m steps, in FP64: a Cholesky-QR pass, done twice
 *   (the second pass restores orthogonality to working precision):
 *     k_gram     deterministic block partials of the k x k Gram matrix
 *     k_chol     one thread: sum of the partials in block order, Cholesky,
 *                R^{-1}, log R_aa added to the log-stretch sums
 *     k_apply    V <- V R^{-1}
 *   The Q and R are those of Gram-Schmidt on the same vectors; the FP64
 *   accumulation is what the stability of the renormalisation needs.
 */
#include "spp_internal.cuh"
#include "spp_lyap.cuh"

namespace {

/* Vectors are handled in groups of 4: uslot holds, per slot, the heading
 * components of all vectors padded to a multiple of 4, so a neighbour's
 * components for one group are one float4 load. */
constexpr int TAN_GROUP = 4;
constexpr int TAN_BLOCK = 128;
constexpr int TAN_LOADS = 3;
#ifndef TAN_PIPE
#define TAN_PIPE 1   /* list entries loaded one group ahead in the neighbour walk */
#endif

__host__ __device__ inline int tan_padded(int K) { return (K + TAN_GROUP - 1) / TAN_GROUP * TAN_GROUP; }

/* The heading components of the stage input, gathered into slot order:
 * uslot[i][v] = u[v][theta][id_i] (v < K; the padding stays 0). */
__global__ void __launch_bounds__(SPP_BLOCK) k_tangent_gather(DevState d, int K, const float* uin, float* uslot) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int v = blockIdx.y;
  if (i >= d.n) return;
  uslot[(size_t)i * tan_padded(K) + v] = uin[(size_t)(v * 3 + 2) * d.n + d.id[i]];
}

/* One thread per (particle slot, group of 4 tangent vectors), blockIdx.y the
 * group: a small system (N = 16,384) still spreads over the GPU, a
 * neighbour's components for the group are one float4 load, and the sum over
 * neighbours for each vector is the same FP32 expression in the same
 * (id-sorted list) order as with one vector per thread.  With LANES = 4
 * (k.lanes) four threads share a particle as in k_abp_stage: lane r sums
 * the neighbours with id % 4 == r and the lane sums combine as
 * (p0 + p1) + (p2 + p3). */
template <int LANES>
__global__ void __launch_bounds__(TAN_BLOCK) k_tangent_stage(SppConsts k, DevState d, LyapState L, TanStage t) {
  const int tg = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = tg / LANES;
  const int lane_r = tg % LANES;
  const int v0 = blockIdx.y * TAN_GROUP;
  if (i >= d.n || d.ctl->frozen) return;
  const int n = d.n;
  const int KP = tan_padded(L.K);
  const uint32_t idi = d.id[i];
  const float4 pi = t.cur[i];
  const float4 ui = *reinterpret_cast<const float4*>(t.us_in + (size_t)i * KP + v0);
  float acc[TAN_GROUP] = {0.0f, 0.0f, 0.0f, 0.0f};
  /* with one vector per lane, that vector's stage inputs (stored by particle
   * id, so scattered) are loaded first: their latency overlaps the
   * neighbour walk.  Only this thread touches these elements. */
  const int vmine = v0 + lane_r;
  float pre_t0[3] = {0.0f, 0.0f, 0.0f}, pre_a[3] = {0.0f, 0.0f, 0.0f};
  if (LANES == TAN_GROUP && vmine < L.K) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const size_t e = (size_t)(vmine * 3 + c) * n + idi;
      pre_t0[c] = L.t0[e];
      if (t.stage != 0) pre_a[c] = L.acc[e];
    }
  }
  int q_begin = 0, q_end = d.nn[i];
  if (LANES > 1) {
    const unsigned long long lc = d.nn_lanes[i];
    for (int r = 0; r < lane_r; ++r) q_begin += (int)((lc >> (16 * r)) & 0xffffull);
    q_end = q_begin + (int)((lc >> (16 * lane_r)) & 0xffffull);
  }
  const int32_t* __restrict__ nb = d.nbr + i;
  /* list entries, then the neighbours' states and components, are loaded
   * TAN_LOADS at a time (independent loads in flight); the terms are added
   * in list order */
#if TAN_PIPE
  /* list entries one group ahead, as in k_abp_stage */
  int jn[TAN_LOADS];
#pragma unroll
  for (int w = 0; w < TAN_LOADS; ++w) jn[w] = q_begin + w < q_end ? __ldg(nb + (size_t)(q_begin + w) * n) : i;
#endif
  for (int q0 = q_begin; q0 < q_end; q0 += TAN_LOADS) {
    int jg[TAN_LOADS];
#pragma unroll
    for (int w = 0; w < TAN_LOADS; ++w) {
#if TAN_PIPE
      jg[w] = jn[w];
#else
      jg[w] = q0 + w < q_end ? __ldg(nb + (size_t)(q0 + w) * n) : i;
#endif
      if (!spp_index_ok(d.ctl, jg[w], n)) jg[w] = i;
    }
    float4 pg[TAN_LOADS], ug[TAN_LOADS];
#pragma unroll
    for (int w = 0; w < TAN_LOADS; ++w) {
      pg[w] = __ldg(t.cur + jg[w]);
      ug[w] = __ldg(reinterpret_cast<const float4*>(t.us_in + (size_t)jg[w] * KP + v0));
    }
#if TAN_PIPE
#pragma unroll
    for (int w = 0; w < TAN_LOADS; ++w) {
      const int q = q0 + TAN_LOADS + w;
      jn[w] = q < q_end ? __ldg(nb + (size_t)q * n) : i;
    }
#endif
#pragma unroll
    for (int w = 0; w < TAN_LOADS; ++w) {
      if (q0 + w < q_end) {
        float dx, dy;
        const float d2 = spp_sep(&k, pi.x, pi.y, pg[w].x, pg[w].y, &dx, &dy);
        if (d2 < k.ral2) {
          const float cij = spp_tangent_coupling(pi.z, pi.w, pg[w].z, pg[w].w);
          acc[0] = acc[0] + cij * (ug[w].x - ui.x);
          acc[1] = acc[1] + cij * (ug[w].y - ui.y);
          acc[2] = acc[2] + cij * (ug[w].z - ui.z);
          acc[3] = acc[3] + cij * (ug[w].w - ui.w);
        }
      }
    }
  }
  if (LANES > 1) {
    const unsigned gmask = ((1u << LANES) - 1u) << ((threadIdx.x & 31) & ~(LANES - 1));
#pragma unroll
    for (int o = 1; o < LANES; o <<= 1)
#pragma unroll
      for (int u = 0; u < TAN_GROUP; ++u) acc[u] = acc[u] + __shfl_xor_sync(gmask, acc[u], o);
  }
  /* every lane now holds the four sums: with four lanes, lane r advances
   * vector v0 + r; with one, the thread advances all four */
  const float gp = k.g * k.one_minus_alpha_over_pi;
  const float uiv[TAN_GROUP] = {ui.x, ui.y, ui.z, ui.w};
#pragma unroll
  for (int u = 0; u < TAN_GROUP; ++u) {
    if (LANES == TAN_GROUP && u != lane_r) continue;
    const int v = v0 + u;
    if (v >= L.K) break;
    const float slope[3] = {-k.v0 * pi.w * uiv[u], k.v0 * pi.z * uiv[u], gp * acc[u]};
    float t0v[3], av[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const size_t e = (size_t)(v * 3 + c) * n + idi;
      t0v[c] = LANES == TAN_GROUP ? pre_t0[c] : L.t0[e];
      av[c] = LANES == TAN_GROUP ? pre_a[c] : (t.stage == 0 ? 0.0f : L.acc[e]);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const size_t e = (size_t)(v * 3 + c) * n + idi;
      float t0 = t0v[c];
      float a = av[c];
      float uo = 0.0f;
      spp_tangent_stage_update(&k, t.stage, t.nstages, slope[c], &t0, &a, &uo);
      if (t.stage == t.nstages - 1) {
        L.t0[e] = t0;
      } else {
        t.uout[e] = uo;
        /* the next stage's heading component, straight into slot order */
        if (c == 2) t.us_out[(size_t)i * KP + v] = uo;
      }
      if (t.nstages == 4 && t.stage < 3) L.acc[e] = a;
    }
  }
}

template <int K>
__global__ void __launch_bounds__(SPP_GRAM_THREADS) k_gram(const float* __restrict__ V, int len,
                                                            double* partial) {
  double g[SPP_GRAM_ENTRIES];
#pragma unroll
  for (int q = 0; q < K * (K + 1) / 2; ++q) g[q] = 0.0;
  const int stride = SPP_GRAM_BLOCKS * SPP_GRAM_THREADS;
  for (int e = blockIdx.x * SPP_GRAM_THREADS + threadIdx.x; e < len; e += stride) {
    double v[K];
#pragma unroll
    for (int a = 0; a < K; ++a) v[a] = (double)V[(size_t)a * len + e];
#pragma unroll
    for (int a = 0; a < K; ++a)
#pragma unroll
      for (int b = 0; b <= a; ++b) g[a * (a + 1) / 2 + b] = g[a * (a + 1) / 2 + b] + v[a] * v[b];
  }
  __shared__ double warp_part[SPP_GRAM_THREADS / 32][SPP_GRAM_ENTRIES];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < K * (K + 1) / 2; ++q) {
    double x = g[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = x + __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) warp_part[warp][q] = x;
  }
  __syncthreads();
  if (threadIdx.x < K * (K + 1) / 2) {
    double x = 0.0;
    for (int w = 0; w < SPP_GRAM_THREADS / 32; ++w) x = x + warp_part[w][threadIdx.x];
    partial[(size_t)blockIdx.x * SPP_GRAM_ENTRIES + threadIdx.x] = x;
  }
}

/* One block of SPP_GRAM_ENTRIES threads: thread q sums entry q of the block
 * partials in block order; thread 0 factors. */
__global__ void k_chol(int K, const double* partial, double* rinv, double* log_stretch,
                       int accumulate, uint32_t* error) {
  __shared__ double Gs[SPP_GRAM_ENTRIES];
  const int q = threadIdx.x;
  if (q < K * (K + 1) / 2) {
    double x = 0.0;
    for (int b = 0; b < SPP_GRAM_BLOCKS; ++b) x = x + partial[(size_t)b * SPP_GRAM_ENTRIES + q];
    Gs[q] = x;
  }
  __syncthreads();
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double G[SPP_GRAM_ENTRIES];
  for (int e = 0; e < K * (K + 1) / 2; ++e) G[e] = Gs[e];
  double lr[SPP_LYAP_MAX];
  if (spp_cholesky_inverse(K, G, rinv, lr)) {
    *error = 1u;
    for (int a = 0; a < SPP_LYAP_MAX * SPP_LYAP_MAX; ++a) rinv[a] = (a % (SPP_LYAP_MAX + 1)) == 0;
    return;
  }
  if (accumulate)
    for (int a = 0; a < K; ++a) log_stretch[a] = log_stretch[a] + lr[a];
}

template <int K>
__global__ void __launch_bounds__(SPP_BLOCK) k_apply(float* V, int len, const double* __restrict__ rinv) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= len) return;
  double v[K];
#pragma unroll
  for (int a = 0; a < K; ++a) v[a] = (double)V[(size_t)a * len + e];
#pragma unroll
  for (int a = 0; a < K; ++a) {
    double x = 0.0;
#pragma unroll
    for (int b = 0; b <= a; ++b) x = x + v[b] * rinv[b * SPP_LYAP_MAX + a];
    V[(size_t)a * len + e] = (float)x;
  }
}

/* Gaussian N(0, 1) entries from the Philox tangent stream: component c of
 * vector v of particle id uses counter (id, v * 3 + c, SPP_RNG_TANGENT). */
__global__ void k_tangent_init(float* V, int K, int n, uint64_t seed, uint32_t system) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= K * 3 * n) return;
  const int id = e % n;
  const int vc = e / n;
  const spp_u32x4 r = spp_draw(seed, system, (uint32_t)id, (uint32_t)vc, SPP_RNG_TANGENT);
  V[e] = spp_normal_f(r.v[0], r.v[1]);
}

}  // namespace

size_t tangent_slot_floats(int K, int n) { return (size_t)tan_padded(K) * (size_t)n; }

void launch_tangent_init(const LyapState& L, uint64_t seed, uint32_t system, cudaStream_t s) {
  const int tot = L.K * 3 * L.n;
  k_tangent_init<<<(tot + SPP_BLOCK - 1) / SPP_BLOCK, SPP_BLOCK, 0, s>>>(L.t0, L.K, L.n, seed, system);
}

#define SPP_K_DISPATCH(K, CALL) \
  switch (K) {                  \
    case 1: CALL(1); break;     \
    case 2: CALL(2); break;     \
    case 3: CALL(3); break;     \
    case 4: CALL(4); break;     \
    case 5: CALL(5); break;     \
    case 6: CALL(6); break;     \
    case 7: CALL(7); break;     \
    default: CALL(8); break;    \
  }

void launch_tangent_stage(const SppConsts& k, const DevState& d, const LyapState& L, int stage,
                          int nstages, const float4* cur, cudaStream_t s, int64_t* launches) {
  TanStage t;
  t.cur = cur;
  t.stage = stage;
  t.nstages = nstages;
  /* stage inputs: stage 0 reads t0; RK2/RK4 alternate ua/ub */
  float* ua = L.ua;
  float* ub = L.ub;
  t.uin = stage == 0 ? L.t0 : ((stage & 1) ? ua : ub);
  t.uout = (stage & 1) ? ub : ua;
  const size_t sf = tangent_slot_floats(L.K, d.n);
  t.us_in = L.uslot + (size_t)(stage & 1) * sf;
  t.us_out = stage < nstages - 1 ? L.uslot + (size_t)((stage + 1) & 1) * sf : nullptr;
  if (stage == 0) {
    /* the step's start vectors (by particle id) into slot order; later
     * stages get theirs from the stage before */
    const dim3 ggrid((unsigned)((d.n + SPP_BLOCK - 1) / SPP_BLOCK), (unsigned)L.K);
    k_tangent_gather<<<ggrid, SPP_BLOCK, 0, s>>>(d, L.K, t.uin, L.uslot);
    if (launches) *launches += 1;
  }
  const int lanes = k.lanes;
  const dim3 tgrid((unsigned)(((size_t)d.n * lanes + TAN_BLOCK - 1) / TAN_BLOCK),
                   (unsigned)(tan_padded(L.K) / TAN_GROUP));
  if (lanes == SPP_GATHER_LANES)
    k_tangent_stage<SPP_GATHER_LANES><<<tgrid, TAN_BLOCK, 0, s>>>(k, d, L, t);
  else
    k_tangent_stage<1><<<tgrid, TAN_BLOCK, 0, s>>>(k, d, L, t);
  if (launches) *launches += 1;
}

void launch_renormalize(const LyapState& L, int accumulate, cudaStream_t s, int64_t* launches) {
  const int len = 3 * L.n;
  const int nb = (len + SPP_BLOCK - 1) / SPP_BLOCK;
  for (int pass = 0; pass < 2; ++pass) {
#define SPP_GRAM(KK) k_gram<KK><<<SPP_GRAM_BLOCKS, SPP_GRAM_THREADS, 0, s>>>(L.t0, len, L.partial)
    SPP_K_DISPATCH(L.K, SPP_GRAM)
#undef SPP_GRAM
    k_chol<<<1, SPP_GRAM_ENTRIES, 0, s>>>(L.K, L.partial, L.rinv, L.log_stretch, accumulate, L.error);
#define SPP_APPLY(KK) k_apply<KK><<<nb, SPP_BLOCK, 0, s>>>(L.t0, len, L.rinv)
    SPP_K_DISPATCH(L.K, SPP_APPLY)
#undef SPP_APPLY
  }
  if (launches) *launches += 6;
}
