/*
 * mlp.cu -- ensemble MLP surrogate of the sweep: forward, backward and Adam.
 *
 * No counterpart in the reference (its sweeps run every point to the end,
 * serial/mpi-main.cpp:157-176).  The surrogate maps a point's parameters and
 * the moments of its polarization over a short start-up window to its
 * stationary polarization; an ensemble of E independent networks gives a
 * spread that decides whether a point may be retired early.
 *
 * Network per member: in (<= 16) -> 128 -> 128 -> 1, GELU (tanh form)
 * after both hidden layers.  Weights are held in FP32 (Adam's master copy)
 * and in BF16; forward and backward read the BF16 copy and accumulate in
 * FP32.  Parameter layout of one member (P floats):
 *   W1[128][in] b1[128] W2[128][128] b2[128] W3[128] b3
 * The problem is tiny (E x B x ~17k MACs per pass), so the kernels are plain
 * FP32-FMA code: one block of 128 threads per (member, sample chunk),
 * gradients summed per parameter over the samples in a fixed order (no
 * atomics, hence reproducible), Adam elementwise.
 */
#include <cuda_bf16.h>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include "spp_internal.cuh"

namespace {

constexpr int H = 128;
constexpr int MAX_IN = 16;
constexpr int CHUNK = 16;  /* samples per forward/backward block */

__host__ __device__ inline int n_params(int in) { return H * in + H + H * H + H + H + 1; }
__host__ __device__ inline int off_b1(int in) { return H * in; }
__host__ __device__ inline int off_w2(int in) { return H * in + H; }
__host__ __device__ inline int off_b2(int in) { return H * in + H + H * H; }
__host__ __device__ inline int off_w3(int in) { return H * in + H + H * H + H; }
__host__ __device__ inline int off_b3(int in) { return H * in + H + H * H + H + H; }

__device__ __forceinline__ float gelu(float z, float* dgelu) {
  const float c = 0.7978845608028654f;  /* sqrt(2/pi) */
  const float u = c * fmaf(0.044715f * z, z * z, z);
  const float t = tanhf(u);
  if (dgelu) *dgelu = 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * c * fmaf(3.0f * 0.044715f, z * z, 1.0f);
  return 0.5f * z * (1.0f + t);
}

struct MlpDev {
  int E, in, B;
  const __nv_bfloat16* w;   /* [E][P] BF16 copy */
  const float* x;           /* [B][in] */
  const float* t;           /* [B] targets */
  const float* sw;          /* [E][B] sample weights, each member's summing to 1 */
  float* z1;                /* [E][B][H] pre-activations */
  float* z2;
  float* h1;                /* [E][B][H] activations gelu(z) */
  float* h2;
  float* y;                 /* [E][B] */
  float* dz1;               /* [E][B][H] */
  float* dz2;
  float* dy;                /* [E][B] */
};

/* W2 of one member in shared memory, row-major with a padded row stride of
 * H + 2 BF16 (65 words): a warp reading a column (forward: row j per thread)
 * or a row (backward: column j per thread) hits 32 different banks. */
constexpr int W2S = H + 2;

__device__ __forceinline__ void load_w2(const __nv_bfloat16* w2, __nv_bfloat16* w2s) {
  for (int idx = threadIdx.x; idx < H * H; idx += blockDim.x) w2s[(idx / H) * W2S + (idx % H)] = w2[idx];
}

/* One block per (member, chunk of CHUNK samples), one thread per hidden unit.
 * The layer sums run over k in order for every sample, as FP32 FMAs on the
 * BF16 weights. */
__global__ void __launch_bounds__(H) k_mlp_forward(MlpDev m) {
  const int e = blockIdx.y;
  const int s0 = blockIdx.x * CHUNK;
  const int j = threadIdx.x;
  const int in = m.in, P = n_params(in);
  const __nv_bfloat16* w = m.w + (size_t)e * P;
  __shared__ __nv_bfloat16 w2s[H * W2S];
  __shared__ float h1s[CHUNK][H];
  __shared__ float red[CHUNK][H / 32];
  load_w2(w + off_w2(in), w2s);
  const int nq = m.B - s0 < CHUNK ? m.B - s0 : CHUNK;
  const float b1j = __bfloat162float(w[off_b1(in) + j]);
  for (int q = 0; q < nq; ++q) {
    const int s = s0 + q;
    float z = b1j;
    for (int k = 0; k < in; ++k) z = fmaf(__bfloat162float(w[j * in + k]), m.x[(size_t)s * in + k], z);
    const size_t es = ((size_t)e * m.B + s) * H + j;
    m.z1[es] = z;
    const float h = gelu(z, nullptr);
    h1s[q][j] = h;
    m.h1[es] = h;
  }
  __syncthreads();
  float z2[CHUNK];
  const float b2j = __bfloat162float(w[off_b2(in) + j]);
#pragma unroll
  for (int q = 0; q < CHUNK; ++q) z2[q] = b2j;
  for (int k = 0; k < H; ++k) {
    const float wv = __bfloat162float(w2s[j * W2S + k]);
#pragma unroll
    for (int q = 0; q < CHUNK; ++q) z2[q] = fmaf(wv, h1s[q < nq ? q : 0][k], z2[q]);
  }
  const float w3j = __bfloat162float(w[off_w3(in) + j]);
#pragma unroll
  for (int q = 0; q < CHUNK; ++q) {
    if (q >= nq) break;
    const size_t es = ((size_t)e * m.B + s0 + q) * H + j;
    m.z2[es] = z2[q];
    const float h2 = gelu(z2[q], nullptr);
    m.h2[es] = h2;
    float part = w3j * h2;
    for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
    if ((j & 31) == 0) red[q][j >> 5] = part;
  }
  __syncthreads();
  if (j < nq) {
    float yy = __bfloat162float(w[off_b3(in)]);
    for (int q2 = 0; q2 < H / 32; ++q2) yy += red[j][q2];
    m.y[(size_t)e * m.B + s0 + j] = yy;
  }
}

/* Per-sample deltas of the weighted squared error L_e = sum_s sw[e][s] (y - t)^2
 * (sw = 1/B without weights: the mean-squared error). */
__global__ void __launch_bounds__(H) k_mlp_backward(MlpDev m) {
  const int e = blockIdx.y;
  const int s0 = blockIdx.x * CHUNK;
  const int j = threadIdx.x;
  const int in = m.in, P = n_params(in);
  const __nv_bfloat16* w = m.w + (size_t)e * P;
  __shared__ __nv_bfloat16 w2s[H * W2S];
  __shared__ float dz2s[CHUNK][H];
  load_w2(w + off_w2(in), w2s);
  const int nq = m.B - s0 < CHUNK ? m.B - s0 : CHUNK;
  const float w3j = __bfloat162float(w[off_w3(in) + j]);
  for (int q = 0; q < nq; ++q) {
    const int s = s0 + q;
    const size_t es = (size_t)e * m.B + s;
    const float dy = 2.0f * m.sw[es] * (m.y[es] - m.t[s]);
    if (j == 0) m.dy[es] = dy;
    float g2;
    gelu(m.z2[es * H + j], &g2);
    const float dz2 = dy * w3j * g2;
    m.dz2[es * H + j] = dz2;
    dz2s[q][j] = dz2;
  }
  __syncthreads();
  /* dh1[j] = sum_r W2[r][j] dz2[r], r in order */
  float dh1[CHUNK];
#pragma unroll
  for (int q = 0; q < CHUNK; ++q) dh1[q] = 0.0f;
  for (int r = 0; r < H; ++r) {
    const float wv = __bfloat162float(w2s[r * W2S + j]);
#pragma unroll
    for (int q = 0; q < CHUNK; ++q) dh1[q] = fmaf(wv, dz2s[q < nq ? q : 0][r], dh1[q]);
  }
#pragma unroll
  for (int q = 0; q < CHUNK; ++q) {
    if (q >= nq) break;
    const size_t es = (size_t)e * m.B + s0 + q;
    float g1;
    gelu(m.z1[es * H + j], &g1);
    m.dz1[es * H + j] = dh1[q] * g1;
  }
}

/* Gradient of W2 (H x H per member): one block per (member, GW_ROWS rows),
 * one thread per column k, the samples streamed through shared memory in
 * chunks; each entry is summed over the samples in order. */
constexpr int GW_ROWS = 16;
constexpr int GW_SAMPLES = 32;

__global__ void __launch_bounds__(H) k_mlp_grad_w2(MlpDev m, float* grad) {
  const int e = blockIdx.y;
  const int j0 = blockIdx.x * GW_ROWS;
  const int k = threadIdx.x;
  const int in = m.in, P = n_params(in);
  __shared__ float hs[GW_SAMPLES][H];
  __shared__ float dzs[GW_SAMPLES][GW_ROWS];
  float acc[GW_ROWS];
#pragma unroll
  for (int r = 0; r < GW_ROWS; ++r) acc[r] = 0.0f;
  const size_t eb = (size_t)e * m.B;
  for (int c0 = 0; c0 < m.B; c0 += GW_SAMPLES) {
    const int nc = m.B - c0 < GW_SAMPLES ? m.B - c0 : GW_SAMPLES;
    for (int ss = 0; ss < nc; ++ss) hs[ss][k] = m.h1[(eb + c0 + ss) * H + k];
    for (int idx = k; idx < nc * GW_ROWS; idx += H)
      dzs[idx / GW_ROWS][idx % GW_ROWS] = m.dz2[(eb + c0 + idx / GW_ROWS) * H + j0 + idx % GW_ROWS];
    __syncthreads();
    for (int ss = 0; ss < nc; ++ss) {
      const float hk = hs[ss][k];
#pragma unroll
      for (int r = 0; r < GW_ROWS; ++r) acc[r] = fmaf(dzs[ss][r], hk, acc[r]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < GW_ROWS; ++r) grad[(size_t)e * P + off_w2(in) + (size_t)(j0 + r) * H + k] = acc[r];
}

/* One thread per (member, parameter) outside W2: the gradient summed over
 * the samples in order. */
__global__ void k_mlp_grad(MlpDev m, float* grad) {
  const int in = m.in, P = n_params(in);
  const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= (long long)m.E * P) return;
  const int e = (int)(gid / P), q = (int)(gid % P);
  float g = 0.0f;
  const size_t eb = (size_t)e * m.B;
  if (q < off_b1(in)) {
    const int j = q / in, k = q % in;
    for (int s = 0; s < m.B; ++s) g = fmaf(m.dz1[(eb + s) * H + j], m.x[(size_t)s * in + k], g);
  } else if (q < off_w2(in)) {
    const int j = q - off_b1(in);
    for (int s = 0; s < m.B; ++s) g += m.dz1[(eb + s) * H + j];
  } else if (q < off_b2(in)) {
    return;  /* W2: k_mlp_grad_w2 */
  } else if (q < off_w3(in)) {
    const int j = q - off_b2(in);
    for (int s = 0; s < m.B; ++s) g += m.dz2[(eb + s) * H + j];
  } else if (q < off_b3(in)) {
    const int j = q - off_w3(in);
    for (int s = 0; s < m.B; ++s) g = fmaf(m.dy[eb + s], m.h2[(eb + s) * H + j], g);
  } else {
    for (int s = 0; s < m.B; ++s) g += m.dy[eb + s];
  }
  grad[gid] = g;
}

__global__ void k_mlp_loss(MlpDev m, float* loss) {
  const int e = threadIdx.x;
  if (e >= m.E) return;
  float l = 0.0f;
  for (int s = 0; s < m.B; ++s) {
    const float d = m.y[(size_t)e * m.B + s] - m.t[s];
    l = fmaf(m.sw[(size_t)e * m.B + s] * d, d, l);
  }
  loss[e] = l;
}

/* Adam (Kingma & Ba, 2015) on the FP32 masters; refreshes the BF16 copy.
 * The bias corrections of step t are bias[*tix] = (1 - b1^t, 1 - b2^t),
 * tabulated on the host for the steps of one training call. */
__global__ void k_mlp_adam(int count, float* master, __nv_bfloat16* w, const float* grad, float* mom,
                           float* vel, float lr, float b1, float b2, float eps, const float2* bias,
                           const int* tix) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float2 c = bias[*tix];
  const float c1 = c.x, c2 = c.y;
  const float g = grad[i];
  const float mm = b1 * mom[i] + (1.0f - b1) * g;
  const float vv = b2 * vel[i] + (1.0f - b2) * g * g;
  mom[i] = mm;
  vel[i] = vv;
  const float th = master[i] - lr * (mm / c1) / (sqrtf(vv / c2) + eps);
  master[i] = th;
  w[i] = __float2bfloat16_rn(th);
}

__global__ void k_mlp_next(int* tix) { *tix += 1; }

__global__ void k_mlp_cast(int count, const float* master, __nv_bfloat16* w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) w[i] = __float2bfloat16_rn(master[i]);
}

int mfail(int status, const std::string& msg) {
  spp_internal_set_error(msg.c_str());
  return status;
}

#define MCUDA(expr)                                                                      \
  do {                                                                                   \
    cudaError_t _e = (expr);                                                             \
    if (_e != cudaSuccess) return mfail(SPP_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

}  // namespace

struct SppMlp {
  int E, in, P;
  float* master = nullptr;
  __nv_bfloat16* w = nullptr;
  float *mom = nullptr, *vel = nullptr, *grad = nullptr;
  int64_t adam_t = 0;
  /* scratch sized for the largest batch seen */
  int cap_B = 0;
  float *x = nullptr, *t = nullptr, *z1 = nullptr, *z2 = nullptr, *h1 = nullptr, *h2 = nullptr, *y = nullptr;
  float *dz1 = nullptr, *dz2 = nullptr, *dy = nullptr, *loss = nullptr, *sw = nullptr;
  std::vector<float> host_sw;
  cudaStream_t stream = nullptr;
  /* Adam bias corrections of one training call, and the index of the step */
  float2* bias = nullptr;
  int bias_cap = 0;
  int* tix = nullptr;
  /* graphs of TRAIN_GRAPH_ITERS training iterations, keyed by (B, lr) */
  struct TrainGraph { int B; float lr; cudaGraph_t graph; cudaGraphExec_t exec; };
  std::vector<TrainGraph> graphs;
};

namespace {

void mlp_drop_graphs(SppMlp* m) {
  for (auto& g : m->graphs) {
    cudaGraphExecDestroy(g.exec);
    cudaGraphDestroy(g.graph);
  }
  m->graphs.clear();
}

void mlp_free_scratch(SppMlp* m) {
  mlp_drop_graphs(m);
  float* ptrs[] = {m->x, m->t, m->z1, m->z2, m->h1, m->h2, m->y, m->dz1, m->dz2, m->dy, m->loss, m->sw};
  for (float* q : ptrs)
    if (q) cudaFree(q);
  m->x = m->t = m->z1 = m->z2 = m->h1 = m->h2 = m->y = m->dz1 = m->dz2 = m->dy = m->loss = m->sw = nullptr;
  m->cap_B = 0;
}

int mlp_reserve(SppMlp* m, int B) {
  if (B <= m->cap_B) return SPP_OK;
  mlp_free_scratch(m);
  size_t eb = (size_t)m->E * B;
  cudaError_t e = cudaSuccess;
  float** targets[] = {&m->x, &m->t, &m->z1, &m->z2, &m->h1, &m->h2, &m->y,
                       &m->dz1, &m->dz2, &m->dy, &m->loss, &m->sw};
  size_t sizes[] = {(size_t)B * m->in, (size_t)B, eb * H, eb * H, eb * H, eb * H, eb,
                    eb * H, eb * H, eb, (size_t)m->E, eb};
  for (int q = 0; q < 12 && e == cudaSuccess; ++q) e = cudaMalloc((void**)targets[q], sizeof(float) * sizes[q]);
  if (e != cudaSuccess) {
    mlp_free_scratch(m);
    return mfail(SPP_ERR_ALLOC, std::string("mlp scratch: ") + cudaGetErrorString(e));
  }
  m->cap_B = B;
  return SPP_OK;
}

MlpDev mlp_dev(SppMlp* m, int B) {
  MlpDev d;
  d.E = m->E;
  d.in = m->in;
  d.B = B;
  d.w = m->w;
  d.x = m->x;
  d.t = m->t;
  d.sw = m->sw;
  d.z1 = m->z1;
  d.z2 = m->z2;
  d.h1 = m->h1;
  d.h2 = m->h2;
  d.y = m->y;
  d.dz1 = m->dz1;
  d.dz2 = m->dz2;
  d.dy = m->dy;
  return d;
}

/* Uploads inputs, targets and the sample weights normalised per member
 * (weights NULL: 1/B each).  Weights must be finite and >= 0 with a positive
 * sum for every member. */
int mlp_upload(SppMlp* m, const float* x, const float* t, const float* weights, int B) {
  int rc = mlp_reserve(m, B);
  if (rc != SPP_OK) return rc;
  MCUDA(cudaMemcpyAsync(m->x, x, sizeof(float) * (size_t)B * m->in, cudaMemcpyHostToDevice, m->stream));
  if (!t) return SPP_OK;
  MCUDA(cudaMemcpyAsync(m->t, t, sizeof(float) * (size_t)B, cudaMemcpyHostToDevice, m->stream));
  /* the previous upload of host_sw may still be in flight */
  MCUDA(cudaStreamSynchronize(m->stream));
  m->host_sw.assign((size_t)m->E * B, 1.0f / (float)B);
  if (weights) {
    for (int e = 0; e < m->E; ++e) {
      double sum = 0.0;
      for (int s = 0; s < B; ++s) {
        const float v = weights[(size_t)e * B + s];
        if (!(v >= 0.0f) || !std::isfinite(v)) return mfail(SPP_ERR_INVALID, "sample weights must be finite and >= 0");
        sum += v;
      }
      if (!(sum > 0.0)) return mfail(SPP_ERR_INVALID, "every member needs a positive weight sum");
      for (int s = 0; s < B; ++s)
        m->host_sw[(size_t)e * B + s] = (float)((double)weights[(size_t)e * B + s] / sum);
    }
  }
  MCUDA(cudaMemcpyAsync(m->sw, m->host_sw.data(), sizeof(float) * m->host_sw.size(), cudaMemcpyHostToDevice,
                        m->stream));
  return SPP_OK;
}

void mlp_fwd_bwd(SppMlp* m, int B, bool backward) {
  MlpDev d = mlp_dev(m, B);
  dim3 grid((B + CHUNK - 1) / CHUNK, m->E);
  k_mlp_forward<<<grid, H, 0, m->stream>>>(d);
  if (!backward) return;
  k_mlp_backward<<<grid, H, 0, m->stream>>>(d);
  const long long tot = (long long)m->E * m->P;
  k_mlp_grad<<<(unsigned)((tot + 255) / 256), 256, 0, m->stream>>>(d, m->grad);
  k_mlp_grad_w2<<<dim3(H / GW_ROWS, m->E), H, 0, m->stream>>>(d, m->grad);
}

constexpr float ADAM_B1 = 0.9f, ADAM_B2 = 0.999f, ADAM_EPS = 1e-8f;
constexpr int TRAIN_GRAPH_ITERS = 50;

/* One training iteration: gradient, Adam with the bias correction at
 * bias[*tix], next step index. */
void mlp_train_iter(SppMlp* m, int B, float lr) {
  mlp_fwd_bwd(m, B, true);
  const int tot = m->E * m->P;
  k_mlp_adam<<<(tot + 255) / 256, 256, 0, m->stream>>>(tot, m->master, m->w, m->grad, m->mom, m->vel, lr,
                                                       ADAM_B1, ADAM_B2, ADAM_EPS, m->bias, m->tix);
  k_mlp_next<<<1, 1, 0, m->stream>>>(m->tix);
}

int mlp_train_graph(SppMlp* m, int B, float lr, cudaGraphExec_t* out) {
  for (auto& g : m->graphs)
    if (g.B == B && g.lr == lr) { *out = g.exec; return SPP_OK; }
  cudaGraph_t graph = nullptr;
  MCUDA(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
  for (int it = 0; it < TRAIN_GRAPH_ITERS; ++it) mlp_train_iter(m, B, lr);
  MCUDA(cudaStreamEndCapture(m->stream, &graph));
  cudaGraphExec_t exec;
  cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    return mfail(SPP_ERR_CUDA, std::string("training graph: ") + cudaGetErrorString(e));
  }
  m->graphs.push_back({B, lr, graph, exec});
  *out = exec;
  return SPP_OK;
}

}  // namespace

extern "C" {

int spp_mlp_create(int ensemble, int in_dim, SppMlp** out) {
  if (!out || ensemble < 1 || ensemble > 32 || in_dim < 1 || in_dim > MAX_IN)
    return mfail(SPP_ERR_INVALID, "need 1 <= ensemble <= 32 and 1 <= in_dim <= 16");
  SppMlp* m = new SppMlp();
  m->E = ensemble;
  m->in = in_dim;
  m->P = n_params(in_dim);
  size_t tot = (size_t)m->E * m->P;
  cudaError_t e = cudaMalloc((void**)&m->master, sizeof(float) * tot);
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->w, sizeof(__nv_bfloat16) * tot);
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->mom, sizeof(float) * tot);
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->vel, sizeof(float) * tot);
  if (e == cudaSuccess) e = cudaMalloc((void**)&m->grad, sizeof(float) * tot);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMemset(m->master, 0, sizeof(float) * tot);
  if (e == cudaSuccess) e = cudaMemset(m->w, 0, sizeof(__nv_bfloat16) * tot);
  if (e == cudaSuccess) e = cudaMemset(m->mom, 0, sizeof(float) * tot);
  if (e == cudaSuccess) e = cudaMemset(m->vel, 0, sizeof(float) * tot);
  if (e != cudaSuccess) {
    cudaFree(m->master); cudaFree(m->w); cudaFree(m->mom); cudaFree(m->vel); cudaFree(m->grad);
    delete m;
    return mfail(SPP_ERR_ALLOC, std::string("mlp: ") + cudaGetErrorString(e));
  }
  *out = m;
  return SPP_OK;
}

int spp_mlp_destroy(SppMlp* m) {
  if (!m) return SPP_OK;
  cudaStreamSynchronize(m->stream);
  mlp_free_scratch(m);
  cudaFree(m->master); cudaFree(m->w); cudaFree(m->mom); cudaFree(m->vel); cudaFree(m->grad);
  cudaFree(m->bias); cudaFree(m->tix);
  cudaStreamDestroy(m->stream);
  delete m;
  return SPP_OK;
}

int spp_mlp_num_params(SppMlp* m) { return m ? m->P : 0; }

int spp_mlp_set_params(SppMlp* m, const float* theta) {
  if (!m || !theta) return mfail(SPP_ERR_INVALID, "NULL argument");
  size_t tot = (size_t)m->E * m->P;
  MCUDA(cudaMemcpyAsync(m->master, theta, sizeof(float) * tot, cudaMemcpyHostToDevice, m->stream));
  k_mlp_cast<<<(unsigned)((tot + 255) / 256), 256, 0, m->stream>>>((int)tot, m->master, m->w);
  MCUDA(cudaMemsetAsync(m->mom, 0, sizeof(float) * tot, m->stream));
  MCUDA(cudaMemsetAsync(m->vel, 0, sizeof(float) * tot, m->stream));
  m->adam_t = 0;
  MCUDA(cudaStreamSynchronize(m->stream));
  return SPP_OK;
}

int spp_mlp_get_params(SppMlp* m, float* theta) {
  if (!m || !theta) return mfail(SPP_ERR_INVALID, "NULL argument");
  MCUDA(cudaMemcpyAsync(theta, m->master, sizeof(float) * (size_t)m->E * m->P, cudaMemcpyDeviceToHost,
                        m->stream));
  MCUDA(cudaStreamSynchronize(m->stream));
  return SPP_OK;
}

int spp_mlp_predict(SppMlp* m, const float* x, int B, float* y) {
  if (!m || !x || !y || B < 1) return mfail(SPP_ERR_INVALID, "bad arguments");
  int rc = mlp_upload(m, x, nullptr, nullptr, B);
  if (rc != SPP_OK) return rc;
  mlp_fwd_bwd(m, B, false);
  MCUDA(cudaMemcpyAsync(y, m->y, sizeof(float) * (size_t)m->E * B, cudaMemcpyDeviceToHost, m->stream));
  MCUDA(cudaStreamSynchronize(m->stream));
  return SPP_OK;
}

int spp_mlp_grad(SppMlp* m, const float* x, const float* t, const float* weights, int B, float* grad,
                 float* loss) {
  if (!m || !x || !t || B < 1) return mfail(SPP_ERR_INVALID, "bad arguments");
  int rc = mlp_upload(m, x, t, weights, B);
  if (rc != SPP_OK) return rc;
  mlp_fwd_bwd(m, B, true);
  MlpDev d = mlp_dev(m, B);
  k_mlp_loss<<<1, 32, 0, m->stream>>>(d, m->loss);
  if (grad)
    MCUDA(cudaMemcpyAsync(grad, m->grad, sizeof(float) * (size_t)m->E * m->P, cudaMemcpyDeviceToHost,
                          m->stream));
  if (loss) MCUDA(cudaMemcpyAsync(loss, m->loss, sizeof(float) * m->E, cudaMemcpyDeviceToHost, m->stream));
  MCUDA(cudaStreamSynchronize(m->stream));
  return SPP_OK;
}

int spp_mlp_train(SppMlp* m, const float* x, const float* t, const float* weights, int B, int iters, float lr,
                  float* loss) {
  if (!m || !x || !t || B < 1 || iters < 0) return mfail(SPP_ERR_INVALID, "bad arguments");
  int rc = mlp_upload(m, x, t, weights, B);
  if (rc != SPP_OK) return rc;
  if (iters > 0) {
    /* the bias corrections of steps adam_t + 1 .. adam_t + iters */
    if (iters > m->bias_cap) {
      mlp_drop_graphs(m);  /* they hold the old table's address */
      cudaFree(m->bias);
      m->bias = nullptr;
      m->bias_cap = 0;
      const int cap = iters > 4096 ? iters : 4096;
      MCUDA(cudaMalloc((void**)&m->bias, sizeof(float2) * cap));
      m->bias_cap = cap;
    }
    if (!m->tix) MCUDA(cudaMalloc((void**)&m->tix, sizeof(int)));
    MCUDA(cudaStreamSynchronize(m->stream));  /* the previous table may still be read */
    std::vector<float2> table((size_t)iters);
    for (int it = 0; it < iters; ++it) {
      const double t = (double)(m->adam_t + 1 + it);
      table[(size_t)it] = make_float2(1.0f - (float)std::pow((double)ADAM_B1, t),
                                      1.0f - (float)std::pow((double)ADAM_B2, t));
    }
    MCUDA(cudaMemcpyAsync(m->bias, table.data(), sizeof(float2) * iters, cudaMemcpyHostToDevice, m->stream));
    MCUDA(cudaMemsetAsync(m->tix, 0, sizeof(int), m->stream));
    int done = 0;
    if (iters >= TRAIN_GRAPH_ITERS) {
      cudaGraphExec_t exec;
      rc = mlp_train_graph(m, B, lr, &exec);
      if (rc != SPP_OK) return rc;
      for (; done + TRAIN_GRAPH_ITERS <= iters; done += TRAIN_GRAPH_ITERS) MCUDA(cudaGraphLaunch(exec, m->stream));
    }
    for (; done < iters; ++done) mlp_train_iter(m, B, lr);
    m->adam_t += iters;
    MCUDA(cudaStreamSynchronize(m->stream));  /* the host table goes out of scope */
  }
  MCUDA(cudaGetLastError());
  if (loss) {
    mlp_fwd_bwd(m, B, false);
    MlpDev d = mlp_dev(m, B);
    k_mlp_loss<<<1, 32, 0, m->stream>>>(d, m->loss);
    MCUDA(cudaMemcpyAsync(loss, m->loss, sizeof(float) * m->E, cudaMemcpyDeviceToHost, m->stream));
  }
  MCUDA(cudaStreamSynchronize(m->stream));
  return SPP_OK;
}

}  // extern "C"
