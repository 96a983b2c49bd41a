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

__global__ void __launch_bounds__(H) k_mlp_forward(MlpDev m) {
  const int e = blockIdx.y;
  const int s0 = blockIdx.x * CHUNK;
  const int j = threadIdx.x;
  const int in = m.in, P = n_params(in);
  const __nv_bfloat16* w = m.w + (size_t)e * P;
  __shared__ float h1[H];
  __shared__ float h2[H];
  __shared__ float red[H / 32];
  for (int q = 0; q < CHUNK; ++q) {
    const int s = s0 + q;
    if (s >= m.B) break;
    float z = __bfloat162float(w[off_b1(in) + j]);
    for (int k = 0; k < in; ++k) z = fmaf(__bfloat162float(w[j * in + k]), m.x[(size_t)s * in + k], z);
    m.z1[((size_t)e * m.B + s) * H + j] = z;
    h1[j] = gelu(z, nullptr);
    m.h1[((size_t)e * m.B + s) * H + j] = h1[j];
    __syncthreads();
    float z2 = __bfloat162float(w[off_b2(in) + j]);
    const __nv_bfloat16* row = w + off_w2(in) + (size_t)j * H;
    for (int k = 0; k < H; ++k) z2 = fmaf(__bfloat162float(row[k]), h1[k], z2);
    m.z2[((size_t)e * m.B + s) * H + j] = z2;
    h2[j] = gelu(z2, nullptr);
    m.h2[((size_t)e * m.B + s) * H + j] = h2[j];
    float part = __bfloat162float(w[off_w3(in) + j]) * h2[j];
    for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
    if ((j & 31) == 0) red[j >> 5] = part;
    __syncthreads();
    if (j == 0) {
      float yy = __bfloat162float(w[off_b3(in)]);
      for (int q2 = 0; q2 < H / 32; ++q2) yy += red[q2];
      m.y[(size_t)e * m.B + s] = yy;
    }
    __syncthreads();
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
  __shared__ float dz2s[H];
  for (int q = 0; q < CHUNK; ++q) {
    const int s = s0 + q;
    if (s >= m.B) break;
    const size_t es = (size_t)e * m.B + s;
    const float dy = 2.0f * m.sw[es] * (m.y[es] - m.t[s]);
    if (j == 0) m.dy[es] = dy;
    float g2;
    gelu(m.z2[es * H + j], &g2);
    const float dz2 = dy * __bfloat162float(w[off_w3(in) + j]) * g2;
    m.dz2[es * H + j] = dz2;
    dz2s[j] = dz2;
    __syncthreads();
    /* dh1[j] = sum_r W2[r][j] dz2[r] */
    float dh1 = 0.0f;
    for (int r = 0; r < H; ++r) dh1 = fmaf(__bfloat162float(w[off_w2(in) + (size_t)r * H + j]), dz2s[r], dh1);
    float g1;
    gelu(m.z1[es * H + j], &g1);
    m.dz1[es * H + j] = dh1 * g1;
    __syncthreads();
  }
}

/* One thread per (member, parameter): the gradient summed over the samples
 * in order. */
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
    const int j = (q - off_w2(in)) / H, k = (q - off_w2(in)) % H;
    for (int s = 0; s < m.B; ++s) g = fmaf(m.dz2[(eb + s) * H + j], m.h1[(eb + s) * H + k], g);
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

/* Adam (Kingma & Ba, 2015) on the FP32 masters; refreshes the BF16 copy. */
__global__ void k_mlp_adam(int count, float* master, __nv_bfloat16* w, const float* grad, float* mom,
                           float* vel, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float g = grad[i];
  const float mm = b1 * mom[i] + (1.0f - b1) * g;
  const float vv = b2 * vel[i] + (1.0f - b2) * g * g;
  mom[i] = mm;
  vel[i] = vv;
  const float th = master[i] - lr * (mm / c1) / (sqrtf(vv / c2) + eps);
  master[i] = th;
  w[i] = __float2bfloat16_rn(th);
}

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
};

namespace {

void mlp_free_scratch(SppMlp* m) {
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
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const int tot = m->E * m->P;
  for (int it = 0; it < iters; ++it) {
    mlp_fwd_bwd(m, B, true);
    m->adam_t += 1;
    const float c1 = 1.0f - (float)std::pow((double)b1, (double)m->adam_t);
    const float c2 = 1.0f - (float)std::pow((double)b2, (double)m->adam_t);
    k_mlp_adam<<<(tot + 255) / 256, 256, 0, m->stream>>>(tot, m->master, m->w, m->grad, m->mom, m->vel, lr,
                                                         b1, b2, eps, c1, c2);
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
