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
#include <cstdlib>
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

/* ------------------------------------------------------------------ */
/* tensor-core path: the 128 x 128 layer on mma.sync (TF32, FP32 sums)  */
/* ------------------------------------------------------------------ */
/* m16n8k8 TF32 products with FP32 accumulation.  BF16 weights are exact in
 * TF32; an FP32 operand x is split into x_hi = tf32(x) and x_lo = tf32(x -
 * x_hi), and the products taken as hi*w + lo*w (weights) or hi*hi + hi*lo +
 * lo*hi (two FP32 operands), which keeps the FP32 accuracy of the scalar
 * kernels (relative error ~2^-21 per product).  Fragment layout of m16n8k8
 * (groupID g = lane / 4, t = lane % 4): A a0 (g, t), a1 (g+8, t), a2 (g,
 * t+4), a3 (g+8, t+4); B b0 (k t, n g), b1 (k t+4, n g); C c0 (g, 2t), c1
 * (g, 2t+1), c2 (g+8, 2t), c3 (g+8, 2t+1). */
__device__ __forceinline__ uint32_t tf32_bits(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ void tf32_split(float x, uint32_t* hi, uint32_t* lo) {
  *hi = tf32_bits(x);
  *lo = tf32_bits(x - __uint_as_float(*hi));
}
__device__ __forceinline__ void mma_tf32(float* c, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

#ifndef SPP_MLP_TS
#define SPP_MLP_TS 16
#endif
constexpr int TS = SPP_MLP_TS; /* samples per block of k_mlp_fused (a multiple of 16) */
constexpr int MT = TS / 16;     /* m16 tiles per block */
constexpr int WP = H + 4;     /* padded row stride of W2 in shared memory (floats) */
constexpr int HP = H + 4;     /* padded row stride of the activation tiles */
constexpr size_t FUSED_SMEM = sizeof(float) * ((size_t)H * WP + 2 * (size_t)TS * HP + (size_t)TS * H + 2 * TS);

/* Forward (and with BACKWARD the per-sample deltas) of one member on TS
 * samples, 4 warps: layer 1 and the output layer as FP32 FMAs, the 128 x
 * 128 layer and its transpose on the tensor cores.  Writes the same arrays
 * as k_mlp_forward / k_mlp_backward. */
template <bool BACKWARD>
__global__ void __launch_bounds__(H) k_mlp_fused(MlpDev m) {
  extern __shared__ float fsm[];
  float* w2f = fsm;                 /* [H][WP]: W2[j][k] */
  float* hs = w2f + H * WP;         /* [TS][HP]: h1 */
  float* t2 = hs + TS * HP;         /* [TS][HP]: h2, then dz2 */
  float* zs1 = t2 + TS * HP;        /* [TS][H]: z1 */
  float* dys = zs1 + TS * H;        /* [TS]: dy */
  float* yts = dys + TS;            /* [TS]: y */
  const int e = blockIdx.y;
  const int s0 = blockIdx.x * TS;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int in = m.in, P = n_params(in);
  const __nv_bfloat16* w = m.w + (size_t)e * P;
  const int nq = m.B - s0 < TS ? m.B - s0 : TS;
  for (int idx = tid; idx < H * H; idx += H) w2f[(idx / H) * WP + (idx % H)] = __bfloat162float(w[off_w2(in) + idx]);
  /* layer 1: thread j, every sample of the tile (rows past the batch: 0) */
  {
    const int j = tid;
    const float b1j = __bfloat162float(w[off_b1(in) + j]);
    for (int q = 0; q < TS; ++q) {
      float z = 0.0f, h = 0.0f;
      if (q < nq) {
        const int sidx = s0 + q;
        z = b1j;
        for (int k = 0; k < in; ++k) z = fmaf(__bfloat162float(w[j * in + k]), m.x[(size_t)sidx * in + k], z);
        h = gelu(z, nullptr);
        const size_t es = ((size_t)e * m.B + sidx) * H + j;
        m.z1[es] = z;
        m.h1[es] = h;
      }
      zs1[q * H + j] = z;
      hs[q * HP + j] = h;
    }
  }
  __syncthreads();
  /* z2 = h1 W2^T + b2: warp w owns columns [32 w, 32 w + 32), every 16-row tile */
  float acc[MT][4][4];
#pragma unroll
  for (int mt = 0; mt < MT; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[mt][nt][c] = 0.0f;
  for (int k0 = 0; k0 < H; k0 += 8) {
    uint32_t ah[MT][4], al[MT][4];
#pragma unroll
    for (int mt = 0; mt < MT; ++mt) {
      const int r = mt * 16 + g;
      tf32_split(hs[r * HP + k0 + t], &ah[mt][0], &al[mt][0]);
      tf32_split(hs[(r + 8) * HP + k0 + t], &ah[mt][1], &al[mt][1]);
      tf32_split(hs[r * HP + k0 + t + 4], &ah[mt][2], &al[mt][2]);
      tf32_split(hs[(r + 8) * HP + k0 + t + 4], &ah[mt][3], &al[mt][3]);
    }
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
      const int n = warp * 32 + nt * 8 + g;
      const uint32_t b0 = __float_as_uint(w2f[n * WP + k0 + t]);
      const uint32_t b1 = __float_as_uint(w2f[n * WP + k0 + t + 4]);
#pragma unroll
      for (int mt = 0; mt < MT; ++mt) {
        mma_tf32(acc[mt][nt], ah[mt], b0, b1);
        mma_tf32(acc[mt][nt], al[mt], b0, b1);
      }
    }
  }
  /* z2, h2 */
#pragma unroll
  for (int mt = 0; mt < MT; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int q = mt * 16 + g + (c >= 2 ? 8 : 0);
        const int j = warp * 32 + nt * 8 + 2 * t + (c & 1);
        const float z2 = acc[mt][nt][c] + __bfloat162float(w[off_b2(in) + j]);
        acc[mt][nt][c] = z2;
        const float h2 = gelu(z2, nullptr);
        t2[q * HP + j] = q < nq ? h2 : 0.0f;
        if (q < nq) {
          const size_t es = ((size_t)e * m.B + s0 + q) * H + j;
          m.z2[es] = z2;
          m.h2[es] = h2;
        }
      }
  __syncthreads();
  /* y = b3 + sum_j W3[j] h2[j], j in order, one thread per sample */
  if (tid < nq) {
    float yy = __bfloat162float(w[off_b3(in)]);
    for (int j = 0; j < H; ++j) yy = fmaf(__bfloat162float(w[off_w3(in) + j]), t2[tid * HP + j], yy);
    yts[tid] = yy;
    m.y[(size_t)e * m.B + s0 + tid] = yy;
    if (BACKWARD) {
      const size_t es = (size_t)e * m.B + s0 + tid;
      const float dy = 2.0f * m.sw[es] * (yy - m.t[s0 + tid]);
      m.dy[es] = dy;
      dys[tid] = dy;
    }
  } else if (tid < TS) {
    dys[tid] = 0.0f;
  }
  if (!BACKWARD) return;
  __syncthreads();
  /* dz2 = dy W3[j] gelu'(z2), into the tile and global memory */
#pragma unroll
  for (int mt = 0; mt < MT; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int q = mt * 16 + g + (c >= 2 ? 8 : 0);
        const int j = warp * 32 + nt * 8 + 2 * t + (c & 1);
        float g2;
        gelu(acc[mt][nt][c], &g2);
        const float dz2 = dys[q] * __bfloat162float(w[off_w3(in) + j]) * g2;
        t2[q * HP + j] = dz2;
        if (q < nq) m.dz2[((size_t)e * m.B + s0 + q) * H + j] = dz2;
      }
  __syncthreads();
  /* dh1 = dz2 W2 (sum over j), dz1 = dh1 gelu'(z1) */
#pragma unroll
  for (int mt = 0; mt < MT; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[mt][nt][c] = 0.0f;
  for (int k0 = 0; k0 < H; k0 += 8) {
    uint32_t ah[MT][4], al[MT][4];
#pragma unroll
    for (int mt = 0; mt < MT; ++mt) {
      const int r = mt * 16 + g;
      tf32_split(t2[r * HP + k0 + t], &ah[mt][0], &al[mt][0]);
      tf32_split(t2[(r + 8) * HP + k0 + t], &ah[mt][1], &al[mt][1]);
      tf32_split(t2[r * HP + k0 + t + 4], &ah[mt][2], &al[mt][2]);
      tf32_split(t2[(r + 8) * HP + k0 + t + 4], &ah[mt][3], &al[mt][3]);
    }
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
      const int n = warp * 32 + nt * 8 + g;
      const uint32_t b0 = __float_as_uint(w2f[(k0 + t) * WP + n]);
      const uint32_t b1 = __float_as_uint(w2f[(k0 + t + 4) * WP + n]);
#pragma unroll
      for (int mt = 0; mt < MT; ++mt) {
        mma_tf32(acc[mt][nt], ah[mt], b0, b1);
        mma_tf32(acc[mt][nt], al[mt], b0, b1);
      }
    }
  }
#pragma unroll
  for (int mt = 0; mt < MT; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const int q = mt * 16 + g + (c >= 2 ? 8 : 0);
        const int k = warp * 32 + nt * 8 + 2 * t + (c & 1);
        if (q < nq) {
          float g1;
          gelu(zs1[q * H + k], &g1);
          m.dz1[((size_t)e * m.B + s0 + q) * H + k] = acc[mt][nt][c] * g1;
        }
      }
}

/* Gradients of the parameters outside W2 (W1, b1, b2, W3, b3: 128 in + 385
 * per member), 8 threads per parameter: thread r sums the samples s = r (mod
 * 8) in order, and the eight partial sums combine through a fixed butterfly
 * of xor shuffles (reproducible, no atomics). */
constexpr int GSPLIT = 8;
__global__ void __launch_bounds__(256) k_mlp_grad_small(MlpDev m, float* grad) {
  const int in = m.in, P = n_params(in);
  const int nsmall = off_w2(in) + (P - off_b2(in));
  const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long item = gid / GSPLIT;
  const int r = (int)(gid % GSPLIT);
  const bool live = item < (long long)m.E * nsmall;   /* whole groups of 8 share it */
  const int e = live ? (int)(item / nsmall) : 0;
  const int u = live ? (int)(item % nsmall) : 0;
  const int q = u < off_w2(in) ? u : u - off_w2(in) + off_b2(in);
  const size_t eb = (size_t)e * m.B;
  float g = 0.0f;
  if (live) {
    if (q < off_b1(in)) {
      const int j = q / in, k = q % in;
      for (int sidx = r; sidx < m.B; sidx += GSPLIT) g = fmaf(m.dz1[(eb + sidx) * H + j], m.x[(size_t)sidx * in + k], g);
    } else if (q < off_w2(in)) {
      const int j = q - off_b1(in);
      for (int sidx = r; sidx < m.B; sidx += GSPLIT) g += m.dz1[(eb + sidx) * H + j];
    } else if (q < off_w3(in)) {
      const int j = q - off_b2(in);
      for (int sidx = r; sidx < m.B; sidx += GSPLIT) g += m.dz2[(eb + sidx) * H + j];
    } else if (q < off_b3(in)) {
      const int j = q - off_w3(in);
      for (int sidx = r; sidx < m.B; sidx += GSPLIT) g = fmaf(m.dy[eb + sidx], m.h2[(eb + sidx) * H + j], g);
    } else {
      for (int sidx = r; sidx < m.B; sidx += GSPLIT) g += m.dy[eb + sidx];
    }
  }
#pragma unroll
  for (int o = 1; o < GSPLIT; o <<= 1) g += __shfl_xor_sync(0xffffffffu, g, o);
  if (live && r == 0) grad[(size_t)e * P + q] = g;
}

/* Gradient of W2 on the tensor cores: dW2[j][k] = sum_s dz2[s][j] h1[s][k]
 * (both FP32: hi*hi + hi*lo + lo*hi), one block of 4 warps per (member, 32 x
 * 32 tile), the samples streamed through shared memory 32 at a time.  Each
 * warp owns a 16 x 16 quarter (two m16n8 tiles).  The other parameters
 * are k_mlp_grad_small's. */
constexpr int GS = 32;            /* samples per chunk */
constexpr int GP = 36;            /* padded row stride of the chunk tiles */
__global__ void __launch_bounds__(H) k_mlp_grads_tc(MlpDev m, float* grad) {
  const int e = blockIdx.y;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int in = m.in, P = n_params(in);
  const size_t eb = (size_t)e * m.B;
  float* ge = grad + (size_t)e * P;
  __shared__ float dzs[GS][GP];   /* dz2[s][j0 + c] */
  __shared__ float hsm[GS][GP];   /* h1[s][k0 + c] */
  const int j0 = (blockIdx.x >> 2) * 32, k0 = (blockIdx.x & 3) * 32;
  const int g = lane >> 2, t = lane & 3;
  const int wm = (warp >> 1) * 16, wn = (warp & 1) * 16;   /* the warp's quarter */
  float acc[2][4];
#pragma unroll
  for (int nt = 0; nt < 2; ++nt)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[nt][c] = 0.0f;
  for (int c0 = 0; c0 < m.B; c0 += GS) {
    const int nc = m.B - c0 < GS ? m.B - c0 : GS;
    for (int idx = tid; idx < GS * 32; idx += H) {
      const int r = idx >> 5, c = idx & 31;
      dzs[r][c] = r < nc ? m.dz2[(eb + c0 + r) * H + j0 + c] : 0.0f;
      hsm[r][c] = r < nc ? m.h1[(eb + c0 + r) * H + k0 + c] : 0.0f;
    }
    __syncthreads();
    for (int s8 = 0; s8 < GS; s8 += 8) {
      /* A[j][s] = dz2[s][j]; B[s][k] = h1[s][k] */
      uint32_t ah[4], al[4];
      tf32_split(dzs[s8 + t][wm + g], &ah[0], &al[0]);
      tf32_split(dzs[s8 + t][wm + g + 8], &ah[1], &al[1]);
      tf32_split(dzs[s8 + t + 4][wm + g], &ah[2], &al[2]);
      tf32_split(dzs[s8 + t + 4][wm + g + 8], &ah[3], &al[3]);
#pragma unroll
      for (int nt = 0; nt < 2; ++nt) {
        uint32_t bh0, bl0, bh1, bl1;
        tf32_split(hsm[s8 + t][wn + nt * 8 + g], &bh0, &bl0);
        tf32_split(hsm[s8 + t + 4][wn + nt * 8 + g], &bh1, &bl1);
        mma_tf32(acc[nt], ah, bh0, bh1);
        mma_tf32(acc[nt], ah, bl0, bl1);
        mma_tf32(acc[nt], al, bh0, bh1);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int nt = 0; nt < 2; ++nt)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int j = j0 + wm + g + (c >= 2 ? 8 : 0);
      const int k = k0 + wn + nt * 8 + 2 * t + (c & 1);
      ge[off_w2(in) + (size_t)j * H + k] = acc[nt][c];
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
  /* the 128 x 128 layer on the tensor cores (k_mlp_fused, k_mlp_grads_tc);
   * SPP_MLP_SCALAR=1 at creation selects the scalar FP32 kernels */
  bool tensor_cores = true;
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
  if (m->tensor_cores) {
    dim3 grid((B + TS - 1) / TS, m->E);
    if (!backward) {
      k_mlp_fused<false><<<grid, H, FUSED_SMEM, m->stream>>>(d);
      return;
    }
    k_mlp_fused<true><<<grid, H, FUSED_SMEM, m->stream>>>(d);
    const long long small = (long long)m->E * (off_w2(m->in) + (m->P - off_b2(m->in))) * GSPLIT;
    k_mlp_grad_small<<<(unsigned)((small + 255) / 256), 256, 0, m->stream>>>(d, m->grad);
    k_mlp_grads_tc<<<dim3(16, m->E), H, 0, m->stream>>>(d, m->grad);
    return;
  }
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
  {
    const char* env = getenv("SPP_MLP_SCALAR");
    m->tensor_cores = !(env && env[0] == '1');
  }
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mlp_fused<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FUSED_SMEM);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mlp_fused<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FUSED_SMEM);
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
