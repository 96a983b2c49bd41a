/*
 * kernels_step.cu -- force sums fused with the integrator stage, on sm_103a.
 *
 * k_abp_stage replaces one Runge-Kutta stage of the reference's step, i.e.
 * Box::Interact (serial/box.h:322-371) followed by Box::Move_Runge_Kutta*_k
 * (serial/box.h:380-424 -> RepulsiveParticle::Move_Runge_Kutta{2,4}_k,
 * shared/particle.h:589-726), in one pass: one thread per particle (cell
 * order) gathers its Verlet neighbours' float4 (x, y, cos, sin) state,
 * sums force and torque in FP32 in ascending neighbour id (the lists are
 * sorted by id at every build, so the sums are reproducible), counts the
 * neighbours, and writes its stage state.  The last stage also
 *   - advances theta / image counters in place,
 *   - reduces the largest squared displacement since the last list build,
 *   - and, in the block that finishes last, decides whether the list must be
 *     rebuilt (max displacement > skin/2), sets the CUDA-graph conditional
 *     that gates the rebuild nodes, and advances the step counter.
 * The reference rebuilds cells after a fixed number of steps
 * (cell_update_period, parallel/box.h:432-438); the displacement trigger
 * rebuilds only when a pair could otherwise be missed.
 *
 * k_vicsek_step replaces VicsekParticle{,2}::Interact/Move
 * (shared/particle.h:145-247) and the configured arg-sum rule, reading the
 * cell-ordered copy and visiting the 3x3 cells directly (the cell list is
 * rebuilt every step at dt = 1).
 */
#include "spp_internal.cuh"
#include <cooperative_groups.h>
#include <mutex>

namespace {

struct StageBufs {
  const float4* cur;   /* state the forces are evaluated on */
  float4* out;         /* stage output (pos for the last stage) */
  int stage, nstages;
};

/* End-of-step bookkeeping shared by the step kernels.  Every block reduces
 * the largest squared displacement since the last list build (my_disp2) and
 * within this step (my_step2); the block that finishes last decides the
 * rebuild.  The list stays valid while no two particles together have moved
 * more than the skin, so the rebuild is scheduled one step ahead: when
 * max_disp + 2 * max_step_disp exceeds skin/2, i.e. before the next step
 * could carry a particle past skin/2.  A rebuild decided when some particle
 * has already passed skin/2 is counted in late_rebuilds (a diagnostic: pairs
 * may have been missed during that step). */
__device__ __forceinline__ void finish_step(const SppConsts& k, const DevState& d, float my_disp2,
                                            float my_step2, cudaGraphConditionalHandle cond,
                                            int use_cond) {
  __shared__ float warp_disp[32];   /* one per warp of the block (at most 32) */
  __shared__ float warp_step[32];
  __shared__ int is_last;
  const float m1 = __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(my_disp2)));
  const float m2 = __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(my_step2)));
  if ((threadIdx.x & 31) == 0) {
    warp_disp[threadIdx.x >> 5] = m1;
    warp_step[threadIdx.x >> 5] = m2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float b1 = 0.0f, b2 = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      b1 = fmaxf(b1, warp_disp[w]);
      b2 = fmaxf(b2, warp_step[w]);
    }
    if (b1 > 0.0f) atomicMax(&d.ctl->dmax2_bits, __float_as_uint(b1));
    if (b2 > 0.0f) atomicMax(&d.ctl->smax2_bits, __float_as_uint(b2));
    __threadfence();
    const unsigned prev = atomicAdd(&d.ctl->blocks_done, 1u);
    is_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (is_last && threadIdx.x == 0) {
    __threadfence();
    volatile Ctl* c = d.ctl;
    const int frozen = c->frozen;
    const float dm = sqrtf(__uint_as_float(c->dmax2_bits));
    const float sm = sqrtf(__uint_as_float(c->smax2_bits));
    unsigned rebuild = 0u;
    if (!frozen && k.half_skin > 0.0f) {
      rebuild = (dm + 2.0f * sm > k.half_skin) ? 1u : 0u;
      if (dm > k.half_skin) c->late_rebuilds = c->late_rebuilds + 1u;
    }
    c->need_rebuild = rebuild;
    c->dmax2_bits = 0u;
    c->smax2_bits = 0u;
    c->blocks_done = 0u;
    if (!frozen) c->step = c->step + 1u;
    if (use_cond) cudaGraphSetConditional(cond, rebuild);
  }
}

/* The same bookkeeping without block-wide barriers, for the stage kernel:
 * each warp folds its maxima into the block's shared words (fin[0..1], the
 * float bits of non-negative values, so unsigned max is float max) and
 * counts itself done in fin[2]; the warp that arrives last does the block's
 * global part.  Warps that finish early leave at once instead of waiting at
 * a barrier for the block's slowest warp.  fin is zeroed by the caller
 * before any warp can arrive. */
__device__ __forceinline__ void finish_step_nb(const SppConsts& k, const DevState& d, float my_disp2,
                                               float my_step2, cudaGraphConditionalHandle cond,
                                               int use_cond, unsigned* fin) {
  const unsigned m1 = __reduce_max_sync(0xffffffffu, __float_as_uint(my_disp2));
  const unsigned m2 = __reduce_max_sync(0xffffffffu, __float_as_uint(my_step2));
  if ((threadIdx.x & 31) != 0) return;
  atomicMax(&fin[0], m1);
  atomicMax(&fin[1], m2);
  __threadfence_block();
  const unsigned done = atomicAdd(&fin[2], 1u);
  if (done != (blockDim.x >> 5) - 1u) return;
  /* the block's last warp */
  __threadfence_block();
  const unsigned b1 = atomicAdd(&fin[0], 0u), b2 = atomicAdd(&fin[1], 0u);
  if (b1 > 0u) atomicMax(&d.ctl->dmax2_bits, b1);
  if (b2 > 0u) atomicMax(&d.ctl->smax2_bits, b2);
  __threadfence();
  const unsigned prev = atomicAdd(&d.ctl->blocks_done, 1u);
  if (prev != gridDim.x - 1) return;
  /* the grid's last block decides, as finish_step does */
  __threadfence();
  volatile Ctl* c = d.ctl;
  const int frozen = c->frozen;
  const float dm = sqrtf(__uint_as_float(c->dmax2_bits));
  const float sm = sqrtf(__uint_as_float(c->smax2_bits));
  unsigned rebuild = 0u;
  if (!frozen && k.half_skin > 0.0f) {
    rebuild = (dm + 2.0f * sm > k.half_skin) ? 1u : 0u;
    if (dm > k.half_skin) c->late_rebuilds = c->late_rebuilds + 1u;
  }
  c->need_rebuild = rebuild;
  c->dmax2_bits = 0u;
  c->smax2_bits = 0u;
  c->blocks_done = 0u;
  if (!frozen) c->step = c->step + 1u;
  if (use_cond) cudaGraphSetConditional(cond, rebuild);
}

/* Stage-kernel shape knobs: SPP_STAGE_UNIFORM 1 walks the neighbour lists
 * in warp-uniform trips up to the warp's longest list, masking the terms of
 * lanes past their own end (no divergent loop exits; measured slower at the
 * 1M workload, 33.3 against 32.7 us per launch: the masked terms cost more
 * than the divergence); SPP_STAGE_FINISH_NB 1 uses finish_step_nb (32.7
 * against 33.0 us). */
#ifndef SPP_STAGE_UNIFORM
#define SPP_STAGE_UNIFORM 0
#endif
#ifndef SPP_STAGE_FINISH_NB
#define SPP_STAGE_FINISH_NB 1
#endif

#ifndef SPP_STAGE_GROUP
#define SPP_STAGE_GROUP 2        /* neighbours whose loads are issued together (1: one-ahead prefetch) */
#endif
/* 1: the walk loads each group's list entries one group ahead (measured at
 * the 1M workload 600 steps in: 31.3 / 32.0 us per stage launch against
 * 32.0 / 32.8 without; with groups of one, 33.5 / 34.7) */
#ifndef SPP_STAGE_PIPE
#define SPP_STAGE_PIPE 1
#endif
#if SPP_STAGE_PIPE && (SPP_STAGE_SMEM_LIST || SPP_STAGE_BULK_ROWS > 0 || SPP_STAGE_UNIFORM)
#error "SPP_STAGE_PIPE is written for list entries read from global memory in the per-lane walk"
#endif
/* 1: with load groups of two, the pair's two 1/d are computed together by
 * two-lane instructions (spp_rsqrtf2).  Measured at the 1M workload 600
 * steps in: 33.2 us per launch against 31.8 (the extra live values spill
 * at the 32-register bound a full SM of threads needs); at 40 registers
 * and 6 blocks per SM it gains 1% (34.6 against 35.0 us), less than the
 * occupancy costs.  Off. */
#ifndef SPP_STAGE_RSQRT2
#define SPP_STAGE_RSQRT2 0
#endif

/* One neighbour's contribution; the chain kind also needs the neighbour's
 * bead count (1 for membrane beads).  valid = 0 marks a padding entry of a
 * load group: the ABP, continuous and bead kinds mask it (no branch), the
 * chain kind skips it. */
template <int LAW, int KIND>
__device__ __forceinline__ void stage_pair(const SppConsts& k, const DevState& d, int wrap, SppAccF* a,
                                           int nbi, int j, float4 pi, float4 pj, int valid) {
  if (KIND == SPP_KIND_CHAIN) {
    if (!valid) return;
    const int nbj = __ldg(d.id + j) < (uint32_t)k.n_beads ? 1 : k.chain_nb;
    spp_pair_chain(&k, LAW, wrap, a, nbi, nbj, pi.x, pi.y, pi.z, pi.w, pj.x, pj.y, pj.z, pj.w);
  } else {
    spp_pair_abp_lkwv(&k, LAW, KIND, wrap, a, pi.x, pi.y, pi.z, pi.w, pj.x, pj.y, pj.z, pj.w, valid);
  }
}

#ifndef SPP_STAGE_BLOCK
#define SPP_STAGE_BLOCK 256      /* threads per block of the stage kernel */
#endif
#ifndef SPP_STAGE_MIN_BLOCKS
#define SPP_STAGE_MIN_BLOCKS (2048 / SPP_STAGE_BLOCK)   /* a full SM: 32 registers */
#endif
/* Where the stage kernel fetches the per-particle inputs that the
 * neighbour walk does not need (heading, the step's noise and start-of-step
 * position, the list-build position, the id for the noise): 0 after the
 * walk; 1 into registers before it (their latency overlaps the walk, at the
 * price of registers held through it); 2 after the walk, with L1 prefetches
 * of their lines issued before it (the overlap without the registers). */
#ifndef SPP_STAGE_PREFETCH
#define SPP_STAGE_PREFETCH 0
#endif
/* List entries of a thread kept in shared memory during the walk (0: read
 * from global memory group by group) and how many of their loads are issued
 * together when they are fetched. */
#ifndef SPP_STAGE_SMEM_LIST
#define SPP_STAGE_SMEM_LIST 0
#endif
#ifndef SPP_STAGE_FILL
#define SPP_STAGE_FILL 8
#endif

/* List rows copied into shared memory by the bulk-copy engine: with one
 * lane per particle and n a multiple of 4 (so that every row segment starts
 * on a 16-byte boundary), lane 0 of each warp copies rows 0 .. R - 1 of the
 * warp's 32 list columns (the column-major list keeps a row's 32 entries
 * contiguous: 128 bytes) with cp.async.bulk, R = min(the warp's longest
 * list, SPP_STAGE_BULK_ROWS), all completing on one mbarrier of the warp.
 * The walk then takes its list entries from shared memory (entries past R
 * from global memory) and only the neighbour states from L1/L2, so each
 * pair waits on one memory round trip instead of two, and the list loads
 * leave the SM's load pipe.  0 disables.  Measured at the 1M workload 600
 * steps in (stage us per launch, same trajectory bits, no copy timed out):
 * 16 rows 38.4, 12 rows 38.6, 8 rows 37.8 against 31.4 without; with the
 * shared-memory carveout at its maximum (SPP_STAGE_CARVEOUT=100) 16 rows
 * 38.2, 8 rows 38.6, 4 rows 37.1.  The warp's walk cannot start before all
 * its rows have landed, and the list loads it saves were not what bound
 * the kernel.  Off. */
#ifndef SPP_STAGE_BULK_ROWS
#define SPP_STAGE_BULK_ROWS 0
#endif
/* try_wait polls before a warp gives up on its copies (each poll may
 * suspend the warp for a while); it then reads the list from global memory
 * and counts itself in Ctl.bulk_timeouts */
#define SPP_BULK_WAIT_LIMIT (1 << 20)

#if SPP_STAGE_BULK_ROWS > 0
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void bulk_issue_rows(uint32_t bar, uint32_t dst, const int32_t* src, size_t stride,
                                                uint32_t bytes, int rows) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes * (uint32_t)rows)
               : "memory");
  for (int q = 0; q < rows; ++q)
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     dst + (uint32_t)q * 128u),
                 "l"(src + (size_t)q * stride), "r"(bytes), "r"(bar)
                 : "memory");
}
/* true once the copies tracked by bar (phase 0) have landed */
__device__ __forceinline__ bool bulk_wait(uint32_t bar) {
  for (int it = 0; it < SPP_BULK_WAIT_LIMIT; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar)
        : "memory");
    if (ok) return true;
  }
  return false;
}
#endif

__device__ __forceinline__ void prefetch_l1(const void* p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

/* The per-particle inputs of a stage besides the state the neighbours read. */
template <bool BEADLIKE>
__device__ __forceinline__ void stage_inputs(const DevState& d, const StageBufs& b, int i, int last,
                                             uint32_t* pid, float* th0, float* dth_in, float2* p0,
                                             float2* rf) {
  if (!BEADLIKE && b.stage == 0) *pid = d.id[i];
  *th0 = d.theta[i];
  if (b.stage > 0) {
    *dth_in = d.dth[i];
    *p0 = reinterpret_cast<const float2*>(d.pos)[2 * (size_t)i];
  }
  if (last) *rf = d.ref[i];
}
/* the chain pair loop (bead offsets, lever-arm torques) needs more than
 * 32 registers: 4 x 256 threads per SM there.
 * LANES threads per particle (LANES = k.lanes: 1, or 4 for small ABP /
 * continuous systems): lane r sums the neighbours with id % 4 == r, one
 * id-ordered segment of the list (spp_list_order), and the lane sums
 * combine through xor shuffles as (p0 + p1) + (p2 + p3); lane 0 then
 * finishes the particle.
 * Latency: every per-particle input of the stage (state, list length,
 * heading, the step's noise and start-of-step position, the list-build
 * position) is loaded before the neighbour walk, so those loads overlap it,
 * and the frozen flag is read alongside rather than ahead of them. */
template <int LAW, int KIND, int LANES, int CLOSED>
__global__ void __launch_bounds__(SPP_STAGE_BLOCK, KIND == SPP_KIND_CHAIN ? 1024 / SPP_STAGE_BLOCK : SPP_STAGE_MIN_BLOCKS) k_abp_stage(SppConsts k, DevState d, StageBufs b,
                                                         cudaGraphConditionalHandle cond,
                                                         int use_cond) {
  constexpr bool BEADLIKE = (KIND == SPP_KIND_BEADS || KIND == SPP_KIND_CHAIN);
  const int tg = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = tg / LANES;
  const int lane_r = tg % LANES;
  const int last = (b.stage == b.nstages - 1);
  const bool inb = i < d.n;
  const bool head = LANES == 1 || lane_r == 0;   /* the lane that finishes the particle */
#if SPP_STAGE_FINISH_NB
  __shared__ unsigned fin[3];
  if (last) {   /* the same for the whole block */
    if (threadIdx.x < 3) fin[threadIdx.x] = 0u;
    __syncthreads();
  }
#endif
  float disp2 = 0.0f, step2 = 0.0f;
  float4 pi = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  int q_begin = 0, q_end = 0;
  uint32_t pid = 0u;
  float th0 = 0.0f, dth_in = 0.0f;
  float2 p0 = make_float2(0.0f, 0.0f), rf = make_float2(0.0f, 0.0f);
  if (inb) {
    pi = b.cur[i];
    q_end = d.nn[i];
    if (LANES > 1) {
      const unsigned long long lc = d.nn_lanes[i];
      for (int r = 0; r < lane_r; ++r) q_begin += (int)((lc >> (16 * r)) & 0xffffull);
      q_end = q_begin + (int)((lc >> (16 * lane_r)) & 0xffffull);
    }
    if (head) {
      if (BEADLIKE) pid = d.id[i];
      if (SPP_STAGE_PREFETCH == 1) {
        stage_inputs<BEADLIKE>(d, b, i, last, &pid, &th0, &dth_in, &p0, &rf);
      } else if (SPP_STAGE_PREFETCH == 2) {
        if (!BEADLIKE && b.stage == 0) prefetch_l1(d.id + i);
        prefetch_l1(d.theta + i);
        if (b.stage > 0) {
          prefetch_l1(d.dth + i);
          prefetch_l1(d.pos + i);
        }
        if (last) prefetch_l1(d.ref + i);
      }
    }
  }
#if SPP_STAGE_BULK_ROWS > 0
  __shared__ __align__(128) int32_t blist[SPP_STAGE_BLOCK / 32][SPP_STAGE_BULK_ROWS][32];
  __shared__ __align__(8) unsigned long long bbar[SPP_STAGE_BLOCK / 32];
  const int wl = threadIdx.x & 31, ww = threadIdx.x >> 5;
  int rows = 0;            /* list rows of this warp in shared memory */
  bool bulk_late = false;  /* copies issued but not seen complete */
  if (LANES == 1 && (d.n & 3) == 0) {
    const int first = tg - wl;   /* the warp's first particle */
    rows = min((int)__reduce_max_sync(0xffffffffu, (unsigned)q_end), SPP_STAGE_BULK_ROWS);
    if (first >= d.n) rows = 0;
    if (rows > 0) {
      const uint32_t bar = smem_u32(&bbar[ww]);
      if (wl == 0)
        bulk_issue_rows(bar, smem_u32(&blist[ww][0][0]), d.nbr + first, (size_t)d.n,
                        (uint32_t)min(32, d.n - first) * 4u, rows);
      __syncwarp();
      if (!__all_sync(0xffffffffu, bulk_wait(bar))) {
        bulk_late = true;
        rows = 0;
        if (wl == 0) atomicAdd(&d.ctl->bulk_timeouts, 1u);
      }
    }
  }
#endif
  const int frozen = d.ctl->frozen;
  if (inb && !frozen) {
    SppAccF a;
    spp_accf_zero(&a);
    const int nbi = (KIND == SPP_KIND_CHAIN && pid >= (uint32_t)k.n_beads) ? k.chain_nb : 1;
    const int32_t* __restrict__ nb = d.nbr + i;
    const size_t stride = (size_t)d.n;
    /* Warps whose particles are all far from the box edges skip the
     * minimum-image corrections (they would not change any separation). */
    const int inner = fabsf(pi.x) < k.interior && fabsf(pi.y) < k.interior;
    const int all_inner = __all_sync(__activemask(), inner);
#if SPP_STAGE_SMEM_LIST
    /* the thread's list entries (up to SPP_STAGE_SMEM_LIST of them) are
     * fetched first, SPP_STAGE_FILL at a time with their loads in flight
     * together, into the thread's column of shared memory: the walk then
     * waits on one global round trip per group (the neighbour states) */
    __shared__ int32_t slist[SPP_STAGE_SMEM_LIST][SPP_STAGE_BLOCK];
    const int q_fill = min(q_end, q_begin + SPP_STAGE_SMEM_LIST);
    for (int q = q_begin; q < q_fill; q += SPP_STAGE_FILL) {
      int32_t v[SPP_STAGE_FILL];
#pragma unroll
      for (int u = 0; u < SPP_STAGE_FILL; ++u) v[u] = q + u < q_fill ? __ldg(nb + (size_t)(q + u) * stride) : 0;
#pragma unroll
      for (int u = 0; u < SPP_STAGE_FILL; ++u)
        if (q + u < q_fill) slist[q + u - q_begin][threadIdx.x] = v[u];
    }
#endif
    /* list entries and neighbour states are loaded SPP_STAGE_GROUP at a time
     * (independent loads in flight), the pairs evaluated in list order */
#if SPP_STAGE_UNIFORM
    /* trips up to the warp's longest list, the same for every lane: lanes
     * past their own end load their own state and mask the term */
    const int my_len = q_end - q_begin;
    const int wmax = (int)__reduce_max_sync(__activemask(), (unsigned)my_len);
    for (int t0 = 0; t0 < wmax; t0 += SPP_STAGE_GROUP) {
      int jg[SPP_STAGE_GROUP];
      float4 pg[SPP_STAGE_GROUP];
#pragma unroll
      for (int u = 0; u < SPP_STAGE_GROUP; ++u) {
        const int q = q_begin + t0 + u;
#if SPP_STAGE_SMEM_LIST
        jg[u] = t0 + u < my_len ? (q < q_fill ? slist[q - q_begin][threadIdx.x] : __ldg(nb + (size_t)q * stride)) : i;
#else
        jg[u] = t0 + u < my_len ? __ldg(nb + (size_t)q * stride) : i;
#endif
        if (!spp_index_ok(d.ctl, jg[u], d.n)) jg[u] = i;
      }
#pragma unroll
      for (int u = 0; u < SPP_STAGE_GROUP; ++u) pg[u] = __ldg(b.cur + jg[u]);
#pragma unroll
      for (int u = 0; u < SPP_STAGE_GROUP; ++u) {
        if (t0 + u < wmax) {   /* warp-uniform */
          if (all_inner || CLOSED)
            stage_pair<LAW, KIND>(k, d, 0, &a, nbi, jg[u], pi, pg[u], t0 + u < my_len);
          else
            stage_pair<LAW, KIND>(k, d, 1, &a, nbi, jg[u], pi, pg[u], t0 + u < my_len);
        }
      }
    }
#else
#if SPP_STAGE_PIPE
    /* list entries one group ahead: the next group's indices are loaded
     * while this group's neighbour states arrive and its terms are summed */
    int jn[SPP_STAGE_GROUP];
#pragma unroll
    for (int u = 0; u < SPP_STAGE_GROUP; ++u) {
      const int q = q_begin + u;
      jn[u] = q < q_end ? __ldg(nb + (size_t)q * stride) : i;
    }
#endif
    for (int q0 = q_begin; q0 < q_end; q0 += SPP_STAGE_GROUP) {
      int jg[SPP_STAGE_GROUP];
      float4 pg[SPP_STAGE_GROUP];
#if SPP_STAGE_PIPE
#pragma unroll
      for (int u = 0; u < SPP_STAGE_GROUP; ++u) {
        jg[u] = jn[u];
        if (!spp_index_ok(d.ctl, jg[u], d.n)) jg[u] = i;
      }
#pragma unroll
      for (int u = 0; u < SPP_STAGE_GROUP; ++u) pg[u] = __ldg(b.cur + jg[u]);
#pragma unroll
      for (int u = 0; u < SPP_STAGE_GROUP; ++u) {
        const int q = q0 + SPP_STAGE_GROUP + u;
        jn[u] = q < q_end ? __ldg(nb + (size_t)q * stride) : i;
      }
#else
#pragma unroll
      for (int u = 0; u < SPP_STAGE_GROUP; ++u) {
        const int q = q0 + u;
#if SPP_STAGE_SMEM_LIST
        jg[u] = q < q_end ? (q < q_fill ? slist[q - q_begin][threadIdx.x] : __ldg(nb + (size_t)q * stride)) : i;
#elif SPP_STAGE_BULK_ROWS > 0
        jg[u] = q < q_end ? (q < rows ? blist[ww][q][wl] : __ldg(nb + (size_t)q * stride)) : i;
#else
        jg[u] = q < q_end ? __ldg(nb + (size_t)q * stride) : i;
#endif
        if (!spp_index_ok(d.ctl, jg[u], d.n)) jg[u] = i;
      }
#pragma unroll
      for (int u = 0; u < SPP_STAGE_GROUP; ++u) pg[u] = __ldg(b.cur + jg[u]);
#endif
#if SPP_STAGE_RSQRT2
      if (SPP_STAGE_GROUP == 2 && KIND != SPP_KIND_CHAIN) {
        /* both separations, then both 1/d in one two-lane Newton sequence
         * (each lane the bits of spp_rsqrtf); a padding entry past the list
         * end (j = i, d2 = 0) gets a finite r and is not applied */
        float dx[2], dy[2], d2[2];
        if (all_inner || CLOSED) {
#pragma unroll
          for (int u = 0; u < 2; ++u) d2[u] = spp_pair_sep(&k, 0, pi.x, pi.y, pg[u].x, pg[u].y, &dx[u], &dy[u]);
        } else {
#pragma unroll
          for (int u = 0; u < 2; ++u) d2[u] = spp_pair_sep(&k, 1, pi.x, pi.y, pg[u].x, pg[u].y, &dx[u], &dy[u]);
        }
        spp_f2 r = spp_f2_make(0.0f, 0.0f);
        if (spp_pair_needs_r(LAW, KIND)) r = spp_rsqrtf2(spp_f2_make(d2[0], d2[1]));
        spp_pair_abp_apply(&k, LAW, KIND, &a, dx[0], dy[0], d2[0], r.x, pi.z, pi.w, pg[0].z, pg[0].w, 1);
        if (q0 + 1 < q_end)
          spp_pair_abp_apply(&k, LAW, KIND, &a, dx[1], dy[1], d2[1], r.y, pi.z, pi.w, pg[1].z, pg[1].w, 1);
        continue;
      }
#endif
#pragma unroll
      for (int u = 0; u < SPP_STAGE_GROUP; ++u) {
        /* entries past the list end are skipped (a warp whose lanes all
         * reached their ends skips the whole term); the term itself has no
         * branches.  The minimum image only off the interior of a periodic
         * box. */
        if (q0 + u < q_end) {
          if (all_inner || CLOSED)
            stage_pair<LAW, KIND>(k, d, 0, &a, nbi, jg[u], pi, pg[u], 1);
          else
            stage_pair<LAW, KIND>(k, d, 1, &a, nbi, jg[u], pi, pg[u], 1);
        }
      }
    }
#endif
    if (LANES > 1) {
      /* the lanes of one particle are consecutive and all present */
      const unsigned gmask = ((1u << LANES) - 1u) << ((threadIdx.x & 31) & ~(LANES - 1));
#pragma unroll
      for (int o = 1; o < LANES; o <<= 1) {
        a.fx = a.fx + __shfl_xor_sync(gmask, a.fx, o);
        a.fy = a.fy + __shfl_xor_sync(gmask, a.fy, o);
        a.ss = a.ss + __shfl_xor_sync(gmask, a.ss, o);
        a.sc = a.sc + __shfl_xor_sync(gmask, a.sc, o);
        a.tq = a.tq + __shfl_xor_sync(gmask, a.tq, o);
        a.cnt += __shfl_xor_sync(gmask, a.cnt, o);
        a.ovf |= __shfl_xor_sync(gmask, a.ovf, o);
      }
    }
  if (head) {
    if (SPP_STAGE_PREFETCH != 1) stage_inputs<BEADLIKE>(d, b, i, last, &pid, &th0, &dth_in, &p0, &rf);
    if (LAW == SPP_FORCE_R12_TRUNC && a.ovf) atomicOr(&d.ctl->fx_overflow, 1u);
    float fx, fy, tau;
    int turns = 1;
    int chain_swimmer = 0;
    if (BEADLIKE) {
      /* membrane beads add their ring forces; positions of the ring
       * neighbours come from the same stage state, found through id -> slot */
      float rfx = 0.0f, rfy = 0.0f;
      const int bead = pid < (uint32_t)k.n_beads;
      if (bead) {
        float px[5], py[5];
#pragma unroll
        for (int o = -2; o <= 2; ++o) {
          uint32_t slot = o == 0 ? (uint32_t)i : d.inv[spp_ring_neighbor(&k, pid, o)];
          if (!spp_index_ok(d.ctl, slot, d.n)) slot = (uint32_t)i;
          const float4 q = o == 0 ? pi : __ldg(b.cur + slot);
          px[o + 2] = q.x;
          py[o + 2] = q.y;
        }
        spp_ring_forces(&k, px, py, &rfx, &rfy);
      }
      if (KIND == SPP_KIND_CHAIN && !bead) {
        chain_swimmer = 1;
        spp_chain_velocity(&k, &a, pi.z, pi.w, pi.z, pi.w, &fx, &fy, &tau);
      } else {
        spp_bead_velocity(&k, !bead, &a, rfx, rfy, pi.z, pi.w, &fx, &fy, &tau);
      }
      turns = !bead;
    } else {
      spp_abp_forces(&k, CLOSED, &a, pi.x, pi.y, pi.z, pi.w, &fx, &fy, &tau);
    }
    float dth;
    if (b.stage == 0) {
      if (!turns) {
        dth = 0.0f;
      } else if (BEADLIKE && k.tumble) {
        dth = spp_tumble_noise(&k, pid, d.ctl->step, d.tumble + pid);
      } else {
        dth = spp_rot_noise(&k, pid, d.ctl->step);
      }
      if (b.nstages > 1) d.dth[i] = dth;
      p0 = make_float2(pi.x, pi.y);
    } else {
      dth = dth_in;
    }
    if (KIND == SPP_KIND_CHAIN && chain_swimmer && b.nstages == 1) {
      /* Move() turns first and projects the force on the new heading */
      float wc, ws;
      spp_sincosf(spp_euler_theta(&k, th0, tau, dth), &ws, &wc);
      spp_chain_velocity(&k, &a, pi.z, pi.w, wc, ws, &fx, &fy, &tau);
    }
    float nx, ny, nt, nc, ns;
    int gx = 0, gy = 0;
    if (b.nstages == 1) {
      spp_euler_update(p0.x, p0.y, th0, fx, fy, tau, dth, &k, &nx, &ny, &nt, &nc, &ns, &gx, &gy, CLOSED);
    } else {
      float h, frac;
      if (b.nstages == 2) {
        h = b.stage == 0 ? k.half_dt : k.dt;
        frac = b.stage == 0 ? 0.5f : 1.0f;
      } else {
        if (b.stage == 0) {
          d.kacc[i] = make_float4(fx, fy, tau, 0.0f);
        } else if (b.stage < 3) {
          const float4 ka = d.kacc[i];
          d.kacc[i] = make_float4(ka.x + 2.0f * fx, ka.y + 2.0f * fy, ka.z + 2.0f * tau, 0.0f);
        } else {
          const float4 ka = d.kacc[i];
          fx = ka.x + fx; fy = ka.y + fy; tau = ka.z + tau;
        }
        h = b.stage < 2 ? k.half_dt : (b.stage == 2 ? k.dt : k.dt6);
        frac = b.stage < 2 ? 0.5f : 1.0f;
      }
      spp_stage_update(h, frac, p0.x, p0.y, th0, fx, fy, tau, dth, &k, &nx, &ny, &nt, &nc, &ns,
                       &gx, &gy, CLOSED);
    }
    b.out[i] = make_float4(nx, ny, nc, ns);
    if (last) {
      d.theta[i] = nt;
      if (gx | gy) {
        const int2 g = d.img[i];
        d.img[i] = make_int2(g.x + gx, g.y + gy);
      }
      float ddx, ddy;
      disp2 = spp_sep_cl(&k, CLOSED, nx, ny, rf.x, rf.y, &ddx, &ddy);
      step2 = spp_sep_cl(&k, CLOSED, nx, ny, p0.x, p0.y, &ddx, &ddy);
    }
  }
  }
#if SPP_STAGE_BULK_ROWS > 0
  /* copies that were late must land before the block's shared memory is
   * released */
  if (bulk_late) bulk_wait(smem_u32(&bbar[ww]));
#endif
#if SPP_STAGE_FINISH_NB
  if (last) finish_step_nb(k, d, disp2, step2, cond, use_cond, fin);
#else
  if (last) finish_step(k, d, disp2, step2, cond, use_cond);
#endif
}

__global__ void __launch_bounds__(SPP_BLOCK) k_vicsek_step(SppConsts k, DevState d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < d.n) {
    const uint32_t step = d.ctl->step;
    const float4 p = d.pos_alt[i];
    const float th0 = d.theta_alt[i];
    const uint32_t id = d.id_alt[i];
    const int cx = spp_cell_coord(p.x, k.L, k.L2, d.D, SPP_BIN_GEOMETRIC);
    const int cy = spp_cell_coord(p.y, k.L, k.L2, d.D, SPP_BIN_GEOMETRIC);
    const int D = d.D;
    const int need_theta = (k.model == SPP_MODEL_VICSEK_REF_ANGLE);
    SppAcc a;
    spp_acc_zero(&a);
    for (int oy = -1; oy <= 1; ++oy) {
      int ny = cy + oy;
      ny = ny < 0 ? ny + D : (ny >= D ? ny - D : ny);
      for (int ox = -1; ox <= 1; ++ox) {
        int nx = cx + ox;
        nx = nx < 0 ? nx + D : (nx >= D ? nx - D : nx);
        const uint32_t kk = spp_morton((uint32_t)nx, (uint32_t)ny);
        if (!spp_index_ok(d.ctl, kk, d.n_keys)) continue;
        const uint32_t s0 = d.cell_start[kk], c = d.cell_count[kk];
        if (!spp_index_ok(d.ctl, (long long)s0 + c, (long long)d.n + 1)) continue;
        for (uint32_t j = s0; j < s0 + c; ++j) {
          const float4 q = __ldg(d.pos_alt + j);
          const float thj = need_theta ? d.theta_alt[j] : 0.0f;
          spp_pair_vicsek(&k, &a, p.x, p.y, q.x, q.y, q.z, q.w, thj, (int)j == i);
        }
      }
    }
    if (k.closed && k.model == SPP_MODEL_VICSEK_REF_ANGLE) spp_vicsek_walls(&k, &a, p.x, p.y, th0);
    if (a.ovf) atomicOr(&d.ctl->fx_overflow, 1u);
    const spp_u32x4 r = spp_draw_k(&k, id, step, SPP_RNG_VICSEK);
    float x, y, t, c, s;
    int gx = 0, gy = 0;
    spp_vicsek_update(&k, &a, p.x, p.y, th0, p.z, p.w, r.v[0], &x, &y, &t, &c, &s, &gx, &gy);
    d.pos[i] = make_float4(x, y, c, s);
    d.theta[i] = t;
    int2 g = d.img_alt[i];
    d.img[i] = make_int2(g.x + gx, g.y + gy);
    d.id[i] = id;
  }
  finish_step(k, d, 0.0f, 0.0f, 0, 0);
}

/* Small Vicsek systems in one thread-block cluster: k_vicsek_small runs
 * nsteps whole steps in a single launch.  Per step every CTA of the cluster
 * bins all particles into its own shared-memory cell table (count, scan,
 * cell-ordered copy of the states; cheap next to the pair sums), then
 * updates its own slice of the particles from that copy.  The state is
 * double-buffered in global memory (pos/theta <-> pos_alt/theta_alt, read
 * through L2): step t reads one buffer and writes the other, so a single
 * cluster barrier per step orders every write before the next step's
 * reads.  The heading sums are exact fixed point and the noise is keyed by
 * particle id and step, so the result is bit-identical to the multi-kernel
 * step (k_bin_count / scan / k_scatter / k_vicsek_step), which at these
 * sizes is bound by launch latency. */
#ifndef SPP_SMALL_THREADS
#define SPP_SMALL_THREADS 1024
#endif
#ifndef SPP_SMALL_LANES
#define SPP_SMALL_LANES 4          /* lanes per particle in the pair sums (1, 2, 4 or 8) */
#endif
#define SPP_SMALL_BATCH 4
#ifndef SPP_SMALL_CLUSTER_MAX
#define SPP_SMALL_CLUSTER_MAX 16   /* CTAs per cluster, tried downwards in powers of 2 */
#endif

__global__ void __launch_bounds__(SPP_SMALL_THREADS, 1) k_vicsek_small(SppConsts k, DevState d, int nsteps) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ float4 small_mem[];
  const int n = d.n, D = d.D, C = D * D;
  const int need_theta = (k.model == SPP_MODEL_VICSEK_REF_ANGLE);
  float4* sp = small_mem;                                        /* n cell-ordered states */
  float* sth = reinterpret_cast<float*>(sp + n);                 /* n headings (REF_ANGLE) */
  int* cnt = reinterpret_cast<int*>(sth + (need_theta ? n : 0)); /* C counts */
  int* start = cnt + C;                                          /* C exclusive starts */
  int* packed = start + C;                                       /* n: cell | rank << 16 */
  __shared__ int warp_tot[SPP_SMALL_THREADS / 32];
  __shared__ unsigned ovf;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int R = (int)cluster.num_blocks(), rk = (int)cluster.block_rank();
  const int per_cta = (n + R - 1) / R;
  const int i0 = rk * per_cta, i1 = min(n, i0 + per_cta);
  if (d.ctl->frozen) return;   /* the same word for every CTA: all return or none */
  uint32_t step = d.ctl->step;
  if (tid == 0) ovf = 0u;
  const int per_c = (C + SPP_SMALL_THREADS - 1) / SPP_SMALL_THREADS;
  for (int t = 0; t < nsteps; ++t, ++step) {
    const float4* __restrict__ src_pos = (t & 1) ? d.pos_alt : d.pos;
    const float* __restrict__ src_th = (t & 1) ? d.theta_alt : d.theta;
    float4* dst_pos = (t & 1) ? d.pos : d.pos_alt;
    float* dst_th = (t & 1) ? d.theta : d.theta_alt;
    for (int c = tid; c < C; c += SPP_SMALL_THREADS) cnt[c] = 0;
    __syncthreads();
    /* loads from L2 issued SPP_SMALL_BATCH at a time */
    for (int ib = tid; ib < n; ib += SPP_SMALL_BATCH * SPP_SMALL_THREADS) {
      float4 pv[SPP_SMALL_BATCH];
#pragma unroll
      for (int u = 0; u < SPP_SMALL_BATCH; ++u) {
        const int i = ib + u * SPP_SMALL_THREADS;
        pv[u] = i < n ? __ldcg(src_pos + i) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      }
#pragma unroll
      for (int u = 0; u < SPP_SMALL_BATCH; ++u) {
        const int i = ib + u * SPP_SMALL_THREADS;
        if (i < n) {
          const int cx = spp_cell_coord(pv[u].x, k.L, k.L2, D, SPP_BIN_GEOMETRIC);
          const int cy = spp_cell_coord(pv[u].y, k.L, k.L2, D, SPP_BIN_GEOMETRIC);
          const int cell = cy * D + cx;
          packed[i] = cell | (atomicAdd(&cnt[cell], 1) << 16);
        }
      }
    }
    __syncthreads();
    /* exclusive scan of the counts: per_c consecutive cells per thread */
    {
      const int c0 = tid * per_c;
      int local = 0;
      for (int c = c0; c < c0 + per_c && c < C; ++c) local += cnt[c];
      int incl = local;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
      }
      if (lane == 31) warp_tot[wid] = incl;
      __syncthreads();
      if (wid == 0) {
        int w = lane < SPP_SMALL_THREADS / 32 ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int v = __shfl_up_sync(0xffffffffu, w, o);
          if (lane >= o) w += v;
        }
        if (lane < SPP_SMALL_THREADS / 32) warp_tot[lane] = w;
      }
      __syncthreads();
      int run = incl - local + (wid > 0 ? warp_tot[wid - 1] : 0);
      for (int c = c0; c < c0 + per_c && c < C; ++c) {
        start[c] = run;
        run += cnt[c];
      }
    }
    __syncthreads();
    for (int ib = tid; ib < n; ib += SPP_SMALL_BATCH * SPP_SMALL_THREADS) {
      float4 pv[SPP_SMALL_BATCH];
      float tv[SPP_SMALL_BATCH];
#pragma unroll
      for (int u = 0; u < SPP_SMALL_BATCH; ++u) {
        const int i = ib + u * SPP_SMALL_THREADS;
        pv[u] = i < n ? __ldcg(src_pos + i) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        tv[u] = (need_theta && i < n) ? __ldcg(src_th + i) : 0.0f;
      }
#pragma unroll
      for (int u = 0; u < SPP_SMALL_BATCH; ++u) {
        const int i = ib + u * SPP_SMALL_THREADS;
        if (i < n) {
          const int pk = packed[i];
          const int slot = start[pk & 0xffff] + (pk >> 16);
          if (!spp_index_ok(d.ctl, slot, n)) continue;
          sp[slot] = pv[u];
          if (need_theta) sth[slot] = tv[u];
        }
      }
    }
    __syncthreads();
    /* SPP_SMALL_LANES consecutive lanes per particle: lane q walks cells
     * q, q + LANES, ... of the 3x3 block; the exact fixed-point partial sums
     * add up to the same integers in any grouping, and lane 0 of the group
     * draws the noise and writes the particle */
    {
      const int q = tid % SPP_SMALL_LANES;
      const int grp = tid / SPP_SMALL_LANES;
      constexpr int GROUPS = SPP_SMALL_THREADS / SPP_SMALL_LANES;
      for (int base = i0; base < i1; base += GROUPS) {
        const int i = base + grp;
        const bool valid = i < i1;
        SppAcc a;
        spp_acc_zero(&a);
        int me = 0;
        float4 p = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (valid) {
          const int pk = packed[i];
          const int cell = pk & 0xffff;
          me = start[cell] + (pk >> 16);
          p = sp[me];
          const int cx = cell % D, cy = cell / D;
          for (int c9 = q; c9 < 9; c9 += SPP_SMALL_LANES) {
            int ny = cy + c9 / 3 - 1;
            ny = ny < 0 ? ny + D : (ny >= D ? ny - D : ny);
            int nx = cx + c9 % 3 - 1;
            nx = nx < 0 ? nx + D : (nx >= D ? nx - D : nx);
            const int kk = ny * D + nx;
            const int s0 = start[kk], s1 = s0 + cnt[kk];
            for (int j = s0; j < s1; ++j) {
              const float4 qq = sp[j];
              spp_pair_vicsek(&k, &a, p.x, p.y, qq.x, qq.y, qq.z, qq.w, need_theta ? sth[j] : 0.0f, j == me);
            }
          }
        }
#pragma unroll
        for (int o = 1; o < SPP_SMALL_LANES; o <<= 1) {
          a.ax.hi += __shfl_xor_sync(0xffffffffu, a.ax.hi, o);
          a.ax.lo += __shfl_xor_sync(0xffffffffu, a.ax.lo, o);
          a.ay.hi += __shfl_xor_sync(0xffffffffu, a.ay.hi, o);
          a.ay.lo += __shfl_xor_sync(0xffffffffu, a.ay.lo, o);
          a.at.hi += __shfl_xor_sync(0xffffffffu, a.at.hi, o);
          a.at.lo += __shfl_xor_sync(0xffffffffu, a.at.lo, o);
          a.cnt += __shfl_xor_sync(0xffffffffu, a.cnt, o);
          a.ovf |= __shfl_xor_sync(0xffffffffu, a.ovf, o);
        }
        if (valid && q == 0) {
          if (k.closed && need_theta) spp_vicsek_walls(&k, &a, p.x, p.y, sth[me]);
          if (a.ovf) ovf = 1u;
          const spp_u32x4 r = spp_draw_k(&k, d.id[i], step, SPP_RNG_VICSEK);
          float x, y, th, c, sn;
          int gx = 0, gy = 0;
          spp_vicsek_update(&k, &a, p.x, p.y, __ldcg(src_th + i), p.z, p.w, r.v[0], &x, &y, &th, &c, &sn,
                            &gx, &gy);
          dst_pos[i] = make_float4(x, y, c, sn);
          dst_th[i] = th;
          if (gx | gy) {   /* only this thread touches particle i's counters */
            const int2 g = d.img[i];
            d.img[i] = make_int2(g.x + gx, g.y + gy);
          }
        }
      }
    }
    /* every write of this step before any read of the next */
    cluster.sync();
  }
  if (nsteps & 1) {
    /* the last step wrote the alternate buffers: move this CTA's slice back */
    for (int i = i0 + tid; i < i1; i += SPP_SMALL_THREADS) {
      d.pos[i] = d.pos_alt[i];
      d.theta[i] = d.theta_alt[i];
    }
  }
  __syncthreads();
  if (tid == 0) {
    if (ovf) atomicOr(&d.ctl->fx_overflow, 1u);
    if (rk == 0) {
      d.ctl->step = step;
      d.ctl->need_rebuild = 0u;
    }
  }
}

/* Euler writes its new state to the half buffer (neighbours read pos during
 * the stage); this commits it. */
__global__ void __launch_bounds__(SPP_BLOCK) k_commit(DevState d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < d.n && !d.ctl->frozen) d.pos[i] = d.half[i];
}

/* Sum of (cos, sin) over all particles in int64 fixed point: exact, hence
 * independent of the particle order (Node::Compute_Polarization,
 * parallel/node.h:1565-1591, replaces its MPI_Reduce). */
__global__ void __launch_bounds__(SPP_BLOCK) k_polarization(DevState d, unsigned long long* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  long long sx = 0, sy = 0;
  if (i < d.n) {
    const float4 p = d.pos[i];
    spp_fx a = {0, 0}, b = {0, 0};
    spp_fx_add(&a, p.z);
    spp_fx_add(&b, p.w);
    sx = spp_fx_units(a);
    sy = spp_fx_units(b);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sx += __shfl_down_sync(0xffffffffu, sx, o);
    sy += __shfl_down_sync(0xffffffffu, sy, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&out[0], (unsigned long long)sx);
    atomicAdd(&out[1], (unsigned long long)sy);
  }
}

inline int blocks_for(int n) { return (n + SPP_BLOCK - 1) / SPP_BLOCK; }

}  // namespace

void launch_abp_stage(const SppConsts& k, const DevState& d, int stage, int nstages,
                      cudaGraphConditionalHandle cond, int use_cond, cudaStream_t s,
                      int64_t* launches) {
  StageBufs b;
  b.stage = stage;
  b.nstages = nstages;
  if (nstages == 1) {
    b.cur = d.pos; b.out = d.half;
  } else if (nstages == 2) {
    b.cur = stage == 0 ? d.pos : d.half;
    b.out = stage == 0 ? d.half : d.pos;
  } else {
    static const int cur_sel[4] = {0, 1, 2, 1};   /* pos, half, half2, half */
    static const int out_sel[4] = {1, 2, 1, 0};
    float4* bufs[3] = {d.pos, d.half, d.half2};
    b.cur = bufs[cur_sel[stage]];
    b.out = bufs[out_sel[stage]];
  }
  const int kind = spp_pair_kind(&k);
  const int lanes = kind == SPP_KIND_CHAIN ? 1 : k.lanes;
  int nb = (d.n * lanes + SPP_STAGE_BLOCK - 1) / SPP_STAGE_BLOCK;
  if (nb == 0) nb = 1;
  /* closed boxes (walls) exist for the ABP and continuous kinds only */
#define SPP_STAGE_CASE(L, K)                                                                   \
  if (k.force_law == L && kind == K) {                                                        \
    if (lanes == SPP_GATHER_LANES)                                                            \
      k_abp_stage<L, K, SPP_GATHER_LANES, 0><<<nb, SPP_STAGE_BLOCK, 0, s>>>(k, d, b, cond, use_cond); \
    else                                                                                      \
      k_abp_stage<L, K, 1, 0><<<nb, SPP_STAGE_BLOCK, 0, s>>>(k, d, b, cond, use_cond);             \
  } else
#define SPP_STAGE_CASE_W(L, K)                                                                 \
  if (k.force_law == L && kind == K) {                                                        \
    if (lanes == SPP_GATHER_LANES && k.closed)                                                \
      k_abp_stage<L, K, SPP_GATHER_LANES, 1><<<nb, SPP_STAGE_BLOCK, 0, s>>>(k, d, b, cond, use_cond); \
    else if (lanes == SPP_GATHER_LANES)                                                       \
      k_abp_stage<L, K, SPP_GATHER_LANES, 0><<<nb, SPP_STAGE_BLOCK, 0, s>>>(k, d, b, cond, use_cond); \
    else if (k.closed)                                                                        \
      k_abp_stage<L, K, 1, 1><<<nb, SPP_STAGE_BLOCK, 0, s>>>(k, d, b, cond, use_cond);             \
    else                                                                                      \
      k_abp_stage<L, K, 1, 0><<<nb, SPP_STAGE_BLOCK, 0, s>>>(k, d, b, cond, use_cond);             \
  } else
  SPP_STAGE_CASE_W(SPP_FORCE_HARMONIC, SPP_KIND_ABP)
  SPP_STAGE_CASE_W(SPP_FORCE_R12_TRUNC, SPP_KIND_ABP)
  SPP_STAGE_CASE_W(SPP_FORCE_NONE, SPP_KIND_ABP)
  SPP_STAGE_CASE_W(SPP_FORCE_NONE, SPP_KIND_CONT)
  SPP_STAGE_CASE_W(SPP_FORCE_NONE, SPP_KIND_CONT_ALPHA)
  SPP_STAGE_CASE(SPP_FORCE_R12_TRUNC, SPP_KIND_BEADS)
  SPP_STAGE_CASE(SPP_FORCE_HARMONIC, SPP_KIND_BEADS)
  SPP_STAGE_CASE(SPP_FORCE_NONE, SPP_KIND_BEADS)
  SPP_STAGE_CASE(SPP_FORCE_R12_TRUNC, SPP_KIND_CHAIN)
  SPP_STAGE_CASE(SPP_FORCE_NONE, SPP_KIND_CHAIN)
  {}
#undef SPP_STAGE_CASE
#undef SPP_STAGE_CASE_W
  if (launches) *launches += 1;
  if (nstages == 1) {
    k_commit<<<blocks_for(d.n), SPP_BLOCK, 0, s>>>(d);
    if (launches) *launches += 1;
  }
}

/* Once per process, before any launch (graph capture included): the
 * shared-memory carveout of the stage kernel of the headline model when it
 * stages list rows in shared memory (SPP_STAGE_CARVEOUT, percent of the
 * maximum), so that a full SM of blocks fits. */
void prepare_abp_stage() {
#if SPP_STAGE_BULK_ROWS > 0 && defined(SPP_STAGE_CARVEOUT)
  static std::once_flag once;
  std::call_once(once, [] {
    cudaFuncSetAttribute(k_abp_stage<SPP_FORCE_HARMONIC, SPP_KIND_ABP, 1, 0>,
                         cudaFuncAttributePreferredSharedMemoryCarveout, SPP_STAGE_CARVEOUT);
    cudaGetLastError();
  });
#endif
}

void launch_vicsek_step(const SppConsts& k, const DevState& d, cudaStream_t s, int64_t* launches) {
  int nb = blocks_for(d.n);
  if (nb == 0) nb = 1;
  k_vicsek_step<<<nb, SPP_BLOCK, 0, s>>>(k, d);
  if (launches) *launches += 1;
}

size_t vicsek_small_smem(const SppConsts& k, const DevState& d) {
  const size_t n = (size_t)d.n, C = (size_t)d.D * d.D;
  return n * sizeof(float4) + (k.model == SPP_MODEL_VICSEK_REF_ANGLE ? n * sizeof(float) : 0) +
         2 * C * sizeof(int) + n * sizeof(int);
}

bool vicsek_small_fits(const SppConsts& k, const DevState& d) {
  return d.n <= SPP_SMALL_MAX_N && (int64_t)d.D * d.D < 65536 &&
         vicsek_small_smem(k, d) <= SPP_SMALL_MAX_SMEM;
}

/* Once per process: the dynamic shared-memory limit of k_vicsek_small set
 * to its maximum (every launch needs at most that, so systems of any size
 * and host threads share the setting), and the largest cluster (16, 8, 4, 2
 * or 1 CTAs) that fits on the device at that shared memory.  0 on failure. */
static int small_cluster_size() {
  static std::once_flag once;
  static int best = 0;
  std::call_once(once, [] {
    if (cudaFuncSetAttribute(k_vicsek_small, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             SPP_SMALL_MAX_SMEM) != cudaSuccess ||
        cudaFuncSetAttribute(k_vicsek_small, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
            cudaSuccess) {
      cudaGetLastError();
      return;
    }
    for (int cs = SPP_SMALL_CLUSTER_MAX; cs >= 1 && !best; cs >>= 1) {
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = cs;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.gridDim = dim3(cs);
      cfg.blockDim = dim3(SPP_SMALL_THREADS);
      cfg.dynamicSmemBytes = SPP_SMALL_MAX_SMEM;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      int nclusters = 0;
      if (cudaOccupancyMaxActiveClusters(&nclusters, k_vicsek_small, &cfg) == cudaSuccess && nclusters > 0)
        best = cs;
      else
        cudaGetLastError();
    }
  });
  return best;
}

int launch_vicsek_small(const SppConsts& k, const DevState& d, int nsteps, cudaStream_t s, int64_t* launches) {
  const int cs = small_cluster_size();
  if (cs < 1) return -1;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(cs);
  cfg.blockDim = dim3(SPP_SMALL_THREADS);
  cfg.dynamicSmemBytes = vicsek_small_smem(k, d);
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelEx(&cfg, k_vicsek_small, k, d, nsteps) != cudaSuccess) return -1;
  if (launches) *launches += 1;
  return 0;
}

void launch_polarization(const DevState& d, cudaStream_t s) {
  if (d.n == 0) return;
  k_polarization<<<blocks_for(d.n), SPP_BLOCK, 0, s>>>(d, reinterpret_cast<unsigned long long*>(d.red));
}

void launch_polarization_into(const DevState& d, unsigned long long* sums, cudaStream_t s) {
  if (d.n == 0) return;
  k_polarization<<<blocks_for(d.n), SPP_BLOCK, 0, s>>>(d, sums);
}
