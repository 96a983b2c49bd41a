/*
 * kernels_step.cu -- force sums fused with the integrator stage, on sm_103a.
 *
 * k_abp_stage replaces one Runge-Kutta stage of the reference's step, i.e.
 * Box::Interact (serial/box.h:322-371) followed by Box::Move_Runge_Kutta*_k
 * (serial/box.h:380-424 -> RepulsiveParticle::Move_Runge_Kutta{2,4}_k,
 * shared/particle.h:589-726), in one pass: one thread per particle (cell
 * order) gathers its Verlet neighbours' float4 (x, y, cos, sin) state,
 * accumulates force, torque and neighbour count in int64 fixed point, and
 * writes its stage state.  The last stage also
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
  __shared__ float warp_disp[SPP_BLOCK / 32];
  __shared__ float warp_step[SPP_BLOCK / 32];
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

#ifndef SPP_STAGE_GROUP
#define SPP_STAGE_GROUP 3        /* neighbours whose loads are issued together (1: one-ahead prefetch) */
#endif

/* One neighbour's contribution; the chain kind also needs the neighbour's
 * bead count (1 for membrane beads). */
template <int LAW, int KIND>
__device__ __forceinline__ void stage_pair(const SppConsts& k, const DevState& d, int wrap, SppAccF* a,
                                           int nbi, int j, float4 pi, float4 pj) {
  if (KIND == SPP_KIND_CHAIN) {
    const int nbj = __ldg(d.id + j) < (uint32_t)k.n_beads ? 1 : k.chain_nb;
    spp_pair_chain(&k, LAW, wrap, a, nbi, nbj, pi.x, pi.y, pi.z, pi.w, pj.x, pj.y, pj.z, pj.w);
  } else {
    spp_pair_abp_lkw(&k, LAW, KIND, wrap, a, pi.x, pi.y, pi.z, pi.w, pj.x, pj.y, pj.z, pj.w);
  }
}

#ifndef SPP_STAGE_MIN_BLOCKS
#define SPP_STAGE_MIN_BLOCKS 8   /* 8 x 256 threads per SM: 32 registers */
#endif
/* the chain pair loop (bead offsets, lever-arm torques) needs more than
 * 32 registers: 4 x 256 threads per SM there */
template <int LAW, int KIND>
__global__ void __launch_bounds__(SPP_BLOCK, KIND == SPP_KIND_CHAIN ? 4 : SPP_STAGE_MIN_BLOCKS) k_abp_stage(SppConsts k, DevState d, StageBufs b,
                                                         cudaGraphConditionalHandle cond,
                                                         int use_cond) {
  constexpr bool BEADLIKE = (KIND == SPP_KIND_BEADS || KIND == SPP_KIND_CHAIN);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int last = (b.stage == b.nstages - 1);
  const int frozen = d.ctl->frozen;
  float disp2 = 0.0f, step2 = 0.0f;
  if (i < d.n && !frozen) {
    const float4 pi = b.cur[i];
    SppAccF a;
    spp_accf_zero(&a);
    const uint32_t pid = BEADLIKE ? d.id[i] : 0u;
    const int nbi = (KIND == SPP_KIND_CHAIN && pid >= (uint32_t)k.n_beads) ? k.chain_nb : 1;
    const int cnt = d.nn[i];
    const int32_t* __restrict__ nb = d.nbr + i;
    const size_t stride = (size_t)d.n;
    /* Warps whose particles are all far from the box edges skip the
     * minimum-image corrections (they would not change any separation). */
    const int inner = fabsf(pi.x) < k.interior && fabsf(pi.y) < k.interior;
    const int all_inner = __all_sync(__activemask(), inner);
#if SPP_STAGE_GROUP > 1
    /* list entries and neighbour states are loaded SPP_STAGE_GROUP at a time
     * (independent loads in flight), the pairs evaluated in list order */
    for (int q0 = 0; q0 < cnt; q0 += SPP_STAGE_GROUP) {
      int jg[SPP_STAGE_GROUP];
      float4 pg[SPP_STAGE_GROUP];
#pragma unroll
      for (int u = 0; u < SPP_STAGE_GROUP; ++u) jg[u] = q0 + u < cnt ? __ldg(nb + (size_t)(q0 + u) * stride) : i;
#pragma unroll
      for (int u = 0; u < SPP_STAGE_GROUP; ++u) pg[u] = __ldg(b.cur + jg[u]);
#pragma unroll
      for (int u = 0; u < SPP_STAGE_GROUP; ++u) {
        if (q0 + u < cnt) {
          if (all_inner)
            stage_pair<LAW, KIND>(k, d, 0, &a, nbi, jg[u], pi, pg[u]);
          else
            stage_pair<LAW, KIND>(k, d, 1, &a, nbi, jg[u], pi, pg[u]);
        }
      }
    }
#else
    /* the next neighbour's index and state are loaded before the current
     * pair is evaluated, so the dependent loads overlap the arithmetic */
    int jn = cnt > 0 ? __ldg(nb) : i;
    float4 pn = __ldg(b.cur + jn);
    if (all_inner) {
      for (int q = 0; q < cnt; ++q) {
        const float4 pj = pn;
        const int j = jn;
        if (q + 1 < cnt) {
          jn = __ldg(nb + (size_t)(q + 1) * stride);
          pn = __ldg(b.cur + jn);
        }
        stage_pair<LAW, KIND>(k, d, 0, &a, nbi, j, pi, pj);
      }
    } else {
      for (int q = 0; q < cnt; ++q) {
        const float4 pj = pn;
        const int j = jn;
        if (q + 1 < cnt) {
          jn = __ldg(nb + (size_t)(q + 1) * stride);
          pn = __ldg(b.cur + jn);
        }
        stage_pair<LAW, KIND>(k, d, 1, &a, nbi, j, pi, pj);
      }
    }
#endif
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
          const uint32_t slot = o == 0 ? (uint32_t)i : d.inv[spp_ring_neighbor(&k, pid, o)];
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
      spp_abp_forces(&k, &a, pi.z, pi.w, &fx, &fy, &tau);
    }
    float dth;
    if (b.stage == 0) {
      if (!turns) {
        dth = 0.0f;
      } else if (BEADLIKE && k.tumble) {
        dth = spp_tumble_noise(&k, pid, d.ctl->step, d.tumble + pid);
      } else {
        dth = spp_rot_noise(&k, BEADLIKE ? pid : d.id[i], d.ctl->step);
      }
      if (b.nstages > 1) d.dth[i] = dth;
    } else {
      dth = d.dth[i];
    }
    const float4 p0 = (b.stage == 0) ? pi : d.pos[i];
    const float th0 = d.theta[i];
    if (KIND == SPP_KIND_CHAIN && chain_swimmer && b.nstages == 1) {
      /* Move() turns first and projects the force on the new heading */
      float wc, ws;
      spp_sincosf(spp_euler_theta(&k, th0, tau, dth), &ws, &wc);
      spp_chain_velocity(&k, &a, pi.z, pi.w, wc, ws, &fx, &fy, &tau);
    }
    float nx, ny, nt, nc, ns;
    int gx = 0, gy = 0;
    if (b.nstages == 1) {
      spp_euler_update(p0.x, p0.y, th0, fx, fy, tau, dth, &k, &nx, &ny, &nt, &nc, &ns, &gx, &gy);
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
                       &gx, &gy);
    }
    b.out[i] = make_float4(nx, ny, nc, ns);
    if (last) {
      d.theta[i] = nt;
      if (gx | gy) {
        const int2 g = d.img[i];
        d.img[i] = make_int2(g.x + gx, g.y + gy);
      }
      const float2 r = d.ref[i];
      float ddx, ddy;
      disp2 = spp_sep(&k, nx, ny, r.x, r.y, &ddx, &ddy);
      step2 = spp_sep(&k, nx, ny, p0.x, p0.y, &ddx, &ddy);
    }
  }
  if (last) finish_step(k, d, disp2, step2, cond, use_cond);
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
        const uint32_t s0 = d.cell_start[kk], c = d.cell_count[kk];
        for (uint32_t j = s0; j < s0 + c; ++j) {
          const float4 q = __ldg(d.pos_alt + j);
          const float thj = need_theta ? d.theta_alt[j] : 0.0f;
          spp_pair_vicsek(&k, &a, p.x, p.y, q.x, q.y, q.z, q.w, thj, (int)j == i);
        }
      }
    }
    if (a.ovf) atomicOr(&d.ctl->fx_overflow, 1u);
    const spp_u32x4 r = spp_draw(k.seed, k.system, id, step, SPP_RNG_VICSEK);
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
  int nb = blocks_for(d.n);
  if (nb == 0) nb = 1;
  const int kind = spp_pair_kind(&k);
#define SPP_STAGE_CASE(L, K)                                                   \
  if (k.force_law == L && kind == K) {                                        \
    k_abp_stage<L, K><<<nb, SPP_BLOCK, 0, s>>>(k, d, b, cond, use_cond);     \
  } else
  SPP_STAGE_CASE(SPP_FORCE_HARMONIC, SPP_KIND_ABP)
  SPP_STAGE_CASE(SPP_FORCE_R12_TRUNC, SPP_KIND_ABP)
  SPP_STAGE_CASE(SPP_FORCE_NONE, SPP_KIND_ABP)
  SPP_STAGE_CASE(SPP_FORCE_NONE, SPP_KIND_CONT)
  SPP_STAGE_CASE(SPP_FORCE_NONE, SPP_KIND_CONT_ALPHA)
  SPP_STAGE_CASE(SPP_FORCE_HARMONIC, SPP_KIND_CONT)
  SPP_STAGE_CASE(SPP_FORCE_HARMONIC, SPP_KIND_CONT_ALPHA)
  SPP_STAGE_CASE(SPP_FORCE_R12_TRUNC, SPP_KIND_CONT)
  SPP_STAGE_CASE(SPP_FORCE_R12_TRUNC, SPP_KIND_CONT_ALPHA)
  SPP_STAGE_CASE(SPP_FORCE_R12_TRUNC, SPP_KIND_BEADS)
  SPP_STAGE_CASE(SPP_FORCE_HARMONIC, SPP_KIND_BEADS)
  SPP_STAGE_CASE(SPP_FORCE_NONE, SPP_KIND_BEADS)
  SPP_STAGE_CASE(SPP_FORCE_R12_TRUNC, SPP_KIND_CHAIN)
  SPP_STAGE_CASE(SPP_FORCE_NONE, SPP_KIND_CHAIN)
  {}
#undef SPP_STAGE_CASE
  if (launches) *launches += 1;
  if (nstages == 1) {
    k_commit<<<nb, SPP_BLOCK, 0, s>>>(d);
    if (launches) *launches += 1;
  }
}

void launch_vicsek_step(const SppConsts& k, const DevState& d, cudaStream_t s, int64_t* launches) {
  int nb = blocks_for(d.n);
  if (nb == 0) nb = 1;
  k_vicsek_step<<<nb, SPP_BLOCK, 0, s>>>(k, d);
  if (launches) *launches += 1;
}

void launch_polarization(const DevState& d, cudaStream_t s) {
  if (d.n == 0) return;
  k_polarization<<<blocks_for(d.n), SPP_BLOCK, 0, s>>>(d, reinterpret_cast<unsigned long long*>(d.red));
}

void launch_polarization_into(const DevState& d, unsigned long long* sums, cudaStream_t s) {
  if (d.n == 0) return;
  k_polarization<<<blocks_for(d.n), SPP_BLOCK, 0, s>>>(d, sums);
}
