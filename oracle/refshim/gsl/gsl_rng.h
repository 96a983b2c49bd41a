/*
 * ORACLE shim -- test infrastructure only.
 *
 * Stand-in for GSL's generator API as the reference calls it
 * (shared/c2dvector.h:19-25, shared/state-hyper-vector.h:43-51).  GSL is not
 * installed here, and its draw order (one global stream consumed in particle
 * iteration order) cannot be shared with a GPU.  Every draw is instead taken
 * from the Philox counter stream of spp_gb300/csrc/spp_fp32.h, keyed by the
 * particle and step that the harness (oracle/ref_harness.cpp) declares
 * before it calls a reference Move*() method.  The k-th draw inside one
 * Move*() call maps to stream k of that (particle, step).
 */
#ifndef ORACLE_SHIM_GSL_RNG_H
#define ORACLE_SHIM_GSL_RNG_H
#include <stdint.h>
#include "../../spp_gb300/csrc/spp_fp32.h"

typedef struct { const char* name; } gsl_rng_type;
typedef struct { unsigned long seed; } gsl_rng;

struct ShimDrawContext {
  uint64_t seed;
  uint32_t system;
  uint32_t pid;
  uint32_t step;
  uint32_t calls;  /* draws taken since the context was set */
};
static ShimDrawContext g_shim_ctx = {0, 0, 0, 0, 0};
static inline void shim_set_context(uint64_t seed, uint32_t system, uint32_t pid, uint32_t step) {
  g_shim_ctx.seed = seed; g_shim_ctx.system = system; g_shim_ctx.pid = pid;
  g_shim_ctx.step = step; g_shim_ctx.calls = 0;
}

static const gsl_rng_type shim_philox_type = {"philox4x32-10 (shim)"};
static const gsl_rng_type* gsl_rng_default = &shim_philox_type;
static unsigned long gsl_rng_default_seed = 0;
static gsl_rng shim_rng_storage[64];
static int shim_rng_used = 0;

static inline void gsl_rng_env_setup(void) {}
static inline gsl_rng* gsl_rng_alloc(const gsl_rng_type*) {
  gsl_rng* r = &shim_rng_storage[shim_rng_used % 64];
  shim_rng_used++;
  r->seed = gsl_rng_default_seed;
  return r;
}
static inline void gsl_rng_set(gsl_rng* r, unsigned long s) { r->seed = s; }
static inline void gsl_rng_free(gsl_rng*) {}
static inline int gsl_rng_memcpy(gsl_rng* dst, const gsl_rng* src) { *dst = *src; return 0; }

/* The stream tag of the k-th call inside one Move*(): the first Gaussian or
 * uniform draw is the one the kernels take. */
static inline spp_u32x4 shim_next_bits(uint32_t first_stream) {
  uint32_t stream = g_shim_ctx.calls == 0 ? first_stream : (100u + g_shim_ctx.calls);
  g_shim_ctx.calls++;
  return spp_draw(g_shim_ctx.seed, g_shim_ctx.system, g_shim_ctx.pid, g_shim_ctx.step, stream);
}
static inline double gsl_rng_uniform(const gsl_rng*) {
  return spp_u01_d(shim_next_bits(SPP_RNG_VICSEK).v[0]);
}
static inline unsigned long gsl_rng_uniform_int(const gsl_rng* r, unsigned long n) {
  return (unsigned long)(gsl_rng_uniform(r) * (double)n);
}
#endif
