// Model-generic entry points (rt_walk, rt_walk_epochs, rt_cftp): one C signature for every
// model, dispatching to the per-model functions, so that a caller binding the library once
// (cgo, ctypes, JNI) reaches all of them.  No counterpart in the reference, whose models are
// separate C++ classes.
#include "rt_internal.h"

using namespace rt;

extern "C" {

RT_API rt_status rt_walk(int32_t model, int32_t* tiling, int32_t n_side, int64_t steps, int64_t seed,
                         const double* weights, const rt_walk_opts* opts) {
  switch (model) {
    case RT_MODEL_DOMINO:
      return rt_domino_walk(tiling, n_side, steps, seed, opts);
    case RT_MODEL_LOZENGE:
      return rt_lozenge_walk(tiling, n_side, steps, seed, opts);
    case RT_MODEL_RECTTRI:
      return rt_recttri_walk(tiling, n_side, steps, seed, weights, opts);
    case RT_MODEL_BIBONE:
      return rt_td_walk(tiling, n_side, steps, seed, opts, nullptr);
    case RT_MODEL_SIX_VERTEX:
      return rt_sv_walk(tiling, n_side, steps, seed, weights, opts, nullptr);
    default:
      clear_error();
      return fail(RT_ERR_INVALID_ARGUMENT, "walk: unknown model");
  }
}

RT_API rt_status rt_walk_epochs(int32_t model, int32_t* tiling, int32_t n_side, const int64_t* steps,
                                const int64_t* seeds, int32_t n_epochs, const rt_walk_opts* opts) {
  if (model == RT_MODEL_DOMINO) return rt_domino_walk_epochs(tiling, n_side, steps, seeds, n_epochs, opts);
  clear_error();
  return fail(RT_ERR_INVALID_ARGUMENT, "walk_epochs: only the domino model has the epoch overload");
}

RT_API rt_status rt_cftp(int32_t model, const int32_t* tmax, const int32_t* tmin, int32_t n_side, int64_t driver_seed,
                         int64_t first_steps, int32_t schedule, int32_t max_attempts, const double* weights,
                         const rt_walk_opts* opts, int32_t* out, rt_cftp_stats* stats) {
  switch (model) {
    case RT_MODEL_DOMINO:
      return rt_domino_cftp(tmax, tmin, n_side, driver_seed, first_steps, schedule, max_attempts, opts, out, stats);
    case RT_MODEL_LOZENGE:
      return rt_lozenge_cftp(tmax, tmin, n_side, driver_seed, first_steps, schedule, max_attempts, opts, out, stats);
    case RT_MODEL_SIX_VERTEX:
      return rt_sv_cftp(tmax, tmin, n_side, driver_seed, first_steps, max_attempts, weights, opts, out, stats);
    case RT_MODEL_RECTTRI:
    case RT_MODEL_BIBONE:
      clear_error();
      return fail(RT_ERR_INVALID_ARGUMENT, "cftp: this model's chain has no monotone coupling");
    default:
      clear_error();
      return fail(RT_ERR_INVALID_ARGUMENT, "cftp: unknown model");
  }
}

}  // extern "C"
