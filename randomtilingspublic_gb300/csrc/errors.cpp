// Status strings, the per-thread error message, defaults and diagnostics of the C ABI.
#include <cstring>
#include <string>

#include "domino_rules.h"
#include "rt_internal.h"

namespace rt {
namespace {
thread_local std::string g_last_error;
}
void set_error(const std::string& msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }
}  // namespace rt

extern "C" {

RT_API void rt_walk_opts_default(rt_walk_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof *o);
  o->rng_mode = RT_RNG_TINYMT;
  o->rule = RT_DOMINO_PLAIN;
  o->weight_a = 0.7;  // dominokerneltwoperiodic.cl:3-4
  o->weight_b = 1.0;
}

RT_API const char* rt_status_string(rt_status s) {
  switch (s) {
    case RT_OK: return "ok";
    case RT_ERR_INVALID_ARGUMENT: return "invalid argument";
    case RT_ERR_CUDA: return "CUDA error";
    case RT_ERR_NOT_TILEABLE: return "domain is not tileable";
    case RT_ERR_TIMEOUT: return "timed out";
    case RT_ERR_OUT_OF_MEMORY: return "out of memory";
    case RT_ERR_NOT_COALESCED: return "chains did not coalesce";
    case RT_ERR_BUFFER_TOO_SMALL: return "output buffer too small";
    case RT_ERR_BUSY: return "busy: no free slot or over the memory budget";
  }
  return "unknown status";
}

RT_API const char* rt_last_error(void) { return rt::g_last_error.c_str(); }

RT_API const char* rt_version(void) { return "rt_tilings 0.1 (sm_103a)"; }

RT_API rt_status rt_domino_rule_table(int32_t rule, int32_t rng_mode, double a, double b, uint32_t* out16) {
  rt::clear_error();
  if (!out16) return rt::fail(RT_ERR_INVALID_ARGUMENT, "rule_table: out is NULL");
  rt::DmRule r;
  const char* err = nullptr;
  if (!rt::dm_rule_build(rule, rng_mode, a, b, &r, &err)) return rt::fail(RT_ERR_INVALID_ARGUMENT, err);
  for (int c = 0; c < 4; ++c) {
    out16[4 * c + 0] = r.lo_up[c];
    out16[4 * c + 1] = r.w_up[c];
    out16[4 * c + 2] = r.lo_dn[c];
    out16[4 * c + 3] = r.w_dn[c];
  }
  return RT_OK;
}

}  // extern "C"
