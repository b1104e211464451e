// Launch-shape table written by the autotuner (randomtilingspublic_gb300/autotune.py) and
// read by the samplers: per model, tiling-side range, swept chains and random mode, the
// resident engine, bands (CTAs) and threads per band that measured fastest on this GPU.
//
// Text format, one entry per line ('#' starts a comment):
//   <model> <n_lo> <n_hi> <chains> <rng> <engine> <bands> <threads> [<us per half-sweep>]
// model: domino; rng: tinymt | fast; engine: 1 per-half-sweep kernels, 2 the run kernel,
// 3 k_persist, 4 the bit-plane kernel; bands, threads: 0 for the engine's default.
#include <cstdlib>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "rt_internal.h"

namespace rt {
namespace {

struct TuneEntry {
  int model, n_lo, n_hi, chains, rng, engine, bands, threads;
};

std::mutex g_tune_mu;
std::vector<TuneEntry> g_tune;
bool g_tune_env_read = false;

rt_status parse_table(const std::string& path, std::vector<TuneEntry>* out) {
  std::ifstream in(path);
  if (!in) return fail(RT_ERR_INVALID_ARGUMENT, "tune table: cannot open " + path);
  std::string line;
  int lineno = 0;
  while (std::getline(in, line)) {
    ++lineno;
    const size_t hash = line.find('#');
    if (hash != std::string::npos) line.resize(hash);
    std::istringstream ss(line);
    std::string model, rng;
    TuneEntry e{};
    if (!(ss >> model)) continue;  // blank or comment
    const std::string where = "tune table " + path + ":" + std::to_string(lineno) + ": ";
    if (!(ss >> e.n_lo >> e.n_hi >> e.chains >> rng >> e.engine >> e.bands >> e.threads))
      return fail(RT_ERR_INVALID_ARGUMENT, where + "expected 8 fields");
    if (model != "domino") return fail(RT_ERR_INVALID_ARGUMENT, where + "unknown model " + model);
    e.model = RT_MODEL_DOMINO;
    if (rng == "tinymt") e.rng = RT_RNG_TINYMT;
    else if (rng == "fast") e.rng = RT_RNG_FAST;
    else return fail(RT_ERR_INVALID_ARGUMENT, where + "rng tinymt or fast");
    if (e.n_lo > e.n_hi || e.chains < 1 || e.engine < 1 || e.engine > 4 || e.bands < 0 || e.threads < 0 ||
        e.threads > 1024 || e.threads % 32)
      return fail(RT_ERR_INVALID_ARGUMENT, where + "field out of range");
    out->push_back(e);
  }
  return RT_OK;
}

}  // namespace

bool tune_lookup(int model, int n_side, int chains, int rng, int* engine, int* bands, int* threads) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  if (!g_tune_env_read) {
    g_tune_env_read = true;
    if (const char* p = std::getenv("RT_TUNE_FILE")) {
      std::vector<TuneEntry> t;
      if (parse_table(p, &t) == RT_OK) g_tune = std::move(t);
      clear_error();
    }
  }
  for (const TuneEntry& e : g_tune)
    if (e.model == model && e.rng == rng && e.chains == chains && n_side >= e.n_lo && n_side <= e.n_hi) {
      *engine = e.engine;
      *bands = e.bands;
      *threads = e.threads;
      return true;
    }
  return false;
}

}  // namespace rt

using namespace rt;

extern "C" {

RT_API rt_status rt_tune_load(const char* path) {
  clear_error();
  if (!path) return fail(RT_ERR_INVALID_ARGUMENT, "tune table: NULL path");
  std::vector<TuneEntry> t;
  if (rt_status st = parse_table(path, &t)) return st;
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune = std::move(t);
  g_tune_env_read = true;
  return RT_OK;
}

RT_API rt_status rt_tune_clear(void) {
  clear_error();
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tune.clear();
  g_tune_env_read = true;
  return RT_OK;
}

RT_API rt_status rt_tune_lookup(int32_t model, int32_t n_side, int32_t chains, int32_t rng_mode, int32_t* out3) {
  clear_error();
  if (!out3) return fail(RT_ERR_INVALID_ARGUMENT, "tune lookup: NULL out");
  int e = 0, b = 0, t = 0;
  if (!tune_lookup(model, n_side, chains, rng_mode, &e, &b, &t))
    return fail(RT_ERR_INVALID_ARGUMENT, "tune lookup: no entry");
  out3[0] = e;
  out3[1] = b;
  out3[2] = t;
  return RT_OK;
}

}  // extern "C"
