// rt_tilings.hpp - C++ drop-in for the reference's domino tiler class.
//
// Same class name, method names, argument meaning and data types as
// src/Domino/DominoTiler.h:46-131 of the reference (domain / tiling / heightfunc are
// std::vector<int>, src/common/common.h:50-52), implemented on the C ABI of
// librt_tilings.so (rt_tilings.h).  Differences a caller sees:
//   * the flip rule and the two-periodic weights, compile-time choices in the reference
//     (which kernel file is built, #define a / b), are constructor arguments;
//   * LoadTinyMT takes the TinyMTDC parameter file the reference's OpenCL path reads; when
//     it is not called, every generator uses the TinyMT32 jump parameters;
//   * failures throw rt::Error instead of printing and calling exit().
// Header-only; link with -lrt_tilings.
#ifndef RT_TILINGS_HPP_
#define RT_TILINGS_HPP_

#include <cmath>
#include <cstdint>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "rt_tilings.h"

namespace rt {

typedef std::vector<int> domain;
typedef std::vector<int> heightfunc;
typedef std::vector<int> tiling;

struct Error : std::runtime_error {
  rt_status status;
  Error(rt_status s, const std::string& what) : std::runtime_error(what), status(s) {}
};

inline void check(rt_status s) {
  if (s != RT_OK) throw Error(s, std::string(rt_status_string(s)) + ": " + rt_last_error());
}

inline int side_of(const std::vector<int>& v) {
  int n = (int)std::lround(std::sqrt((double)v.size()));
  if ((size_t)n * n != v.size()) throw Error(RT_ERR_INVALID_ARGUMENT, "array is not square");
  return n;
}

class DominoTiler {
 public:
  // rule: RT_DOMINO_PLAIN (dominokernel), RT_DOMINO_CFTP, RT_DOMINO_TWOPERIODIC,
  // RT_DOMINO_CFTP_TWOPERIODIC; rng_mode: RT_RNG_TINYMT or RT_RNG_FAST.
  explicit DominoTiler(int rule = RT_DOMINO_PLAIN, int rng_mode = RT_RNG_TINYMT, double a = 0.7, double b = 1.0) {
    rt_walk_opts_default(&opts_);
    opts_.rule = rule;
    opts_.rng_mode = rng_mode;
    opts_.weight_a = a;
    opts_.weight_b = b;
  }

  // DominoTiler::LoadTinyMT(params, size) (DominoTiler.cpp:235-237): `size` parameter sets
  // from a TinyMTDC file (lines not starting with '#'; mat1, mat2, tmat after the 3rd, 4th
  // and 5th comma, in hex).
  void LoadTinyMT(const std::string& path, int size) {
    std::ifstream in(path);
    if (!in) throw Error(RT_ERR_INVALID_ARGUMENT, "cannot open " + path);
    params_.clear();
    std::string line;
    while ((int)params_.size() < 3 * size && std::getline(in, line)) {
      if (line.empty() || line[0] == '#') continue;
      size_t p = 0;
      for (int c = 0; c < 3; ++c) p = line.find(',', p) + 1;
      for (int f = 0; f < 3; ++f) {
        params_.push_back((uint32_t)std::stoul(line.substr(p), nullptr, 16));
        p = line.find(',', p) + 1;
      }
    }
    if ((int)params_.size() < 3 * size) throw Error(RT_ERR_INVALID_ARGUMENT, path + ": too few parameter sets");
    opts_.tinymt_params = params_.data();
    opts_.tinymt_params_count = size;
  }

  // Present for source compatibility with the reference's CUDA build; the MTGP32
  // generators it loads are not used by this library (see rt_tilings.h, RNG modes).
  void LoadMTGP() {}

  void Walk(tiling& t, long steps, long seed) {
    check(rt_domino_walk(t.data(), side_of(t), steps, seed, &opts_));
  }

  void Walk(tiling& t, std::vector<long> steps, std::vector<long> seeds) {
    if (steps.size() != seeds.size()) throw Error(RT_ERR_INVALID_ARGUMENT, "steps and seeds differ in length");
    std::vector<int64_t> st(steps.begin(), steps.end()), sd(seeds.begin(), seeds.end());
    check(rt_domino_walk_epochs(t.data(), side_of(t), st.data(), sd.data(), (int32_t)st.size(), &opts_));
  }

  // Coupling from the past with the reference example's driver (AztecDiamondCftpEx.cpp).
  tiling CFTP(const tiling& tmax, const tiling& tmin, long driver_seed, long first_steps = 128, int schedule = 0,
              int max_attempts = 30, rt_cftp_stats* stats = nullptr) {
    tiling out(tmax.size());
    check(rt_domino_cftp(tmax.data(), tmin.data(), side_of(tmax), driver_seed, first_steps, schedule, max_attempts,
                         &opts_, out.data(), stats));
    return out;
  }

  static domain Rectangle(int M, int N) {
    int dim = std::max(M, N) + 5;
    domain d((size_t)dim * dim);
    int32_t side = 0;
    check(rt_domino_rectangle(M, N, d.data(), (int64_t)d.size(), &side));
    d.resize((size_t)side * side);
    return d;
  }

  static domain AztecRectangle(int N, const std::vector<int>& remove) {
    int dim = 2 * N - (int)remove.size() + 5;
    domain d((size_t)dim * dim);
    int32_t side = 0;
    check(rt_domino_aztec_rectangle(N, remove.data(), (int32_t)remove.size(), d.data(), (int64_t)d.size(), &side));
    d.resize((size_t)side * side);
    return d;
  }

  static domain AztecDiamond(int N) { return AztecRectangle(N, std::vector<int>()); }

  static tiling MaxTiling(const domain& d) {
    int m = side_of(d);
    tiling t((size_t)(m + 1) * (m + 1));
    check(rt_domino_max_tiling(d.data(), m, t.data()));
    return t;
  }

  static tiling MinTiling(const domain& d) {
    int m = side_of(d);
    tiling t((size_t)(m + 1) * (m + 1));
    check(rt_domino_min_tiling(d.data(), m, t.data()));
    return t;
  }

  static std::vector<int> DomainToVertices(const domain& d) {
    int m = side_of(d);
    std::vector<int> v((size_t)(m + 1) * (m + 1));
    check(rt_domino_domain_to_vertices(d.data(), m, v.data()));
    return v;
  }

  static domain TilingToDomain(const tiling& t) {
    int n = side_of(t);
    domain d((size_t)(n - 1) * (n - 1));
    check(rt_domino_tiling_to_domain(t.data(), n, d.data()));
    return d;
  }

  static tiling HeightfuncToTiling(const heightfunc& hf, const domain& d) {
    int n = side_of(hf);
    tiling t((size_t)n * n);
    check(rt_domino_heightfunc_to_tiling(hf.data(), d.data(), n, t.data()));
    return t;
  }

  static heightfunc TilingToHeightfunc(const tiling& t, const domain& d) {
    int n = side_of(t);
    heightfunc h((size_t)n * n);
    check(rt_domino_tiling_to_heightfunc(t.data(), d.data(), n, h.data()));
    return h;
  }

  rt_walk_opts& options() { return opts_; }

 private:
  rt_walk_opts opts_;
  std::vector<uint32_t> params_;
};

}  // namespace rt

#endif  // RT_TILINGS_HPP_
