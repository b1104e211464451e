// rt_tilings.hpp - C++ drop-in for the reference's tiler classes.
//
// Same class names, method names, argument meaning and data types as the reference's
// src/Domino/DominoTiler.h:46-131, src/Lozenge/LozengeTiler.h:46-92,
// src/RectTriangle/RectTriangleTiler.h:32-86 and src/TriangleDimer/TriangleDimerTiler.h:84-216
// (domain / tiling / heightfunc are std::vector<int>, src/common/common.h:50-52), plus a
// six-vertex class of the same shape, implemented on the C ABI of librt_tilings.so
// (rt_tilings.h).  Differences a caller sees:
//   * the flip rule and the two-periodic weights, compile-time choices in the reference
//     (which kernel file is built, #define a / b), are constructor arguments;
//   * LoadTinyMT takes the TinyMTDC parameter file the reference's OpenCL path reads; when
//     it is not called, every generator uses the TinyMT32 jump parameters;
//   * failures throw rt::Error instead of printing and calling exit();
//   * the OpenCL constructors (context, queue, devices, kernel source) are replaced by
//     default construction; LoadTinyMT / LoadMTGP are accepted where the reference has them
//     (every tiler's LoadMTGP selects the cuRAND MTGP32 mode, as in the reference's CUDA
//     build).
// Header-only; link with -lrt_tilings.
#ifndef RT_TILINGS_HPP_
#define RT_TILINGS_HPP_

#include <cmath>
#include <cstdint>
#include <fstream>
#include <algorithm>
#include <utility>
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

// The options every tiler passes to the C ABI, and LoadTinyMT(params, size) of the reference's
// tilers (DominoTiler.cpp:235-237, LozengeTiler.cpp:161-164, RectTriangleTiler.cpp:22-25,
// TriangleDimerTiler.cpp:24-27): `size` parameter sets read from a TinyMTDC file as
// src/TinyMT/file_reader.cpp:22-38 reads them (lines not starting with '#'; mat1, mat2, tmat
// after the 3rd, 4th and 5th comma, in hex), set k for TinyMT generator k.
class TinyMTOpts {
 public:
  void LoadTinyMT(const std::string& path, int size) {
    std::ifstream in(path);
    if (!in) throw Error(RT_ERR_INVALID_ARGUMENT, "cannot open " + path);
    std::vector<uint32_t> p;
    std::string line;
    while ((int)p.size() < 3 * size && std::getline(in, line)) {
      if (line.empty() || line[0] == '#') continue;
      size_t at = 0;
      for (int c = 0; c < 3; ++c) at = line.find(',', at) + 1;
      for (int f = 0; f < 3; ++f) {
        p.push_back((uint32_t)std::stoul(line.substr(at), nullptr, 16));
        at = line.find(',', at) + 1;
      }
    }
    if ((int)p.size() < 3 * size) throw Error(RT_ERR_INVALID_ARGUMENT, path + ": too few parameter sets");
    params_ = std::move(p);
  }

  rt_walk_opts& options() { return opts_; }

 protected:
  // The options of a call, pointing at the loaded table (set on every call, so that a copied
  // tiler points at its own copy).
  const rt_walk_opts* wopts() {
    if (!params_.empty()) {
      opts_.tinymt_params = params_.data();
      opts_.tinymt_params_count = (int64_t)(params_.size() / 3);
    }
    return &opts_;
  }
  rt_walk_opts opts_{};
  std::vector<uint32_t> params_;
};

class DominoTiler : public TinyMTOpts {
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

  // DominoTiler::LoadMTGP (DominoTiler.cpp:239-242): as in the reference's CUDA build, the
  // walks then draw from cuRAND MTGP32 generators, one per 8 x 8 block of sites seeded
  // seed + block (RT_RNG_MTGP), so they see the reference's random stream.
  void LoadMTGP() { opts_.rng_mode = RT_RNG_MTGP; }

  void Walk(tiling& t, long steps, long seed) {
    check(rt_domino_walk(t.data(), side_of(t), steps, seed, wopts()));
  }

  void Walk(tiling& t, std::vector<long> steps, std::vector<long> seeds) {
    if (steps.size() != seeds.size()) throw Error(RT_ERR_INVALID_ARGUMENT, "steps and seeds differ in length");
    std::vector<int64_t> st(steps.begin(), steps.end()), sd(seeds.begin(), seeds.end());
    check(rt_domino_walk_epochs(t.data(), side_of(t), st.data(), sd.data(), (int32_t)st.size(), wopts()));
  }

  // Coupling from the past with the reference example's driver (AztecDiamondCftpEx.cpp).
  tiling CFTP(const tiling& tmax, const tiling& tmin, long driver_seed, long first_steps = 128, int schedule = 0,
              int max_attempts = 30, rt_cftp_stats* stats = nullptr) {
    tiling out(tmax.size());
    check(rt_domino_cftp(tmax.data(), tmin.data(), side_of(tmax), driver_seed, first_steps, schedule, max_attempts,
                         wopts(), out.data(), stats));
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

  // Not in the reference: the exact edge-placement probabilities of AztecDiamond(order) under
  // the two-periodic weights a / b (a = b: uniform), in the layout of
  // rt_domino_edge_indicators (2 N^2 values, N = 2 order + 6), computed on the device.
  static std::vector<double> AztecEdgeProbabilities(int order, double a = 1.0, double b = 1.0) {
    const size_t n = (size_t)2 * order + 6;
    std::vector<double> p(2 * n * n);
    check(rt_domino_aztec_edge_probs(order, a, b, p.data(), (int64_t)p.size(), nullptr));
    return p;
  }
};


// Shared by the three-colour models: TinyMT (the reference's OpenCL path, default
// parameters) or fast mode.
inline rt_walk_opts model_opts(int rng_mode, uint32_t fast_stream) {
  rt_walk_opts o;
  rt_walk_opts_default(&o);
  o.rng_mode = rng_mode;
  o.fast_stream = fast_stream;
  return o;
}

inline int tri_rows(const domain& d) {
  int m = (int)std::lround(std::sqrt(d.size() / 2.0));
  if ((size_t)2 * m * m != d.size()) throw Error(RT_ERR_INVALID_ARGUMENT, "expected an M x 2M triangle array");
  return m;
}

// src/Lozenge/LozengeTiler.h:46-92.
class LozengeTiler : public TinyMTOpts {
 public:
  explicit LozengeTiler(int rng_mode = RT_RNG_TINYMT, uint32_t fast_stream = 0) {
    opts_ = model_opts(rng_mode, fast_stream);
  }
  // LozengeTiler::LoadMTGP: as in the reference's CUDA build, walks then draw from cuRAND
  // MTGP32 block generators (RT_RNG_MTGP).
  void LoadMTGP() { opts_.rng_mode = RT_RNG_MTGP; }

  void Walk(tiling& t, int steps, long seed) { check(rt_lozenge_walk(t.data(), side_of(t), steps, seed, wopts())); }

  tiling CFTP(const tiling& tmax, const tiling& tmin, long driver_seed, long first_steps = 128, int schedule = 0,
              int max_attempts = 30, rt_cftp_stats* stats = nullptr) {
    tiling out(tmax.size());
    check(rt_lozenge_cftp(tmax.data(), tmin.data(), side_of(tmax), driver_seed, first_steps, schedule, max_attempts,
                          wopts(), out.data(), stats));
    return out;
  }

  static domain AlmostHexDomain(int n, int m) {
    int r = 2 * n + 9;
    domain d((size_t)2 * r * r);
    int32_t rows = 0;
    check(rt_lozenge_almost_hex_domain(n, m, d.data(), (int64_t)d.size(), &rows));
    d.resize((size_t)2 * rows * rows);
    return d;
  }
  static domain Hexagon(int n) { return AlmostHexDomain(n, 0); }

  static std::vector<int> DomainToVertices(const domain& d) {
    int m = tri_rows(d);
    std::vector<int> v((size_t)(m + 1) * (m + 1));
    check(rt_lozenge_domain_to_vertices(d.data(), m, v.data()));
    return v;
  }
  static tiling MaxTiling(const domain& d) {
    int m = tri_rows(d);
    tiling t((size_t)(m + 1) * (m + 1));
    check(rt_lozenge_max_tiling(d.data(), m, t.data()));
    return t;
  }
  static tiling MinTiling(const domain& d) {
    int m = tri_rows(d);
    tiling t((size_t)(m + 1) * (m + 1));
    check(rt_lozenge_min_tiling(d.data(), m, t.data()));
    return t;
  }
  static heightfunc TilingToHeightfunc(const tiling& t, const domain& d) {
    heightfunc h(t.size());
    check(rt_lozenge_tiling_to_heightfunc(t.data(), d.data(), side_of(t), h.data()));
    return h;
  }
  static tiling HeightfuncToTiling(const heightfunc& h, const domain& d) {
    tiling t(h.size());
    check(rt_lozenge_heightfunc_to_tiling(h.data(), d.data(), side_of(h), t.data()));
    return t;
  }
  static domain TilingToDomain(const tiling& t) {
    int n = side_of(t);
    domain d((size_t)2 * (n - 1) * (n - 1));
    check(rt_lozenge_tiling_to_domain(t.data(), n, d.data()));
    return d;
  }

};

// src/RectTriangle/RectTriangleTiler.h:32-86.  The nine weights {wt1, wt2, wt3, wm1, wm2, wm3,
// wr1, wr2, wr3} are #defines in the reference's kernel (all 1); here a constructor argument.
class RectTriangleTiler : public TinyMTOpts {
 public:
  explicit RectTriangleTiler(int rng_mode = RT_RNG_TINYMT, uint32_t fast_stream = 0,
                             std::vector<double> weights = std::vector<double>(9, 1.0))
      : w_(std::move(weights)) {
    if (w_.size() != 9) throw Error(RT_ERR_INVALID_ARGUMENT, "nine weights");
    opts_ = model_opts(rng_mode, fast_stream);
  }
  // RectTriangleTiler::LoadMTGP (RectTriangleTiler.cpp:27-30): walks then draw from cuRAND
  // MTGP32 block generators, as in the reference's CUDA build (RT_RNG_MTGP).
  void LoadMTGP() { opts_.rng_mode = RT_RNG_MTGP; }

  void Walk(tiling& t, int steps, long seed) {
    check(rt_recttri_walk(t.data(), side_of(t), steps, seed, w_.data(), wopts()));
  }

  static tiling maxHex(int n) { return hex(n, 1); }
  static tiling minHex(int n) { return hex(n, 0); }
  static tiling slopeHex(int n) { return hex(n, 2); }
  static tiling LozengeToRectTriangle(const tiling& tL, const domain& dL) {
    tiling t(tL.size());
    check(rt_recttri_from_lozenge(tL.data(), side_of(tL), dL.data(), tri_rows(dL), t.data()));
    return t;
  }

 private:
  static tiling hex(int n, int top) {
    int s = 2 * n + 9;
    tiling t((size_t)s * s);
    int32_t side = 0;
    check(rt_recttri_hex_tiling(n, top, t.data(), (int64_t)t.size(), &side));
    t.resize((size_t)side * side);
    return t;
  }
  std::vector<double> w_;
};

// src/TriangleDimer/TriangleDimerTiler.h:84-216 (bibone tilings).
class TriangleDimerTiler : public TinyMTOpts {
 public:
  explicit TriangleDimerTiler(int rng_mode = RT_RNG_TINYMT, uint32_t fast_stream = 0)
  {
    opts_ = model_opts(rng_mode, fast_stream);
  }
  // TriangleDimerTiler::LoadMTGP (TriangleDimerTiler.cpp:29-32): walks then draw from cuRAND
  // MTGP32 block generators, as in the reference's CUDA build (RT_RNG_MTGP).
  void LoadMTGP() { opts_.rng_mode = RT_RNG_MTGP; }

  void Walk(tiling& t, int steps, long seed, rt_cftp_stats* stats = nullptr) {
    check(rt_td_walk(t.data(), side_of(t), steps, seed, wopts(), stats));
  }

  static tiling IceCreamCone(int n, int m) {
    int s = 2 * (n + 4);
    tiling t((size_t)s * s);
    int32_t side = 0;
    check(rt_td_icecream_cone(n, m, t.data(), (int64_t)t.size(), &side));
    return t;
  }
  // No counterpart in the reference: the rows x cols rhombus from the brick covering.
  static tiling RhombusBrick(int rows, int cols) {
    int s = 2 * (std::max(rows, cols) + 6);
    tiling t((size_t)s * s);
    int32_t side = 0;
    check(rt_td_rhombus_brick(rows, cols, t.data(), (int64_t)t.size(), &side));
    return t;
  }
  static tiling TestButterfly(int type) {
    tiling t(16 * 16);
    int32_t side = 0;
    check(rt_td_test_butterfly(type, t.data(), (int64_t)t.size(), &side));
    return t;
  }
  static std::vector<int> TilingToTriangleFlips(const tiling& t) {
    int n = side_of(t);
    std::vector<int> v((size_t)(n / 2) * n);
    check(rt_td_triangle_flips(t.data(), n, v.data()));
    return v;
  }
  static std::vector<int> TilingToButterflyFlips(const tiling& t) {
    int n = side_of(t);
    std::vector<int> v((size_t)n * n);
    check(rt_td_butterfly_flips(t.data(), n, v.data()));
    return v;
  }
  static std::vector<int> TilingToVertices(const tiling& t) {
    int n = side_of(t);
    std::vector<int> v((size_t)(n / 2 + 1) * (n / 2 + 1));
    check(rt_td_vertices(t.data(), n, v.data()));
    return v;
  }
  static domain TilingToDomain(const tiling& t) {
    int n = side_of(t);
    domain d((size_t)(n / 2) * n);
    check(rt_td_domain(t.data(), n, d.data()));
    return d;
  }
  static std::vector<int> DimerIndicator(const tiling& t, int c) {
    int n = side_of(t);
    std::vector<int> v((size_t)(n / 2) * (n / 2));
    check(rt_td_dimer_indicator(t.data(), n, c, v.data()));
    return v;
  }

};

// Six-vertex model (no counterpart in the reference); the state is the height function.
class SixVertexTiler {
 public:
  explicit SixVertexTiler(double a = 1.0, double b = 1.0, double c = 1.0, uint32_t fast_stream = 0)
      : opts_(model_opts(RT_RNG_FAST, fast_stream)), abc_{a, b, c} {}

  void Walk(heightfunc& h, long sweeps, long seed, rt_cftp_stats* stats = nullptr) {
    check(rt_sv_walk(h.data(), side_of(h) - 1, sweeps, seed, abc_, &opts_, stats));
  }
  heightfunc CFTP(const heightfunc& hmax, const heightfunc& hmin, long seed, long first_sweeps = 16,
                  int max_attempts = 20, rt_cftp_stats* stats = nullptr) {
    heightfunc out(hmax.size());
    check(rt_sv_cftp(hmax.data(), hmin.data(), side_of(hmax) - 1, seed, first_sweeps, max_attempts, abc_, &opts_,
                     out.data(), stats));
    return out;
  }
  static heightfunc MaxHeight(int n) { return dwbc(n, 1); }
  static heightfunc MinHeight(int n) { return dwbc(n, 0); }
  static std::vector<int> HeightToASM(const heightfunc& h) {
    int n = side_of(h) - 1;
    std::vector<int> a((size_t)n * n);
    check(rt_sv_height_to_asm(h.data(), n, a.data()));
    return a;
  }
  static heightfunc ASMToHeight(const std::vector<int>& a) {
    int n = side_of(a);
    heightfunc h((size_t)(n + 1) * (n + 1));
    check(rt_sv_asm_to_height(a.data(), n, h.data()));
    return h;
  }

 private:
  static heightfunc dwbc(int n, int top) {
    heightfunc h((size_t)(n + 1) * (n + 1));
    check(rt_sv_dwbc_height(n, top, h.data()));
    return h;
  }
  rt_walk_opts opts_;
  double abc_[3];
};

}  // namespace rt

#endif  // RT_TILINGS_HPP_
