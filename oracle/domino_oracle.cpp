// TEST INFRASTRUCTURE ONLY - the oracle for the domino path.
//
// CPU restatement of the reference's domino tiler:
//   * domains            src/Domino/DominoTiler.cpp:249-324  (Rectangle, AztecDiamond, AztecRectangle)
//   * vertices           src/Domino/DominoTiler.cpp:611-631  (DomainToVertices)
//   * Thurston max/min   src/Domino/DominoTiler.cpp:345-531
//   * height functions   src/Domino/DominoTiler.cpp:534-609
//   * colour split/merge src/Domino/DominoTiler.cpp:24-33, 109-114
//   * the sweep, as the OpenCL path runs it (TinyMT32 per generator, one uniform per
//     generator per step): rotate kernels src/Domino/dominokernel.cl:4-18,
//     dominokernelCFTP.cl:10-30, dominokerneltwoperiodic.cl:7-35,
//     dominokernelCFTPtwoperiodic.cl:14-43; update kernel dominokernel.cl:22-31;
//     InitTinyMT dominokernel.cl:33-40; host loop DominoTiler.cpp:50-97 (single walk: the
//     generators are seeded with the first mt19937 draw) and :125-209 (epochs: seeded with
//     seeds[k] itself)
//   * the sweep as the CUDA path runs it, given its MTGP32 draws: rotate kernels
//     dominokernel.cu:8-24, dominokernelCFTP.cu:14-33, dominokerneltwoperiodic.cu:11-43,
//     dominokernelCFTPtwoperiodic.cu:18-47; host loop DominoTiler.cpp:51-97 (colours from
//     the first mt19937 draw) and :155-190 (epochs).  cuRAND's MTGP32 generator itself is
//     library code and is not restated here: its draws come in as data.
//   * the CFTP driver    Examples/AztecDiamondCftpEx.cpp:51-77
// plus the library's own counter-based fast mode (no reference counterpart), stated here
// as the checker of its CUDA kernels.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this.
#include <algorithm>
#include <atomic>
#include <barrier>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <queue>
#include <random>
#include <thread>
#include <utility>
#include <vector>

#include "philox_ref.h"
#include "tinymt32_ref.h"

namespace {

constexpr int kInf = INT_MAX;  // common.h:47

// ----------------------------------------------------------------------------------------
// Domains (DominoTiler.cpp:249-324)
// ----------------------------------------------------------------------------------------
std::vector<int> rectangle_domain(int rows, int cols) {
  int dim = std::max(rows, cols) + 4;
  if (dim % 2 == 0) dim++;
  std::vector<int> d((size_t)dim * dim, 0);
  for (int r = 0; r < rows; ++r)
    for (int c = 0; c < cols; ++c) d[(size_t)(r + 2) * dim + (c + 2)] = 1;
  return d;
}

std::vector<int> aztec_rectangle_domain(int n, const std::vector<int>& remove) {
  const int k = (int)remove.size();
  const int M = 2 * n - k;
  std::vector<int> d((size_t)M * M, 0);
  for (int i = 0; i < M; ++i) {
    for (int j = 0; j < M; ++j) {
      bool in;
      if (i == 0 || i == M - 1) {
        int c = (n - k) + (i == M - 1 ? k : 0);
        in = (j == c - 1 || j == c);
      } else if (i < n - k) {
        in = (j >= n - k - i - 1 && j <= n - k + i);
      } else if (i > n - 1) {
        in = (j >= i - n + k && j <= 3 * n - k - i - 1);
      } else {
        in = (j >= i - (n - k) && j <= i + (n - k));
      }
      if (in) d[(size_t)i * M + j] = 1;
    }
  }
  for (int r = 0; r < k; ++r) d[(size_t)(n - k + remove[r]) * M + remove[r]] = 0;
  const int M2 = M + 4 + (1 - M % 2);
  std::vector<int> out((size_t)M2 * M2, 0);
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < M; ++j) out[(size_t)(i + 2) * M2 + j + 2] = d[(size_t)i * M + j];
  return out;
}

// ----------------------------------------------------------------------------------------
// Vertices / height functions / Thurston (DominoTiler.cpp:345-631)
// ----------------------------------------------------------------------------------------
// neighbour order and the edge bit toward each neighbour (DominoTiler.cpp:335-337)
const int kNb[4][2] = {{1, 0}, {-1, 0}, {0, 1}, {0, -1}};
const int kNbFace[4][2][2] = {{{0, -1}, {0, 0}}, {{-1, -1}, {-1, 0}}, {{-1, 0}, {0, 0}}, {{-1, -1}, {0, -1}}};
const int kBit[4] = {2, 1, 8, 4};

std::vector<int> domain_to_vertices(const std::vector<int>& d, int M) {
  const int N = M + 1;
  std::vector<int> v((size_t)N * N, 0);
  auto D = [&](int r, int c) { return d[(size_t)r * M + c]; };
  for (int i = 0; i < N; ++i) {
    for (int j = 0; j < N; ++j) {
      if (i == 0 || j == 0 || i == M || j == M) {
        int ri = i - (i == M), rj = j - (j == M);
        int ui = i - 1 + (i == 0), uj = j - 1 + (j == 0);
        if (D(ri, rj) || D(ui, rj) || D(ri, uj) || D(ui, uj)) v[(size_t)i * N + j] = 2;
      } else {
        int a = D(i - 1, j - 1), b = D(i - 1, j), c = D(i, j - 1), e = D(i, j);
        if (a && b && c && e) v[(size_t)i * N + j] = 1;
        else if (a || b || c || e) v[(size_t)i * N + j] = 2;
      }
    }
  }
  return v;
}

inline int step_sign(int i0, int j0, int nb) {
  return (nb > 1 ? 1 : -1) * ((i0 + j0) % 2 == 0 ? 1 : -1);
}

std::vector<int> heightfunc_to_tiling(const std::vector<int>& hf, const std::vector<int>& d, int N) {
  std::vector<int> t((size_t)N * N, 0);
  const int M = N - 1;
  for (int i0 = 0; i0 < N; ++i0) {
    for (int j0 = 0; j0 < N; ++j0) {
      if (hf[(size_t)i0 * N + j0] == kInf) continue;
      for (int nb = 0; nb < 4; ++nb) {
        int i = i0 + kNb[nb][0], j = j0 + kNb[nb][1];
        int fa = (i0 - (nb == 1) - (nb > 1)) * M + j0 - (nb <= 1) - (nb == 3);
        int fb = (i0 - (nb == 1)) * M + j0 - (nb == 3);
        if (hf[(size_t)i * N + j] != kInf && (d[fa] || d[fb]))
          t[(size_t)i0 * N + j0] += kBit[nb] * std::abs((hf[(size_t)i * N + j] - hf[(size_t)i0 * N + j0]) / 2);
      }
    }
  }
  return t;
}

struct ByHeightAsc {  // common.h:94-98 (pops the lowest height first)
  bool operator()(const std::pair<std::pair<int, int>, int>& x, const std::pair<std::pair<int, int>, int>& y) const {
    return x.second > y.second;
  }
};
struct ByHeightDesc {  // common.h:88-92 (pops the highest height first)
  bool operator()(const std::pair<std::pair<int, int>, int>& x, const std::pair<std::pair<int, int>, int>& y) const {
    return x.second < y.second;
  }
};

// Returns 0 and the tiling, or -1 and the partial height function (the reference returns
// the height function in that case, DominoTiler.cpp:407-409,426-427).
template <class Cmp, bool kMax>
int thurston(const std::vector<int>& d, int M, std::vector<int>& out) {
  std::vector<int> v = domain_to_vertices(d, M);
  const int N = M + 1;
  std::vector<int> hf((size_t)N * N, kInf);
  std::queue<std::pair<int, int>> ring;
  bool found = false;
  for (int i = 0; i < N && !found; ++i)
    for (int j = 0; j < N && !found; ++j)
      if (v[(size_t)i * N + j] == 2) {
        found = true;
        ring.push({i, j});
        hf[(size_t)i * N + j] = 0;
      }
  std::priority_queue<std::pair<std::pair<int, int>, int>, std::vector<std::pair<std::pair<int, int>, int>>, Cmp> pq{Cmp()};
  while (!ring.empty()) {
    auto [i0, j0] = ring.front();
    ring.pop();
    for (int nb = 0; nb < 4; ++nb) {
      int i = i0 + kNb[nb][0], j = j0 + kNb[nb][1];
      if (v[(size_t)i * N + j] != 2) continue;
      int fa = (i0 + kNbFace[nb][0][0]) * M + j0 + kNbFace[nb][0][1];
      int fb = (i0 + kNbFace[nb][1][0]) * M + j0 + kNbFace[nb][1][1];
      if (!(d[fa] ^ d[fb])) continue;
      int h = hf[(size_t)i0 * N + j0] + step_sign(i0, j0, nb);
      if (hf[(size_t)i * N + j] == kInf) {
        hf[(size_t)i * N + j] = h;
        ring.push({i, j});
        pq.push({{i, j}, h});
      } else if (hf[(size_t)i * N + j] != h) {
        out = hf;
        return -1;
      }
    }
  }
  while (!pq.empty()) {
    auto top = pq.top();
    pq.pop();
    int i0 = top.first.first, j0 = top.first.second;
    for (int nb = 0; nb < 4; ++nb) {
      int i = i0 + kNb[nb][0], j = j0 + kNb[nb][1];
      if (!(i >= 0 && j >= 0 && i < N && j < N && v[(size_t)i * N + j] > 0)) continue;
      int dir = ((i0 + j0) % 2 == 0 ? 1 : -1) * (nb > 1 ? 1 : -1);
      if (kMax ? dir <= 0 : dir >= 0) continue;
      int here = hf[(size_t)i0 * N + j0];
      if (kMax) {
        if (v[(size_t)i * N + j] == 2 && hf[(size_t)i * N + j] > here + 1 && v[(size_t)i0 * N + j0] != 2) {
          out = hf;
          return -1;
        }
        if (hf[(size_t)i * N + j] == kInf) {
          hf[(size_t)i * N + j] = here + 1;
          pq.push({{i, j}, here + 1});
        }
      } else {
        // DominoTiler.cpp:519 compares the height (not the vertex class) with 2; kept as is.
        if (v[(size_t)i * N + j] == 2 && hf[(size_t)i * N + j] < here - 1 && here != 2) {
          out = hf;
          return -1;
        }
        if (hf[(size_t)i * N + j] == kInf) {
          hf[(size_t)i * N + j] = here - 1;
          pq.push({{i, j}, here - 1});
        }
      }
    }
  }
  out = heightfunc_to_tiling(hf, d, N);
  return 0;
}

std::vector<int> tiling_to_heightfunc(const std::vector<int>& t, const std::vector<int>& d, int N) {
  const int M = N - 1;
  std::vector<int> v = domain_to_vertices(d, M);
  std::vector<int> hf((size_t)N * N, kInf);
  std::queue<std::pair<int, int>> q;
  bool found = false;
  for (int i = 0; i < N && !found; ++i)
    for (int j = 0; j < N && !found; ++j)
      if (v[(size_t)i * N + j] == 2) {
        found = true;
        q.push({i, j});
        hf[(size_t)i * N + j] = 0;
      }
  while (!q.empty()) {
    auto [i0, j0] = q.front();
    q.pop();
    for (int nb = 0; nb < 4; ++nb) {
      int i = i0 + kNb[nb][0], j = j0 + kNb[nb][1];
      if ((t[(size_t)i0 * N + j0] & kBit[nb]) != 0) continue;
      if (!(v[(size_t)i * N + j] > 0 && hf[(size_t)i * N + j] == kInf)) continue;
      int fa = (i0 + kNbFace[nb][0][0]) * M + j0 + kNbFace[nb][0][1];
      int fb = (i0 + kNbFace[nb][1][0]) * M + j0 + kNbFace[nb][1][1];
      if (d[fa] || d[fb]) {
        hf[(size_t)i * N + j] = hf[(size_t)i0 * N + j0] + step_sign(i0, j0, nb);
        q.push({i, j});
      }
    }
  }
  return hf;
}

// ----------------------------------------------------------------------------------------
// The sweep (OpenCL-path semantics)
// ----------------------------------------------------------------------------------------
enum Variant { kPlain = 0, kCftp = 1, kTwoPeriodic = 2, kCftpTwoPeriodic = 3 };

struct Chain {
  int N = 0, H = 0;  // H = N/2 colour-array width
  std::vector<uint8_t> B, W;
};

void split_tiling(const int* t, int N, Chain& c) {
  c.N = N;
  c.H = N / 2;
  c.B.assign((size_t)N * c.H, 0);
  c.W.assign((size_t)N * c.H, 0);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      auto& dst = ((i + j) % 2 == 0) ? c.B : c.W;
      dst[(size_t)i * c.H + j / 2] = (uint8_t)t[(size_t)i * N + j];
    }
}

void merge_tiling(const Chain& c, int* t) {
  const int N = c.N;
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      const auto& src = ((i + j) % 2 == 0) ? c.B : c.W;
      t[(size_t)i * N + j] = src[(size_t)i * c.H + j / 2];
    }
}

// Flip decision for one site given the float uniform rd in [0,1), as the .cl kernels
// evaluate it.  Returns the new state.
inline uint8_t rotate_cl(uint8_t e, float rd, int variant, int i, int t, double a, double b) {
  switch (variant) {
    case kPlain:  // dominokernel.cl:14-17
      if ((double)rd < .8) {
        if (e == 3) return 12;
        if (e == 12) return 3;
      }
      return e;
    case kCftp:  // dominokernelCFTP.cl:65-69
      if ((double)rd < 0.5) {
        if (e == 3) return 12;
      } else {
        if (e == 12) return 3;
      }
      return e;
    case kTwoPeriodic: {  // dominokerneltwoperiodic.cl:17-32
      float pp = 0.8;
      if (rd < pp) {
        float thr = rd / pp;
        if (e == 3) {
          float wI = b * b * ((i + t + 1) % 2) + a * a * ((i + t) % 2);
          float wF = a * a * (i % 2) + b * b * ((i + 1) % 2);
          if (wF / wI > thr) return 12;
        } else if (e == 12) {
          float wI = a * a * (i % 2) + b * b * ((i + 1) % 2);
          float wF = b * b * ((i + t + 1) % 2) + a * a * ((i + t) % 2);
          if (wF / wI > thr) return 3;
        }
      }
      return e;
    }
    case kCftpTwoPeriodic: {  // dominokernelCFTPtwoperiodic.cl:84-99
      if ((double)rd < 0.5) {
        float thr = (double)rd / 0.5;
        if (e == 3) {
          float wI = b * b * ((i + t + 1) % 2) + a * a * ((i + t) % 2);
          float wF = a * a * (i % 2) + b * b * ((i + 1) % 2);
          if (wF / wI > thr) return 12;
        }
      } else {
        float thr = ((double)rd - 0.5) / 0.5;
        if (e == 12) {
          float wI = a * a * (i % 2) + b * b * ((i + 1) % 2);
          float wF = b * b * ((i + t + 1) % 2) + a * a * ((i + t) % 2);
          if (wF / wI > thr) return 3;
        }
      }
      return e;
    }
  }
  return e;
}

// The same decision as the reference's CUDA kernels make it, rd the float from cuRAND's
// MTGP32 (dominokernel.cu:19-22, dominokernelCFTP.cu:26-31, dominokerneltwoperiodic.cu:23-40,
// dominokernelCFTPtwoperiodic.cu:30-46).  Three rules read as the .cl kernels do; in the
// two-periodic rule the CUDA kernel compares the draw with the double PROB_PROPOSE and
// divides in double, where the .cl kernel uses a float propose.
inline uint8_t rotate_cu(uint8_t e, float rd, int variant, int i, int t, double a, double b) {
  if (variant != kTwoPeriodic) return rotate_cl(e, rd, variant, i, t, a, b);
  if ((double)rd < 0.8) {
    float thr = (double)rd / 0.8;
    if (e == 3) {
      float wI = b * b * ((i + t + 1) % 2) + a * a * ((i + t) % 2);
      float wF = a * a * (i % 2) + b * b * ((i + 1) % 2);
      if (wF / wI > thr) return 12;
    } else if (e == 12) {
      float wI = a * a * (i % 2) + b * b * ((i + 1) % 2);
      float wF = b * b * ((i + t + 1) % 2) + a * a * ((i + t) % 2);
      if (wF / wI > thr) return 3;
    }
  }
  return e;
}

// The library's fast-mode acceptance rule (its own specification): the same move
// probabilities as the reference kernels, resolved against a 32-bit uniform u by
// u < ceil(p * 2^32) (proposal-only variants) or, for the monotone CFTP variants, by
// u < 2^31 for the up-half and u >= 2^31 for the down-half, each accepting with
// ceil(min(1, ratio) * 2^31).
inline float ratio_up(int i, int t, double a, double b) {
  float wI = b * b * ((i + t + 1) % 2) + a * a * ((i + t) % 2);
  float wF = a * a * (i % 2) + b * b * ((i + 1) % 2);
  return wF / wI;
}
inline float ratio_dn(int i, int t, double a, double b) {
  float wI = a * a * (i % 2) + b * b * ((i + 1) % 2);
  float wF = b * b * ((i + t + 1) % 2) + a * a * ((i + t) % 2);
  return wF / wI;
}
inline uint64_t ceil_scaled(double p, double scale) {
  double x = std::ceil(p * scale);
  if (x < 0) x = 0;
  return (uint64_t)x;
}

inline uint8_t rotate_fast(uint8_t e, uint32_t u, int variant, int i, int t, double a, double b) {
  const double P32 = 4294967296.0, P31 = 2147483648.0;
  switch (variant) {
    case kPlain: {
      uint64_t c = ceil_scaled(0.8, P32);
      if (u < c) {
        if (e == 3) return 12;
        if (e == 12) return 3;
      }
      return e;
    }
    case kCftp:
      if (u < 0x80000000u) {
        if (e == 3) return 12;
      } else if (e == 12) {
        return 3;
      }
      return e;
    case kTwoPeriodic: {
      if (e == 3) {
        double r = std::min(1.0, (double)ratio_up(i, t, a, b));
        if (u < ceil_scaled(0.8 * r, P32)) return 12;
      } else if (e == 12) {
        double r = std::min(1.0, (double)ratio_dn(i, t, a, b));
        if (u < ceil_scaled(0.8 * r, P32)) return 3;
      }
      return e;
    }
    case kCftpTwoPeriodic: {
      if (u < 0x80000000u) {
        if (e == 3) {
          double r = std::min(1.0, (double)ratio_up(i, t, a, b));
          if (u < ceil_scaled(r, P31)) return 12;
        }
      } else if (e == 12) {
        double r = std::min(1.0, (double)ratio_dn(i, t, a, b));
        if ((uint64_t)(u - 0x80000000u) < ceil_scaled(r, P31)) return 3;
      }
      return e;
    }
  }
  return e;
}

// dominokernel.cl:22-31: passive colour rebuilt from the active colour.
inline uint8_t update_site(const uint8_t* A, int H, int i, int j, int t) {
  return (uint8_t)(((A[(size_t)(i - 1) * H + j] & 2) / 2) + 2 * (A[(size_t)(i + 1) * H + j] & 1) +
                   ((A[(size_t)i * H + j - (i + t + 1) % 2] & 8) / 2) + 2 * (A[(size_t)i * H + j + (i + t) % 2] & 4));
}

// A team of host threads splitting the rows of each phase; used for the CPU baseline.
struct Team {
  int n;
  explicit Team(int threads) : n(threads < 1 ? 1 : threads) {}
  // Runs body(tid, r0, r1) for every phase in sequence over rows [lo, hi) with a barrier
  // between phases.  phases(tid, run) is the per-thread driver.
  void run(const std::function<void(int, std::function<void()>&)>& driver) {
    if (n == 1) {
      std::function<void()> nop = [] {};
      driver(0, nop);
      return;
    }
    std::barrier bar(n);
    std::function<void()> sync = [&bar] { bar.arrive_and_wait(); };
    std::vector<std::thread> th;
    for (int k = 1; k < n; ++k) th.emplace_back([&, k] {
      std::function<void()> s = [&bar] { bar.arrive_and_wait(); };
      driver(k, s);
    });
    driver(0, sync);
    for (auto& x : th) x.join();
  }
};

// One coupled set of chains that share the per-generator random stream.
struct SweepJob {
  int N, H, rows, cols;            // cells: rows = N-2, cols = N/2-2
  int variant;
  double a, b;
  std::vector<Chain*> chains;
};

// Runs the half-sweeps colour[0..steps) on all chains with TinyMT generators g (one per
// cell, index (i-1)*cols + (j-1)), threads splitting rows.
void run_tinymt(SweepJob& J, std::vector<oracle::TinyMT32>& g, const std::vector<uint8_t>& colour, int threads) {
  Team team(threads);
  const int nthreads = team.n;
  const int64_t steps = (int64_t)colour.size();
  team.run([&](int tid, std::function<void()>& sync) {
    const int r0 = 1 + (int)((int64_t)J.rows * tid / nthreads);
    const int r1 = 1 + (int)((int64_t)J.rows * (tid + 1) / nthreads);
    for (int64_t s = 0; s < steps; ++s) {
      const int t = colour[s];  // 1: rotate black, update white; 0: the reverse
      for (int i = r0; i < r1; ++i) {
        for (int j = 1; j <= J.cols; ++j) {
          auto& gen = g[(size_t)(i - 1) * J.cols + (j - 1)];
          float rd = oracle::tmt_u23_to_float(oracle::tmt_next_u23(gen));
          for (Chain* c : J.chains) {
            uint8_t* A = t ? c->B.data() : c->W.data();
            uint8_t& e = A[(size_t)i * J.H + j];
            e = rotate_cl(e, rd, J.variant, i, t, J.a, J.b);
          }
        }
      }
      sync();
      for (Chain* c : J.chains) {
        const uint8_t* A = t ? c->B.data() : c->W.data();
        uint8_t* P = t ? c->W.data() : c->B.data();
        for (int i = r0; i < r1; ++i)
          for (int j = 1; j <= J.cols; ++j) P[(size_t)i * J.H + j] = update_site(A, J.H, i, j, t);
      }
      sync();
    }
  });
}

// Fast mode: half-sweep h rotates black when h is even, white when h is odd.
void run_fast(SweepJob& J, uint64_t seed, uint32_t stream, int64_t h0, int64_t steps, int threads) {
  Team team(threads);
  const int nthreads = team.n;
  team.run([&](int tid, std::function<void()>& sync) {
    const int r0 = 1 + (int)((int64_t)J.rows * tid / nthreads);
    const int r1 = 1 + (int)((int64_t)J.rows * (tid + 1) / nthreads);
    for (int64_t s = 0; s < steps; ++s) {
      const int64_t h = h0 + s;
      const int t = (h & 1) ? 0 : 1;
      for (int i = r0; i < r1; ++i) {
        for (int j = 1; j <= J.cols; ++j) {
          uint32_t u = oracle::fast_draw(seed, stream, h, (uint32_t)i, (uint32_t)j);
          for (Chain* c : J.chains) {
            uint8_t* A = t ? c->B.data() : c->W.data();
            uint8_t& e = A[(size_t)i * J.H + j];
            e = rotate_fast(e, u, J.variant, i, t, J.a, J.b);
          }
        }
      }
      sync();
      for (Chain* c : J.chains) {
        const uint8_t* A = t ? c->B.data() : c->W.data();
        uint8_t* P = t ? c->W.data() : c->B.data();
        for (int i = r0; i < r1; ++i)
          for (int j = 1; j <= J.cols; ++j) P[(size_t)i * J.H + j] = update_site(A, J.H, i, j, t);
      }
      sync();
    }
  });
}

// The reference's CUDA path with its draws supplied: step s takes draws[s][i-1][j-1] for
// candidate (i, j) (the curand_uniform value of that thread, dominokernel.cu:14-15), rotates
// colour[s] as the CUDA kernels decide, then rebuilds the other colour.
void run_draws(SweepJob& J, const float* draws, const std::vector<uint8_t>& colour) {
  const size_t per = (size_t)J.rows * J.cols;
  for (size_t s = 0; s < colour.size(); ++s) {
    const int t = colour[s];
    const float* d = draws + s * per;
    for (int i = 1; i <= J.rows; ++i)
      for (int j = 1; j <= J.cols; ++j) {
        const float rd = d[(size_t)(i - 1) * J.cols + (j - 1)];
        for (Chain* c : J.chains) {
          uint8_t* A = t ? c->B.data() : c->W.data();
          uint8_t& e = A[(size_t)i * J.H + j];
          e = rotate_cu(e, rd, J.variant, i, t, J.a, J.b);
        }
      }
    for (Chain* c : J.chains) {
      const uint8_t* A = t ? c->B.data() : c->W.data();
      uint8_t* P = t ? c->W.data() : c->B.data();
      for (int i = 1; i <= J.rows; ++i)
        for (int j = 1; j <= J.cols; ++j) P[(size_t)i * J.H + j] = update_site(A, J.H, i, j, t);
    }
  }
}

void init_generators(std::vector<oracle::TinyMT32>& g, size_t count, uint32_t seed, const uint32_t* params,
                     int64_t nparams) {
  g.resize(count);
  for (size_t id = 0; id < count; ++id) {
    oracle::TinyMT32& x = g[id];
    if (params && (int64_t)id < nparams) {
      x.mat1 = params[3 * id + 0];
      x.mat2 = params[3 * id + 1];
      x.tmat = params[3 * id + 2];
    } else {
      x.mat1 = oracle::kTmtMat1;
      x.mat2 = oracle::kTmtMat2;
      x.tmat = oracle::kTmtTmat;
    }
    oracle::tmt_init(x, seed + (uint32_t)id);
  }
}

std::vector<uint8_t> colour_stream(std::mt19937& mt, int64_t steps) {
  std::vector<uint8_t> c((size_t)steps);
  for (int64_t s = 0; s < steps; ++s) c[(size_t)s] = (uint8_t)(mt() % 2);
  return c;
}

SweepJob make_job(int N, int variant, double a, double b) {
  SweepJob J;
  J.N = N;
  J.H = N / 2;
  J.rows = N - 2;
  J.cols = N / 2 - 2;
  J.variant = variant;
  J.a = a;
  J.b = b;
  return J;
}

}  // namespace

extern "C" {

// --- domains / vertices / height functions ------------------------------------------------
int orc_dm_aztec_rectangle(int n, const int* remove, int k, int* out, long cap) {
  std::vector<int> rm(remove, remove + k);
  std::vector<int> d = aztec_rectangle_domain(n, rm);
  int side = (int)std::lround(std::sqrt((double)d.size()));
  if ((long)d.size() > cap) return -side;
  std::memcpy(out, d.data(), d.size() * sizeof(int));
  return side;
}

int orc_dm_rectangle(int rows, int cols, int* out, long cap) {
  std::vector<int> d = rectangle_domain(rows, cols);
  int side = (int)std::lround(std::sqrt((double)d.size()));
  if ((long)d.size() > cap) return -side;
  std::memcpy(out, d.data(), d.size() * sizeof(int));
  return side;
}

void orc_dm_domain_to_vertices(const int* d, int M, int* out) {
  std::vector<int> dv(d, d + (size_t)M * M);
  std::vector<int> v = domain_to_vertices(dv, M);
  std::memcpy(out, v.data(), v.size() * sizeof(int));
}

int orc_dm_max_tiling(const int* d, int M, int* out) {
  std::vector<int> dv(d, d + (size_t)M * M), o;
  int rc = thurston<ByHeightAsc, true>(dv, M, o);
  std::memcpy(out, o.data(), o.size() * sizeof(int));
  return rc;
}

int orc_dm_min_tiling(const int* d, int M, int* out) {
  std::vector<int> dv(d, d + (size_t)M * M), o;
  int rc = thurston<ByHeightDesc, false>(dv, M, o);
  std::memcpy(out, o.data(), o.size() * sizeof(int));
  return rc;
}

void orc_dm_heightfunc_to_tiling(const int* hf, const int* d, int N, int* out) {
  std::vector<int> h(hf, hf + (size_t)N * N), dv(d, d + (size_t)(N - 1) * (N - 1));
  std::vector<int> t = heightfunc_to_tiling(h, dv, N);
  std::memcpy(out, t.data(), t.size() * sizeof(int));
}

void orc_dm_tiling_to_heightfunc(const int* t, const int* d, int N, int* out) {
  std::vector<int> tv(t, t + (size_t)N * N), dv(d, d + (size_t)(N - 1) * (N - 1));
  std::vector<int> h = tiling_to_heightfunc(tv, dv, N);
  std::memcpy(out, h.data(), h.size() * sizeof(int));
}

void orc_dm_tiling_to_domain(const int* t, int N, int* out) {
  const int M = N - 1;
  for (int i = 0; i < M; ++i)
    for (int j = 0; j < M; ++j)
      out[(size_t)i * M + j] = ((t[(size_t)i * N + j] & (2 + 8)) != 0) || ((t[(size_t)(i + 1) * N + j + 1] & (1 + 4)) != 0);
}

// --- walks ---------------------------------------------------------------------------------
// DominoTiler::Walk(t, steps, seed), OpenCL path: generators seeded with the first draw of
// mt19937(seed), colours from the following draws.
int orc_dm_walk_tinymt(int* t, int N, long steps, long seed, int variant, double a, double b,
                       const uint32_t* params, long nparams, int threads) {
  if (N % 2 || N < 6) return -1;
  Chain c;
  split_tiling(t, N, c);
  std::mt19937 mt((uint32_t)seed);
  std::vector<oracle::TinyMT32> g;
  uint32_t s0 = (uint32_t)mt();
  SweepJob J = make_job(N, variant, a, b);
  init_generators(g, (size_t)J.rows * J.cols, s0, params, nparams);
  std::vector<uint8_t> col = colour_stream(mt, steps);
  J.chains = {&c};
  run_tinymt(J, g, col, threads);
  merge_tiling(c, t);
  return 0;
}

// DominoTiler::Walk(t, steps[], seeds[]), OpenCL path.
int orc_dm_walk_epochs_tinymt(int* t, int N, const long* steps, const long* seeds, int nepochs, int variant,
                              double a, double b, const uint32_t* params, long nparams, int threads) {
  if (N % 2 || N < 6) return -1;
  Chain c;
  split_tiling(t, N, c);
  SweepJob J = make_job(N, variant, a, b);
  J.chains = {&c};
  std::vector<oracle::TinyMT32> g;
  for (int k = 0; k < nepochs; ++k) {
    std::mt19937 mt((uint32_t)seeds[k]);
    init_generators(g, (size_t)J.rows * J.cols, (uint32_t)seeds[k], params, nparams);
    std::vector<uint8_t> col = colour_stream(mt, steps[k]);
    run_tinymt(J, g, col, threads);
  }
  merge_tiling(c, t);
  return 0;
}

// Examples/AztecDiamondCftpEx.cpp:51-77 with the coupled chains run side by side.
// schedule 0: the reference's rule (prepend 2 * steps.back()); 1: prepend 2 * steps.front().
// Returns the number of attempts, or -1 when max_attempts ran out.
int orc_dm_cftp_tinymt(const int* tmax, const int* tmin, int N, long driver_seed, long first_steps, int schedule,
                       int max_attempts, int variant, double a, double b, const uint32_t* params, long nparams,
                       int threads, int* out, long* total_steps) {
  std::mt19937 drv((uint32_t)driver_seed);
  std::vector<long> steps{first_steps}, seeds{(long)drv()};
  SweepJob J = make_job(N, variant, a, b);
  std::vector<oracle::TinyMT32> g;
  long total = 0;
  for (int attempt = 1; attempt <= max_attempts; ++attempt) {
    Chain top, bot;
    split_tiling(tmax, N, top);
    split_tiling(tmin, N, bot);
    J.chains = {&bot, &top};
    for (size_t k = 0; k < steps.size(); ++k) {
      std::mt19937 mt((uint32_t)seeds[k]);
      init_generators(g, (size_t)J.rows * J.cols, (uint32_t)seeds[k], params, nparams);
      std::vector<uint8_t> col = colour_stream(mt, steps[k]);
      run_tinymt(J, g, col, threads);
      total += steps[k];  // half-sweeps per chain
    }
    if (top.B == bot.B && top.W == bot.W) {
      merge_tiling(top, out);
      if (total_steps) *total_steps = total;
      return attempt;
    }
    long next = schedule == 0 ? steps.back() * 2 : steps.front() * 2;
    steps.insert(steps.begin(), next);
    seeds.insert(seeds.begin(), (long)drv());
  }
  if (total_steps) *total_steps = total;
  return -1;
}

// DominoTiler::Walk(t, steps, seed), CUDA path, with the MTGP32 draws supplied (steps x
// (N-2) x (N/2-2) floats): colours from mt19937(seed) starting with its first draw
// (DominoTiler.cpp:51, 69; no draw is spent on seeding, unlike the OpenCL path).
int orc_dm_walk_draws(int* t, int N, const float* draws, long steps, long seed, int variant, double a, double b) {
  if (N % 2 || N < 6) return -1;
  Chain c;
  split_tiling(t, N, c);
  SweepJob J = make_job(N, variant, a, b);
  J.chains = {&c};
  std::mt19937 mt((uint32_t)seed);
  run_draws(J, draws, colour_stream(mt, steps));
  merge_tiling(c, t);
  return 0;
}

// DominoTiler::Walk(t, steps[], seeds[]), CUDA path (DominoTiler.cpp:155-190): epoch k takes
// its colours from mt19937(seeds[k]) and its draws from the next steps[k] blocks of draws.
int orc_dm_walk_epochs_draws(int* t, int N, const float* draws, const long* steps, const long* seeds, int nepochs,
                             int variant, double a, double b) {
  if (N % 2 || N < 6) return -1;
  Chain c;
  split_tiling(t, N, c);
  SweepJob J = make_job(N, variant, a, b);
  J.chains = {&c};
  const size_t per = (size_t)J.rows * J.cols;
  size_t off = 0;
  for (int k = 0; k < nepochs; ++k) {
    std::mt19937 mt((uint32_t)seeds[k]);
    run_draws(J, draws + off * per, colour_stream(mt, steps[k]));
    off += (size_t)steps[k];
  }
  merge_tiling(c, t);
  return 0;
}

// The CUDA kernels' rotation of one colour array in the reference's layout (N rows x N/2
// bytes), draws per candidate (N-2) x (N/2-2).
void orc_dm_rotate_cuda_grid(uint8_t* colour, int N, int t, const float* draws, int variant, double a, double b) {
  const int H = N / 2, cols = H - 2;
  for (int i = 1; i <= N - 2; ++i)
    for (int j = 1; j <= cols; ++j) {
      uint8_t& e = colour[(size_t)i * H + j];
      e = rotate_cu(e, draws[(size_t)(i - 1) * cols + (j - 1)], variant, i, t, a, b);
    }
}

// The CUDA kernels' decision for n draws of one (state, variant, row, colour) case.
void orc_dm_rotate_cuda_many(const float* rd, long n, int e, int variant, int i, int t, double a, double b,
                             uint8_t* out) {
  for (long k = 0; k < n; ++k) out[k] = rotate_cu((uint8_t)e, rd[k], variant, i, t, a, b);
}

// n outputs of std::mt19937(seed) (the drivers' seed and colour streams).
void orc_mt19937(uint32_t seed, long n, uint32_t* out) {
  std::mt19937 mt(seed);
  for (long k = 0; k < n; ++k) out[k] = (uint32_t)mt();
}

// Fast mode walk over half-sweeps [h0, h0 + steps).
int orc_dm_walk_fast(int* t, int N, long h0, long steps, unsigned long seed, unsigned stream, int variant, double a,
                     double b, int threads) {
  if (N % 2 || N < 6) return -1;
  Chain c;
  split_tiling(t, N, c);
  SweepJob J = make_job(N, variant, a, b);
  J.chains = {&c};
  run_fast(J, seed, stream, h0, steps, threads);
  merge_tiling(c, t);
  return 0;
}

// Fast-mode CFTP: attempt j runs the coupled max/min chains over half-sweeps
// [-2*T_j, 0) with T_j = first_sweeps * 2^j sweeps; the first coalesced attempt wins.
int orc_dm_cftp_fast(const int* tmax, const int* tmin, int N, unsigned long seed, unsigned stream, long first_sweeps,
                     int max_attempts, int variant, double a, double b, int threads, int* out, long* sweeps_used) {
  SweepJob J = make_job(N, variant, a, b);
  long T = first_sweeps;
  for (int attempt = 1; attempt <= max_attempts; ++attempt, T *= 2) {
    Chain top, bot;
    split_tiling(tmax, N, top);
    split_tiling(tmin, N, bot);
    J.chains = {&bot, &top};
    run_fast(J, seed, stream, -2 * T, 2 * T, threads);
    if (top.B == bot.B && top.W == bot.W) {
      merge_tiling(top, out);
      if (sweeps_used) *sweeps_used = T;
      return attempt;
    }
  }
  return -1;
}

// Raw generator outputs for known-answer checks.
unsigned orc_tinymt_u32(unsigned seed, unsigned mat1, unsigned mat2, unsigned tmat, int skip) {
  oracle::TinyMT32 g{0, 0, 0, 0, mat1, mat2, tmat};
  oracle::tmt_init(g, seed);
  for (int s = 0; s < skip; ++s) oracle::tmt_next_state(g);
  oracle::tmt_next_state(g);
  return oracle::tmt_temper(g);
}

void orc_philox4x32_10(const unsigned* ctr, const unsigned* key, unsigned* out) {
  oracle::U32x4 c{{ctr[0], ctr[1], ctr[2], ctr[3]}};
  oracle::U32x4 o = oracle::philox4x32_10(c, key[0], key[1]);
  for (int k = 0; k < 4; ++k) out[k] = o.v[k];
}

}  // extern "C"

extern "C" {

// Exhaustive scan of the reference decision over all 2^23 TinyMT draws for one (rule, row
// parity, colour): writes {lo_up, width_up, lo_dn, width_dn} and returns 0 when each accept
// set is a single interval, -1 otherwise.
int orc_dm_scan_intervals(int rule, int ip, int t, double a, double b, uint32_t* out) {
  const int i = 2 + ip;
  for (int move = 0; move < 2; ++move) {
    const uint8_t from = move == 0 ? 3 : 12, to = move == 0 ? 12 : 3;
    long lo = -1, hi = -1;
    bool gap = false;
    for (uint32_t u = 0; u < (1u << 23); ++u) {
      bool acc = rotate_cl(from, oracle::tmt_u23_to_float(u), rule, i, t, a, b) == to;
      if (acc) {
        if (lo < 0) lo = u;
        else if (hi >= 0) gap = true;
      } else if (lo >= 0 && hi < 0) {
        hi = u;
      }
    }
    if (gap) return -1;
    if (lo < 0) lo = 0, hi = 0;
    if (hi < 0) hi = 1L << 23;
    out[2 * move] = (uint32_t)lo;
    out[2 * move + 1] = (uint32_t)(hi - lo);
  }
  return 0;
}

int orc_dm_rotate_fast(int e, uint32_t u, int rule, int i, int t, double a, double b) {
  return rotate_fast((uint8_t)e, u, rule, i, t, a, b);
}

}  // extern "C"

extern "C" {

// Seeded TinyMT generator states (default parameters) for generators 0 .. count-1 seeded
// with seed + k, as InitTinyMT does (dominokernel.cl:33-40): out is count x {s0, s1, s2, s3}.
void orc_tmt_seed_states(uint32_t seed, long count, uint32_t* out) {
  for (long k = 0; k < count; ++k) {
    oracle::TinyMT32 g{0, 0, 0, 0, oracle::kTmtMat1, oracle::kTmtMat2, oracle::kTmtTmat};
    oracle::tmt_init(g, seed + (uint32_t)k);
    out[4 * k] = g.s0;
    out[4 * k + 1] = g.s1;
    out[4 * k + 2] = g.s2;
    out[4 * k + 3] = g.s3;
  }
}

}  // extern "C"
