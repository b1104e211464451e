/*
 * rt_tilings.h - C ABI of librt_tilings.so, the GB300 (sm_103a) random-tiling sampler.
 *
 * The entry points replace the domino tiler of the reference library
 * (src/Domino/DominoTiler.h:78-130) for callers that bind it over an FFI: plain pointers,
 * sizes and status codes, no C++ or CUDA types.  include/rt_tilings.hpp keeps the
 * reference's C++ class shape (DominoTiler::Walk, MaxTiling, ...) on top of this ABI.
 *
 * Conventions shared by every entry point
 *  - A domain is an M x M int32 0/1 array of squares, a tiling an N x N int32 array of
 *    vertex edge-indicator masks with N = M + 1 (src/Domino/DominoTiler.h:19-37): bit 1 for
 *    the edge toward row i-1, 2 toward row i+1, 4 toward column j-1, 8 toward column j+1.
 *  - The caller owns every buffer; tilings are updated in place, as the reference's
 *    Walk(tiling&, ...) does (DominoTiler.cpp:18-122).
 *  - Errors are returned, never exit(): the reference prints and calls exit() from
 *    checkCudaErrors (src/common/helper_cuda.h:566-579).  rt_last_error() gives the
 *    message of the last failing call on the calling thread.
 *  - Sweeps run on the GPU only.  There is no CPU fallback: without a usable CUDA device
 *    every sweep entry point returns RT_ERR_CUDA.
 */
#ifndef RT_TILINGS_H_
#define RT_TILINGS_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define RT_API __attribute__((visibility("default")))
#else
#define RT_API
#endif

typedef int32_t rt_status;
#define RT_OK 0
#define RT_ERR_INVALID_ARGUMENT 1
#define RT_ERR_CUDA 2
#define RT_ERR_NOT_TILEABLE 3
#define RT_ERR_TIMEOUT 4
#define RT_ERR_OUT_OF_MEMORY 5
#define RT_ERR_NOT_COALESCED 6
#define RT_ERR_BUFFER_TOO_SMALL 7
#define RT_ERR_BUSY 8

/* Random-number modes of the sweep. */
#define RT_RNG_TINYMT 0 /* one TinyMT32 generator per site, the reference's OpenCL path
                           (src/TinyMT/tinymt32.clh, dominokernel.cl:4-40): bit-exact with it */
#define RT_RNG_FAST 1   /* counter-based Philox4x32-10 keyed by (seed, stream, half-sweep,
                           site); no generator state in memory */
#define RT_RNG_MTGP 2   /* cuRAND MTGP32, one generator per 8 x 8 block of sites seeded
                           seed + block, the reference's CUDA path (DominoTiler.cpp:51-66,
                           dominokernel*.cu; LozengeTiler.cpp:71-80, lozengekernel.cu;
                           RectTriangleTiler.cpp:75-85, TriangleDimerTiler.cpp:279-291):
                           domino, uniform lozenge, rectangle-triangle and bibone walks,
                           epochs and CFTP through the per-step kernels; the same draws as
                           the reference's build */

/* Flip rules: the reference picks one by compiling one of four kernel files. */
#define RT_DOMINO_PLAIN 0            /* src/Domino/dominokernel.cl:4-18 (propose 0.8) */
#define RT_DOMINO_CFTP 1             /* src/Domino/dominokernelCFTP.cl:51-71 (monotone 1/2-1/2) */
#define RT_DOMINO_TWOPERIODIC 2      /* src/Domino/dominokerneltwoperiodic.cl:7-35 */
#define RT_DOMINO_CFTP_TWOPERIODIC 3 /* src/Domino/dominokernelCFTPtwoperiodic.cl:72-101 */

typedef struct rt_walk_opts {
  int32_t rng_mode;  /* RT_RNG_* */
  int32_t rule;      /* RT_DOMINO_* */
  double weight_a;   /* two-periodic weights; the reference hard-codes a = 0.7, b = 1. */
  double weight_b;   /* (dominokerneltwoperiodic.cl:3-4).  Both must be > 0. */
  /* Optional TinyMT parameter table: count triples (mat1, mat2, tmat), one per generator
     in the order of the reference's parameter file (LoadTinyMT, DominoTiler.cpp:235-237).
     NULL selects the TinyMT32 jump parameters for every generator. */
  const uint32_t* tinymt_params;
  int64_t tinymt_params_count;
  uint32_t fast_stream; /* RT_RNG_FAST: stream id (< 65536), e.g. the instance number */
  int32_t engine;       /* 0: automatic; 1: per-half-sweep kernels; 2: resident persistent
                           kernel (the run kernel, which rebuilds the passive colour only where
                           the colour switches, else k_persist); 3: k_persist, the resident
                           kernel that exchanges band rows every half-sweep; 4: the bit-plane
                           kernel (one bit per lattice edge, TinyMT mode, 1 or 2 swept chains,
                           tilings whose flip candidates keep off the array's outer cells; 0
                           prefers it where it applies).  Lozenges: 0
                           automatic, 1 per-step kernels, 2 the resident band kernel (TinyMT
                           without MTGP, or fast mode); the same tilings from every engine */
  void* cuda_stream;    /* cudaStream_t to run on; NULL = the library's own stream */
} rt_walk_opts;

/* Fills *o with the reference's defaults: TinyMT, RT_DOMINO_PLAIN, a = 0.7, b = 1. */
RT_API void rt_walk_opts_default(rt_walk_opts* o);

RT_API const char* rt_status_string(rt_status s);
RT_API const char* rt_last_error(void);
RT_API const char* rt_version(void);

/* ---- domino host utilities (no GPU needed) ------------------------------------------- */

/* DominoTiler::AztecRectangle (DominoTiler.cpp:267-324) / AztecDiamond (:262-265).
   Writes the padded side^2 domain into out (capacity cap ints); *side receives M. */
RT_API rt_status rt_domino_aztec_rectangle(int32_t n, const int32_t* remove, int32_t n_remove, int32_t* out,
                                           int64_t cap, int32_t* side);
RT_API rt_status rt_domino_aztec_diamond(int32_t n, int32_t* out, int64_t cap, int32_t* side);
/* DominoTiler::Rectangle (DominoTiler.cpp:249-260). */
RT_API rt_status rt_domino_rectangle(int32_t rows, int32_t cols, int32_t* out, int64_t cap, int32_t* side);
/* DominoTiler::DomainToVertices (DominoTiler.cpp:611-631): out is (M+1)^2. */
RT_API rt_status rt_domino_domain_to_vertices(const int32_t* domain, int32_t m_side, int32_t* out);
/* DominoTiler::MaxTiling / MinTiling, Thurston's algorithm (DominoTiler.cpp:345-531).
   RT_ERR_NOT_TILEABLE when the boundary or bulk height check fails (the reference prints
   "NOT tileable" and returns a height function in that case). */
RT_API rt_status rt_domino_max_tiling(const int32_t* domain, int32_t m_side, int32_t* out);
RT_API rt_status rt_domino_min_tiling(const int32_t* domain, int32_t m_side, int32_t* out);
/* Thurston's extremal tiling on the GPU (no counterpart in the reference): the same tiling
   and the same errors as rt_domino_max_tiling (top != 0) / rt_domino_min_tiling, with the
   bulk filled by parallel relaxation to the reference's shortest-path fixed point.  Domains
   whose boundary is not one connected walk (holes) return RT_ERR_INVALID_ARGUMENT. */
RT_API rt_status rt_domino_extremal_tiling_device(const int32_t* domain, int32_t m_side, int32_t top, int32_t* out,
                                                  void* cuda_stream);
/* DominoTiler::TilingToHeightfunc / HeightfuncToTiling / TilingToDomain
   (DominoTiler.cpp:555-593, 534-553, 595-609).  Heights outside the domain are INT32_MAX. */
RT_API rt_status rt_domino_tiling_to_heightfunc(const int32_t* tiling, const int32_t* domain, int32_t n_side,
                                                int32_t* out);
RT_API rt_status rt_domino_heightfunc_to_tiling(const int32_t* hf, const int32_t* domain, int32_t n_side,
                                                int32_t* out);
RT_API rt_status rt_domino_tiling_to_domain(const int32_t* tiling, int32_t n_side, int32_t* out);

/* ---- domino sweeps (GPU) ---------------------------------------------------------------- */

/* DominoTiler::Walk(tiling&, long steps, long seed) (DominoTiler.cpp:18-122).  One step is
   one half-sweep: a colour drawn from mt19937(seed) (TinyMT mode: the generators are seeded
   with the first draw, as on the reference's OpenCL path; MTGP mode: block generator k is
   seeded seed + k and the colours start with the first draw, as on its CUDA path) or
   alternating black/white (fast mode), a flip attempt at every site of that colour, then
   the other colour rebuilt.
   n_side = N must be even and >= 6; the outermost two rings must be empty (padded). */
RT_API rt_status rt_domino_walk(int32_t* tiling, int32_t n_side, int64_t steps, int64_t seed,
                                const rt_walk_opts* opts);

/* DominoTiler::Walk(tiling&, vector steps, vector seeds) (DominoTiler.cpp:125-231): epoch k
   re-seeds the generators with seeds[k] and draws its colours from mt19937(seeds[k]). */
RT_API rt_status rt_domino_walk_epochs(int32_t* tiling, int32_t n_side, const int64_t* steps, const int64_t* seeds,
                                       int32_t n_epochs, const rt_walk_opts* opts);

/* Coupling from the past for the monotone rules (RT_DOMINO_CFTP, RT_DOMINO_CFTP_TWOPERIODIC).
   TinyMT mode follows Examples/AztecDiamondCftpEx.cpp:51-77: epoch seeds from
   mt19937(driver_seed); the first epoch has first_steps steps; each failed attempt prepends
   an epoch of 2*steps.back() steps (schedule 0, the reference's rule) or 2*steps.front()
   (schedule 1, doubling).  Fast mode: attempt j runs half-sweeps [-2T, 0) with
   T = first_steps * 2^j sweeps, randomness keyed by (driver_seed, fast_stream, half-sweep).
   The coupled max/min chains run in one kernel on the shared stream and coalescence is a
   device XOR-popcount.  RT_ERR_NOT_COALESCED after max_attempts attempts; out then holds the
   top chain after the last attempt and *stats is filled. */
typedef struct rt_cftp_stats {
  int32_t attempts;     /* attempts run (the last one coalesced on success) */
  int64_t total_steps;  /* half-sweeps run per chain over all attempts */
  int64_t final_steps;  /* half-sweeps of the coalesced attempt (its look-back) */
  int64_t flip_attempts;/* interior-site evaluations over both chains and all attempts */
  double seconds;       /* device time of the sweeps */
} rt_cftp_stats;

RT_API rt_status rt_domino_cftp(const int32_t* tmax, const int32_t* tmin, int32_t n_side, int64_t driver_seed,
                                int64_t first_steps, int32_t schedule, int32_t max_attempts,
                                const rt_walk_opts* opts, int32_t* out, rt_cftp_stats* stats);

/* ---- lozenge tilings (src/Lozenge/LozengeTiler.h:63-92) ---------------------------------
   Vertices of the triangular lattice, N x N, each an edge mask over its six neighbours
   (0,+1):8 (-1,+1):2 (-1,0):1 (0,-1):4 (+1,-1):16 (+1,0):32, set where a lozenge crosses
   the edge; N must be a multiple of 3.  A domain is an M x 2M array of triangles, N = M+1. */

/* Lozenge rules (rt_walk_opts.rule for the rt_lozenge_* sweeps): the reference's uniform
   rotation (lozengekernel.cl, 0.4 / 0.4), or the q^volume rotation of qlozengekernel.cl with
   q = rt_walk_opts.weight_a (the reference's #define q 0.99) and its down-move rescaling
   corrected (identical decisions for q <= 1). */
#define RT_LOZENGE_UNIFORM 0
#define RT_LOZENGE_Q 1

/* LozengeTiler::AlmostHexDomain(n, m) (LozengeTiler.cpp:422-467): hexagon of side n with an
   m x m corner removed (m = 0: the regular a = b = c = n hexagon), padded.  *rows = M. */
RT_API rt_status rt_lozenge_almost_hex_domain(int32_t n, int32_t m, int32_t* out, int64_t cap, int32_t* rows);
/* LozengeTiler::DomainToVertices / MaxTiling / MinTiling / HeightfuncToTiling /
   TilingToHeightfunc / TilingToDomain (LozengeTiler.cpp:173-556). */
RT_API rt_status rt_lozenge_domain_to_vertices(const int32_t* domain, int32_t m_rows, int32_t* out);
RT_API rt_status rt_lozenge_max_tiling(const int32_t* domain, int32_t m_rows, int32_t* out);
RT_API rt_status rt_lozenge_min_tiling(const int32_t* domain, int32_t m_rows, int32_t* out);
RT_API rt_status rt_lozenge_heightfunc_to_tiling(const int32_t* hf, const int32_t* domain, int32_t n_side,
                                                 int32_t* out);
RT_API rt_status rt_lozenge_tiling_to_heightfunc(const int32_t* tiling, const int32_t* domain, int32_t n_side,
                                                 int32_t* out);
RT_API rt_status rt_lozenge_tiling_to_domain(const int32_t* tiling, int32_t n_side, int32_t* out);
/* LozengeTiler::Walk(tiling&, int steps, long seed) (LozengeTiler.cpp:27-159): per step a
   colour from default_random_engine(seed) + uniform_int_distribution(0, 2) (TinyMT mode,
   generators seeded with seed itself; MTGP mode, block generator k seeded seed + k as the
   CUDA branch does, LozengeTiler.cpp:71-80) or h mod 3 (fast mode), then the rotation
   25 <-> 38 (0.4 / 0.4, lozengekernel.cl:74-105, lozengekernel.cu:15-29) and the rebuild of
   the two other colours (lozengekernel.cl:107-125).  opts->rule selects RT_LOZENGE_UNIFORM
   or RT_LOZENGE_Q (q in opts->weight_a; TinyMT and fast modes only). */
RT_API rt_status rt_lozenge_walk(int32_t* tiling, int32_t n_side, int64_t steps, int64_t seed,
                                 const rt_walk_opts* opts);
/* The float draws RT_RNG_MTGP makes for the first `launches` steps of a lozenge walk on an
   n_side tiling whose block generators are seeded seed + k: out[h][i][j] (launches x n_side x
   n_side/3 floats, host memory) is the draw of slot (i, j) of the rotated colour at step h
   (lozengekernel.cu:20-21). */
RT_API rt_status rt_lozenge_mtgp_draws(int32_t n_side, int64_t seed, int64_t launches, float* out);
/* Coupling from the past from the max and min tilings with the reference's primitives: each
   epoch is one Walk(t, steps_k, seed_k) of both chains on the shared stream, seeds from
   mt19937(driver_seed), look-back prepending 2*steps.back() (schedule 0) or 2*steps.front()
   (schedule 1); fast mode runs steps [-3T, 0), T = first_steps * 2^j. */
RT_API rt_status rt_lozenge_cftp(const int32_t* tmax, const int32_t* tmin, int32_t n_side, int64_t driver_seed,
                                 int64_t first_steps, int32_t schedule, int32_t max_attempts,
                                 const rt_walk_opts* opts, int32_t* out, rt_cftp_stats* stats);

/* ---- rectangle-triangle tilings (src/RectTriangle/RectTriangleTiler.h:32-86) -----------
   Vertices of the triangular lattice, N x N with N a multiple of 3 and three rows/columns of
   zero padding, each holding six hexadecimal digits: the covering codes of the six triangles
   around it (RectTriangleTiler.h:14-22); a digit d of a tiling weighs wt_d (d = 1-3),
   wr_((d-4) mod 3 + 1) (d = 4-9) or wm_((d-10) mod 3 + 1) (d = 10-15), as the weight table at
   recttrianglekernel.cl:13. */

/* RectTriangleTiler::maxHex (top = 1) / minHex (top = 0) / slopeHex (top = 2)
   (RectTriangleTiler.cpp:173-600): start tilings of the hexagon of side n >= 2 after the
   reference's shear and padding.
   *side receives the side N; out needs N * N entries (cap). */
RT_API rt_status rt_recttri_hex_tiling(int32_t n, int32_t top, int32_t* out, int64_t cap, int32_t* side);
/* RectTriangleTiler::LozengeToRectTriangle(tiling&, domain&) (RectTriangleTiler.cpp:602-644):
   a lozenge tiling (edge masks as rt_lozenge_*, N x N) of a domain of m_rows x 2 m_rows
   triangles, read as an all-triangle rectangle-triangle tiling, N x N. */
RT_API rt_status rt_recttri_from_lozenge(const int32_t* lozenge, int32_t n_side, const int32_t* domain,
                                         int32_t m_rows, int32_t* out);
/* RectTriangleTiler::Walk(tiling&, int steps, long seed) (RectTriangleTiler.cpp:33-171):
   per step a colour ((i - j) mod 3) from default_random_engine(seed) +
   uniform_int_distribution(0, 2) (TinyMT mode, generator k seeded with seed + k; MTGP mode,
   block generator k seeded seed + k as the CUDA branch does, RectTriangleTiler.cpp:75-85)
   or h mod 3 (fast mode), then flipTiles (recttrianglekernel.cl:25-118) on that colour and
   updateTiles1/2 (:120-146) on the two others.  weights9 = {wt1, wt2, wt3, wm1, wm2, wm3,
   wr1, wr2, wr3}, the compile-time constants of recttrianglekernel.cl:3-11 (NULL: all 1, the
   reference's values); float arithmetic as the reference kernel.  opts->rule is ignored. */
RT_API rt_status rt_recttri_walk(int32_t* tiling, int32_t n_side, int64_t steps, int64_t seed,
                                 const double* weights9, const rt_walk_opts* opts);
/* The MTGP mode's float draws of a rectangle-triangle walk: the layout of
   rt_lozenge_mtgp_draws (launches x n_side x n_side/3; flipTilesKernel draws at
   recttrianglekernel.cu:39-40 on the same grid). */
RT_API rt_status rt_recttri_mtgp_draws(int32_t n_side, int64_t seed, int64_t launches, float* out);

/* ---- six-vertex model ----------------------------------------------------------------------
   No counterpart in the reference (which has no six-vertex model); the entry points follow the
   shape of the per-model classes (domain / extremal states / Walk / CFTP / height function).
   State: the height function on the (n+1) x (n+1) corners of an n x n vertex grid, int32,
   h(below) - h(above) = +1 across a horizontal edge whose arrow points right and
   h(right) - h(left) = +1 across a vertical edge whose arrow points up.  Vertex types from
   the corner heights: a (NE == SW, NW != SE), b (NW == SE, NE != SW), c (both equal), weights
   abc = {a, b, c} (NULL: all 1).  The boundary heights are never changed.
   Sweep: four point classes (x mod 2, y mod 2), sub-sweep s updates class s mod 4 by heat
   bath (h' +- 1 at points whose four edge neighbours equal h'), draws from Philox4x32-10
   bit planes keyed by (seed, opts->fast_stream, s).  Only RT_RNG_FAST exists for this model
   (opts NULL: fast mode, stream 0). */

/* Heat-bath thresholds T[3 k1 + k2] = min(floor(P 2^32), 2^32 - 1), P = W+ / (W+ + W-). */
RT_API rt_status rt_sv_thresholds(double a, double b, double c, uint32_t* out9);
/* Domain-wall boundary, maximal (top != 0: min(x + y, 2n - x - y)) or minimal (|x - y|)
   height function, (n+1)^2 entries. */
RT_API rt_status rt_sv_dwbc_height(int32_t n, int32_t top, int32_t* out);
/* Domain-wall height function <-> alternating sign matrix (n x n, entries (NE + SW - NW - SE)/2). */
RT_API rt_status rt_sv_height_to_asm(const int32_t* h, int32_t n, int32_t* out);
RT_API rt_status rt_sv_asm_to_height(const int32_t* a, int32_t n, int32_t* out);
/* 4 * sweeps sub-sweeps (s = 0 .. 4 sweeps - 1) on h in place.  stats (optional): flip
   attempts ((n-1)^2 per sweep) and the device time of the sweeps. */
RT_API rt_status rt_sv_walk(int32_t* h, int32_t n, int64_t sweeps, int64_t seed, const double* abc,
                            const rt_walk_opts* opts, rt_cftp_stats* stats);
/* Coupling from the past from hmax >= hmin (same boundary): attempt j runs sub-sweeps
   [-4 T, 0), T = first_sweeps * 2^j, both chains on the same draws.  Exact for
   c >= max(a, b) (the heat-bath update is then monotone); RT_ERR_INVALID_ARGUMENT otherwise.
   RT_ERR_NOT_COALESCED after max_attempts (out then holds the top chain). */
RT_API rt_status rt_sv_cftp(const int32_t* hmax, const int32_t* hmin, int32_t n, int64_t seed, int64_t first_sweeps,
                            int32_t max_attempts, const double* abc, const rt_walk_opts* opts, int32_t* out,
                            rt_cftp_stats* stats);

/* ---- bibone tilings: dimers of the triangular lattice (src/TriangleDimer/TriangleDimerTiler.h:
   84-216) -------------------------------------------------------------------------------------
   Tiling format of the reference: side N = 2M, vertex (a, b); t[2a][2b+1], t[2a+1][2b] and
   t[2a+1][2b+1] hold the edge states of the lozenges around the horizontal, up-left and
   up-right edges (TriangleDimerTiler.h:17-28); the first and last three rows and columns are
   zero.  Dimer form: one byte per vertex, bit 1 the edge (a,b)-(a,b+1), bit 2 (a,b)-(a-1,b),
   bit 4 (a,b)-(a-1,b+1). */

/* TriangleDimerTiler::IceCreamCone(n, m) (TriangleDimerTiler.cpp:697-793): the downward
   triangle of side n with a side-m triangle cut from its top-left corner.  *side = 2 (n + 4). */
RT_API rt_status rt_td_icecream_cone(int32_t n, int32_t m, int32_t* out, int64_t cap, int32_t* side);
/* No counterpart in the reference: the rows x cols rhombus of vertices (cols even) covered by
   horizontal dimers in a brick pattern, padded by three vertices; *side = 2 (max(rows, cols) + 6). */
RT_API rt_status rt_td_rhombus_brick(int32_t rows, int32_t cols, int32_t* out, int64_t cap, int32_t* side);
/* Tiling format <-> dimer bytes ((N/2)^2 of them). */
RT_API rt_status rt_td_dimers(const int32_t* tiling, int32_t n_side, uint8_t* out);
RT_API rt_status rt_td_from_dimers(const uint8_t* dimers, int32_t n_side, int32_t* out);
/* TriangleDimerTiler::TestButterfly(type) (TriangleDimerTiler.cpp:795-845, side 16; types
   other than 0 H, 1 L, 2 R give the all-zero tiling), TilingToTriangleFlips (:846-873,
   (N/2) x N) and TilingToButterflyFlips (:875-921, N x N): the move states the reference
   derives from a tiling. */
RT_API rt_status rt_td_test_butterfly(int32_t type, int32_t* out, int64_t cap, int32_t* side);
RT_API rt_status rt_td_triangle_flips(const int32_t* tiling, int32_t n_side, int32_t* out);
RT_API rt_status rt_td_butterfly_flips(const int32_t* tiling, int32_t n_side, int32_t* out);
/* TriangleDimerTiler::TilingToVertices / TilingToDomain / DimerIndicator
   (TriangleDimerTiler.cpp:923-982, 35-99): the covered-vertex grid ((N/2+1)^2), the domain of
   triangles ((N/2) x N) and the M x M indicator of dimers of orientation c (0 horizontal,
   1 up-left, 2 up-right). */
RT_API rt_status rt_td_vertices(const int32_t* tiling, int32_t n_side, int32_t* out);
RT_API rt_status rt_td_domain(const int32_t* tiling, int32_t n_side, int32_t* out);
RT_API rt_status rt_td_dimer_indicator(const int32_t* tiling, int32_t n_side, int32_t c, int32_t* out);
/* TriangleDimerTiler::Walk(tiling&, int steps, long seed) (TriangleDimerTiler.cpp:101-695):
   per step a move type, orientation and colour (plus slice and parity for butterflies) from
   default_random_engine(seed) (TinyMT mode; every generator draws each step, generator
   row * M + column seeded seed + k) or from Philox keyed by (seed, opts->fast_stream, step)
   (fast mode); sites of that class toggle their lozenge / triangle / butterfly cycle with
   probability 1/2 when one half of it is covered.  stats (optional): flip attempts (sites of
   the chosen class on covered vertices) and the device time. */
RT_API rt_status rt_td_walk(int32_t* tiling, int32_t n_side, int64_t steps, int64_t seed, const rt_walk_opts* opts,
                            rt_cftp_stats* stats);
/* The MTGP mode's float draws of a bibone walk: out[h][a][b] (launches x M x M, M = n_side/2)
   is the curand_uniform value of site (a, b) at step h, in the launch of the reference's
   Rotate*Kernel (triangledimerkernel.cu, 8 x 8 blocks over M x M). */
RT_API rt_status rt_td_mtgp_draws(int32_t n_side, int64_t seed, int64_t launches, float* out);

/* ---- the reference's text matrix format (src/common/common.cpp:84-178) --------------------
   rt_save_matrix: rows x cols values, each followed by a space, one line per row
   (SaveMatrix(v, M, N, file)); rt_save_matrix_square: SaveMatrix(v, file), floor(sqrt(size))
   rows and columns.  rt_load_matrix: every run of decimal digits is one value (LoadMatrix;
   like the reference it reads no sign); *count = values found, at most cap written. */
RT_API rt_status rt_save_matrix(const int32_t* a, int64_t rows, int64_t cols, const char* path);
RT_API rt_status rt_save_matrix_square(const int32_t* a, int64_t size, const char* path);
RT_API rt_status rt_load_matrix(const char* path, int32_t* out, int64_t cap, int64_t* count);

/* ---- batched coupling from the past --------------------------------------------------------
   No counterpart in the reference (which runs one instance at a time).  Many independent
   fast-mode CFTP instances of uneven sizes, dominoes and lozenges mixed, in one persistent
   launch: each CTA takes instances from a device work queue and runs an instance's whole
   CFTP in shared memory.  Instance k returns exactly what rt_domino_cftp / rt_lozenge_cftp
   return with rng_mode RT_RNG_FAST, fast_stream = stream and driver_seed = seed. */
#define RT_MODEL_DOMINO 0
#define RT_MODEL_LOZENGE 1
#define RT_MODEL_RECTTRI 2
#define RT_MODEL_BIBONE 3
#define RT_MODEL_SIX_VERTEX 4

typedef struct rt_cftp_instance {
  int32_t model;        /* RT_MODEL_DOMINO or RT_MODEL_LOZENGE */
  int32_t n_side;       /* tiling side N */
  int32_t rule;         /* dominoes: RT_DOMINO_CFTP or RT_DOMINO_CFTP_TWOPERIODIC */
  int32_t max_attempts; /* <= 40 */
  double weight_a, weight_b;
  uint64_t seed;        /* driver seed of the instance's draws */
  uint32_t stream;      /* < 65536 */
  int32_t pad;
  int64_t first_steps;  /* sweeps of the first attempt; attempt j uses first_steps * 2^j */
  const int32_t* tmax;  /* host N x N extremal tilings */
  const int32_t* tmin;
  int32_t* out;         /* host N x N sample (the top chain of the last attempt) */
  int32_t attempts;     /* out: attempts run; negative when the instance did not coalesce */
  int32_t pad2;
  int64_t final_steps;  /* out: half-sweeps (steps) of the last attempt */
} rt_cftp_instance;

typedef struct rt_batch_stats {
  int32_t instances, coalesced, ctas, pad;
  double seconds;             /* device time of the batch kernels (and of the one-at-a-time runs) */
  int32_t cluster_instances;  /* instances held by a thread-block cluster */
  int32_t single_instances;   /* instances run one at a time through the single-instance path */
} rt_batch_stats;

/* Runs every instance; RT_ERR_NOT_COALESCED if any instance ran out of attempts (its out
   and attempts are still written).  Instances whose two chains fit one CTA's shared memory
   (about 2 x N^2 bytes: N up to about 330 for dominoes, 340 for lozenges) run in the
   persistent one-CTA kernel; larger ones in a cluster kernel, each instance held by a
   thread-block cluster of 2-16 CTAs exchanging its halo rows through distributed shared
   memory (N up to about 1300); any larger instance runs
   after them, one at a time, through rt_domino_cftp / rt_lozenge_cftp on the same stream.
   All three give the same samples for the same (seed, stream). */
RT_API rt_status rt_cftp_batch(rt_cftp_instance* inst, int32_t count, void* cuda_stream, rt_batch_stats* stats);

/* ---- model-generic entry points ------------------------------------------------------------
   One signature for every model (RT_MODEL_*), dispatching to the per-model functions above,
   for callers that bind the library once.  weights: RT_MODEL_RECTTRI the nine weights of
   rt_recttri_walk, RT_MODEL_SIX_VERTEX {a, b, c} (NULL: all 1), unused by the other models
   (domino and lozenge take theirs in opts).  For RT_MODEL_SIX_VERTEX the state is the height
   function, n_side is n and steps count sweeps; for RT_MODEL_BIBONE the state is the
   reference's tiling format of rt_td_walk.  rt_walk_epochs exists for dominoes only (the
   reference's epoch overload), rt_cftp for dominoes, lozenges and the six-vertex model
   (schedule is ignored there); the others return RT_ERR_INVALID_ARGUMENT. */
RT_API rt_status rt_walk(int32_t model, int32_t* tiling, int32_t n_side, int64_t steps, int64_t seed,
                         const double* weights, const rt_walk_opts* opts);
RT_API rt_status rt_walk_epochs(int32_t model, int32_t* tiling, int32_t n_side, const int64_t* steps,
                                const int64_t* seeds, int32_t n_epochs, const rt_walk_opts* opts);
RT_API rt_status rt_cftp(int32_t model, const int32_t* tmax, const int32_t* tmin, int32_t n_side, int64_t driver_seed,
                         int64_t first_steps, int32_t schedule, int32_t max_attempts, const double* weights,
                         const rt_walk_opts* opts, int32_t* out, rt_cftp_stats* stats);

/* ---- serving: continuous batching ----------------------------------------------------------
   No counterpart in the reference.  A request is one fast-mode CFTP instance
   (rt_cftp_instance).  Submitted requests go to a ring of slots in pinned host memory that
   the GPU reads directly; a persistent kernel's CTAs claim them in order as they free up
   (requests that arrive while others run join without waiting for them), run each one's
   CFTP in shared memory and flag it done.  The kernel leaves after idle_seconds without
   work and is relaunched by the next submit / poll / wait.  Admission: a request needs a
   free slot and its footprint (3 colour-split tilings) within memory_budget_bytes, else
   RT_ERR_BUSY.  Results equal rt_cftp_batch's and the plain entry points'.  One host thread
   per server. */
typedef struct rt_server rt_server;
typedef struct rt_server_opts {
  int32_t slots;                 /* ring capacity: requests submitted and not yet collected */
  int32_t max_side;              /* largest tiling side accepted, <= 330 */
  int64_t memory_budget_bytes;   /* cap on the staged state of requests in flight */
  double idle_seconds;           /* the kernel leaves after this long without work (0: 0.25 s) */
  void* cuda_stream;             /* NULL: the server's own stream */
} rt_server_opts;

RT_API rt_status rt_server_create(const rt_server_opts* opts, rt_server** out);
/* Copies the request (its tmax / tmin) and returns its ticket; req->out is not used here. */
RT_API rt_status rt_server_submit(rt_server* s, const rt_cftp_instance* req, int64_t* ticket);
RT_API rt_status rt_server_poll(rt_server* s, int64_t ticket, int32_t* done);
/* Waits up to timeout_s, writes the sample to result->out (N x N) and result->attempts /
   final_steps, and frees the ticket's slot. */
RT_API rt_status rt_server_wait(rt_server* s, int64_t ticket, double timeout_s, rt_cftp_instance* result);
/* Asks the kernel to leave, waits for it and frees everything. */
RT_API rt_status rt_server_destroy(rt_server* s);

/* ---- device-resident chains --------------------------------------------------------------
   A sampler keeps n_chains coupled chains of one N x N domain on the GPU; all chains see
   the same random stream (CFTP couples the max and min chains this way).  The building
   block of the entry points above, exposed for callers that keep state on the device. */
typedef struct rt_dm_sampler rt_dm_sampler;

RT_API rt_status rt_dm_sampler_create(int32_t n_side, int32_t n_chains, const rt_walk_opts* opts,
                                      rt_dm_sampler** out);
RT_API rt_status rt_dm_sampler_destroy(rt_dm_sampler* s);
/* Host int32 N x N tiling -> chain (copy and colour split run on the device). */
RT_API rt_status rt_dm_sampler_load(rt_dm_sampler* s, int32_t chain, const int32_t* tiling);
/* Chain -> host int32 N x N tiling. */
RT_API rt_status rt_dm_sampler_store(rt_dm_sampler* s, int32_t chain, int32_t* tiling);
/* Copies chain src onto chain dst on the device. */
RT_API rt_status rt_dm_sampler_copy_chain(rt_dm_sampler* s, int32_t dst, int32_t src);
/* Only chains [0, k) are swept by later runs (the others keep their state), 1 <= k <= n_chains. */
RT_API rt_status rt_dm_sampler_set_active(rt_dm_sampler* s, int32_t k);
/* TinyMT mode: InitTinyMT (dominokernel.cl:33-40): generator k <- seed + k.  MTGP mode: block
   generator k <- seed + k (DominoTiler.cpp:62-65), after the sampler's stream has drained. */
RT_API rt_status rt_dm_sampler_seed(rt_dm_sampler* s, uint32_t seed);
/* TinyMT or MTGP mode: runs steps half-sweeps, colours[s] = 1 rotates black (t = 1), 0 white.
   MTGP mode needs a prior rt_dm_sampler_seed (RT_ERR_INVALID_ARGUMENT otherwise). */
RT_API rt_status rt_dm_sampler_run(rt_dm_sampler* s, const uint8_t* colours, int64_t steps);
/* Fast mode: runs half-sweeps h0 .. h0+steps-1 (even h black, odd h white). */
RT_API rt_status rt_dm_sampler_run_fast(rt_dm_sampler* s, uint64_t seed, int64_t h0, int64_t steps);
/* Number of sites where chains a and b differ (device XOR-popcount). */
RT_API rt_status rt_dm_sampler_diff(rt_dm_sampler* s, int32_t a, int32_t b, int64_t* ndiff);
/* Waits for the sampler's stream. */
RT_API rt_status rt_dm_sampler_sync(rt_dm_sampler* s);
/* The cudaStream_t the sampler launches on. */
RT_API void* rt_dm_sampler_stream(rt_dm_sampler* s);
/* Flip attempts (interior sites of one colour class) per half-sweep of one chain: the
   average over the two colours is interior_vertices / 2. */
RT_API int64_t rt_dm_sampler_interior_vertices(rt_dm_sampler* s);
/* Kernels launched by this sampler since creation. */
RT_API int64_t rt_dm_sampler_launches(rt_dm_sampler* s);
/* Device-side statistics: adds the edge-placement indicators of a chain to a caller-owned
   device array of 2 N^2 uint32 counters on the sampler's stream, no copy to the host.
   counts[i N + j] counts vertex (i, j)'s bit 2 (a horizontal domino on faces (i, j-1), (i, j));
   counts[N^2 + i N + j] its bit 8 (a vertical domino on faces (i-1, j), (i, j)).  No
   counterpart in the reference; rt_domino_edge_indicators is the same on a host tiling. */
RT_API rt_status rt_dm_sampler_accumulate_edges(rt_dm_sampler* s, int32_t chain, uint32_t* counts_device);
/* Height functions on the device: TilingToHeightfunc (DominoTiler.cpp:555-593) of a chain,
   for the domain given once (the (N-1)^2 face array the chains tile).  sums_device (int64,
   N^2, may be NULL) receives += the heights of the vertices that have one; heights_device
   (int32, N^2, may be NULL) the heights themselves (INT32_MAX where unset, as the
   reference's infty).  For tilings (not arbitrary masks) the heights equal the host
   function's. */
RT_API rt_status rt_dm_sampler_set_domain(rt_dm_sampler* s, const int32_t* domain, int32_t m_side);
RT_API rt_status rt_dm_sampler_accumulate_heights(rt_dm_sampler* s, int32_t chain, long long* sums_device,
                                                  int32_t* heights_device);
/* The same for one tiling in host memory. */
RT_API rt_status rt_domino_heightfunc_device(const int32_t* tiling, const int32_t* domain, int32_t n_side,
                                             int32_t* out, void* cuda_stream);
RT_API rt_status rt_domino_edge_indicators(const int32_t* tiling, int32_t n_side, uint32_t* counts);
/* Exact edge-placement probabilities of the Aztec diamond of the given order (the tiling of
   rt_domino_aztec_diamond, N = 2 order + 6) under the reference's weights: a horizontal
   domino weighs a when its left face's column is odd, else b; a vertical one a when its top
   face's row is even, else b (a = b: uniform).  out (2 N^2 doubles, cap entries) receives
   them in the layout of the edge counters above, so counts / samples estimates out.
   Generalized domino shuffling (Propp 2003) on the device, one launch per order level, on
   cuda_stream (NULL: the default stream); synchronous.  No counterpart in the reference. */
RT_API rt_status rt_domino_aztec_edge_probs(int32_t order, double a, double b, double* out, int64_t cap,
                                            void* cuda_stream);
/* The engine the next run will use: out4 = {engine (1 per-half-sweep kernels, 2 the
   resident run kernel, 3 the resident k_persist, 4 the bit-plane kernel), flip-candidate
   generators held by the resident kernel (sites with a TinyMT generator: units), CTAs
   (bands), units per thread (column quads for the run kernel, sites or quads for k_persist,
   32-cell words for the bit-plane kernel)}. */
RT_API rt_status rt_dm_sampler_engine_info(rt_dm_sampler* s, int64_t* out4);
/* Launch shape of the sampler's next runs (no counterpart in the reference: its kernels use
   one compile-time block shape, BLOCK_DIM 8 in src/Domino/dominokernel.cuh:4): engine (0
   automatic, 1 per-half-sweep kernels, 2 the run kernel, 3 k_persist, 4 the bit-plane
   kernel), bands (CTAs, 0: one per SM) and threads per band (a multiple of 32 up to 1024,
   0: 1024) of the run kernel.
   Results do not depend on the shape: every draw is keyed by its site.  Without this call,
   and with rt_walk_opts.engine 0, the autotuner's table (rt_tune_load) chooses when it has an
   entry.  out6 of rt_dm_sampler_launch_info = {engine, units, bands, units per thread,
   threads per band, 1 when the table chose}. */
RT_API rt_status rt_dm_sampler_set_launch(rt_dm_sampler* s, int32_t engine, int32_t bands, int32_t threads);
RT_API rt_status rt_dm_sampler_launch_info(rt_dm_sampler* s, int64_t* out6);

/* ---- autotuner table -------------------------------------------------------------------
   No counterpart in the reference.  A text table of measured launch shapes, written by
   `python -m randomtilingspublic_gb300.autotune`: one entry per line,
     domino <n_lo> <n_hi> <chains> <tinymt|fast> <engine> <bands> <threads> [<us>]
   ('#' starts a comment).  rt_tune_load replaces the process's table (also read from the
   file named by the environment variable RT_TUNE_FILE at the first lookup); samplers with
   engine 0 and no rt_dm_sampler_set_launch take the entry whose tiling-side range holds
   theirs.  rt_tune_lookup returns {engine, bands, threads} of that entry, or
   RT_ERR_INVALID_ARGUMENT when there is none. */
RT_API rt_status rt_tune_load(const char* path);
RT_API rt_status rt_tune_clear(void);
RT_API rt_status rt_tune_lookup(int32_t model, int32_t n_side, int32_t chains, int32_t rng_mode, int32_t* out3);

/* Test hook for the resident engine's failure detection (no counterpart in the reference):
   in the sampler's next runs band `band` publishes none of its boundary rows (band < 0:
   none) and every wait gives up after max_spin polls (0: the default, 2^22).  The
   neighbours' waits then run out, every CTA leaves its loop, and the run (or the next sync
   or store) returns RT_ERR_TIMEOUT, with the CUDA context intact.  Nothing faults. */
RT_API rt_status rt_dm_sampler_test_silent_band(rt_dm_sampler* s, int32_t band, int64_t max_spin);

/* ---- allocation-free sweep -------------------------------------------------------------
   No counterpart in the reference.  For callers that cannot allocate device memory (a
   host application that hands the library a fixed device arena up front, or code that must
   not allocate inside a latency-critical loop or under a hard memory cap): runs steps
   half-sweeps of the resident sweep kernel on chains the caller already holds on the
   device, and allocates nothing - no cudaMalloc, cudaFree or allocating library call.
   The kernel's scratch (neighbour exchange rows, flags, band plan, colours) is a fixed
   static device array of about 2.2 MiB in the library's device code module; a GPU holds it
   from the time that module is loaded on it until the process exits.
   Layout: dev_chains holds n_chains chains back to back, n_chains * 2 * N * P bytes in all
   (P = N/2 rounded up to a multiple of 16).  Each chain is two colour arrays, white (colour
   0) then black (colour 1: the vertices (i, j) with i + j even), each N rows of P bytes;
   byte m of row i of colour c is the edge mask of the vertex of that colour in columns
   2m, 2m+1 of row i of the N x N tiling.  The size cannot be checked, as no size is passed.
   dev_generators (TinyMT mode) holds one uint4 state per site (i, m), i in [1, N-2], m in
   [1, N/2-2], index (i-1)*(N/2-2) + (m-1), advanced in place; colours (host) gives the
   colour of each half-sweep (1 black, 0 white).  Fast mode ignores both and runs
   half-sweeps h0 .. h0+steps-1 keyed by fast_seed.
   Limits: N <= 1024, n_chains <= 2, steps <= 65536 per call; larger requests return
   RT_ERR_INVALID_ARGUMENT.  Per-generator parameter tables are not supported here.
   Set-up: every call takes the array's device address (cudaGetSymbolAddress) with the
   current device, which under CUDA's default lazy module loading loads the module (the
   array and the kernels) at the first call on a device.  A call with steps = 0 does all of
   this set-up and sweeps nothing: make it first, before any stream capture and outside any
   loop that must not see the module load (or set CUDA_MODULE_LOADING=EAGER).  Every call
   shares the array and clears the flags it relies on; calls that overlap on the GPU race on
   it, so order them (one stream, or synchronise between calls).  Synchronous: returns after
   the sweep ends. */
RT_API rt_status rt_dm_sweep_noalloc(uint8_t* dev_chains, void* dev_generators, int32_t n_side, int32_t n_chains,
                                     const uint8_t* colours, int64_t steps, uint64_t fast_seed, int64_t h0,
                                     const rt_walk_opts* opts);

/* ---- diagnostics ---------------------------------------------------------------------
   The acceptance intervals a rule compiles to: for c = (row & 1) | (colour << 1),
   out16[4c .. 4c+3] = {lo_up, width_up, lo_down, width_down}; a site in state 3 flips to 12
   when (u - lo_up) < width_up, a site in state 12 flips to 3 when (u - lo_down) < width_down,
   u the 23-bit TinyMT draw, the 32-bit fast draw or the bit pattern of the MTGP mode's float
   draw.  No reference counterpart: the reference evaluates its float thresholds per draw
   (dominokernel*.cl, dominokernel*.cu). */
RT_API rt_status rt_domino_rule_table(int32_t rule, int32_t rng_mode, double a, double b, uint32_t* out16);

/* The float draws RT_RNG_MTGP makes for the first `launches` half-sweeps of a domino walk on
   an n_side tiling whose block generators are seeded seed + k: out[h][i-1][m-1] (launches x
   (n_side-2) x (n_side/2-2) floats, host memory) is the draw of candidate site (i, m) at
   half-sweep h, the value the reference's rotate kernel receives from curand_uniform at that
   site (dominokernel.cu:14-15). */
RT_API rt_status rt_domino_mtgp_draws(int32_t n_side, int64_t seed, int64_t launches, float* out);

#ifdef __cplusplus
}
#endif
#endif /* RT_TILINGS_H_ */
