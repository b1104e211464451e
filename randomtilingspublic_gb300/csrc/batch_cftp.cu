// Batched coupling from the past: many independent domino and lozenge instances in one
// persistent launch.
//
// A CTA takes the next instance from a device work queue (an atomic counter), keeps that
// instance's coupled max and min chains in shared memory and runs its whole CFTP there:
// attempt j resets the chains to the extremal tilings and runs the half-sweeps [-S T, 0)
// (S = 2 colours for dominoes, 3 for lozenges, T = first * 2^j sweeps) with fast-mode draws
// keyed by (instance seed, instance stream, half-sweep, row, column quad), then tests
// coalescence with a block reduction.  No CTA ever waits on another, so uneven instance
// sizes only change how many instances each CTA ends up taking.  The draws, rules and
// schedule are those of the single-instance fast mode, so every sample equals what
// rt_domino_cftp / rt_lozenge_cftp return for the same (seed, stream): the batch changes
// the throughput, not the samples.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "batch_cftp.cuh"
#include "domino_rules.h"
#include "rng.cuh"
#include "rt_internal.h"

namespace rt {
namespace {

constexpr int kBatchThreads = 256;

#define BT_CUDA(expr)                                                                   \
  do {                                                                                  \
    cudaError_t _e = (expr);                                                            \
    if (_e != cudaSuccess)                                                              \
      return fail(RT_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e));     \
  } while (0)

// Per-instance state of a batched launch, in which an instance's attempts are separate work
// items: the CTA that takes an instance from the queue runs its attempts in order, and CTAs
// with nothing left to take run the next attempt of an unfinished instance beside it.
struct InstState {
  int next_att;             // attempts handed out
  int best;                 // smallest attempt that coalesced (kNoAttempt: none yet)
  unsigned long long done;  // bit j: attempt j has finished and recorded its output
  int lock;                 // guards the instance's output
  int finished;             // the instance's result is final
};
constexpr int kNoAttempt = 0x7fffffff;

struct BatchArgs {
  DevInstance* inst;
  InstState* state;
  int count;
  uint8_t* tilings;
  unsigned* queue;
  unsigned* finished;  // instances whose result is final
  int* error;          // set when a bounded wait for an instance's lock gave up
  long max_spin;       // bound of that wait, and of a helper's rounds without work
};

// One domino half-sweep of colour t on both chains of an instance held whole in shared
// memory (chain c, colour k at sm + (c * 2 + k) * N * P): flips on rows [1, N-1), then the
// rebuild of the passive colour.
__device__ void domino_half_sweep(uint8_t* sm, const DevInstance& in, int t, int64_t h) {
  const RowView v{sm, (size_t)in.N * in.P, 0};
  dm_flip_rows<kBatchThreads>(v, in, t, h, 1, in.N - 1, nullptr, -1, nullptr, -1);
  __syncthreads();
  dm_rebuild_rows<kBatchThreads>(v, in, t, 1, in.N - 1);
  __syncthreads();
}

// One lozenge step of colour r on both chains (chain c, colour k at sm + (c * 3 + k) * N * P):
// rotation on every row, then the rebuild of the two other colours on rows [1, N-1).
__device__ void lozenge_step(uint8_t* sm, const DevInstance& in, int r, int64_t h, uint32_t c4, uint32_t c8) {
  const RowView v{sm, (size_t)in.N * in.P, 0};
  lz_rotate_rows<kBatchThreads>(v, in, r, h, c4, c8, 0, in.N, nullptr, -1, nullptr, -1);
  __syncthreads();
  lz_rebuild_rows<kBatchThreads>(v, in, r, 1, in.N - 1);
  __syncthreads();
}

// Runs one instance's CFTP in shared memory: tmax / tmin / out are its colour arrays in
// global or mapped host memory (loaded with volatile reads, since a serving slot is reused).
// Returns the attempts run (negative when it did not coalesce) and the last look-back.
__device__ void run_instance(uint8_t* sm, const DevInstance& in, const uint8_t* tmax, const uint8_t* tmin, uint8_t* out,
                             uint32_t lz_c4, uint32_t lz_c8, uint32_t* red, int* attempts_out, int64_t* look_out) {
  const int ncol = in.model == 0 ? 2 : 3;
  const size_t chain = (size_t)ncol * in.N * in.P;
  const uint32_t* gmax = reinterpret_cast<const uint32_t*>(tmax);
  const uint32_t* gmin = reinterpret_cast<const uint32_t*>(tmin);
  uint32_t* s32 = reinterpret_cast<uint32_t*>(sm);
  const int words = (int)(chain / 4);
  int attempts = 0;
  int64_t look = 0;
  bool done = false;
  for (int att = 0; att < in.max_attempts && !done; ++att) {
    // chain 0 starts at the min tiling, chain 1 at the max tiling
    for (int w = threadIdx.x; w < words; w += kBatchThreads) {
      s32[w] = __ldcv(gmin + w);
      s32[words + w] = __ldcv(gmax + w);
    }
    __syncthreads();
    const int64_t T = in.first_sweeps << att;
    look = ncol * T;
    for (int64_t h = -look; h < 0; ++h) {
      if (in.model == 0) domino_half_sweep(sm, in, (h & 1) ? 0 : 1, h);
      else lozenge_step(sm, in, (int)(((h % 3) + 3) % 3), h, lz_c4, lz_c8);
    }
    uint32_t differ = 0;
    for (int w = threadIdx.x; w < words; w += kBatchThreads) differ += s32[w] != s32[words + w];
    differ = block_sum<kBatchThreads>(differ, red);
    attempts = att + 1;
    done = differ == 0;
  }
  uint32_t* gout = reinterpret_cast<uint32_t*>(out);
  for (int w = threadIdx.x; w < words; w += kBatchThreads) __stcg(gout + w, s32[words + w]);
  *attempts_out = done ? attempts : -attempts;
  *look_out = look;
}

__device__ __forceinline__ int ld_volatile_i(const int* p) { return *reinterpret_cast<const volatile int*>(p); }
__device__ __forceinline__ unsigned long long ld_volatile_u64(const unsigned long long* p) {
  return *reinterpret_cast<const volatile unsigned long long*>(p);
}

// Attempt att of an instance in shared memory (chain 0 from the min tiling, chain 1 from the
// max tiling, half-sweeps [-look, 0)): 1 coalesced, 0 not, -1 abandoned because a smaller
// attempt of the instance coalesced meanwhile (checked every 256 steps).
__device__ int run_attempt(uint8_t* sm, const DevInstance& in, const InstState* st, int att, const uint8_t* tilings,
                           uint32_t lz_c4, uint32_t lz_c8, uint32_t* red, int* s_flag) {
  const int ncol = in.model == 0 ? 2 : 3;
  const int words = (int)((size_t)ncol * in.N * in.P / 4);
  const uint32_t* gmax = reinterpret_cast<const uint32_t*>(tilings + in.off_max);
  const uint32_t* gmin = reinterpret_cast<const uint32_t*>(tilings + in.off_min);
  uint32_t* s32 = reinterpret_cast<uint32_t*>(sm);
  for (int w = threadIdx.x; w < words; w += kBatchThreads) {
    s32[w] = __ldcv(gmin + w);
    s32[words + w] = __ldcv(gmax + w);
  }
  __syncthreads();
  const int64_t look = ncol * (in.first_sweeps << att);
  for (int64_t h = -look; h < 0; ++h) {
    if (in.model == 0) domino_half_sweep(sm, in, (h & 1) ? 0 : 1, h);
    else lozenge_step(sm, in, (int)(((h % 3) + 3) % 3), h, lz_c4, lz_c8);
    if (((h + look) & 255) == 255) {  // uniform over the CTA
      if (threadIdx.x == 0) *s_flag = ld_volatile_i(&st->best) < att;
      __syncthreads();
      const int stop = *s_flag;
      __syncthreads();
      if (stop) return -1;
    }
  }
  uint32_t differ = 0;
  for (int w = threadIdx.x; w < words; w += kBatchThreads) differ += s32[w] != s32[words + w];
  differ = block_sum<kBatchThreads>(differ, red);
  return differ == 0 ? 1 : 0;
}

// Records attempt att (outcome of run_attempt).  A coalesced attempt smaller than any
// recorded one, or the last attempt while none has coalesced, writes its top chain as the
// instance's output under the instance's lock.  The CTA whose record completes the instance
// (a coalesced attempt and every smaller one finished, or every attempt finished) writes the
// attempt count and the look-back: the result is that of running the attempts in order.
__device__ void record_attempt(uint8_t* sm, DevInstance* g, const DevInstance& in, InstState* st, int att, int outcome,
                               uint8_t* tilings, const BatchArgs& a, int* s_flag) {
  const int ncol = in.model == 0 ? 2 : 3;
  const int words = (int)((size_t)ncol * in.N * in.P / 4);
  if (outcome == 1 || (outcome == 0 && att == in.max_attempts - 1)) {
    if (threadIdx.x == 0) {
      int write = 0;
      long it = 0;
      bool locked = true;
      while (atomicCAS(&st->lock, 0, 1) != 0) {
        if (++it > a.max_spin) {
          atomicExch(a.error, 1);
          locked = false;
          break;
        }
      }
      if (locked) {
        __threadfence();
        const int best = ld_volatile_i(&st->best);
        write = outcome == 1 ? att < best : best == kNoAttempt;
        if (!write) atomicExch(&st->lock, 0);
      }
      *s_flag = write;
    }
    __syncthreads();
    if (*s_flag) {
      const uint32_t* s32 = reinterpret_cast<const uint32_t*>(sm);
      uint32_t* gout = reinterpret_cast<uint32_t*>(tilings + in.off_out);
      for (int w = threadIdx.x; w < words; w += kBatchThreads) __stcg(gout + w, s32[words + w]);
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0) {
        if (outcome == 1) atomicExch(&st->best, att);
        __threadfence();
        atomicExch(&st->lock, 0);
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned long long bit = 1ull << att;
    const unsigned long long done = atomicOr(&st->done, bit) | bit;
    const int best = ld_volatile_i(&st->best);
    int attempts = 0, last = -1;
    if (best != kNoAttempt) {
      const unsigned long long need = (2ull << best) - 1;  // attempts 0 .. best (best < 40)
      if ((done & need) == need) attempts = best + 1, last = best;
    } else {
      const unsigned long long all = in.max_attempts >= 64 ? ~0ull : ((1ull << in.max_attempts) - 1);
      if ((done & all) == all) attempts = -in.max_attempts, last = in.max_attempts - 1;
    }
    if (last >= 0 && atomicCAS(&st->finished, 0, 1) == 0) {
      g->attempts = attempts;
      g->final_half_sweeps = ncol * (in.first_sweeps << last);
      __threadfence();
      atomicAdd(a.finished, 1u);
    }
  }
  __syncthreads();
}

// Claims the next attempt of an instance if it is below limit (compare-and-swap, so that an
// attempt handed out is always run); -1 otherwise.
__device__ int claim_attempt(InstState* st, int limit) {
  int cur = ld_volatile_i(&st->next_att);
  while (cur < limit) {
    const int prev = atomicCAS(&st->next_att, cur, cur + 1);
    if (prev == cur) return cur;
    cur = prev;
  }
  return -1;
}

// Attempts an instance's owner may still take: below max_attempts and below any attempt
// that coalesced.  Helpers may run up to kSpeculate attempts beyond the smallest unfinished
// one (attempt j costs 2^j units, so the deepest attempt in flight is most of the work left).
constexpr int kSpeculate = 3;
__device__ int owner_limit(const DevInstance& in, const InstState* st) {
  return min(in.max_attempts, ld_volatile_i(&st->best));
}
__device__ int helper_limit(const DevInstance& in, const InstState* st) {
  const unsigned long long done = ld_volatile_u64(&st->done);
  const int lowest_unfinished = __ffsll((long long)~done) - 1;  // done < all-ones: attempts are below 64
  return min(owner_limit(in, st), lowest_unfinished + 1 + kSpeculate);
}

__global__ void __launch_bounds__(kBatchThreads, 4) k_batch_cftp(BatchArgs a, uint32_t lz_c4, uint32_t lz_c8) {
  extern __shared__ __align__(16) uint8_t sm[];
  __shared__ DevInstance s_in;
  __shared__ int s_idx, s_att, s_flag, s_pick;
  __shared__ uint32_t red[kBatchThreads / 32];
  int own = -1;            // the instance this CTA took from the queue (thread 0's view)
  bool drained = false;
  long idle_rounds = 0;
  for (;;) {
    __syncthreads();  // every thread has read the previous round's shared picks
    if (threadIdx.x == 0) {
      int idx = -1, att = -1;
      if (own >= 0) {
        att = claim_attempt(&a.state[own], owner_limit(a.inst[own], &a.state[own]));
        if (att >= 0) idx = own;
        else own = -1;
      }
      while (idx < 0 && !drained) {
        const int q = (int)atomicAdd(a.queue, 1u);
        if (q >= a.count) {
          drained = true;
          break;
        }
        att = claim_attempt(&a.state[q], owner_limit(a.inst[q], &a.state[q]));
        if (att >= 0) idx = own = q;
      }
      s_idx = idx;
      s_att = att;
      s_pick = drained && idx < 0 ? (ld_volatile_i(reinterpret_cast<const int*>(a.finished)) < a.count ? 1 : 2) : 0;
    }
    __syncthreads();
    if (s_pick == 2) break;  // every instance is final
    if (s_pick == 1) {
      // Help: the CTA scans the unfinished instances that are under way for an attempt to take.
      if (threadIdx.x == 0) s_idx = kNoAttempt;
      __syncthreads();
      const int start = (int)((blockIdx.x * 2654435761u) % (unsigned)a.count);
      for (int k = threadIdx.x; k < a.count; k += kBatchThreads) {
        const int i = (start + k) % a.count;
        const InstState* st = &a.state[i];
        if (ld_volatile_i(&st->finished) || ld_volatile_i(&st->next_att) == 0) continue;
        if (ld_volatile_i(&st->next_att) < helper_limit(a.inst[i], st)) atomicMin(&s_idx, k);
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        int idx = -1, att = -1;
        if (s_idx != kNoAttempt) {
          const int i = (start + s_idx) % a.count;
          att = claim_attempt(&a.state[i], helper_limit(a.inst[i], &a.state[i]));
          if (att >= 0) idx = i;
        }
        if (idx < 0) {
          // Nothing to take now: wait and rescan.  A helper that has waited long leaves (the
          // owners finish their instances on their own, so this bounds the wait and changes
          // no result).
          if (++idle_rounds > a.max_spin) s_pick = 2;
          else __nanosleep(8000);
        }
        s_idx = idx;
        s_att = att;
      }
      __syncthreads();
      if (s_pick == 2) break;
      if (s_idx < 0) continue;
    }
    const int idx = s_idx, att = s_att;
    DevInstance* g = &a.inst[idx];
    if (threadIdx.x == 0) s_in = *g;  // read by every thread from shared memory
    __syncthreads();
    const DevInstance& in = s_in;
    const int outcome = run_attempt(sm, in, &a.state[idx], att, a.tilings, lz_c4, lz_c8, red, &s_flag);
    record_attempt(sm, g, in, &a.state[idx], att, outcome, a.tilings, a, &s_flag);
  }
}

// ---- serving: continuous batching on a persistent kernel ------------------------------------
// Shared with the host in pinned, device-mapped memory.
struct ServeRing {
  uint64_t tail;       // requests published by the host (release store after the slot is written)
  uint32_t shutdown;   // host asks the kernel to leave
  uint32_t pad;
};

struct ServeArgs {
  ServeRing* ring;             // mapped host memory
  DevInstance* desc;           // [slots], mapped host memory
  uint8_t* data;               // [slots][slot_bytes], mapped host memory
  uint64_t* done;              // [slots], mapped host memory: ticket + 1 once finished
  unsigned long long* head;    // device memory: tickets claimed so far
  int slots;
  size_t slot_bytes;
  long idle_polls;             // polls without work before a CTA leaves
};

__device__ __forceinline__ uint64_t ld_acquire_sys(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_sys(uint64_t* p, uint64_t v) {
  asm volatile("st.release.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Each CTA claims the next published ticket (compare-and-swap on the device head, only
// when head < tail, so an idle CTA never takes a ticket it will not serve), runs that
// request's CFTP and releases its done word.  A CTA leaves after idle_polls polls without
// work or when the host sets shutdown; the host relaunches the kernel when it finds
// published work and no kernel running.
__global__ void __launch_bounds__(kBatchThreads) k_serve(ServeArgs a, uint32_t lz_c4, uint32_t lz_c8) {
  extern __shared__ __align__(16) uint8_t sm[];
  __shared__ long long s_ticket;
  __shared__ uint32_t red[kBatchThreads / 32];
  __shared__ DevInstance s_in;
  for (;;) {
    if (threadIdx.x == 0) {
      long long claimed = -1;
      long polls = 0;
      while (true) {
        if (*(volatile uint32_t*)&a.ring->shutdown) break;
        const uint64_t tail = ld_acquire_sys(&a.ring->tail);
        const unsigned long long h = *(volatile unsigned long long*)a.head;
        if (h < tail) {
          if (atomicCAS(a.head, h, h + 1) == h) {
            claimed = (long long)h;
            break;
          }
          continue;
        }
        if (++polls > a.idle_polls) break;
        __nanosleep(256);
      }
      s_ticket = claimed;
    }
    __syncthreads();
    const long long ticket = s_ticket;
    __syncthreads();
    if (ticket < 0) break;
    const int slot = (int)(ticket % a.slots);
    if (threadIdx.x < (int)(sizeof(DevInstance) / 4))  // the request, into shared memory
      reinterpret_cast<uint32_t*>(&s_in)[threadIdx.x] =
          reinterpret_cast<const volatile uint32_t*>(a.desc + slot)[threadIdx.x];
    __syncthreads();
    const DevInstance& in = s_in;
    uint8_t* base = a.data + (size_t)slot * a.slot_bytes;
    int att;
    int64_t look;
    run_instance(sm, in, base + in.off_max, base + in.off_min, base + in.off_out, lz_c4, lz_c8, red, &att, &look);
    __threadfence_system();
    __syncthreads();
    if (threadIdx.x == 0) {
      volatile DevInstance* d = a.desc + slot;
      d->attempts = att;
      d->final_half_sweeps = look;
      __threadfence_system();
      st_release_sys(a.done + slot, (uint64_t)ticket + 1);
    }
    __syncthreads();
  }
}

// Packs an instance request into a DevInstance and its colour-split extremal tilings.
rt_status pack_instance(const rt_cftp_instance& x, DevInstance* d, size_t* chain_bytes) {
  if (!x.tmax || !x.tmin) return fail(RT_ERR_INVALID_ARGUMENT, "cftp instance: NULL tiling");
  if (x.first_steps < 1 || x.max_attempts < 1 || x.max_attempts > 40)
    return fail(RT_ERR_INVALID_ARGUMENT, "cftp instance: first_steps >= 1 and 1 <= max_attempts <= 40");
  if (x.stream >= 65536u) return fail(RT_ERR_INVALID_ARGUMENT, "cftp instance: stream must be < 65536");
  std::memset(d, 0, sizeof *d);
  d->model = x.model;
  d->N = x.n_side;
  if (x.model == RT_MODEL_DOMINO) {
    if (x.n_side < 6 || x.n_side % 2) return fail(RT_ERR_INVALID_ARGUMENT, "cftp instance: domino side must be even >= 6");
    if (x.rule != RT_DOMINO_CFTP && x.rule != RT_DOMINO_CFTP_TWOPERIODIC)
      return fail(RT_ERR_INVALID_ARGUMENT, "cftp instance: domino instances need a monotone rule");
    DmRule r;
    const char* err = nullptr;
    if (!dm_rule_build(x.rule, RT_RNG_FAST, x.weight_a, x.weight_b, &r, &err)) return fail(RT_ERR_INVALID_ARGUMENT, err);
    std::memcpy(d->lo_up, r.lo_up, sizeof r.lo_up);
    std::memcpy(d->w_up, r.w_up, sizeof r.w_up);
    std::memcpy(d->lo_dn, r.lo_dn, sizeof r.lo_dn);
    std::memcpy(d->w_dn, r.w_dn, sizeof r.w_dn);
    d->cols = x.n_side / 2 - 1;
    d->P = ((x.n_side / 2) + 15) / 16 * 16;
  } else if (x.model == RT_MODEL_LOZENGE) {
    if (x.n_side < 9 || x.n_side % 3)
      return fail(RT_ERR_INVALID_ARGUMENT, "cftp instance: lozenge side must be a multiple of 3 >= 9");
    d->cols = x.n_side / 3;
    d->P = ((x.n_side / 3) + 15) / 16 * 16;
  } else {
    return fail(RT_ERR_INVALID_ARGUMENT, "cftp instance: model must be RT_MODEL_DOMINO or RT_MODEL_LOZENGE");
  }
  d->seed = x.seed;
  d->stream = x.stream;
  d->max_attempts = x.max_attempts;
  d->first_sweeps = x.first_steps;
  *chain_bytes = (size_t)(x.model == RT_MODEL_DOMINO ? 2 : 3) * d->N * d->P;
  return RT_OK;
}

// Colour split of an N x N tiling into ncol arrays of N x P bytes at dst.
rt_status split_into(const int32_t* t, const DevInstance& d, uint8_t* dst) {
  const int N = d.N, ncol = d.model == RT_MODEL_DOMINO ? 2 : 3;
  const size_t plane = (size_t)N * d.P;
  std::memset(dst, 0, plane * ncol);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      const int32_t v = t[(size_t)i * N + j];
      if ((uint32_t)v > 63u) return fail(RT_ERR_INVALID_ARGUMENT, "cftp instance: tiling values out of range");
      const int c = ncol == 2 ? (((i + j) & 1) == 0 ? 1 : 0) : ((j - i) % 3 + 3) % 3;
      dst[(size_t)c * plane + (size_t)i * d.P + (ncol == 2 ? j / 2 : j / 3)] = (uint8_t)v;
    }
  return RT_OK;
}

// The split for the batch's host threads: false when a value is out of range.
bool split_ok(const int32_t* t, const DevInstance& d, uint8_t* dst) {
  const int N = d.N, ncol = d.model == RT_MODEL_DOMINO ? 2 : 3;
  const size_t plane = (size_t)N * d.P;
  std::memset(dst, 0, plane * ncol);
  for (int i = 0; i < N; ++i) {
    const int32_t* row = t + (size_t)i * N;
    if (ncol == 2) {
      uint8_t* b = dst + (size_t)i * d.P;  // black (i + j even) in plane 1, white in plane 0
      for (int j = 0; j < N; ++j) {
        const int32_t v = row[j];
        if ((uint32_t)v > 63u) return false;
        b[(((i + j) & 1) == 0 ? plane : 0) + (size_t)(j >> 1)] = (uint8_t)v;
      }
    } else {
      for (int j = 0; j < N; ++j) {
        const int32_t v = row[j];
        if ((uint32_t)v > 63u) return false;
        const int c = ((j - i) % 3 + 3) % 3;
        dst[(size_t)c * plane + (size_t)i * d.P + j / 3] = (uint8_t)v;
      }
    }
  }
  return true;
}

size_t chain_bytes_of(const DevInstance& d) { return (size_t)(d.model == RT_MODEL_DOMINO ? 2 : 3) * d.N * d.P; }

// Runs `work` (which takes items off a shared counter) on up to 32 host threads, fewer for
// few items.
template <class F>
void run_on_host_threads(F work, size_t items) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const unsigned n = (unsigned)std::min<size_t>(std::min(32u, hw), std::max<size_t>(1, items / 4));
  std::vector<std::thread> pool;
  for (unsigned k = 1; k < n; ++k) pool.emplace_back(work);
  work();
  for (std::thread& th : pool) th.join();
}

void merge_from(const uint8_t* src, const DevInstance& d, int32_t* t) {
  const int N = d.N, ncol = d.model == RT_MODEL_DOMINO ? 2 : 3;
  const size_t plane = (size_t)N * d.P;
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      const int c = ncol == 2 ? (((i + j) & 1) == 0 ? 1 : 0) : ((j - i) % 3 + 3) % 3;
      t[(size_t)i * N + j] = src[(size_t)c * plane + (size_t)i * d.P + (ncol == 2 ? j / 2 : j / 3)];
    }
}

uint32_t lz_cut(double p) { return (uint32_t)std::ceil(p * 4294967296.0); }

}  // namespace
}  // namespace rt

using namespace rt;

extern "C" {

RT_API rt_status rt_cftp_batch(rt_cftp_instance* inst, int32_t count, void* cuda_stream, rt_batch_stats* stats) {
  clear_error();
  if (!inst || count < 1) return fail(RT_ERR_INVALID_ARGUMENT, "cftp_batch: need at least one instance");
  int dev = 0, sms = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return fail(RT_ERR_CUDA, "no CUDA device: the sweep has no CPU fallback");
  }
  BT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  BT_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  // Host side: validate every instance and sort it by where it runs.  Instances whose two
  // chains fit one CTA's shared memory go to the one-CTA persistent kernel; larger ones to the
  // cluster kernel, grouped by cluster size (one launch per size); instances too large for a
  // 16-CTA cluster run one by one through the single-instance entry points.  All three draw
  // the same (seed, stream, half-sweep) keyed randomness and so return the same samples.
  const size_t smem_limit = (size_t)optin - 1024;
  std::vector<DevInstance> dv;  // packed instances: the one-CTA ones, then the groups in order
  std::vector<int> packed_idx, large_idx, csize((size_t)count, 0);
  std::vector<DevInstance> all((size_t)count);
  size_t smem_max = 0;
  int n_small = 0;
  for (int k = 0; k < count; ++k) {
    const rt_cftp_instance& x = inst[k];
    if (!x.out) return fail(RT_ERR_INVALID_ARGUMENT, "cftp_batch: NULL output in instance");
    size_t chain = 0;
    if (rt_status st = pack_instance(x, &all[(size_t)k], &chain)) return st;
    if (2 * chain <= smem_limit) {
      smem_max = std::max(smem_max, 2 * chain);
      packed_idx.push_back(k);
      ++n_small;
    } else {
      csize[(size_t)k] = cluster_size_for(all[(size_t)k], smem_limit);
      if (csize[(size_t)k] == 0) large_idx.push_back(k);
    }
  }
  std::vector<ClusterGroup> groups;
  for (int C = 2; C <= 16; ++C) {
    ClusterGroup g;
    g.C = C;
    for (int k = 0; k < count; ++k)
      if (csize[(size_t)k] == C) {
        g.smem = std::max(g.smem, cluster_smem_bytes(all[(size_t)k], C));
        g.members.push_back(k);
      }
    if (g.members.empty()) continue;
    const int cap = cluster_capacity(C, g.smem);
    if (cap < 1) {  // no such cluster fits the device: the single-instance path
      large_idx.insert(large_idx.end(), g.members.begin(), g.members.end());
      continue;
    }
    g.clusters = std::min((int)g.members.size(), cap);
    packed_idx.insert(packed_idx.end(), g.members.begin(), g.members.end());
    groups.push_back(g);
  }
  std::sort(large_idx.begin(), large_idx.end());
  // One tiling buffer: every packed instance's max and min chains, then every output chain
  // (so that the copy back is one contiguous region of the outputs alone).
  size_t bytes_in = 0, bytes = 0;
  for (int k : packed_idx) bytes_in += 2 * chain_bytes_of(all[(size_t)k]);
  bytes = bytes_in;
  for (int k : packed_idx) {
    DevInstance d = all[(size_t)k];
    const size_t chain = chain_bytes_of(d);
    d.off_max = (int64_t)(dv.empty() ? 0 : dv.back().off_min + chain_bytes_of(dv.back()));
    d.off_min = d.off_max + (int64_t)chain;
    d.off_out = (int64_t)bytes;
    bytes += chain;
    dv.push_back(d);
  }
  // The colour splits of all instances, on the host's cores (the staging buffer is not
  // zero-filled first: each split writes its whole region).
  std::unique_ptr<uint8_t[]> host_buf(new uint8_t[std::max<size_t>(bytes, 1)]);
  uint8_t* const host = host_buf.get();
  {
    std::atomic<int> next{0}, bad{0};
    auto work = [&] {
      for (int s2 = next++; s2 < (int)dv.size(); s2 = next++) {
        const rt_cftp_instance& x = inst[packed_idx[(size_t)s2]];
        if (!split_ok(x.tmax, dv[(size_t)s2], host + dv[(size_t)s2].off_max) ||
            !split_ok(x.tmin, dv[(size_t)s2], host + dv[(size_t)s2].off_min))
          bad = 1;
      }
    };
    run_on_host_threads(work, dv.size());
    if (bad) return fail(RT_ERR_INVALID_ARGUMENT, "cftp instance: tiling values out of range");
  }
  for (int k : large_idx)
    for (const int32_t* t : {inst[k].tmax, inst[k].tmin})
      for (size_t v = 0; v < (size_t)inst[k].n_side * inst[k].n_side; ++v)
        if ((uint32_t)t[v] > 63u) return fail(RT_ERR_INVALID_ARGUMENT, "cftp_batch: tiling values out of range");
  cudaStream_t stream = (cudaStream_t)cuda_stream;
  const int n_packed = (int)dv.size();
  const int nq = 3 + (int)groups.size();  // [queue, finished, error, one queue per cluster group]
  uint8_t* d_tilings = nullptr;
  DevInstance* d_inst = nullptr;
  unsigned* d_queue = nullptr;
  InstState* d_state = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  rt_status status = RT_OK;
  int coalesced = 0, grid = 0;
  double seconds = 0.0;
  do {
    if (n_packed == 0) break;
    if ((status = dev_alloc(&d_tilings, bytes, stream)) != RT_OK ||
        (status = dev_alloc(&d_inst, dv.size() * sizeof(DevInstance), stream)) != RT_OK ||
        (status = dev_alloc(&d_queue, nq * sizeof(unsigned), stream)) != RT_OK ||
        (status = dev_alloc(&d_state, (size_t)std::max(1, n_small) * sizeof(InstState), stream)) != RT_OK)
      break;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaMemcpyAsync(d_tilings, host, bytes_in, cudaMemcpyHostToDevice, stream);
    cudaMemsetAsync(d_tilings + bytes_in, 0, bytes - bytes_in, stream);
    cudaMemcpyAsync(d_inst, dv.data(), dv.size() * sizeof(DevInstance), cudaMemcpyHostToDevice, stream);
    cudaMemsetAsync(d_queue, 0, nq * sizeof(unsigned), stream);
    std::vector<InstState> st0((size_t)std::max(1, n_small));
    for (InstState& x : st0) {
      std::memset(&x, 0, sizeof x);
      x.best = kNoAttempt;
    }
    cudaMemcpyAsync(d_state, st0.data(), st0.size() * sizeof(InstState), cudaMemcpyHostToDevice, stream);
    const uint32_t c4 = (uint32_t)std::ceil(0.4 * 4294967296.0), c8 = (uint32_t)std::ceil(0.8 * 4294967296.0);
    cudaEventRecord(e0, stream);
    if (n_small > 0) {
      cudaFuncSetAttribute(k_batch_cftp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max);
      int per_sm = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_cftp, kBatchThreads, smem_max);
      grid = std::max(1, std::min(n_small, std::max(1, per_sm) * sms));
      BatchArgs ba{d_inst, d_state, n_small, d_tilings, d_queue, d_queue + 1, reinterpret_cast<int*>(d_queue + 2),
                   1L << 24};
      k_batch_cftp<<<grid, kBatchThreads, smem_max, stream>>>(ba, c4, c8);
      cudaError_t le = cudaGetLastError();
      if (le != cudaSuccess) {
        status = fail(RT_ERR_CUDA, std::string("cftp_batch launch: ") + cudaGetErrorString(le));
        break;
      }
    }
    int first = n_small;
    for (size_t gi = 0; gi < groups.size() && status == RT_OK; ++gi) {
      const int n = (int)groups[gi].members.size();
      status = launch_cluster_group(groups[gi], d_inst + first, n, d_tilings, d_queue + 3 + gi, c4, c8, stream);
      grid += groups[gi].C * groups[gi].clusters;
      first += n;
    }
    if (status != RT_OK) break;
    cudaEventRecord(e1, stream);
    cudaMemcpyAsync(host + bytes_in, d_tilings + bytes_in, bytes - bytes_in, cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(dv.data(), d_inst, dv.size() * sizeof(DevInstance), cudaMemcpyDeviceToHost, stream);
    unsigned err_word = 0;
    cudaMemcpyAsync(&err_word, d_queue + 2, sizeof err_word, cudaMemcpyDeviceToHost, stream);
    cudaError_t se = cudaStreamSynchronize(stream);
    if (se != cudaSuccess) {
      status = fail(RT_ERR_CUDA, std::string("cftp_batch: ") + cudaGetErrorString(se));
      break;
    }
    if (err_word) {
      status = fail(RT_ERR_TIMEOUT, "cftp_batch: a bounded wait for an instance's output lock gave up");
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    seconds += ms * 1e-3;
    std::atomic<int> next{0};
    run_on_host_threads(
        [&] {
          for (int s2 = next++; s2 < n_packed; s2 = next++)
            merge_from(host + dv[(size_t)s2].off_out, dv[(size_t)s2], inst[packed_idx[(size_t)s2]].out);
        },
        (size_t)n_packed);
    for (int s2 = 0; s2 < n_packed; ++s2) {
      rt_cftp_instance& x = inst[packed_idx[(size_t)s2]];
      x.attempts = dv[(size_t)s2].attempts;
      x.final_steps = dv[(size_t)s2].final_half_sweeps;
      coalesced += dv[(size_t)s2].attempts > 0;
    }
  } while (false);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  for (void* ptr : {(void*)d_tilings, (void*)d_inst, (void*)d_queue, (void*)d_state})
    if (ptr) dev_free(ptr, stream);
  if (status != RT_OK) return status;
  // Instances too large for a cluster: the single-instance path (the resident engine or the
  // per-half-sweep kernels), one at a time on the same stream.
  for (int k : large_idx) {
    rt_cftp_instance& x = inst[k];
    rt_walk_opts o;
    rt_walk_opts_default(&o);
    o.rng_mode = RT_RNG_FAST;
    o.fast_stream = x.stream;
    o.cuda_stream = cuda_stream;
    rt_cftp_stats st;
    std::memset(&st, 0, sizeof st);
    rt_status r;
    if (x.model == RT_MODEL_DOMINO) {
      o.rule = x.rule;
      o.weight_a = x.weight_a;
      o.weight_b = x.weight_b;
      r = rt_domino_cftp(x.tmax, x.tmin, x.n_side, (int64_t)x.seed, x.first_steps, 1, x.max_attempts, &o, x.out, &st);
    } else {
      o.rule = RT_LOZENGE_UNIFORM;
      r = rt_lozenge_cftp(x.tmax, x.tmin, x.n_side, (int64_t)x.seed, x.first_steps, 1, x.max_attempts, &o, x.out, &st);
    }
    if (r != RT_OK && r != RT_ERR_NOT_COALESCED) return r;  // the entry point has set the message
    x.attempts = r == RT_OK ? st.attempts : -st.attempts;
    x.final_steps = st.final_steps;
    coalesced += r == RT_OK;
    seconds += st.seconds;
  }
  if (stats) {
    stats->instances = count;
    stats->coalesced = coalesced;
    stats->seconds = seconds;
    stats->ctas = grid;
    stats->cluster_instances = n_packed - n_small;
    stats->single_instances = (int32_t)large_idx.size();
  }
  if (coalesced != count) return fail(RT_ERR_NOT_COALESCED, "cftp_batch: some instances did not coalesce");
  return RT_OK;
}

}  // extern "C"

// ---- server (host side) ----------------------------------------------------------------------
struct rt_server {
  int slots = 0, max_side = 0;
  size_t slot_bytes = 0, smem = 0;
  int64_t budget = 0, in_flight_bytes = 0;
  long idle_polls = 0;
  ServeRing* ring = nullptr;           // pinned + mapped
  DevInstance* desc = nullptr;
  uint8_t* data = nullptr;
  uint64_t* done = nullptr;
  ServeRing* d_ring = nullptr;         // device views of the mapped memory
  DevInstance* d_desc = nullptr;
  uint8_t* d_data = nullptr;
  uint64_t* d_done = nullptr;
  unsigned long long* d_head = nullptr;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaEvent_t ev_exit = nullptr;
  bool launched = false;
  int grid = 0;
  int64_t next_ticket = 0;
  std::vector<int64_t> owner;          // ticket held by each slot, -1 when free
  std::vector<int64_t> footprint;

  // Releases whatever was set up, so that a create that fails half-way leaks nothing: a
  // running serving kernel is told to leave and waited for first.
  ~rt_server() {
    if (ring) __atomic_store_n(&ring->shutdown, 1u, __ATOMIC_RELEASE);
    if (stream) cudaStreamSynchronize(stream);
    if (ev_exit) cudaEventDestroy(ev_exit);
    if (own_stream && stream) cudaStreamDestroy(stream);
    if (d_head) cudaFree(d_head);
    for (void* p : {(void*)ring, (void*)desc, (void*)data, (void*)done})
      if (p) cudaFreeHost(p);
  }
};

static rt_status server_launch(rt_server* s) {
  ServeArgs a{s->d_ring, s->d_desc, s->d_data, s->d_done, s->d_head, s->slots, s->slot_bytes, s->idle_polls};
  k_serve<<<s->grid, kBatchThreads, s->smem, s->stream>>>(a, lz_cut(0.4), lz_cut(0.8));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(RT_ERR_CUDA, std::string("server launch: ") + cudaGetErrorString(e));
  BT_CUDA(cudaEventRecord(s->ev_exit, s->stream));
  s->launched = true;
  return RT_OK;
}

// Relaunches the persistent kernel when none is running (it leaves after idle_polls polls).
static rt_status server_ensure_running(rt_server* s) {
  if (s->launched) {
    cudaError_t q = cudaEventQuery(s->ev_exit);
    if (q == cudaErrorNotReady) return RT_OK;
    if (q != cudaSuccess) return fail(RT_ERR_CUDA, std::string("server kernel: ") + cudaGetErrorString(q));
  }
  return server_launch(s);
}

extern "C" {

RT_API rt_status rt_server_create(const rt_server_opts* o, rt_server** out) {
  clear_error();
  if (!o || !out) return fail(RT_ERR_INVALID_ARGUMENT, "server_create: NULL argument");
  *out = nullptr;
  if (o->slots < 1 || o->slots > (1 << 20) || o->max_side < 9 || o->max_side > 330 || o->memory_budget_bytes < 1)
    return fail(RT_ERR_INVALID_ARGUMENT, "server_create: 1 <= slots <= 2^20, 9 <= max_side <= 330, budget > 0");
  int dev = 0, sms = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return fail(RT_ERR_CUDA, "no CUDA device: the sweep has no CPU fallback");
  }
  BT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  BT_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  auto s = std::make_unique<rt_server>();
  s->slots = o->slots;
  s->max_side = o->max_side;
  const size_t pd = (size_t)((o->max_side / 2) + 15) / 16 * 16, pl = (size_t)((o->max_side / 3) + 15) / 16 * 16;
  const size_t chain = std::max((size_t)2 * o->max_side * pd, (size_t)3 * o->max_side * pl);
  s->slot_bytes = (3 * chain + 255) / 256 * 256;
  s->smem = 2 * chain;
  if (s->smem > (size_t)optin - 1024) return fail(RT_ERR_INVALID_ARGUMENT, "server_create: max_side too large for one CTA");
  s->budget = o->memory_budget_bytes;
  s->idle_polls = (long)std::max(1.0, (o->idle_seconds > 0 ? o->idle_seconds : 0.25) * 2.0e6);
  BT_CUDA(cudaHostAlloc(&s->ring, sizeof(ServeRing), cudaHostAllocMapped));
  BT_CUDA(cudaHostAlloc(&s->desc, sizeof(DevInstance) * s->slots, cudaHostAllocMapped));
  BT_CUDA(cudaHostAlloc(&s->data, s->slot_bytes * s->slots, cudaHostAllocMapped));
  BT_CUDA(cudaHostAlloc(&s->done, sizeof(uint64_t) * s->slots, cudaHostAllocMapped));
  std::memset(s->ring, 0, sizeof(ServeRing));
  std::memset(s->done, 0, sizeof(uint64_t) * s->slots);
  BT_CUDA(cudaHostGetDevicePointer((void**)&s->d_ring, s->ring, 0));
  BT_CUDA(cudaHostGetDevicePointer((void**)&s->d_desc, s->desc, 0));
  BT_CUDA(cudaHostGetDevicePointer((void**)&s->d_data, s->data, 0));
  BT_CUDA(cudaHostGetDevicePointer((void**)&s->d_done, s->done, 0));
  BT_CUDA(cudaMalloc(&s->d_head, sizeof(unsigned long long)));
  BT_CUDA(cudaMemset(s->d_head, 0, sizeof(unsigned long long)));
  if (o->cuda_stream) {
    s->stream = (cudaStream_t)o->cuda_stream;
  } else {
    BT_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    s->own_stream = true;
  }
  BT_CUDA(cudaEventCreateWithFlags(&s->ev_exit, cudaEventDisableTiming));
  BT_CUDA(cudaFuncSetAttribute(k_serve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->smem));
  int per_sm = 0;
  BT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_serve, kBatchThreads, s->smem));
  s->grid = std::max(1, per_sm) * sms;
  s->owner.assign(s->slots, -1);
  s->footprint.assign(s->slots, 0);
  *out = s.release();
  return RT_OK;
}

RT_API rt_status rt_server_submit(rt_server* s, const rt_cftp_instance* req, int64_t* ticket) {
  clear_error();
  if (!s || !req || !ticket) return fail(RT_ERR_INVALID_ARGUMENT, "server_submit: NULL argument");
  if (req->n_side > s->max_side) return fail(RT_ERR_INVALID_ARGUMENT, "server_submit: tiling side above the server's max_side");
  DevInstance d;
  size_t chain = 0;
  if (rt_status st = pack_instance(*req, &d, &chain)) return st;
  const int64_t foot = (int64_t)(3 * chain);  // extremal tilings + result staged for the request
  const int64_t t = s->next_ticket;
  const int slot = (int)(t % s->slots);
  if (s->owner[slot] >= 0) return fail(RT_ERR_BUSY, "server_submit: no free slot (collect finished requests first)");
  if (s->in_flight_bytes + foot > s->budget) return fail(RT_ERR_BUSY, "server_submit: memory budget reached");
  uint8_t* base = s->data + (size_t)slot * s->slot_bytes;
  d.off_max = 0;
  d.off_min = (int64_t)chain;
  d.off_out = (int64_t)(2 * chain);
  if (rt_status st = split_into(req->tmax, d, base)) return st;
  if (rt_status st = split_into(req->tmin, d, base + chain)) return st;
  std::memcpy(s->desc + slot, &d, sizeof d);
  s->owner[slot] = t;
  s->footprint[slot] = foot;
  s->in_flight_bytes += foot;
  s->next_ticket = t + 1;
  __atomic_store_n(&s->ring->tail, (uint64_t)(t + 1), __ATOMIC_RELEASE);
  *ticket = t;
  return server_ensure_running(s);
}

RT_API rt_status rt_server_poll(rt_server* s, int64_t ticket, int32_t* done) {
  clear_error();
  if (!s || !done || ticket < 0 || ticket >= s->next_ticket) return fail(RT_ERR_INVALID_ARGUMENT, "server_poll: bad ticket");
  const int slot = (int)(ticket % s->slots);
  if (s->owner[slot] != ticket) return fail(RT_ERR_INVALID_ARGUMENT, "server_poll: ticket already collected");
  *done = __atomic_load_n(s->done + slot, __ATOMIC_ACQUIRE) == (uint64_t)ticket + 1;
  if (!*done) return server_ensure_running(s);
  return RT_OK;
}

RT_API rt_status rt_server_wait(rt_server* s, int64_t ticket, double timeout_s, rt_cftp_instance* result) {
  clear_error();
  if (!s || !result || !result->out || ticket < 0 || ticket >= s->next_ticket)
    return fail(RT_ERR_INVALID_ARGUMENT, "server_wait: bad arguments");
  const int slot = (int)(ticket % s->slots);
  if (s->owner[slot] != ticket) return fail(RT_ERR_INVALID_ARGUMENT, "server_wait: ticket already collected");
  const auto t0 = std::chrono::steady_clock::now();
  for (int spins = 0;; ++spins) {
    if (__atomic_load_n(s->done + slot, __ATOMIC_ACQUIRE) == (uint64_t)ticket + 1) break;
    if (rt_status st = server_ensure_running(s)) return st;
    if (std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() > timeout_s)
      return fail(RT_ERR_TIMEOUT, "server_wait: request not finished within the timeout");
    if (spins > 64) std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
  DevInstance d;
  std::memcpy(&d, s->desc + slot, sizeof d);
  merge_from(s->data + (size_t)slot * s->slot_bytes + d.off_out, d, result->out);
  result->attempts = d.attempts;
  result->final_steps = d.final_half_sweeps;
  s->owner[slot] = -1;
  s->in_flight_bytes -= s->footprint[slot];
  s->footprint[slot] = 0;
  if (d.attempts < 0) return fail(RT_ERR_NOT_COALESCED, "server_wait: the request did not coalesce");
  return RT_OK;
}

RT_API rt_status rt_server_destroy(rt_server* s) {
  clear_error();
  delete s;  // the destructor stops the serving kernel and frees everything
  return RT_OK;
}

}  // extern "C"
