// pps_batch.cu -- the batched persistent form: many uneven jobs (different k,
// n and p ranges, mixed +/- sides) in one persistent walk kernel fed by a
// device work queue.
//
// A job's p range is cut into batches (contiguous sieve segments of 2^18 odd
// candidates).  Batches of many jobs fill a wave (up to WAVE_SEGS segments).
// Per wave, one fixed launch sequence -- large-prime scatter, segment sieve,
// scan, expansion, chunking, scan, persistent walk -- reads every count from
// device tables, so it is captured once as a CUDA graph and replayed for each
// wave after the wave's tables are copied in.  The walk kernel's warps pop
// chunks of CHUNK primes (all of one job, so every lane of a warp has the same
// n loop) from a device counter until the wave is exhausted.  Raw candidates
// carry their job slot; a filter launch after each wave applies each job's
// output rule.  Jobs live in device slots (parameters, prime counters), so the
// serving loop can admit and retire jobs between waves.
//
// Reference counterpart: none in one piece -- the reference runs one range per
// process (main.c:887-1266) and one kernel per n slice (pps/appcu.cu:1194-1261).
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "pps_device.cuh"
#include "pps_engine_impl.h"
#include "pps_sieve.cuh"

namespace pps {

constexpr uint32_t WAVE_SEGS = 1u << 14;        // segments per wave (2^32 odd candidates)
constexpr uint32_t BATCH_SEGS = 1u << 12;       // segments per batch
constexpr uint32_t WAVE_BATCHES = WAVE_SEGS;    // at most one batch per segment
constexpr uint32_t MAX_JOBS = 1u << 16;
constexpr int BW_THREADS = 256;
constexpr uint32_t BQ_CAP = 512;  // queued blocks per warp
constexpr uint32_t MAX_CHUNK = 8192;  // primes per work chunk, at most (a multiple of 32)

struct BJob {
  uint64_t kmin, kmax, kstep, koffset;
  uint32_t nmin, nmax, step, nsteps;
  uint32_t proth, win_hi, win_mask, qmax;
  int32_t sign;
  uint32_t chunk;  // primes per work chunk: about the same walk steps for every job
  // win_sh < 32: the small-p window, K < 2^win_sh or the low bits in win_mask
  // all zero; 32: K < (win_hi + 1) * 2^32 or the low bits in win_mask zero
  uint32_t win_sh;
  uint32_t shift_ok;  // step < 32 and pmax <= 2^(32+step): walk form 1
  uint32_t win_u;     // win_hi == 2^win_u - 1 (32: every hi word passes)
  // bound_hi < 2^32 - 1: the single-bound test (hi word <= bound_hi), exact for
  // 32-bit steps when kmax < 2^32 and p > kmax 2^43 (false-pass rate < 2^-12)
  uint32_t bound_hi;
  // sw_mask != 0: walk form 1 with test 4 (the window K < 2^s read off the step)
  uint32_t sw_mask;
  // n parts per prime (1, 2, 4, 8): each chunk of primes is walked as nsplit
  // work items, item j holding blocks [j L, (j+1) L) of the n range,
  // L = ceil(blocks / nsplit), so a long-n job's work comes in pieces of
  // about the same size as a short-n job's
  uint32_t nsplit;
};

struct BBatch {
  uint64_t lo, nbits;
  uint32_t seg0, job;
  uint32_t nq, nq_tiny, nq_seg, limit;  // limit = largest sieving prime allowed
};

struct BSeg {
  uint64_t lo;
  uint32_t bits, batch;
};

struct WaveTables {  // pinned host staging == device layout
  uint32_t nseg, nbatch, pad0, pad1;
  BSeg seg[WAVE_SEGS];
  BBatch batch[WAVE_BATCHES];
};

}  // namespace pps

using namespace pps;

struct BatchState {
  bool ready = false;
  DevBuf<uint8_t> tables;       // WaveTables
  WaveTables* h_tables = nullptr;
  DevBuf<BJob> jobs;
  DevBuf<uint32_t> bitmap;      // WAVE_SEGS * SEG_WORDS
  DevBuf<uint32_t> seg_count, seg_off, chunk_count, chunk_off, chunk_seg;
  DevBuf<uint32_t> large_items, large_off;  // per batch: large-prime work items, their prefix sums
  DevBuf<uint64_t> P, Pinv;
  DevBuf<uint64_t> tot;         // [0] primes, [1] sum, [2] chunks, [3] work counter, [4] large items
  DevBuf<unsigned long long> job_primes, job_sum;
  DevBuf<pps_hit> hits, out;
  DevBuf<uint32_t> counters;    // [0] raw, [1] survivors, [2] tuning hits, [3] large-sieve items
  DevBuf<uint64_t> qm;          // Barrett constants of the sieving primes
  const uint32_t* qm_q = nullptr;  // sieving-prime table the constants belong to
  uint32_t qm_n = 0;
  uint64_t prime_cap = 0;
  // the wave's launch sequence as two captured graphs: the sieve part (clear,
  // scatter, segment sieve, scans, expansion, chunking) and the walk, so that
  // events between the two launches time each part
  cudaGraphExec_t graph = nullptr, graph_walk = nullptr;
  cudaEvent_t ev_wave[3] = {nullptr, nullptr, nullptr};
  double sieve_ms = 0, walk_ms = 0;  // device time of the waves so far, per part
  int graph_unroll = 0;
  const uint32_t* graph_q = nullptr;  // sieving-prime table the graph was captured with
  uint32_t graph_nq = 0;
  uint32_t graph_hcap = 0, graph_qcap = 0;  // candidate and warp-queue capacities it was captured with
  cudaEvent_t copied = nullptr;
  uint32_t wave_segs = WAVE_SEGS;  // segments one wave holds (pps_engine_set_wave_segments)
  int tuned_work = 0, tuned_unroll = 0;  // walk steps per chunk (x32 lanes), walk kernel code (timed)
  int walk_code = 0;                     // the walk kernel code of the last wave (tuned or forced)
  std::vector<BJob> hjobs;               // host mirror of the device job slots
  std::vector<uint64_t> slot_pmax;       // each slot's pmax (sieving-prime bound)
  DevBuf<unsigned long long> bak_primes, bak_sum;  // slot counters before a wave
};

void drop_graphs(BatchState* b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->graph_walk) cudaGraphExecDestroy(b->graph_walk);
  b->graph = nullptr;
  b->graph_walk = nullptr;
}

void batch_state_free(pps_engine* e) {
  BatchState* b = e->batch;
  if (!b) return;
  drop_graphs(b);
  for (auto& v : b->ev_wave)
    if (v) cudaEventDestroy(v);
  if (b->copied) cudaEventDestroy(b->copied);
  if (b->h_tables) cudaFreeHost(b->h_tables);
  b->tables.release();
  b->jobs.release();
  b->bitmap.release();
  b->seg_count.release();
  b->seg_off.release();
  b->chunk_count.release();
  b->chunk_off.release();
  b->chunk_seg.release();
  b->large_items.release();
  b->large_off.release();
  b->P.release();
  b->Pinv.release();
  b->tot.release();
  b->job_primes.release();
  b->job_sum.release();
  b->hits.release();
  b->out.release();
  b->counters.release();
  b->qm.release();
  b->bak_primes.release();
  b->bak_sum.release();
  delete b;
  e->batch = nullptr;
}

namespace pps {

__device__ __forceinline__ const WaveTables* wt(const uint8_t* t) { return (const WaveTables*)t; }

constexpr uint32_t LARGE_Q_PER_ITEM = 256;  // large sieving primes per work item

// per batch: how many of the ascending sieving primes are <= its limit, and
// its number of large-prime work items (0 past the last batch)
__global__ void k_bcounts(uint8_t* tables, const uint32_t* q, uint32_t nq_all, uint32_t* large_items) {
  WaveTables* T = (WaveTables*)tables;
  for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < WAVE_BATCHES; b += gridDim.x * blockDim.x) {
    if (b >= T->nbatch) {
      large_items[b] = 0;
      continue;
    }
    BBatch& B = T->batch[b];
    uint32_t lo = 0, hi = nq_all;
    while (lo < hi) {
      const uint32_t mid = lo + (hi - lo) / 2;
      if (q[mid] <= B.limit) lo = mid + 1; else hi = mid;
    }
    B.nq = lo;
    uint32_t t = 0, s = 0;
    {
      uint32_t l2 = 0, h2 = lo;
      while (l2 < h2) {
        const uint32_t mid = l2 + (h2 - l2) / 2;
        if (q[mid] < TINY_Q_LIMIT) l2 = mid + 1; else h2 = mid;
      }
      t = l2;
      l2 = 0;
      h2 = lo;
      while (l2 < h2) {
        const uint32_t mid = l2 + (h2 - l2) / 2;
        if (q[mid] < SEG_BITS) l2 = mid + 1; else h2 = mid;
      }
      s = l2;
    }
    B.nq_tiny = t;
    B.nq_seg = s;
    large_items[b] = (lo - s + LARGE_Q_PER_ITEM - 1) / LARGE_Q_PER_ITEM;
  }
}

__device__ __forceinline__ uint64_t b_first_odd_multiple(uint64_t q, uint64_t lo) {
  uint64_t st = q * q;
  if (st < lo) {
    const uint64_t r = lo % q;
    st = r ? lo + (q - r) : lo;
    if ((st & 1ull) == 0ull) st += q;
  }
  return st;
}

// Barrett constants of the sieving primes: m = floor((2^64 - 1) / q), which is
// floor(2^64 / q) for every odd q > 1 (Barrett, CRYPTO '86).
__global__ void k_brecip(const uint32_t* q, uint32_t nq, uint64_t* m) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += gridDim.x * blockDim.x)
    m[i] = ~0ull / (uint64_t)q[i];
}

// x mod q from the Barrett constant: the estimate umulhi(x, m) is at most 2
// below floor(x / q), so at most two corrections.
__device__ __forceinline__ uint64_t b_mod(uint64_t x, uint64_t q, uint64_t m) {
  uint64_t r = x - __umul64hi(x, m) * q;
  if (r >= q) r -= q;
  if (r >= q) r -= q;
  return r;
}

// Large sieving primes (q >= SEG_BITS) into the wave bitmap.  Work items of
// LARGE_Q_PER_ITEM primes each are numbered batch by batch (item_off = prefix
// sums of the per-batch item counts) and taken in order from a device counter,
// so the GPU works on one or two batches at a time: their bitmap (at most
// 128 MB) stays in L2 while its bits are cleared.  A block's items only ever
// increase, so it finds each item's batch by galloping forward from the last one.
__global__ void k_bsieve_large(const uint8_t* tables, const uint32_t* q, const uint64_t* qm, uint32_t* bitmap,
                               const uint32_t* item_off, const uint64_t* item_total, uint32_t* item_counter) {
  __shared__ uint32_t s_item, s_batch;
  const WaveTables* T = wt(tables);
  const uint32_t nitems = (uint32_t)*item_total, nb = T->nbatch;
  uint32_t cur = 0;  // thread 0: batch of the block's last item
  for (;;) {
    if (threadIdx.x == 0) {
      const uint32_t item = atomicAdd(item_counter, 1u);
      if (item < nitems) {
        // last batch b >= cur with item_off[b] <= item
        uint32_t step = 1, lo = cur, hi = cur + 1;
        while (hi < nb && item_off[hi] <= item) {
          lo = hi;
          hi = lo + step;
          step <<= 1;
        }
        if (hi > nb) hi = nb;
        while (hi - lo > 1) {
          const uint32_t mid = lo + (hi - lo) / 2;
          if (item_off[mid] <= item) lo = mid; else hi = mid;
        }
        cur = lo;
      }
      s_item = item;
      s_batch = cur;
    }
    __syncthreads();
    const uint32_t item = s_item, bidx = s_batch;
    __syncthreads();
    if (item >= nitems) return;
    const BBatch B = T->batch[bidx];
    uint32_t* bm = bitmap + (size_t)B.seg0 * SEG_WORDS;
    const uint64_t hi = B.lo + 2ull * B.nbits;
    const uint32_t i0 = B.nq_seg + (item - item_off[bidx]) * LARGE_Q_PER_ITEM;
    const uint32_t i1 = min(B.nq, i0 + LARGE_Q_PER_ITEM);
    for (uint32_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      const uint64_t qq = q[i];
      if (qq * qq >= hi) continue;
      uint64_t st = qq * qq;
      if (st < B.lo) {
        const uint64_t r = b_mod(B.lo, qq, qm[i]);
        st = r ? B.lo + (qq - r) : B.lo;
        if ((st & 1ull) == 0ull) st += qq;
      }
      for (uint64_t j = (st - B.lo) >> 1; j < B.nbits; j += qq) atomicAnd(&bm[j >> 5], ~(1u << (j & 31u)));
    }
  }
}

// All bits set in the segments of this wave only (the large-prime scatter
// clears bits in them next); a wave of few segments does not pay for the
// whole 512 MB bitmap.
__global__ void k_bclear(const uint8_t* tables, uint32_t* bitmap) {
  const uint64_t words = (uint64_t)wt(tables)->nseg * SEG_WORDS;
  uint4* b4 = (uint4*)bitmap;
  const uint4 ones = make_uint4(0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < words / 4;
       i += (uint64_t)gridDim.x * blockDim.x)
    b4[i] = ones;
}

// The segment sieve of a wave: as k_sieve_seg (pps_kernels.cu), with the
// pre-sieve table for 3, 5, 7, 11 and 13 and Barrett reductions (qm) for the
// start offsets of the small primes.
__global__ void __launch_bounds__(SIEVE_THREADS) k_bsieve_seg(const uint8_t* tables, const uint32_t* q,
                                                              const uint64_t* qm, const uint32_t* presieve,
                                                              uint32_t* bitmap, uint32_t* seg_count) {
  __shared__ uint32_t sb[SEG_WORDS];
  __shared__ uint32_t warp_cnt[SIEVE_THREADS / 32];
  const WaveTables* T = wt(tables);
  const uint32_t seg = blockIdx.x;
  if (seg >= T->nseg) {
    if (threadIdx.x == 0) seg_count[seg] = 0;
    return;
  }
  const BSeg S = T->seg[seg];
  const BBatch B = T->batch[S.batch];
  const uint32_t bits = S.bits;
  const uint64_t seg_lo = S.lo, seg_hi = seg_lo + 2ull * bits;
  const int have_large = B.nq > B.nq_seg;
  uint32_t* gw = bitmap + (size_t)seg * SEG_WORDS;
  // pieces start above 2^32, so the pre-sieved primes never lie in a segment
  const bool pre = presieve != nullptr && B.nq_tiny >= PRESIEVE_PRIMES;
  const uint32_t xstep = (64u * SIEVE_THREADS) % PRESIEVE_MOD;
  uint32_t x = pre ? (uint32_t)((seg_lo % PRESIEVE_MOD + 64u * threadIdx.x) % PRESIEVE_MOD) : 0u;
  for (uint32_t w = threadIdx.x; w < SEG_WORDS; w += blockDim.x) {
    uint32_t v = have_large ? gw[w] : 0xffffffffu;
    if (pre) {
      v &= ~__ldg(presieve + x);
      x += xstep;
      if (x >= PRESIEVE_MOD) x -= PRESIEVE_MOD;
    }
    const uint32_t j0 = w * 32u;
    if (j0 >= bits) v = 0u;
    else if (bits - j0 < 32u) v &= (1u << (bits - j0)) - 1u;
    sb[w] = v;
  }
  __syncthreads();
  for (uint32_t i = pre ? PRESIEVE_PRIMES : 0u; i < B.nq_tiny; ++i) {
    const uint64_t qq = q[i];
    if (qq * qq >= seg_hi) break;
    const uint64_t st = b_first_odd_multiple(qq, seg_lo);
    for (uint64_t j = ((st - seg_lo) >> 1) + (uint64_t)threadIdx.x * qq; j < bits; j += (uint64_t)blockDim.x * qq)
      atomicAnd(&sb[j >> 5], ~(1u << (j & 31u)));
  }
  const uint32_t qend = B.nq_seg < B.nq ? B.nq_seg : B.nq;
  for (uint32_t i = B.nq_tiny + threadIdx.x; i < qend; i += blockDim.x) {
    const uint64_t qq = q[i];
    if (qq * qq >= seg_hi) continue;
    uint64_t st;
    if (qq * qq <= seg_lo) {  // the first odd multiple >= seg_lo, by a Barrett reduction
      const uint64_t r = b_mod(seg_lo, qq, qm[i]);
      st = r ? seg_lo + (qq - r) : seg_lo;
      if ((st & 1ull) == 0ull) st += qq;
    } else {
      st = b_first_odd_multiple(qq, seg_lo);
    }
    for (uint64_t j = (st - seg_lo) >> 1; j < bits; j += (uint32_t)qq) atomicAnd(&sb[j >> 5], ~(1u << (j & 31u)));
  }
  __syncthreads();
  uint32_t cnt = 0;
  for (uint32_t w = threadIdx.x; w < SEG_WORDS; w += blockDim.x) {
    const uint32_t v = sb[w];
    gw[w] = v;
    cnt += __popc(v);
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0) warp_cnt[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += warp_cnt[i];
    seg_count[seg] = t;
  }
}

// exclusive scan of n counts (one CTA); total into *total
__global__ void __launch_bounds__(1024) k_bscan(const uint32_t* cnt, uint32_t* off, uint32_t n, uint64_t* total) {
  __shared__ uint64_t part[1024];
  const uint32_t per = (n + blockDim.x - 1) / blockDim.x;
  const uint32_t a = threadIdx.x * per;
  const uint32_t e = a + per < n ? a + per : n;
  uint64_t s = 0;
  for (uint32_t i = a; i < e; ++i) s += cnt[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (uint32_t d = 1; d < blockDim.x; d <<= 1) {
    const uint64_t v = threadIdx.x >= d ? part[threadIdx.x - d] : 0ull;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  uint64_t run = part[threadIdx.x] - s;
  for (uint32_t i = a; i < e; ++i) {
    off[i] = (uint32_t)run;
    run += cnt[i];
  }
  if (threadIdx.x == blockDim.x - 1) *total = part[threadIdx.x];
}

__global__ void __launch_bounds__(SIEVE_THREADS) k_bexpand(const uint8_t* tables, const uint32_t* bitmap,
                                                           const uint32_t* seg_off, uint64_t* P, uint64_t* Pinv,
                                                           unsigned long long* job_primes,
                                                           unsigned long long* job_sum, uint64_t cap) {
  __shared__ ExpandShared sh;
  const WaveTables* T = wt(tables);
  const uint32_t seg = blockIdx.x;
  if (seg >= T->nseg) return;
  const BSeg S = T->seg[seg];
  const uint32_t job = T->batch[S.batch].job;
  const uint64_t sum = expand_segment<false>(bitmap + (size_t)seg * SEG_WORDS, S.lo, seg_off[seg], cap, P, Pinv,
                                             nullptr, &sh);
  if (threadIdx.x == 0) {
    atomicAdd(&job_primes[job], (unsigned long long)sh.total);
    atomicAdd(&job_sum[job], (unsigned long long)sum);
  }
}

__global__ void k_bchunks(const uint8_t* tables, const BJob* jobs, const uint32_t* seg_count,
                          uint32_t* chunk_count) {
  const WaveTables* T = wt(tables);
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < WAVE_SEGS; s += gridDim.x * blockDim.x) {
    uint32_t n = 0;
    if (s < T->nseg) {
      const BJob& J = jobs[T->batch[T->seg[s].batch].job];
      n = (seg_count[s] + J.chunk - 1) / J.chunk * J.nsplit;
    }
    chunk_count[s] = n;
  }
}

// chunk -> segment map (one CTA per segment writes its chunks' entries)
__global__ void k_bchunkmap(const uint8_t* tables, const uint32_t* chunk_count, const uint32_t* chunk_off,
                            uint32_t* chunk_seg, uint64_t map_cap) {
  const WaveTables* T = wt(tables);
  const uint32_t s = blockIdx.x;
  if (s >= T->nseg) return;
  const uint32_t c0 = chunk_off[s], n = chunk_count[s];
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
    if ((uint64_t)c0 + i < map_cap) chunk_seg[c0 + i] = s;
}

// Candidates carry their job slot in idx bits 0-30 and their side in bit 31
// (1: k*2^n+1, 0: k*2^n-1), which a twin job needs per candidate.
constexpr uint32_t SIDE_PROTH = BATCH_SIDE_PROTH;

__device__ __forceinline__ void b_record(uint32_t klo, uint32_t khi, uint32_t n, uint32_t step, uint64_t p,
                                         uint32_t tag, const BJob& J, pps_hit* hits, uint32_t* hit_count,
                                         uint32_t hit_cap) {
  const uint32_t i = klo ? (uint32_t)(__ffs(klo) - 1) : (uint32_t)(31 + __ffs(khi));
  const uint64_t k = mk64(klo, khi) >> (i & 63u);
  const bool hit = (i < step) && (k <= J.kmax) && (k >= J.kmin) && (n + i < J.nmax);
  const unsigned act = __activemask();
  const unsigned hm = __ballot_sync(act, hit);
  if (hm) {
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(hm) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(hit_count, (uint32_t)__popc(hm));
    base = __shfl_sync(act, base, leader);
    if (hit) {
      const uint32_t pos = base + (uint32_t)__popc(hm & ((1u << lane) - 1u));
      if (pos < hit_cap) {
        pps_hit h;
        h.p = p;
        h.k = k;
        h.n = n + i;
        h.idx = tag;
        hits[pos] = h;
      }
    }
  }
}

// Walk-step forms of the batched walk:
//   0  s == 32: the REDC by 2^32 without low-word carries (step_neg32);
//   1  s < 32 and p <= 2^(32+s): K' = K * 2^(32-s) (< 2^64) through the same
//      step, since (K + m p) / 2^s == (K' + m' p) / 2^32 with
//      m' = lo32(K') * (-p^-1) mod 2^32 = m * 2^(32-s);
//   2  s < 32, larger p: the shift-REDC with a wide multiply-add.
// pinv is lo32(-p^-1) for form 0 and that << (32-s) for forms 1 and 2; the
// words (pa, pb) of p are (neg_lo(p), neg_hi(p)) for forms 0 and 1 and
// (lo32(p), hi32(p)) for form 2 (b_words).
template <int FORM>
__device__ __forceinline__ void b_step(uint32_t& klo, uint32_t& khi, uint32_t pa, uint32_t pb, uint32_t pinv,
                                       uint32_t s) {
  if (FORM == 0) {
    step_neg32(klo, khi, pa, pb, pinv);
  } else if (FORM == 1) {
    step_neg32s(klo, khi, pa, pb, pinv, 32u - s);
  } else {
    step_form0<false>(klo, khi, pa, pb, pinv, s);
  }
}

template <int FORM>
__device__ __forceinline__ void b_words(uint64_t p, uint32_t* pa, uint32_t* pb) {
  *pa = FORM == 2 ? lo32(p) : neg_lo(p);
  *pb = FORM == 2 ? hi32(p) : neg_hi(p);
}

template <int FORM>
__device__ __forceinline__ uint32_t b_pinv(uint64_t ps, uint32_t s) {
  return FORM == 0 ? lo32(ps) : (lo32(ps) << (32u - s));
}

// One round: every lane walks one prime of the same job; flagged blocks of U
// steps (and the partial last block) go to the warp's queue and are re-checked
// exactly once the round's walks are done.  A twin job (TW) walks K = 2^-n, the
// -1 side's value, and tests p - K, the +1 side's, at the same step.
// Pre-test (TEST), an exact superset of the hits K = k 2^i (k < 2^kb, i < s),
// kept as a running minimum over the block:
//   0  the window: K < 2^(32+win_u), i.e. hi >> win_u == 0, or the low bits in
//      win_mask zero (a hit below the window, or with i past it);
//   1  the small-p window: K < 2^win_sh (a funnel shift) or the low bits zero;
//   2  the single bound: hi <= bound_hi (32-bit steps, p > kmax 2^43);
//   3  the window with win_u == 0 (test 0 without the shift);
//   4  walk form 1: K < 2^s, i.e. the step's own high word K >> s is zero,
//      or the low s+1-kb bits of K zero (sw_mask).
// `part` (< J.nsplit) is the part of the n range this round walks: blocks
// [b_lo, b_hi) and, in the last part, the partial last block.
template <int FORM, int U, int TEST, bool TW>
__device__ __forceinline__ void b_round(const BJob& J, uint32_t job, uint32_t part, uint64_t p, uint64_t ps,
                                        bool valid, uint32_t* qe, uint32_t* qc, uint64_t* qp, uint64_t* qk,
                                        uint32_t qcap, pps_hit* hits, uint32_t* hit_count, uint32_t hit_cap) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t s = FORM == 0 ? 32u : J.step;
  const uint32_t nsteps = J.nsteps, full = nsteps / (uint32_t)U;
  const uint32_t nsplit = J.nsplit > 1u ? J.nsplit : 1u;
  const uint32_t per = (full + nsplit - 1u) / nsplit;
  const uint32_t b_lo = min(full, part * per), b_hi = min(full, b_lo + per);
  const bool last_part = part == nsplit - 1u;
  const uint32_t tag = job | (J.proth == 1u ? SIDE_PROTH : 0u);  // the walked value's side
  qp[lane] = p;
  if (valid) {
    uint32_t pa, pb;
    b_words<FORM>(p, &pa, &pb);
    const uint32_t pinv_s = b_pinv<FORM>(ps, s);
    const uint64_t x = inv_pow2(J.nmin + s * (uint32_t)U * b_lo, p, ps);
    const uint64_t K = J.proth == 1u ? p - x : x;
    uint32_t klo = lo32(K), khi = hi32(K);
    const uint32_t win_hi = J.win_hi, win_mask = J.win_mask, win_sh = J.win_sh, win_u = J.win_u;
    const uint32_t bound_hi = J.bound_hi, sw_mask = J.sw_mask;
    constexpr bool WSH = TEST == 1;
    // twin: p - K is below the window bound `lim` iff K > p - lim, and its low
    // bits are zero iff K's equal p's
    uint64_t tw_above = 0;
    uint32_t tw_low = 0;
    if (TW) {
      // lim = 0 stands for 2^64 (every value inside)
      const uint64_t lim = WSH ? (1ull << win_sh) : (win_hi == 0xffffffffu ? 0ull : ((uint64_t)win_hi + 1ull) << 32);
      tw_above = (lim != 0ull && p > lim) ? p - lim : 0ull;
      tw_low = lo32(p) & win_mask;
    }
    for (uint32_t b = b_lo; b < b_hi; ++b) {
      bool f = false;
      uint32_t acc = 0xffffffffu;
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (TEST == 0)
          acc = min(acc, min(__funnelshift_rc(khi, 0u, win_u), klo & win_mask));
        else if (TEST == 3)
          acc = min(acc, min(khi, klo & win_mask));
        else if (TEST == 4) {
          const uint32_t hi = __funnelshift_l(klo, khi, 32u - s);
          acc = min(acc, min(hi, klo & sw_mask));
          neg_sum(klo * pinv_s, hi, pa, pb, klo, khi);
          continue;
        }
        else if (TEST == 1)
          acc = min(acc, min(__funnelshift_rc(klo, khi, win_sh), klo & win_mask));
        else
          acc = min(acc, khi);
        if (TW) f |= (mk64(klo, khi) > tw_above) | ((klo & win_mask) == tw_low);
        b_step<FORM>(klo, khi, pa, pb, pinv_s, s);
      }
      f |= TEST == 2 ? acc <= bound_hi : acc == 0u;
      if (f) {
        const uint32_t pos = atomicAdd(qc, 1u);
        if (pos < qcap) qe[pos] = (lane << 27) | b;
      }
    }
    if (last_part && full * (uint32_t)U < nsteps) {
      // the partial last block: its start value is at hand, keep it
      qk[lane] = mk64(klo, khi);
      const uint32_t pos = atomicAdd(qc, 1u);
      if (pos < qcap) qe[pos] = (lane << 27) | full;
    }
  }
  __syncwarp();
  const uint32_t cnt = *qc;
  if (cnt <= qcap) {
    for (uint32_t e = lane; e < cnt; e += 32u) {
      const uint32_t ent = qe[e];
      const uint32_t owner = ent >> 27, blk = ent & ((1u << 27) - 1u);
      const uint64_t op = qp[owner];
      const uint64_t ops = neg_inv64(op);
      const uint32_t t0 = (uint32_t)U * blk;
      const uint32_t nblk = min((uint32_t)U, nsteps - t0);
      const uint32_t n0 = J.nmin + s * t0;
      uint64_t K;
      if (blk == full) {
        K = qk[owner];
      } else {
        const uint64_t x = inv_pow2(n0, op, ops);
        K = J.proth == 1u ? op - x : x;
      }
      uint32_t klo = lo32(K), khi = hi32(K);
      uint32_t opa, opb;
      b_words<FORM>(op, &opa, &opb);
      const uint32_t opinv = b_pinv<FORM>(ops, s);
#pragma unroll 1
      for (uint32_t u = 0; u < nblk; ++u) {
        b_record(klo, khi, n0 + s * u, s, op, tag, J, hits, hit_count, hit_cap);
        if (TW) {
          const uint64_t v = op - mk64(klo, khi);
          b_record(lo32(v), hi32(v), n0 + s * u, s, op, job | SIDE_PROTH, J, hits, hit_count, hit_cap);
        }
        b_step<FORM>(klo, khi, opa, opb, opinv, s);
      }
    }
  } else if (valid) {
    // queue overflow: the exact test at every step of this part
    uint32_t pa, pb;
    b_words<FORM>(p, &pa, &pb);
    const uint32_t pinv_s = b_pinv<FORM>(ps, s);
    const uint32_t t_lo = (uint32_t)U * b_lo, t_hi = last_part ? nsteps : (uint32_t)U * b_hi;
    const uint64_t x = inv_pow2(J.nmin + s * t_lo, p, ps);
    const uint64_t K = J.proth == 1u ? p - x : x;
    uint32_t klo = lo32(K), khi = hi32(K);
#pragma unroll 1
    for (uint32_t t = t_lo; t < t_hi; ++t) {
      b_record(klo, khi, J.nmin + s * t, s, p, tag, J, hits, hit_count, hit_cap);
      if (TW) {
        const uint64_t v = p - mk64(klo, khi);
        b_record(lo32(v), hi32(v), J.nmin + s * t, s, p, job | SIDE_PROTH, J, hits, hit_count, hit_cap);
      }
      b_step<FORM>(klo, khi, pa, pb, pinv_s, s);
    }
  }
  __syncwarp();
  if (lane == 0) *qc = 0;
  __syncwarp();
}

// Two primes per lane (32-bit steps, one side, hi-word windows or the single
// bound): the same walk and queue as b_round for FORM 0, with lane l walking
// primes l and 32 + l of the round side by side (two independent step chains);
// queue entries carry the prime's slot (0..63) in their top 6 bits.
template <int U, int TEST>
__device__ __forceinline__ void b_round2(const BJob& J, uint32_t job, uint32_t part, uint64_t p0, uint64_t ps0,
                                         bool v0, uint64_t p1, uint64_t ps1, bool v1, uint32_t* qe, uint32_t* qc,
                                         uint64_t* qp, uint64_t* qk, uint32_t qcap, pps_hit* hits,
                                         uint32_t* hit_count, uint32_t hit_cap) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t nsteps = J.nsteps, full = nsteps / (uint32_t)U;
  const uint32_t nsplit = J.nsplit > 1u ? J.nsplit : 1u;
  const uint32_t per = (full + nsplit - 1u) / nsplit;
  const uint32_t b_lo = min(full, part * per), b_hi = min(full, b_lo + per);
  const bool last_part = part == nsplit - 1u;
  const uint32_t tag = job | (J.proth == 1u ? SIDE_PROTH : 0u);
  qp[lane] = p0;
  qp[32 + lane] = p1;
  if (v0) {
    const uint32_t pa0 = neg_lo(p0), pb0 = neg_hi(p0), pi0 = lo32(ps0);
    const uint32_t pa1 = neg_lo(p1), pb1 = neg_hi(p1), pi1 = lo32(ps1);
    const uint32_t n0 = J.nmin + 32u * (uint32_t)U * b_lo;
    const uint64_t x0 = inv_pow2(n0, p0, ps0), x1 = inv_pow2(n0, p1, ps1);
    const uint64_t K0 = J.proth == 1u ? p0 - x0 : x0, K1 = J.proth == 1u ? p1 - x1 : x1;
    uint32_t klo0 = lo32(K0), khi0 = hi32(K0), klo1 = lo32(K1), khi1 = hi32(K1);
    const uint32_t win_mask = J.win_mask, win_u = J.win_u, bound_hi = J.bound_hi;
    for (uint32_t b = b_lo; b < b_hi; ++b) {
      uint32_t acc0 = 0xffffffffu, acc1 = 0xffffffffu;
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (TEST == 0) {
          acc0 = min(acc0, min(__funnelshift_rc(khi0, 0u, win_u), klo0 & win_mask));
          acc1 = min(acc1, min(__funnelshift_rc(khi1, 0u, win_u), klo1 & win_mask));
        } else if (TEST == 3) {
          acc0 = min(acc0, min(khi0, klo0 & win_mask));
          acc1 = min(acc1, min(khi1, klo1 & win_mask));
        } else {
          acc0 = min(acc0, khi0);
          acc1 = min(acc1, khi1);
        }
        step_neg32(klo0, khi0, pa0, pb0, pi0);
        step_neg32(klo1, khi1, pa1, pb1, pi1);
      }
      const bool f0 = TEST == 2 ? acc0 <= bound_hi : acc0 == 0u;
      const bool f1 = v1 && (TEST == 2 ? acc1 <= bound_hi : acc1 == 0u);
      if (f0 | f1) {
        const uint32_t pos = atomicAdd(qc, (uint32_t)f0 + (uint32_t)f1);
        if (f0 && pos < qcap) qe[pos] = (lane << 26) | b;
        if (f1 && pos + (uint32_t)f0 < qcap) qe[pos + (uint32_t)f0] = ((32u + lane) << 26) | b;
      }
    }
    if (last_part && full * (uint32_t)U < nsteps) {
      qk[lane] = mk64(klo0, khi0);
      qk[32 + lane] = mk64(klo1, khi1);
      const uint32_t pos = atomicAdd(qc, 1u + (uint32_t)v1);
      if (pos < qcap) qe[pos] = (lane << 26) | full;
      if (v1 && pos + 1u < qcap) qe[pos + 1u] = ((32u + lane) << 26) | full;
    }
  }
  __syncwarp();
  const uint32_t cnt = *qc;
  if (cnt <= qcap) {
    for (uint32_t e = lane; e < cnt; e += 32u) {
      const uint32_t ent = qe[e];
      const uint32_t owner = ent >> 26, blk = ent & ((1u << 26) - 1u);
      const uint64_t op = qp[owner];
      const uint64_t ops = neg_inv64(op);
      const uint32_t t0 = (uint32_t)U * blk;
      const uint32_t nblk = min((uint32_t)U, nsteps - t0);
      const uint32_t n0 = J.nmin + 32u * t0;
      uint64_t K;
      if (blk == full) {
        K = qk[owner];
      } else {
        const uint64_t x = inv_pow2(n0, op, ops);
        K = J.proth == 1u ? op - x : x;
      }
      uint32_t klo = lo32(K), khi = hi32(K);
      const uint32_t opa = neg_lo(op), opb = neg_hi(op), opinv = lo32(ops);
#pragma unroll 1
      for (uint32_t u = 0; u < nblk; ++u) {
        b_record(klo, khi, n0 + 32u * u, 32u, op, tag, J, hits, hit_count, hit_cap);
        step_neg32(klo, khi, opa, opb, opinv);
      }
    }
  } else {
    // queue overflow: the exact test at every step of this part, both primes
    for (int which = 0; which < 2; ++which) {
      if (which ? !v1 : !v0) continue;
      const uint64_t p = which ? p1 : p0, ps = which ? ps1 : ps0;
      const uint32_t pa = neg_lo(p), pb = neg_hi(p), pinv = lo32(ps);
      const uint32_t t_lo = (uint32_t)U * b_lo, t_hi = last_part ? nsteps : (uint32_t)U * b_hi;
      const uint64_t x = inv_pow2(J.nmin + 32u * t_lo, p, ps);
      const uint64_t K = J.proth == 1u ? p - x : x;
      uint32_t klo = lo32(K), khi = hi32(K);
#pragma unroll 1
      for (uint32_t t = t_lo; t < t_hi; ++t) {
        b_record(klo, khi, J.nmin + 32u * t, 32u, p, tag, J, hits, hit_count, hit_cap);
        step_neg32(klo, khi, pa, pb, pinv);
      }
    }
  }
  __syncwarp();
  if ((threadIdx.x & 31u) == 0) *qc = 0;
  __syncwarp();
}

// TWO: rounds of the eligible jobs walk two primes per lane (b_round2); the
// kernel then holds 64 registers a thread (4 CTAs per SM) instead of 48 (5).
template <int U, bool TWO>
__global__ void __launch_bounds__(BW_THREADS, TWO ? 4 : 5) k_bwalk(const uint8_t* tables, const BJob* jobs,
                                                         const uint32_t* seg_count, const uint32_t* seg_off,
                                                         const uint32_t* chunk_off, const uint32_t* chunk_seg,
                                                         const uint64_t* P, const uint64_t* Pinv, uint64_t* tot,
                                                         uint64_t chunk_limit, uint32_t qcap, pps_hit* hits,
                                                         uint32_t* hit_count, uint32_t hit_cap) {
  __shared__ uint32_t q_ent[BW_THREADS / 32][BQ_CAP];
  __shared__ uint64_t q_p[BW_THREADS / 32][64];
  __shared__ uint64_t q_k[BW_THREADS / 32][64];
  __shared__ uint32_t q_cnt[BW_THREADS / 32];
  const WaveTables* T = wt(tables);
  const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
  uint64_t nchunks = tot[2];
  if (chunk_limit && chunk_limit < nchunks) nchunks = chunk_limit;
  if (lane == 0) q_cnt[wib] = 0;
  __syncwarp();
  for (;;) {
    uint64_t c = 0;
    if (lane == 0) c = atomicAdd((unsigned long long*)&tot[3], 1ull);
    c = __shfl_sync(0xffffffffu, c, 0);
    if (c >= nchunks) break;
    const uint32_t s = chunk_seg[c];
    const uint32_t job = T->batch[T->seg[s].batch].job;
    const BJob J = jobs[job];
    // work items of a segment: its chunks of primes, each as nsplit n parts
    const uint32_t w = (uint32_t)(c - chunk_off[s]);
    const uint32_t nsplit = J.nsplit > 1u ? J.nsplit : 1u;
    const uint32_t part = w % nsplit;
    const uint32_t within = (w / nsplit) * J.chunk;
    const uint32_t count = min(J.chunk, seg_count[s] - within);
    const uint64_t first = (uint64_t)seg_off[s] + within;
    // two primes per lane where the job's steps are 32 n with a hi-word window
    // or the single bound, and more than one warp's worth of primes remain
    const bool two = TWO && J.step == 32 && J.proth != 2u && J.win_sh >= 32u;
    for (uint32_t r = 0; r < count;) {
      if (two && count - r > 32u) {
        const bool v1 = r + 32u + lane < count;
        const uint64_t pi0 = first + r + lane, pi1 = first + r + 32u + (v1 ? lane : 0u);
        const uint64_t p0 = P[pi0], ps0 = Pinv[pi0], p1 = P[pi1], ps1 = Pinv[pi1];
        if (J.bound_hi != 0xffffffffu)
          b_round2<U, 2>(J, job, part, p0, ps0, true, p1, ps1, v1, q_ent[wib], &q_cnt[wib], q_p[wib], q_k[wib],
                         qcap, hits, hit_count, hit_cap);
        else if (J.win_u == 0u)
          b_round2<U, 3>(J, job, part, p0, ps0, true, p1, ps1, v1, q_ent[wib], &q_cnt[wib], q_p[wib], q_k[wib],
                         qcap, hits, hit_count, hit_cap);
        else
          b_round2<U, 0>(J, job, part, p0, ps0, true, p1, ps1, v1, q_ent[wib], &q_cnt[wib], q_p[wib], q_k[wib],
                         qcap, hits, hit_count, hit_cap);
        r += 64u;
        continue;
      }
      const bool valid = r + lane < count;
      const uint64_t pi = first + r + (valid ? lane : 0u);
      const uint64_t p = P[pi], ps = Pinv[pi];
#define PPS_BROUND(FORM_, TEST_, TW_)                                                                    \
  b_round<FORM_, U, TEST_, TW_>(J, job, part, p, ps, valid, q_ent[wib], &q_cnt[wib], q_p[wib], q_k[wib], \
                                qcap, hits, hit_count, hit_cap)
#define PPS_BROUND_F(FORM_)                                                                             \
  do {                                                                                                  \
    if (wsh) {                                                                                          \
      if (tw) PPS_BROUND(FORM_, 1, true); else PPS_BROUND(FORM_, 1, false);                             \
    } else {                                                                                            \
      if (tw) PPS_BROUND(FORM_, 0, true); else if (u0) PPS_BROUND(FORM_, 3, false);                     \
      else PPS_BROUND(FORM_, 0, false);                                                                 \
    }                                                                                                   \
  } while (0)
      const bool wsh = J.win_sh < 32u, tw = J.proth == 2u, u0 = J.win_u == 0u;
      if (J.step == 32 && !tw && J.bound_hi != 0xffffffffu) PPS_BROUND(0, 2, false);
      else if (J.step == 32) PPS_BROUND_F(0);
      else if (J.shift_ok && !tw && J.sw_mask) PPS_BROUND(1, 4, false);
      else if (J.shift_ok) PPS_BROUND_F(1);
      else PPS_BROUND_F(2);
#undef PPS_BROUND_F
#undef PPS_BROUND
      r += 32u;
    }
  }
}

// output rule per candidate with its job's parameters
__global__ void __launch_bounds__(FILTER_THREADS) k_bfilter(const pps_hit* hits, const uint32_t* d_nhits,
                                                            uint32_t hit_cap, const BJob* jobs,
                                                            const uint16_t* small_q, uint32_t nsmall, pps_hit* out,
                                                            uint32_t* out_count, uint32_t out_cap) {
  uint32_t nh = *d_nhits;
  if (nh > hit_cap) nh = hit_cap;
  for (uint32_t h = blockIdx.x; h < nh; h += gridDim.x) {
    const pps_hit x = hits[h];
    const BJob J = jobs[x.idx & ~SIDE_PROTH];
    const int32_t c = (x.idx & SIDE_PROTH) ? 1 : -1;
    bool ok = (x.k == J.kstep * (x.k / J.kstep) + J.koffset) && x.n >= J.nmin && x.n < J.nmax;
    if (ok) ok = !cta_small_factor(x.k, x.n, c, small_q, nsmall);  // the same in every thread
    if (ok && threadIdx.x == 0) {
      const uint32_t pos = atomicAdd(out_count, 1u);
      if (pos < out_cap) out[pos] = x;
    }
  }
}

}  // namespace pps

// --------------------------------------------------------------- host side

namespace {

int ensure_state(pps_engine* e) {
  if (!e->batch) e->batch = new BatchState();
  BatchState* b = e->batch;
  int rc;
  if (!b->ready) {
    // (a failure below leaves ready false; the next call resumes here)
    if ((rc = b->tables.ensure(sizeof(WaveTables)))) return rc;
    if (!b->h_tables && cudaMallocHost(&b->h_tables, sizeof(WaveTables)) != cudaSuccess) {
      b->h_tables = nullptr;
      return set_err(PPS_ERR_INSUFFICIENT_RESOURCE, "pinned table staging");
    }
    b->wave_segs = e->wave_segs_req ? e->wave_segs_req : WAVE_SEGS;
    if ((rc = b->bitmap.ensure((size_t)b->wave_segs * SEG_WORDS))) return rc;
    if ((rc = b->seg_count.ensure(WAVE_SEGS)) || (rc = b->seg_off.ensure(WAVE_SEGS)) ||
        (rc = b->chunk_count.ensure(WAVE_SEGS)) || (rc = b->chunk_off.ensure(WAVE_SEGS)) ||
        (rc = b->large_items.ensure(WAVE_BATCHES)) || (rc = b->large_off.ensure(WAVE_BATCHES)))
      return rc;
    // p > 2^32: odd primes are fewer than 1/10 of the odd candidates
    b->prime_cap = (uint64_t)b->wave_segs * SEG_BITS / 10 + 4096;
    if ((rc = b->P.ensure(b->prime_cap)) || (rc = b->Pinv.ensure(b->prime_cap))) return rc;
    // at most prime_cap/32 + one partial chunk per segment (smallest chunk: 32),
    // each as up to 8 n parts
    if ((rc = b->chunk_seg.ensure(8 * (b->prime_cap / 32 + b->wave_segs)))) return rc;
    if ((rc = b->tot.ensure(8))) return rc;
    if ((rc = b->counters.ensure(4))) return rc;
    if ((rc = b->hits.ensure(1u << 22)) || (rc = b->out.ensure(1u << 20))) return rc;
    if (!b->copied && cudaEventCreateWithFlags(&b->copied, cudaEventDisableTiming) != cudaSuccess) {
      b->copied = nullptr;
      return set_err(PPS_ERR_CUDA, "event");
    }
    for (auto& v : b->ev_wave)
      if (!v && cudaEventCreate(&v) != cudaSuccess) {
        v = nullptr;
        return set_err(PPS_ERR_CUDA, "event");
      }
    // job slots at their maximum size once: the captured graph holds these pointers
    if ((rc = b->jobs.ensure(MAX_JOBS)) || (rc = b->job_primes.ensure(MAX_JOBS)) ||
        (rc = b->job_sum.ensure(MAX_JOBS)) || (rc = b->bak_primes.ensure(MAX_JOBS)) ||
        (rc = b->bak_sum.ensure(MAX_JOBS)))
      return rc;
    CU(cudaMemsetAsync(b->jobs.p, 0, MAX_JOBS * sizeof(BJob), e->st));
    CU(cudaMemsetAsync(b->counters.p, 0, 4 * sizeof(uint32_t), e->st));
    b->hjobs.assign(MAX_JOBS, BJob{});
    b->slot_pmax.assign(MAX_JOBS, 0);
    b->ready = true;
  }
  return PPS_OK;
}

constexpr uint64_t WAVE_KERNELS = 11;  // kernels in one wave's launch sequence

// The fixed per-wave launch sequence (everything reads counts from the
// tables): the sieve part, then the walk.
int launch_wave_sieve(pps_engine* e, const uint32_t* dq, uint32_t nq_all) {
  BatchState* b = e->batch;
  cudaStream_t st = e->st;
  k_bclear<<<e->num_sms * 8, 256, 0, st>>>(b->tables.p, b->bitmap.p);
  CU(cudaMemsetAsync(b->tot.p, 0, 8 * sizeof(uint64_t), st));
  k_bcounts<<<(WAVE_BATCHES + 255) / 256, 256, 0, st>>>(b->tables.p, dq, nq_all, b->large_items.p);
  k_bscan<<<1, 1024, 0, st>>>(b->large_items.p, b->large_off.p, WAVE_BATCHES, b->tot.p + 4);
  CU(cudaMemsetAsync(b->counters.p + 3, 0, sizeof(uint32_t), st));
  k_bsieve_large<<<e->num_sms * 8, 256, 0, st>>>(b->tables.p, dq, b->qm.p, b->bitmap.p, b->large_off.p,
                                                 b->tot.p + 4, b->counters.p + 3);
  k_bsieve_seg<<<WAVE_SEGS, SIEVE_THREADS, 0, st>>>(b->tables.p, dq, b->qm.p, e->presieve.p, b->bitmap.p,
                                                     b->seg_count.p);
  k_bscan<<<1, 1024, 0, st>>>(b->seg_count.p, b->seg_off.p, WAVE_SEGS, b->tot.p);
  k_bexpand<<<WAVE_SEGS, SIEVE_THREADS, 0, st>>>(b->tables.p, b->bitmap.p, b->seg_off.p, b->P.p, b->Pinv.p,
                                                  b->job_primes.p, b->job_sum.p, b->prime_cap);
  k_bchunks<<<(WAVE_SEGS + 255) / 256, 256, 0, st>>>(b->tables.p, b->jobs.p, b->seg_count.p, b->chunk_count.p);
  k_bscan<<<1, 1024, 0, st>>>(b->chunk_count.p, b->chunk_off.p, WAVE_SEGS, b->tot.p + 2);
  k_bchunkmap<<<WAVE_SEGS, 256, 0, st>>>(b->tables.p, b->chunk_count.p, b->chunk_off.p, b->chunk_seg.p,
                                         b->chunk_seg.n);
  CU(cudaGetLastError());
  e->launches += WAVE_KERNELS - 1;
  return PPS_OK;
}

// The walk kernel of a tuning code: the unroll (8 or 16) plus WALK_TWO for two
// primes per lane.
constexpr int WALK_TWO = 0x100;
typedef void (*bwalk_fn)(const uint8_t*, const BJob*, const uint32_t*, const uint32_t*, const uint32_t*,
                         const uint32_t*, const uint64_t*, const uint64_t*, uint64_t*, uint64_t, uint32_t,
                         pps_hit*, uint32_t*, uint32_t);
bwalk_fn bwalk_kernel(int code) {
  const bool two = (code & WALK_TWO) != 0;
  if ((code & 0xff) == 16) return two ? k_bwalk<16, true> : k_bwalk<16, false>;
  return two ? k_bwalk<8, true> : k_bwalk<8, false>;
}

int launch_wave_walk(pps_engine* e, int unroll, uint64_t chunk_limit, pps_hit* hits, uint32_t* hit_count,
                     uint32_t hit_cap) {
  BatchState* b = e->batch;
  cudaStream_t st = e->st;
  int per_sm = 0;
  auto fn = bwalk_kernel(unroll);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, BW_THREADS, 0);
  const int grid = (per_sm > 0 ? per_sm : 1) * e->num_sms;
  fn<<<grid, BW_THREADS, 0, st>>>(b->tables.p, b->jobs.p, b->seg_count.p, b->seg_off.p, b->chunk_off.p,
                                  b->chunk_seg.p, b->P.p, b->Pinv.p, b->tot.p, chunk_limit,
                                  std::min(debug_queue_cap(), BQ_CAP), hits, hit_count, hit_cap);
  CU(cudaGetLastError());
  e->launches += 1;
  return PPS_OK;
}

int launch_wave(pps_engine* e, const uint32_t* dq, uint32_t nq_all, int unroll, uint64_t chunk_limit,
                pps_hit* hits, uint32_t* hit_count, uint32_t hit_cap) {
  int rc = launch_wave_sieve(e, dq, nq_all);
  return rc ? rc : launch_wave_walk(e, unroll, chunk_limit, hits, hit_count, hit_cap);
}

int floor_lg2(uint64_t x) { return 63 - __builtin_clzll(x | 1ull); }

// The one-job window tests K < 2^(32+u) with u >= 0; when p is below about
// 2^(64-kb) (kmax < 2^kb) that bound passes most steps.  There the window is
// placed at t = (lg p + kb - 1) / 2, which balances P(K < 2^t) ~ 2^(t - lg p)
// against P(low t+1-kb bits zero) = 2^-(t+1-kb).  It stays exact while
// K < p <= 2^(t+32), so that the funnel shift sees all of K >> t.
void small_p_window(const pps_job_params& jp, BJob* J) {
  uint32_t t, mask;
  small_p_window_of(&jp, &t, &mask);
  J->win_sh = t;
  if (t < 32) J->win_mask = mask;
}

BJob make_job(const pps_job_params& jp) {
  WalkArgs a;
  walk_args_for_job(&jp, &a);
  BJob J;
  memset(&J, 0, sizeof J);
  J.kmin = jp.kmin;
  J.kmax = jp.kmax;
  J.kstep = jp.kstep;
  J.koffset = jp.koffset;
  J.nmin = jp.nmin;
  J.nmax = jp.nmax;
  J.step = jp.step;
  J.nsteps = a.nsteps;
  J.proth = jp.sign == PPS_SIGN_TWIN ? 2u : a.proth;  // 2: both sides (twin)
  J.win_hi = a.win_hi;
  J.win_mask = a.win_mask;
  J.qmax = jp.qmax;
  J.sign = jp.sign;
  J.chunk = 32;
  J.nsplit = 1;
  J.win_u = a.win_hi == 0xffffffffu ? 32u : (uint32_t)__builtin_popcount(a.win_hi);
  J.bound_hi = 0xffffffffu;
  if (jp.step == 32 && jp.kmax < (1ull << 32) && jp.pmin / jp.kmax >= (1ull << 43)) J.bound_hi = a.bound_hi;
  small_p_window(jp, &J);
  // The small-p window costs a funnel shift per step; the plain window (hi
  // word below 2^u, no shift when u == 0) is kept where it passes at most
  // 1 step in 1024 and a round's expected queue (32 lanes x nsteps x rate)
  // stays within half the warp queue.
  if (J.win_sh < 32) {
    const double plain = ldexp(1.0, 32 + (int)J.win_u) / (double)jp.pmin +
                         (a.win_mask == 0xffffffffu ? ldexp(1.0, -32) : 1.0 / ((double)a.win_mask + 1.0));
    if (plain <= 1.0 / 1024.0 && 32.0 * (double)J.nsteps * plain <= BQ_CAP / 2) {
      J.win_sh = 32;
      J.win_mask = a.win_mask;
    }
  }
  // form 1 keeps K * 2^(32-step) below 2^64: every K < p <= pmax <= 2^(32+step)
  J.shift_ok = jp.step < 32 && (jp.pmax - 1) >> (32 + jp.step) == 0 ? 1u : 0u;
  // Form-1 jobs take test 4 (no shift of its own: the step computes K >> s
  // anyway) where its pass rate 2^s / pmin + 2^-(s+1-kb) is at most 1.25 times
  // the rate of the window chosen above and a round's expected queue fits in
  // half the warp queue.
  J.sw_mask = 0;
  if (J.shift_ok && J.proth != 2u && a.sw_mask) {
    const int kb = floor_lg2(jp.kmax) + 1;
    const double pmin = (double)jp.pmin;
    const double sw = ldexp(1.0, (int)jp.step) / pmin + ldexp(1.0, kb - 1 - (int)jp.step);
    const double cur = J.win_sh < 32
                           ? ldexp(1.0, (int)J.win_sh) / pmin + ldexp(1.0, kb - 1 - (int)J.win_sh)
                           : ldexp(1.0, 32 + (int)J.win_u) / pmin +
                                 (J.win_mask == 0xffffffffu ? ldexp(1.0, -32) : 1.0 / ((double)J.win_mask + 1.0));
    if (sw <= 1.25 * cur && 32.0 * (double)J.nsteps * sw <= BQ_CAP / 2) J.sw_mask = a.sw_mask;
  }
  return J;
}

// Each job's work item holds about `work` walk steps per lane, so an item of
// a short-n job and one of a long-n job take about the same time: a long n
// range is cut into up to 8 parts (n-chunks of at least 32 blocks of 16 steps,
// and at most 8 times `work` steps where a cut is possible), and a chunk holds
// `work` x 32 / (steps per part) primes (at least 32: one per lane).
// A forced split (pps_engine_set_split) replaces the choice for every job.
void chunk_for(BJob* J, int work, int forced_split) {
  const uint64_t nsteps = std::max<uint64_t>(1, J->nsteps);
  uint32_t t = 1;
  while (t < 8 && nsteps / t > 8ull * (uint64_t)work && nsteps / (2ull * t) >= 32ull * 16ull) t *= 2;
  if (forced_split > 0) t = (uint32_t)forced_split;
  const uint64_t per = (nsteps + t - 1) / t;
  const uint64_t c = ((uint64_t)work * 32u / per + 31u) & ~31ull;
  // jobs the walk may take two primes per lane for get at least 64 (a round of two)
  const uint64_t cmin = J->step == 32 && J->proth != 2u && J->win_sh >= 32u ? 64 : 32;
  J->nsplit = t;
  J->chunk = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(c, cmin), MAX_CHUNK);
}

// Copy mirror slots [lo, hi) to the device.  The source is pageable: the call
// returns once it is staged, so the mirror may change right afterwards.
int upload_slots(pps_engine* e, uint32_t lo, uint32_t hi) {
  BatchState* b = e->batch;
  if (hi > lo)
    CU(cudaMemcpyAsync(b->jobs.p + lo, b->hjobs.data() + lo, (size_t)(hi - lo) * sizeof(BJob),
                       cudaMemcpyHostToDevice, e->st));
  return PPS_OK;
}

// Chunk sizes of slots [lo, hi] for a work target; uploads what changed.
int set_chunks(pps_engine* e, uint32_t lo, uint32_t hi, int work) {
  BatchState* b = e->batch;
  bool changed = false;
  for (uint32_t s = lo; s <= hi; ++s) {
    if (!b->slot_pmax[s]) continue;
    BJob J = b->hjobs[s];
    chunk_for(&J, work, e->forced_split);
    if (J.chunk != b->hjobs[s].chunk || J.nsplit != b->hjobs[s].nsplit) {
      b->hjobs[s].chunk = J.chunk;
      b->hjobs[s].nsplit = J.nsplit;
      changed = true;
    }
  }
  return changed ? upload_slots(e, lo, hi + 1) : PPS_OK;
}

}  // namespace

uint32_t batch_max_slots() { return MAX_JOBS; }
uint64_t batch_wave_segments(const pps_engine* e) {
  return e && e->batch && e->batch->ready ? e->batch->wave_segs : WAVE_SEGS;
}
uint64_t batch_max_piece_span() { return 2ull * SEG_BITS * BATCH_SEGS; }
uint64_t batch_piece_span(const pps_engine* e) {
  return 2ull * SEG_BITS * std::min<uint64_t>(BATCH_SEGS, batch_wave_segments(e));
}
uint64_t batch_piece_segments(uint64_t lo, uint64_t hi) {
  const uint64_t lo0 = lo | 1ull;
  if (hi <= lo0) return 0;
  const uint64_t span = batch_max_piece_span(), bits = (hi - lo0 + 1) / 2;
  // whole batches of BATCH_SEGS segments, then the remainder
  const uint64_t full = (hi - lo0) / span;
  const uint64_t rest = bits - full * (span / 2);
  return full * BATCH_SEGS + (rest + SEG_BITS - 1) / SEG_BITS;
}

int batch_prepare(pps_engine* e) {
  if (!e) return set_err(PPS_ERR_INVALID_PARAM, "null engine");
  CU(cudaSetDevice(e->device));
  return ensure_state(e);
}

void batch_tuning(pps_engine* e, uint32_t* work, uint32_t* unroll) {
  const BatchState* b = e ? e->batch : nullptr;
  if (work) *work = b ? (uint32_t)b->tuned_work : 0;
  if (unroll) *unroll = b ? (uint32_t)b->walk_code & 0xffu : 0;
}

int batch_set_jobs(pps_engine* e, uint32_t slot0, const pps_job_params* jobs, size_t n) {
  int rc;
  if ((rc = batch_prepare(e))) return rc;
  if (!jobs && n) return set_err(PPS_ERR_INVALID_PARAM, "null jobs");
  if ((uint64_t)slot0 + n > MAX_JOBS) return set_err(PPS_ERR_INVALID_PARAM, "at most %u job slots", MAX_JOBS);
  for (size_t j = 0; j < n; ++j)
    if (jobs[j].step < 1 || jobs[j].step > 32 || jobs[j].pmin <= (1ull << 32) || jobs[j].pmax <= jobs[j].pmin)
      return set_err(PPS_ERR_INVALID_PARAM, "job %zu not normalized", j);
  BatchState* b = e->batch;
  const int work = b->tuned_work > 0 ? b->tuned_work : 1024;
  for (size_t j = 0; j < n; ++j) {
    BJob J = make_job(jobs[j]);
    chunk_for(&J, work, e->forced_split);
    b->hjobs[slot0 + j] = J;
    b->slot_pmax[slot0 + j] = jobs[j].pmax;
  }
  if ((rc = upload_slots(e, slot0, (uint32_t)(slot0 + n)))) return rc;
  if (n) {
    CU(cudaMemsetAsync(b->job_primes.p + slot0, 0, n * sizeof(unsigned long long), e->st));
    CU(cudaMemsetAsync(b->job_sum.p + slot0, 0, n * sizeof(unsigned long long), e->st));
  }
  return PPS_OK;
}

int batch_job_counts(pps_engine* e, uint32_t slot0, size_t n, uint64_t* primes, uint64_t* sums) {
  int rc;
  if ((rc = batch_prepare(e))) return rc;
  if ((uint64_t)slot0 + n > MAX_JOBS) return set_err(PPS_ERR_INVALID_PARAM, "slot range");
  BatchState* b = e->batch;
  CU(cudaStreamSynchronize(e->st));
  if (primes && n) CU(cudaMemcpy(primes, b->job_primes.p + slot0, n * 8, cudaMemcpyDeviceToHost));
  if (sums && n) CU(cudaMemcpy(sums, b->job_sum.p + slot0, n * 8, cudaMemcpyDeviceToHost));
  return PPS_OK;
}

int batch_wave(pps_engine* e, const BatchPiece* pieces, size_t n, std::vector<pps_hit>* survivors,
               uint64_t* raw_hits, double* filter_ms) {
  int rc;
  if ((rc = batch_prepare(e))) return rc;
  if (!pieces && n) return set_err(PPS_ERR_INVALID_PARAM, "null pieces");
  if (n == 0) return PPS_OK;
  BatchState* b = e->batch;
  cudaStream_t st = e->st;

  // the pieces' slots, and the sieving bound over them
  uint32_t smin = MAX_JOBS, smax = 0;
  uint64_t need_q = SEG_BITS;
  for (size_t i = 0; i < n; ++i) {
    const BatchPiece& pc = pieces[i];
    if (pc.slot >= MAX_JOBS || !b->slot_pmax[pc.slot] || pc.hi <= pc.lo || pc.hi > b->slot_pmax[pc.slot] ||
        pc.lo <= (1ull << 32))
      return set_err(PPS_ERR_INVALID_PARAM, "piece %zu: bad slot or range", i);
    smin = std::min(smin, pc.slot);
    smax = std::max(smax, pc.slot);
    need_q = std::max<uint64_t>(need_q, std::min<uint64_t>(b->hjobs[pc.slot].qmax, isqrt64(pc.hi - 1)));
  }
  // The whole cached table of sieving primes serves the wave (each batch stops
  // at its own limit on the device); it only grows, so the graph stays valid.
  const uint32_t want = (uint32_t)std::max<uint64_t>(need_q, e->base_limit);
  const uint32_t* dq = nullptr;
  BaseTable bt;
  if ((rc = prepare_sieving_primes(e, want, (uint64_t)want * want + 1, &dq, &bt))) return rc;
  const uint32_t nq_all = e->base_count;
  if (b->qm_q != dq || b->qm_n != nq_all) {
    // a new sieving-prime table: its Barrett constants (the graph, which holds
    // the old qm pointer, is recaptured too)
    drop_graphs(b);
    b->qm_q = nullptr;
    b->qm_n = 0;
    if ((rc = b->qm.ensure(std::max<uint32_t>(nq_all, 1)))) return rc;
    if (nq_all) {
      k_brecip<<<std::min<uint32_t>((nq_all + 255) / 256, 4096), 256, 0, st>>>(dq, nq_all, b->qm.p);
      CU(cudaGetLastError());
      e->launches++;
    }
    b->qm_q = dq;
    b->qm_n = nq_all;
  }

  // wave tables: each piece as batches of at most BATCH_SEGS segments
  CU(cudaEventSynchronize(b->copied));  // staging free again
  WaveTables* T = b->h_tables;
  uint32_t nseg = 0, nb = 0;
  const uint64_t span = batch_max_piece_span();
  for (size_t i = 0; i < n; ++i) {
    const BatchPiece& pc = pieces[i];
    const BJob& J = b->hjobs[pc.slot];
    for (uint64_t lo = pc.lo | 1ull; lo < pc.hi; lo += span) {
      const uint64_t hi = std::min(pc.hi, lo + span);
      BBatch B;
      memset(&B, 0, sizeof B);
      B.lo = lo;
      B.nbits = (hi - lo + 1) / 2;
      B.job = pc.slot;
      B.limit = (uint32_t)std::min<uint64_t>(J.qmax, isqrt64(hi - 1));
      const uint32_t ns = (uint32_t)((B.nbits + SEG_BITS - 1) / SEG_BITS);
      if (nseg + ns > b->wave_segs || nb >= WAVE_BATCHES)
        return set_err(PPS_ERR_INVALID_PARAM, "pieces exceed one wave (%u segments)", b->wave_segs);
      B.seg0 = nseg;
      for (uint32_t s = 0; s < ns; ++s) {
        BSeg& S = T->seg[nseg + s];
        S.lo = B.lo + 2ull * (uint64_t)s * SEG_BITS;
        S.bits = (uint32_t)std::min<uint64_t>(B.nbits - (uint64_t)s * SEG_BITS, SEG_BITS);
        S.batch = nb;
      }
      T->batch[nb++] = B;
      nseg += ns;
    }
  }
  T->nseg = nseg;
  T->nbatch = nb;
  const size_t bytes = offsetof(WaveTables, seg) + sizeof(BSeg) * WAVE_SEGS + sizeof(BBatch) * nb;
  CU(cudaMemcpyAsync(b->tables.p, T, bytes, cudaMemcpyHostToDevice, st));
  CU(cudaEventRecord(b->copied, st));

  // slot counters before the wave: the tuning runs and an overflow re-run put them back
  const size_t nsl = (size_t)(smax - smin) + 1;
  CU(cudaMemcpyAsync(b->bak_primes.p + smin, b->job_primes.p + smin, nsl * 8, cudaMemcpyDeviceToDevice, st));
  CU(cudaMemcpyAsync(b->bak_sum.p + smin, b->job_sum.p + smin, nsl * 8, cudaMemcpyDeviceToDevice, st));
  auto restore = [&]() -> int {
    CU(cudaMemcpyAsync(b->job_primes.p + smin, b->bak_primes.p + smin, nsl * 8, cudaMemcpyDeviceToDevice, st));
    CU(cudaMemcpyAsync(b->job_sum.p + smin, b->bak_sum.p + smin, nsl * 8, cudaMemcpyDeviceToDevice, st));
    return PPS_OK;
  };

  if (!b->tuned_work) {
    // time each (work per chunk, unroll) on the first chunks of this wave, the
    // same number of walk steps for every candidate.  The kernels take two
    // primes per lane: on the 512-job mix, each kind of job alone walked as
    // fast or faster with them than with one prime per lane at the same unroll
    // (pps_engine_set_batch_walk still forces one prime per lane).
    const int works[] = {256, 1024, 4096};
    const int unrolls[] = {8 | WALK_TWO, 16 | WALK_TWO};
    float best = 1e30f;
    for (int w : works)
      for (int u : unrolls) {
        if ((rc = set_chunks(e, smin, smax, w))) return rc;
        CU(cudaMemsetAsync(b->counters.p + 2, 0, sizeof(uint32_t), st));
        // tuning hits go to the survivors' buffer (its count is reset), then are dropped
        const uint64_t lim = std::max<uint64_t>(16, (uint64_t)nseg * 4096 / (uint64_t)w);
        if ((rc = launch_wave(e, dq, nq_all, u, lim, b->out.p, b->counters.p + 2, (uint32_t)b->out.n)))
          return rc;
        CU(cudaEventRecord(e->ev[0], st));
        CU(cudaMemsetAsync(b->tot.p + 3, 0, sizeof(uint64_t), st));
        auto fn = bwalk_kernel(u);
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, BW_THREADS, 0);
        fn<<<std::max(per_sm, 1) * e->num_sms, BW_THREADS, 0, st>>>(
            b->tables.p, b->jobs.p, b->seg_count.p, b->seg_off.p, b->chunk_off.p, b->chunk_seg.p, b->P.p,
            b->Pinv.p, b->tot.p, lim, std::min(debug_queue_cap(), BQ_CAP), b->out.p, b->counters.p + 2,
            (uint32_t)b->out.n);
        CU(cudaGetLastError());
        e->launches++;
        CU(cudaEventRecord(e->ev[1], st));
        CU(cudaEventSynchronize(e->ev[1]));
        float ms = 0;
        CU(cudaEventElapsedTime(&ms, e->ev[0], e->ev[1]));
        // steps timed: the work items walked (the wave may hold fewer than lim),
        // each with the chunk size and n part of the wave's first job, whose
        // primes come first
        uint64_t nch = 0;
        CU(cudaMemcpy(&nch, b->tot.p + 2, sizeof nch, cudaMemcpyDeviceToHost));
        const BJob& J0 = b->hjobs[T->batch[0].job];
        const double part_steps = (double)std::max<uint32_t>(J0.nsteps, 1) / std::max<uint32_t>(J0.nsplit, 1);
        const double steps = (double)std::min<uint64_t>(lim, nch) * J0.chunk * part_steps;
        const float per_step = (float)(ms / std::max(steps, 1.0));
        if (per_step < best) {
          best = per_step;
          b->tuned_work = w;
          b->tuned_unroll = u;
        }
      }
    if ((rc = restore())) return rc;
  }
  // the walk kernel of this wave: the tuner's, unless pps_engine_set_batch_walk forces one
  b->walk_code = e->forced_bwalk ? e->forced_bwalk : b->tuned_unroll;
  if ((rc = set_chunks(e, smin, smax, b->tuned_work))) return rc;

  // the wave itself: a captured graph of the fixed sequence, replayed
  CU(cudaMemsetAsync(b->counters.p, 0, 2 * sizeof(uint32_t), st));
  uint32_t raw = 0;
  // the first attempt's candidate capacity (less under pps_debug_limits)
  uint32_t hcap = (uint32_t)std::min<size_t>(b->hits.n, 0xffffffffu);
  if (debug_first_hit_cap() && debug_first_hit_cap() < hcap) hcap = debug_first_hit_cap();
  for (;;) {
    const uint32_t qcap = std::min(debug_queue_cap(), BQ_CAP);
    if (!b->graph || !b->graph_walk || b->graph_unroll != b->walk_code || b->graph_q != dq ||
        b->graph_nq != nq_all || b->graph_hcap != hcap || b->graph_qcap != qcap) {
      drop_graphs(b);
      for (int part = 0; part < 2; ++part) {
        cudaGraph_t g;
        CU(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        const uint64_t launches0 = e->launches;
        rc = part == 0 ? launch_wave_sieve(e, dq, nq_all)
                       : launch_wave_walk(e, b->walk_code, 0, b->hits.p, b->counters.p, hcap);
        cudaError_t ce = cudaStreamEndCapture(st, &g);
        e->launches = launches0;
        if (rc) return rc;
        if (ce != cudaSuccess) return set_err(PPS_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
        ce = cudaGraphInstantiate(part == 0 ? &b->graph : &b->graph_walk, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) {
          drop_graphs(b);
          return set_err(PPS_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
        }
      }
      b->graph_unroll = b->walk_code;
      b->graph_q = dq;
      b->graph_nq = nq_all;
      b->graph_hcap = hcap;
      b->graph_qcap = qcap;
    }
    CU(cudaEventRecord(b->ev_wave[0], st));
    CU(cudaGraphLaunch(b->graph, st));
    CU(cudaEventRecord(b->ev_wave[1], st));
    CU(cudaGraphLaunch(b->graph_walk, st));
    CU(cudaEventRecord(b->ev_wave[2], st));
    e->launches += WAVE_KERNELS;
    CU(cudaMemcpyAsync(e->h_pinned, b->counters.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    {
      float ms0 = 0, ms1 = 0;
      CU(cudaEventElapsedTime(&ms0, b->ev_wave[0], b->ev_wave[1]));
      CU(cudaEventElapsedTime(&ms1, b->ev_wave[1], b->ev_wave[2]));
      b->sieve_ms += ms0;
      b->walk_ms += ms1;
    }
    raw = ((uint32_t*)e->h_pinned)[0];
    if (raw <= hcap) break;
    // more candidates than the buffer: grow it (a new graph), put the slot
    // counters back and walk the wave again
    drop_graphs(b);  // the walk graph holds the old hits pointer
    if (raw > b->hits.n && (rc = b->hits.ensure((size_t)raw * 2))) return rc;
    hcap = (uint32_t)std::min<size_t>(b->hits.n, 0xffffffffu);
    if ((rc = restore())) return rc;
    CU(cudaMemsetAsync(b->counters.p, 0, 2 * sizeof(uint32_t), st));
  }
  if (raw_hits) *raw_hits += raw;

  // output rule per candidate, with its job's parameters
  if (raw) {
    CU(cudaEventRecord(e->ev[4], st));
    uint32_t nf = 0;
    for (;;) {
      CU(cudaMemsetAsync(b->counters.p + 1, 0, sizeof(uint32_t), st));
      k_bfilter<<<filter_blocks(raw), FILTER_THREADS, 0, st>>>(b->hits.p, b->counters.p, (uint32_t)b->hits.n,
                                                               b->jobs.p, e->small_q.p, e->nsmall, b->out.p,
                                                               b->counters.p + 1, (uint32_t)b->out.n);
      CU(cudaGetLastError());
      e->launches++;
      CU(cudaMemcpyAsync(e->h_pinned, b->counters.p + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
      CU(cudaStreamSynchronize(st));
      nf = ((uint32_t*)e->h_pinned)[0];
      if (nf <= b->out.n) break;
      if ((rc = b->out.ensure((size_t)nf * 2))) return rc;  // the filter is re-run into the larger buffer
    }
    CU(cudaEventRecord(e->ev[5], st));
    if (nf && survivors) {
      const size_t at = survivors->size();
      survivors->resize(at + nf);
      CU(cudaMemcpyAsync(survivors->data() + at, b->out.p, nf * sizeof(pps_hit), cudaMemcpyDeviceToHost, st));
      CU(cudaStreamSynchronize(st));
      std::sort(survivors->begin() + at, survivors->end(), batch_hit_less);
    }
    CU(cudaEventSynchronize(e->ev[5]));
    float fms = 0;
    CU(cudaEventElapsedTime(&fms, e->ev[4], e->ev[5]));
    if (filter_ms) *filter_ms += fms;
  }
  return PPS_OK;
}

extern "C" int pps_run_batch(pps_engine* e, const pps_job_params* jobs, size_t njobs, pps_factor* out,
                             size_t cap, size_t* nout, size_t* job_offsets, pps_batch_stats* bst) {
  if (!e || (!jobs && njobs)) return set_err(PPS_ERR_INVALID_PARAM, "null argument");
  if (njobs > MAX_JOBS) return set_err(PPS_ERR_INVALID_PARAM, "at most %u jobs per batch", MAX_JOBS);
  for (size_t j = 0; j < njobs; ++j)
    if (jobs[j].step < 1 || jobs[j].step > 32 || jobs[j].pmin <= (1ull << 32))
      return set_err(PPS_ERR_INVALID_PARAM, "job %zu not normalized", j);
  int rc;
  if ((rc = batch_prepare(e))) return rc;
  BatchState* b = e->batch;
  if (bst) memset(bst, 0, sizeof *bst);
  b->sieve_ms = b->walk_ms = 0;
  CU(cudaEventRecord(e->ev[6], e->st));

  // jobs j in slots j; pieces of at most one batch, most expensive jobs first
  // (steps per prime x range width), packed into waves in that order
  if ((rc = batch_set_jobs(e, 0, jobs, njobs))) return rc;
  std::vector<size_t> order(njobs);
  for (size_t j = 0; j < njobs; ++j) order[j] = j;
  std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) {
    const double cx = (double)b->hjobs[x].nsteps * (double)(jobs[x].pmax - jobs[x].pmin);
    const double cy = (double)b->hjobs[y].nsteps * (double)(jobs[y].pmax - jobs[y].pmin);
    return cx > cy;
  });
  std::vector<BatchPiece> pieces;
  const uint64_t span = batch_piece_span(e);
  for (size_t j : order)
    for (uint64_t lo = jobs[j].pmin | 1ull; lo < jobs[j].pmax; lo += span)
      pieces.push_back(BatchPiece{lo, std::min(jobs[j].pmax, lo + span), (uint32_t)j});
  std::vector<pps_hit> surv;
  uint64_t raw = 0;
  double fms = 0;
  int waves = 0;
  for (size_t a = 0; a < pieces.size();) {
    uint64_t segs = 0;
    size_t z = a;
    while (z < pieces.size() && z - a < WAVE_BATCHES) {
      const uint64_t ns = batch_piece_segments(pieces[z].lo, pieces[z].hi);
      if (segs + ns > b->wave_segs) break;
      segs += ns;
      ++z;
    }
    if ((rc = batch_wave(e, pieces.data() + a, z - a, &surv, &raw, &fms))) return rc;
    ++waves;
    a = z;
  }
  CU(cudaEventRecord(e->ev[7], e->st));
  CU(cudaEventSynchronize(e->ev[7]));
  // survivors by job, each job's in (p, k, n) order
  std::sort(surv.begin(), surv.end(), batch_hit_less);
  const size_t nf = surv.size();
  if (nout) *nout = nf;
  if (job_offsets) {
    size_t k = 0;
    for (size_t j = 0; j <= njobs; ++j) {
      while (k < nf && batch_hit_slot(surv[k]) < j) ++k;
      job_offsets[j] = k;
    }
  }
  if (out) {
    for (size_t i = 0; i < nf && i < cap; ++i) {
      out[i].p = surv[i].p;
      out[i].k = surv[i].k;
      out[i].n = surv[i].n;
      out[i].c = batch_hit_sign(surv[i]);
    }
  }
  if (bst) {
    std::vector<uint64_t> jp(njobs), js(njobs);
    if (njobs && (rc = batch_job_counts(e, 0, njobs, jp.data(), js.data()))) return rc;
    for (size_t j = 0; j < njobs; ++j) {
      bst->primes += jp[j];
      bst->prime_sum += js[j];
      bst->steps += jp[j] * b->hjobs[j].nsteps;
    }
    bst->raw_hits = raw;
    bst->factors = nf;
    bst->waves = (uint32_t)waves;
    bst->chunk = (uint32_t)b->tuned_work;
    bst->unroll = (uint32_t)b->walk_code & 0xffu;
    bst->primes_per_lane = (b->walk_code & WALK_TWO) ? 2u : 1u;
    float ms = 0;
    CU(cudaEventElapsedTime(&ms, e->ev[6], e->ev[7]));
    bst->total_ms = ms;
    bst->filter_ms = fms;
    bst->sieve_ms = b->sieve_ms;
    bst->walk_ms = b->walk_ms;
  }
  if (out && nf > cap) return set_err(PPS_ERR_OVERFLOW, "%zu factors, buffer holds %zu", nf, cap);
  return PPS_OK;
}

extern "C" int pps_batch_job_primes(pps_engine* e, size_t njobs, uint64_t* primes, uint64_t* sums) {
  if (!e || !e->batch || !e->batch->ready) return set_err(PPS_ERR_INVALID_PARAM, "no batch has run");
  if (njobs > MAX_JOBS) return set_err(PPS_ERR_INVALID_PARAM, "njobs too large");
  return batch_job_counts(e, 0, njobs, primes, sums);
}

extern "C" int pps_engine_set_wave_segments(pps_engine* e, uint32_t segments) {
  if (!e || segments > WAVE_SEGS) return set_err(PPS_ERR_INVALID_PARAM, "wave segments above %u", WAVE_SEGS);
  if (e->batch && e->batch->ready)
    return set_err(PPS_ERR_BUSY, "the batched form's buffers are already sized for this engine");
  e->wave_segs_req = segments;
  return PPS_OK;
}

extern "C" int pps_engine_set_batch_walk(pps_engine* e, int unroll, int primes_per_lane) {
  if (!e) return set_err(PPS_ERR_INVALID_PARAM, "null engine");
  if (unroll == 0 && primes_per_lane == 0) {
    e->forced_bwalk = 0;
    return PPS_OK;
  }
  if ((unroll != 8 && unroll != 16) || (primes_per_lane != 1 && primes_per_lane != 2))
    return set_err(PPS_ERR_INVALID_PARAM, "batched walk: unroll 8 or 16, 1 or 2 primes per lane");
  e->forced_bwalk = unroll | (primes_per_lane == 2 ? WALK_TWO : 0);
  return PPS_OK;
}
