// pps_internal.h -- kernel launchers and device-side structures shared by the
// library's translation units.  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "ppsgpu.h"

namespace pps {

// ------------------------------------------------------------------ sieve
// Odd candidates are numbered j = 0, 1, ... for values lo + 2j (lo odd).  One
// CTA sieves one segment of SEG_BITS candidates in shared memory; primes
// q >= SEG_BITS are scattered into the batch bitmap in global memory first.
constexpr int SEG_LOG2 = 18;
constexpr uint32_t SEG_BITS = 1u << SEG_LOG2;
constexpr uint32_t SEG_WORDS = SEG_BITS / 32;
constexpr int SIEVE_THREADS = 512;
constexpr uint32_t TINY_Q_LIMIT = 128;  // q below this: whole CTA strides one q

struct SieveBatch {
  uint64_t lo;        // first odd candidate
  uint64_t nbits;     // odd candidates in the batch
  uint32_t nseg;      // ceil(nbits / SEG_BITS)
  const uint32_t* q;  // sieving primes, ascending, odd, q <= qmax
  uint32_t nq;        // number of sieving primes used (q*q < hi is checked too)
  uint32_t nq_tiny;   // q < TINY_Q_LIMIT
  uint32_t nq_seg;    // q < SEG_BITS (sieved per segment)
  uint32_t* bitmap;   // nseg * SEG_WORDS words
  uint32_t* seg_count;
  uint32_t* seg_off;  // exclusive scan of seg_count
  uint64_t* d_total;  // [0] = primes in batch (written by scan), [1] = wrapping sum
  // optional: the pre-sieve table (PRESIEVE_WORDS words: bit b of word x set
  // when the value x + 2b (mod PRESIEVE_MOD) has a factor 3, 5, 7, 11 or 13),
  // replacing the marking by those five primes; and per-batch residues of the
  // sieving primes q[nq_tiny .. nq_seg): res[2i] = lo mod q, res[2i+1] =
  // 2 SEG_BITS mod q, so a segment's start offsets need no 64-bit division
  const uint32_t* presieve = nullptr;
  uint32_t* res = nullptr;
};

constexpr uint32_t PRESIEVE_MOD = 3u * 5u * 7u * 11u * 13u;  // 15015
constexpr uint32_t PRESIEVE_WORDS = PRESIEVE_MOD;
constexpr uint32_t PRESIEVE_PRIMES = 5;  // 3, 5, 7, 11, 13: the first five sieving primes
// The pre-sieve table (host side, to copy to the device once).
void presieve_table(uint32_t* out);

// Launch the full sieve of one batch on `st`: large-prime scatter, segment
// sieve, scan, expansion into out64 (+ Montgomery constants into pinv64 when
// non-null) or out32.  Returns the number of kernel launches issued.
int launch_sieve_batch(const SieveBatch& b, uint64_t* out64, uint64_t* pinv64, uint32_t* out32,
                       cudaStream_t st);

// Number of entries <= x of the ascending table q[0..n), into *out (one thread).
cudaError_t launch_count_le(const uint32_t* q, uint32_t n, uint32_t x, uint32_t* out, cudaStream_t st);

// ------------------------------------------------------------------- walk
struct WalkArgs {
  const uint64_t* P;        // primes
  const uint64_t* Pinv;     // -p^-1 mod 2^64 per prime, or null (computed)
  const uint64_t* d_np;     // device-side prime count (or null: use np)
  uint64_t np;
  uint64_t kmin, kmax;
  uint32_t nmin, nmax;
  uint32_t step;            // s, 1..32
  uint32_t nsteps;          // ceil((nmax - nmin) / s)
  uint32_t proth;           // 1: K0 = p - 2^-nmin, 0: K0 = 2^-nmin
  uint32_t win_hi;          // window pre-test: hi word <= win_hi ...
  uint32_t win_mask;        // ... or (lo word & win_mask) == 0
  uint32_t kmax32;          // low-bit pre-test (kmax < 2^32)
  uint32_t bound_hi;        // single-bound pre-test: hi word <= bound_hi
  uint32_t sh_t, sh_mask;   // small-p window: K < 2^sh_t or (lo & sh_mask) == 0; sh_t 32: none
  uint32_t shift_ok;        // step < 32 and pmax <= 2^(32+step): the shifted chain step
  uint32_t sw_mask;         // steps s < 32: K < 2^s (hi word of K 2^(32-s) zero) or (lo & sw_mask) == 0,
                            // sw_mask = 2^(s+1-kb) - 1 (0 where s < kb)
  uint32_t nsplit;          // queued walks: threads per prime (1, 2, 4, 8): thread j of a
                            // prime walks blocks [j L, (j+1) L) of its n range,
                            // L = ceil(blocks / nsplit); 0 counts as 1
  uint32_t qcap;            // queued walks: warp-queue entries used (<= WALK_QUEUE_CAP)
  uint32_t idx_base;        // added to the prime index in hit records
  pps_hit* hits;
  uint32_t* hit_count;      // may exceed hit_cap: overflow is detected by host
  uint32_t hit_cap;
};

// Variant v in [0, PPS_NUM_VARIANTS): step formulation x pre-test x unroll.
// Flagged blocks a warp of the queued walks (variants 10 and up) holds for its
// exact re-check; beyond it each lane re-walks its prime with the exact test.
constexpr int WALK_QUEUE_CAP = 512;

const char* walk_variant_name(int v);
// What a walk variant is: the queued walks (k_walk32q, k_walk32q2) hold no
// exact-check code in their hot loop and take threads per prime; the others
// (k_walk) branch or replay per block.  Pre-test kinds: window (hi word below
// 2^u or the low bits zero), min (the window as a running minimum, u == 0),
// bound (hi word <= kmax/2: 32-bit steps, p > kmax 2^43), lowbit (kmax <
// 2^32), smallp (K < 2^t or the low bits zero, p far below 2^(64-bits(kmax))),
// stepwin (K < 2^s read off the step, s < 32).
struct VariantTraits {
  const char* name;
  bool queued;
  bool twin;       // both sides of a twin job from one walk
  bool s32;        // 32-bit steps only
  bool shifted;    // s < 32 through the carry-free step on K 2^(32-s) (p <= 2^(32+s))
  bool smallp;
  bool min_window; // needs u == 0
  bool bound;
  bool lowbit;
  bool stepwin;
  int unroll;      // steps per block
  int per_thread;  // primes per thread (queued walks: a warp covers 32 x this)
};
const VariantTraits& walk_variant_traits(int v);
// Pre-test constants of a normalised job, and whether variant v is exact for it
// (defined in pps_engine.cu).
void walk_args_for_job(const pps_job_params* jp, WalkArgs* a);
// The small-p window of a job: where p is far below 2^(64 - bits(kmax)) the
// hi-word window passes most steps; there K < 2^t or the low t+1-bits(kmax)
// bits zero is tested instead (*t = 32: not used).
void small_p_window_of(const pps_job_params* jp, uint32_t* t, uint32_t* mask);
int walk_variant_exact(const pps_job_params* jp, int v);
// Record an error message for pps_last_error(); returns code.
int set_error_text(int code, const char* msg);
// Largest useful grid for the walk kernel of variant v with `threads` threads
// per block (occupancy-derived); 0 if the variant cannot run this step size.
int walk_max_blocks(int v, int threads, uint32_t step, int num_sms);
// Threads per block of variant v's launch.
int walk_block_threads(int v);
cudaError_t launch_walk(int v, const WalkArgs& a, int blocks, int threads, cudaStream_t st);

// ----------------------------------------------------------------- filter
struct FilterArgs {
  const pps_hit* hits;
  const uint32_t* d_nhits;  // device-side count (clamped to hit_cap inside)
  uint32_t hit_cap;
  uint64_t kstep, koffset;
  uint32_t nmin, nmax;
  int32_t sign;
  const uint16_t* small_q;  // odd primes 3..32749
  uint32_t nsmall;
  pps_factor* out;
  uint32_t* out_count;
  uint32_t out_cap;
  // input sieve file as the output rule instead of small_q: sorted keys
  // (n - nmin) * in_width + (k - kmin) / kstep (pps/app.c:180-183)
  const uint64_t* in_keys = nullptr;
  uint64_t in_n = 0, in_width = 0;
  uint64_t kmin = 0, kmax = 0;
};
cudaError_t launch_filter(const FilterArgs& a, uint32_t max_hits, cudaStream_t st);
// The filters run one CTA of FILTER_THREADS per candidate, over a grid of at
// most FILTER_MAX_BLOCKS that loops over the device-side count.
constexpr uint32_t FILTER_THREADS = 256, FILTER_MAX_BLOCKS = 2048;
inline uint32_t filter_blocks(uint32_t max_hits) {
  return max_hits == 0 ? 1u : (max_hits < FILTER_MAX_BLOCKS ? max_hits : FILTER_MAX_BLOCKS);
}

// ------------------------------------------------------------- utilities
cudaError_t launch_imad_probe(uint32_t* sink, uint32_t iters, int blocks, int threads,
                              cudaStream_t st);

}  // namespace pps
