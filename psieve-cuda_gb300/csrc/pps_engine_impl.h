// pps_engine_impl.h -- engine state shared by the library's host translation
// units (pps_engine.cu, pps_batch.cu, pps_server.cu).  Not part of the ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <vector>

#include "pps_internal.h"
#include "ppsgpu.h"

// Record an error for pps_last_error(); returns code.
int set_err(int code, const char* fmt, ...);

#define CU(call)                                                                         \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return set_err(PPS_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_),      \
                     __FILE__, __LINE__);                                                \
  } while (0)

// Host-side fault injection (pps_debug_fail_allocs): true when this device
// allocation is to fail as if device memory were exhausted.
bool alloc_fault_injected();
// pps_debug_limits: the warp-queue cap of the queued walks (512 unless set) and
// the raw-candidate cap of each call's first attempt (0: none).
uint32_t debug_queue_cap();
uint32_t debug_first_hit_cap();

// Device buffer that only grows (contents are not preserved on growth).  A
// failed growth leaves it empty (p null, n 0): whatever cached a pointer into
// it must be invalidated before the call.
template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  int ensure(size_t want) {
    if (want <= n) return PPS_OK;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    size_t grow = want + want / 8;
    if (alloc_fault_injected())
      return set_err(PPS_ERR_INSUFFICIENT_RESOURCE, "cudaMalloc(%zu bytes): injected failure",
                     grow * sizeof(T));
    cudaError_t e = cudaMalloc(&p, grow * sizeof(T));
    if (e != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      return set_err(PPS_ERR_INSUFFICIENT_RESOURCE, "cudaMalloc(%zu bytes): %s",
                     grow * sizeof(T), cudaGetErrorString(e));
    }
    n = grow;
    return PPS_OK;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  size_t bytes() const { return n * sizeof(T); }
};

struct BatchState;  // pps_batch.cu

struct pps_engine {
  int device = 0;
  int num_sms = 0;
  cudaStream_t st = nullptr;
  cudaEvent_t ev[8] = {};
  uint64_t batch_span = 1ull << 31;
  int forced_variant = -1;
  // tuned walk variant per set of exact variants (bit v: variant v is exact),
  // with the work (primes x steps) of the sample it was timed on
  struct Tuned {
    uint64_t mask;
    int variant;
    uint64_t work;
  };
  std::vector<Tuned> tuned_variant;
  // threads per prime of the queued walks: forced (0: tuned), and the tuned
  // choice per (variant set, variant, log2 primes, log2 steps)
  int forced_split = 0;
  uint32_t wave_segs_req = 0;  // batched form: segments per wave (0: the maximum)
  int forced_bwalk = 0;        // batched form: forced walk kernel code (0: tuned)
  uint32_t hit_cap_limit = 0;  // the raw-candidate cap of this attempt (0: the buffer's size)
  struct TunedSplit {
    uint64_t mask;
    int variant;
    int lg_np, lg_steps;
    uint32_t split;
  };
  std::vector<TunedSplit> tuned_split;
  uint64_t launches = 0;

  // sieving primes (ascending odd primes <= base_limit), u32
  DevBuf<uint32_t> base_q;
  uint32_t base_limit = 0;
  uint32_t base_count = 0;
  std::map<uint32_t, uint32_t> base_le;  // primes <= limit in the table, per limit asked
  std::vector<uint32_t> host_seed;  // odd primes < SEG_BITS (host copy)
  DevBuf<uint32_t> seed_q;

  DevBuf<uint32_t> bitmap, seg_count, seg_off;
  DevBuf<uint64_t> P, Pinv;
  DevBuf<uint64_t> totals;  // [0] count, [1] sum
  DevBuf<pps_hit> hits;
  DevBuf<pps_factor> factors;
  DevBuf<uint32_t> counters;  // [0] raw hits, [1] factors
  DevBuf<uint16_t> small_q;
  DevBuf<uint32_t> presieve;  // the pre-sieve table for 3, 5, 7, 11, 13 (PRESIEVE_WORDS)
  DevBuf<uint32_t> sieve_res; // per-batch residues of the small sieving primes
  uint32_t nsmall = 0;
  DevBuf<uint32_t> probe_sink;
  uint64_t* h_pinned = nullptr;  // 16 words of pinned host scratch

  BatchState* batch = nullptr;  // state of the batched persistent form

  // input sieve file as the output rule (pps_engine_set_input), and its key
  // table for the job it was last built for
  const pps_input* input = nullptr;
  DevBuf<uint64_t> in_keys;
  uint64_t in_n = 0, in_width = 0;
  bool in_built = false;
  pps_job_params in_job{};
};

// Sorted bit numbers of the input file's bitmap for one job (pps_input.cu).
int input_keys_for_job(const pps_input* in, const pps_job_params* jp, std::vector<uint64_t>* keys,
                       uint64_t* width);

struct BaseTable {
  uint32_t nq, nq_tiny, nq_seg;
};

uint32_t isqrt64(uint64_t x);
// Device table of odd sieving primes q <= min(qmax, sqrt(pmax-1)), with counts.
int prepare_sieving_primes(pps_engine* e, uint32_t qmax, uint64_t pmax, const uint32_t** dq,
                           BaseTable* bt);
void batch_state_free(pps_engine* e);

// ---- wave-level interface of the batched form (pps_batch.cu), shared by
// pps_run_batch and the serving loop (pps_server.cu).  Jobs live in device
// slots; a wave walks pieces (p sub-ranges of slotted jobs) and returns the
// survivors of the output rule, sorted by (slot, p, k, n).
struct BatchPiece {
  uint64_t lo, hi;  // p in [lo, hi)
  uint32_t slot;
};
// A wave's candidates and survivors: idx = job slot | side bit (set: k*2^n+1).
constexpr uint32_t BATCH_SIDE_PROTH = 0x80000000u;
inline uint32_t batch_hit_slot(const pps_hit& h) { return h.idx & ~BATCH_SIDE_PROTH; }
inline int32_t batch_hit_sign(const pps_hit& h) { return (h.idx & BATCH_SIDE_PROTH) ? 1 : -1; }
inline bool batch_hit_less(const pps_hit& x, const pps_hit& y) {  // (slot, p, k, n)
  if (batch_hit_slot(x) != batch_hit_slot(y)) return batch_hit_slot(x) < batch_hit_slot(y);
  if (x.p != y.p) return x.p < y.p;
  if (x.k != y.k) return x.k < y.k;
  return x.n < y.n;
}
uint32_t batch_max_slots();
uint64_t batch_wave_segments(const pps_engine* e);  // segments one wave holds
uint64_t batch_piece_segments(uint64_t lo, uint64_t hi);
uint64_t batch_max_piece_span();         // p range of one full batch
uint64_t batch_piece_span(const pps_engine* e);     // widest p range of one piece on this engine
int batch_prepare(pps_engine* e);
// normalised jobs into slots [slot0, slot0 + n); their prime counters start at zero
int batch_set_jobs(pps_engine* e, uint32_t slot0, const pps_job_params* jobs, size_t n);
int batch_wave(pps_engine* e, const BatchPiece* pieces, size_t n, std::vector<pps_hit>* survivors,
               uint64_t* raw_hits, double* filter_ms);
int batch_job_counts(pps_engine* e, uint32_t slot0, size_t n, uint64_t* primes, uint64_t* sums);
void batch_tuning(pps_engine* e, uint32_t* work, uint32_t* unroll);
