// pps_sieve.cuh -- device helpers shared by the one-job sieve (pps_kernels.cu)
// and the batched form's wave sieve (pps_batch.cu).
#pragma once
#include <stdint.h>

#include "pps_device.cuh"
#include "pps_internal.h"

namespace pps {

// Writing the primes of one segment in order.  The segment is taken 32 words
// (a chunk) per warp at a time: a scan of the chunk counts gives each chunk's
// place, each lane ranks its word's primes within the chunk (warp scan), the
// warp stages them in shared memory in order and stores them with consecutive
// lanes on consecutive addresses, so the 16 B per prime reach HBM in whole
// lines.
constexpr int EXP_WARPS = SIEVE_THREADS / 32;
constexpr int EXP_CHUNKS = SEG_WORDS / 32;  // chunks of 32 words per segment
constexpr int EXP_STAGE = 256;              // staged primes per warp and round

struct ExpandShared {
  uint32_t chunk_off[EXP_CHUNKS];
  uint64_t stage[EXP_WARPS][EXP_STAGE];
  unsigned long long sum;
  uint32_t total;
};

__device__ __forceinline__ uint32_t warp_excl_scan(uint32_t v, uint32_t lane, uint32_t* total) {
  uint32_t inc = v;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= (uint32_t)o) inc += t;
  }
  *total = __shfl_sync(0xffffffffu, inc, 31);
  return inc - v;
}

// The whole CTA (SIEVE_THREADS threads) expands the segment whose words are gw
// and whose bit 0 is the value seg_val: its primes go to positions seg_base,
// seg_base + 1, ... (those at or past cap are counted, not written), with
// -p^-1 mod 2^64 into pinv64 when it is non-null, or as 32-bit values into
// out32 (OUT32).  Returns, in thread 0, the 64-bit wrapping sum of the
// segment's primes; sh->total holds their count for every thread.
template <bool OUT32>
__device__ uint64_t expand_segment(const uint32_t* gw, uint64_t seg_val, uint64_t seg_base, uint64_t cap,
                                   uint64_t* out64, uint64_t* pinv64, uint32_t* out32, ExpandShared* sh) {
  const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) sh->sum = 0ull;
  for (uint32_t c = wid; c < (uint32_t)EXP_CHUNKS; c += EXP_WARPS) {
    uint32_t t = __popc(gw[c * 32u + lane]);
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (lane == 0) sh->chunk_off[c] = t;
  }
  __syncthreads();
  if (wid == 0) {  // exclusive scan of the chunk counts, 8 chunks per lane
    constexpr int PER = EXP_CHUNKS / 32;
    uint32_t loc[PER], s = 0;
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      loc[i] = sh->chunk_off[lane * PER + i];
      s += loc[i];
    }
    uint32_t tot;
    uint32_t run = warp_excl_scan(s, lane, &tot);
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      sh->chunk_off[lane * PER + i] = run;
      run += loc[i];
    }
    if (lane == 0) sh->total = tot;
  }
  __syncthreads();
  uint64_t sum = 0;
  for (uint32_t c = wid; c < (uint32_t)EXP_CHUNKS; c += EXP_WARPS) {
    const uint32_t v = gw[c * 32u + lane];
    uint32_t total;
    const uint32_t excl = warp_excl_scan(__popc(v), lane, &total);
    const uint64_t out_base = seg_base + sh->chunk_off[c];
    const uint64_t word_val = seg_val + 2ull * ((c * 32u + lane) * 32u);
    for (uint32_t done = 0; done < total; done += EXP_STAGE) {
      uint32_t vv = v, r = excl;
      while (vv) {
        const uint32_t bit = __ffs(vv) - 1u;
        vv &= vv - 1u;
        if (r >= done && r < done + EXP_STAGE) sh->stage[wid][r - done] = word_val + 2ull * bit;
        ++r;
      }
      __syncwarp();
      const uint32_t n = min((uint32_t)EXP_STAGE, total - done);
      for (uint32_t i = lane; i < n; i += 32u) {
        const uint64_t p = sh->stage[wid][i];
        const uint64_t pos = out_base + done + i;
        sum += p;
        if (pos < cap) {
          if (OUT32) {
            out32[pos] = (uint32_t)p;
          } else {
            out64[pos] = p;
            if (pinv64) pinv64[pos] = neg_inv64(p);
          }
        }
      }
      __syncwarp();
    }
  }
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
  if (lane == 0) atomicAdd(&sh->sum, (unsigned long long)sum);
  __syncthreads();
  return sh->sum;
}

}  // namespace pps
