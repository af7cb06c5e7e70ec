// pps_kernels.cu -- sm_103a kernels of the PPSieve hot path.
//
//   k_sieve_large / k_sieve_seg / k_scan_counts / k_expand
//       segmented sieve of Eratosthenes (reference: sieve.c:168-608 on the host).
//       Candidates live as bits in shared memory; the primes and their
//       Montgomery constants are written to HBM in order.
//   k_walk<...>
//       per-prime walk over n (reference: pps/appcu.cu:1120-1190 + 803-1115 for
//       the flags, pps/app.c:1037-1121 for the exact (k, n)).  One thread owns
//       one prime; 2^-nmin mod p by Montgomery exponentiation, then one
//       reduction per `step` values of n, a cheap pre-test per step, and an
//       exact count-trailing-zeros test on the rare candidates.  Hits are
//       appended through one atomic per warp (ballot + popc ranks).
//   k_filter
//       output rule of pps/app.c:159-186 + pps/factor_proth.c:247-253 on the raw
//       hits: one CTA per hit, its threads split the odd primes below 32768.
//   k_imad_probe
//       multiply-pipe throughput probe on the walk's multiply mix.
#include <cuda_runtime.h>
#include <stdint.h>

#include "pps_device.cuh"
#include "pps_internal.h"
#include "pps_sieve.cuh"

namespace pps {

// ===================================================================== sieve

__device__ __forceinline__ uint64_t first_odd_multiple(uint64_t q, uint64_t lo) {
  // smallest odd multiple of odd q that is >= max(lo, q*q); lo odd
  uint64_t st = q * q;
  if (st < lo) {
    const uint64_t r = lo % q;
    st = r ? lo + (q - r) : lo;
    if ((st & 1ull) == 0ull) st += q;
  }
  return st;
}

// Primes q >= SEG_BITS hit a segment at most once: one thread per prime walks
// its multiples through the whole batch and clears them in the global bitmap.
__global__ void k_sieve_large(SieveBatch b) {
  const uint64_t hi = b.lo + 2ull * b.nbits;
  for (uint32_t i = b.nq_seg + blockIdx.x * blockDim.x + threadIdx.x; i < b.nq;
       i += gridDim.x * blockDim.x) {
    const uint64_t q = b.q[i];
    if (q * q >= hi) continue;
    const uint64_t st = first_odd_multiple(q, b.lo);
    for (uint64_t j = (st - b.lo) >> 1; j < b.nbits; j += q)
      atomicAnd(&b.bitmap[j >> 5], ~(1u << (j & 31u)));
  }
}

void presieve_table(uint32_t* out) {
  for (uint32_t x = 0; x < PRESIEVE_MOD; ++x) {
    uint32_t m = 0;
    for (uint32_t bit = 0; bit < 32; ++bit) {
      const uint32_t v = (x + 2u * bit) % PRESIEVE_MOD;
      if (v % 3u == 0 || v % 5u == 0 || v % 7u == 0 || v % 11u == 0 || v % 13u == 0) m |= 1u << bit;
    }
    out[x] = m;
  }
}

// Per-batch residues of the small sieving primes (see SieveBatch::res).
__global__ void k_sieve_res(SieveBatch b) {
  for (uint32_t i = b.nq_tiny + blockIdx.x * blockDim.x + threadIdx.x; i < b.nq_seg; i += gridDim.x * blockDim.x) {
    const uint32_t q = b.q[i];
    b.res[2 * (i - b.nq_tiny)] = (uint32_t)(b.lo % q);
    b.res[2 * (i - b.nq_tiny) + 1] = (2u * SEG_BITS) % q;
  }
}

__global__ void __launch_bounds__(SIEVE_THREADS) k_sieve_seg(SieveBatch b, int have_large) {
  __shared__ uint32_t sb[SEG_WORDS];
  __shared__ uint32_t warp_cnt[SIEVE_THREADS / 32];
  const uint32_t seg = blockIdx.x;
  const uint64_t seg_first = (uint64_t)seg * SEG_BITS;
  const uint64_t left = b.nbits - seg_first;
  const uint32_t bits = left < SEG_BITS ? (uint32_t)left : SEG_BITS;
  const uint64_t seg_lo = b.lo + 2ull * seg_first;
  const uint64_t seg_hi = seg_lo + 2ull * bits;
  uint32_t* gw = b.bitmap + (size_t)seg * SEG_WORDS;
  // the pre-sieve table's entry for word w is at (seg_lo + 64 w) mod 15015
  const bool pre = b.presieve != nullptr && b.nq_tiny >= PRESIEVE_PRIMES;
  const uint32_t x0 = pre ? (uint32_t)(seg_lo % PRESIEVE_MOD) : 0u;
  const uint32_t xstep = (64u * SIEVE_THREADS) % PRESIEVE_MOD;
  uint32_t x = pre ? (x0 + 64u * threadIdx.x) % PRESIEVE_MOD : 0u;

  for (uint32_t w = threadIdx.x; w < SEG_WORDS; w += blockDim.x) {
    uint32_t v = have_large ? gw[w] : 0xffffffffu;
    if (pre) {
      v &= ~__ldg(b.presieve + x);
      x += xstep;
      if (x >= PRESIEVE_MOD) x -= PRESIEVE_MOD;
    }
    const uint32_t j0 = w * 32u;
    if (j0 >= bits) v = 0u;
    else if (bits - j0 < 32u) v &= (1u << (bits - j0)) - 1u;
    sb[w] = v;
  }
  __syncthreads();
  if (pre && seg_lo <= 13u && threadIdx.x == 0) {
    // the five pre-sieved primes themselves are primes
    for (uint32_t q = 3; q <= 13; q += 2)
      if (q != 9 && q >= seg_lo && q < seg_hi) {
        const uint32_t j = (uint32_t)((q - seg_lo) >> 1);
        sb[j >> 5] |= 1u << (j & 31u);
      }
  }
  __syncthreads();

  // tiny primes: the CTA strides one q at a time
  for (uint32_t i = pre ? PRESIEVE_PRIMES : 0; i < b.nq_tiny; ++i) {
    const uint64_t q = b.q[i];
    if (q * q >= seg_hi) break;
    const uint64_t st = first_odd_multiple(q, seg_lo);
    for (uint64_t j = ((st - seg_lo) >> 1) + (uint64_t)threadIdx.x * q; j < bits;
         j += (uint64_t)blockDim.x * q)
      atomicAnd(&sb[j >> 5], ~(1u << (j & 31u)));
  }
  // small primes: one thread per q
  const uint32_t qend = b.nq_seg < b.nq ? b.nq_seg : b.nq;
  for (uint32_t i = b.nq_tiny + threadIdx.x; i < qend; i += blockDim.x) {
    const uint64_t q = b.q[i];
    if (q * q >= seg_hi) continue;
    const uint32_t qq = (uint32_t)q;
    uint32_t j;
    if (b.res != nullptr && q * q <= seg_lo) {
      // seg_lo mod q from the batch's residues, in 32 bits (seg < 2^13, q < 2^18)
      const uint32_t r = (b.res[2 * (i - b.nq_tiny)] + b.res[2 * (i - b.nq_tiny) + 1] * seg) % qq;
      uint32_t d = r ? qq - r : 0u;  // seg_lo + d is the first multiple of q >= seg_lo
      if (d & 1u) d += qq;           // seg_lo is odd: the odd multiple
      j = d >> 1;
    } else {
      j = (uint32_t)((first_odd_multiple(q, seg_lo) - seg_lo) >> 1);
    }
    for (; j < bits; j += qq) atomicAnd(&sb[j >> 5], ~(1u << (j & 31u)));
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
    b.seg_count[seg] = t;
  }
}

// Exclusive scan of the per-segment counts (one CTA).
__global__ void __launch_bounds__(1024) k_scan_counts(const uint32_t* cnt, uint32_t* off, uint32_t n,
                                                      uint64_t* d_total) {
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
  if (threadIdx.x == blockDim.x - 1) d_total[0] = part[threadIdx.x];
}

// One CTA per segment: rank the set bits and write the primes in order
// (expand_segment, pps_sieve.cuh).
template <bool OUT32>
__global__ void __launch_bounds__(SIEVE_THREADS) k_expand(SieveBatch b, uint64_t* out64, uint64_t* pinv64,
                                                          uint32_t* out32) {
  __shared__ ExpandShared sh;
  const uint32_t seg = blockIdx.x;
  const uint64_t sum = expand_segment<OUT32>(b.bitmap + (size_t)seg * SEG_WORDS,
                                             b.lo + 2ull * (uint64_t)seg * SEG_BITS, b.seg_off[seg], ~0ull,
                                             out64, pinv64, out32, &sh);
  if (threadIdx.x == 0) atomicAdd((unsigned long long*)&b.d_total[1], (unsigned long long)sum);
}

__global__ void k_count_le(const uint32_t* q, uint32_t n, uint32_t x, uint32_t* out) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = lo + (hi - lo) / 2;
    if (q[mid] <= x) lo = mid + 1; else hi = mid;
  }
  *out = lo;
}

cudaError_t launch_count_le(const uint32_t* q, uint32_t n, uint32_t x, uint32_t* out, cudaStream_t st) {
  k_count_le<<<1, 1, 0, st>>>(q, n, x, out);
  return cudaGetLastError();
}

int launch_sieve_batch(const SieveBatch& b, uint64_t* out64, uint64_t* pinv64, uint32_t* out32,
                       cudaStream_t st) {
  int launches = 0;
  if (b.res && b.nq_seg > b.nq_tiny) {
    const uint32_t n = b.nq_seg - b.nq_tiny;
    k_sieve_res<<<(n + 255) / 256, 256, 0, st>>>(b);
    ++launches;
  }
  const int have_large = b.nq > b.nq_seg;
  if (have_large) {
    cudaMemsetAsync(b.bitmap, 0xff, (size_t)b.nseg * SEG_WORDS * sizeof(uint32_t), st);
    const uint32_t nl = b.nq - b.nq_seg;
    uint32_t blocks = (nl + 255) / 256;
    if (blocks > 65535u * 4u) blocks = 65535u * 4u;
    k_sieve_large<<<blocks, 256, 0, st>>>(b);
    ++launches;
  }
  k_sieve_seg<<<b.nseg, SIEVE_THREADS, 0, st>>>(b, have_large);
  k_scan_counts<<<1, 1024, 0, st>>>(b.seg_count, b.seg_off, b.nseg, b.d_total);
  if (out32)
    k_expand<true><<<b.nseg, SIEVE_THREADS, 0, st>>>(b, nullptr, nullptr, out32);
  else
    k_expand<false><<<b.nseg, SIEVE_THREADS, 0, st>>>(b, out64, pinv64, nullptr);
  launches += 3;
  return launches;
}

// ====================================================================== walk

// Pre-tests: never reject a true candidate K = k 2^i (k <= kmax, i < step).
// Window: if i < t then K < kmax 2^t <= 2^(32+u), i.e. hi word < 2^u; otherwise
// the low t bits are zero.  win_hi = 2^u - 1, win_mask = 2^t - 1, t = 32+u-bits(kmax).
// Low bit: with 2^i the lowest set bit of the low word, K <= kmax 2^i implies
// hi word <= hi32(kmax 2^i); a zero low word always passes.
template <int TEST>
__device__ __forceinline__ bool pretest(uint32_t klo, uint32_t khi, const WalkArgs& a) {
  if (TEST == 0) {
    return (khi <= a.win_hi) | ((klo & a.win_mask) == 0u);
  } else {
    const uint32_t lb = klo & (0u - klo);
    return (lb == 0u) | (khi <= __umulhi(a.kmax32, lb));
  }
}

__device__ __forceinline__ void exact_check(const WalkArgs& a, uint32_t klo, uint32_t khi, uint32_t n,
                                            uint64_t p, uint32_t idx) {
  const uint32_t i = klo ? (uint32_t)(__ffs(klo) - 1) : (uint32_t)(31 + __ffs(khi));
  const uint64_t k = mk64(klo, khi) >> (i & 63u);
  const bool hit = (i < a.step) && (k <= a.kmax) && (k >= a.kmin) && (n + i < a.nmax);
  const unsigned act = __activemask();
  const unsigned hm = __ballot_sync(act, hit);
  if (hm) {
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(hm) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(a.hit_count, (uint32_t)__popc(hm));
    base = __shfl_sync(act, base, leader);
    if (hit) {
      const uint32_t pos = base + (uint32_t)__popc(hm & ((1u << lane) - 1u));
      if (pos < a.hit_cap) {
        pps_hit h;
        h.p = p;
        h.k = k;
        h.n = n + i;
        h.idx = idx;
        a.hits[pos] = h;
      }
    }
  }
}

template <int FORM, bool S32>
__device__ __forceinline__ void walk_step(uint32_t& klo, uint32_t& khi, uint32_t plo, uint32_t phi,
                                          uint32_t pinv_s, uint32_t s) {
  if (FORM == 1 && S32) {
    step_chain32(klo, khi, plo, phi, pinv_s);
  } else if (FORM == 2) {
    step_form2<S32>(klo, khi, plo, phi, pinv_s, s);
  } else {
    step_form0<S32>(klo, khi, plo, phi, pinv_s, s);
  }
}

// One thread walks ILP primes side by side.  With BLOCK, the pre-test result is
// OR-ed into a flag over U unrolled steps and only a flagged block is replayed
// from its saved starting value with the exact test (the replay recomputes the
// same values, so the walk continues from the already computed end value).
// Without BLOCK the pre-test branches every step.
template <int FORM, int TEST, int U, bool S32, int ILP, bool BLOCK>
__global__ void __launch_bounds__(256) k_walk(WalkArgs a) {
  const uint64_t np = a.d_np ? *a.d_np : a.np;
  const uint32_t s = S32 ? 32u : a.step;
  const uint64_t gstride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; base < np;
       base += gstride * ILP) {
    uint32_t klo[ILP], khi[ILP], plo[ILP], phi[ILP], pinv_s[ILP], idx[ILP];
    uint64_t p[ILP];
    bool valid[ILP];
#pragma unroll
    for (int j = 0; j < ILP; ++j) {
      const uint64_t pi = base + (uint64_t)j * gstride;
      valid[j] = pi < np;
      p[j] = a.P[valid[j] ? pi : base];
      const uint64_t ps = a.Pinv ? a.Pinv[valid[j] ? pi : base] : neg_inv64(p[j]);
      const uint64_t x = inv_pow2(a.nmin, p[j], ps);
      const uint64_t K = a.proth ? p[j] - x : x;
      klo[j] = lo32(K);
      khi[j] = hi32(K);
      plo[j] = lo32(p[j]);
      phi[j] = hi32(p[j]);
      pinv_s[j] = S32 ? lo32(ps) : (lo32(ps) << (32u - s));
      idx[j] = a.idx_base + (uint32_t)pi;
    }
    uint32_t n = a.nmin;
    uint32_t t = 0;
    for (; t + U <= a.nsteps; t += U) {
      if (BLOCK) {
        uint32_t slo[ILP], shi[ILP];
        bool f[ILP];
#pragma unroll
        for (int j = 0; j < ILP; ++j) {
          slo[j] = klo[j];
          shi[j] = khi[j];
          f[j] = false;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
#pragma unroll
          for (int j = 0; j < ILP; ++j) {
            f[j] |= pretest<TEST>(klo[j], khi[j], a);
            walk_step<FORM, S32>(klo[j], khi[j], plo[j], phi[j], pinv_s[j], s);
          }
        }
        bool any = false;
#pragma unroll
        for (int j = 0; j < ILP; ++j) any |= f[j] & valid[j];
        if (any) {
#pragma unroll
          for (int j = 0; j < ILP; ++j) {
            if (f[j] && valid[j]) {
              uint32_t rlo = slo[j], rhi = shi[j];
#pragma unroll 1
              for (int u = 0; u < U; ++u) {
                if (pretest<TEST>(rlo, rhi, a)) exact_check(a, rlo, rhi, n + (uint32_t)u * s, p[j], idx[j]);
                walk_step<FORM, S32>(rlo, rhi, plo[j], phi[j], pinv_s[j], s);
              }
            }
          }
        }
      } else {
#pragma unroll
        for (int u = 0; u < U; ++u) {
#pragma unroll
          for (int j = 0; j < ILP; ++j) {
            if (valid[j] && pretest<TEST>(klo[j], khi[j], a))
              exact_check(a, klo[j], khi[j], n + (uint32_t)u * s, p[j], idx[j]);
            walk_step<FORM, S32>(klo[j], khi[j], plo[j], phi[j], pinv_s[j], s);
          }
        }
      }
      n += (uint32_t)U * s;
    }
    for (; t < a.nsteps; ++t) {
#pragma unroll
      for (int j = 0; j < ILP; ++j) {
        if (valid[j] && pretest<TEST>(klo[j], khi[j], a)) exact_check(a, klo[j], khi[j], n, p[j], idx[j]);
        walk_step<FORM, S32>(klo[j], khi[j], plo[j], phi[j], pinv_s[j], s);
      }
      n += s;
    }
  }
}

// ---- queued 32-bit-step walk.  The hot loop only appends (lane, block) to a
// per-warp queue in shared memory when a block of U steps is flagged; after the
// warp's primes finish their walk, the warp re-checks the queued blocks together
// (one block per lane), recomputing each block's starting value as
// -/+2^-(nmin + 32 U b) mod p.  The hot loop thus holds no exact-check code.
//
// Threads per prime (a.nsplit = T): the n range's blocks are cut into T parts
// of L = ceil(blocks / T) blocks, and part j of every prime is walked by its
// own thread, starting from -/+2^-(nmin + s U j L) mod p (the same start value
// the queue re-check computes).  Virtual threads are numbered part-major over
// the prime count rounded up to 32, so each warp holds 32 consecutive primes
// of one part (every lane runs the same number of blocks).  A job with fewer
// primes than the GPU holds threads then still fills every SM (the
// reference's per-launch n slices, pps/appcu.cu:337-357, split n the same way
// but across launches).
constexpr int WQ_CAP = WALK_QUEUE_CAP;   // queue entries per warp
constexpr int WQ_WARPS = 8;   // warps per 256-thread block

__device__ __forceinline__ void record_exact(uint32_t klo, uint32_t khi, uint32_t n, uint64_t p, uint32_t idx,
                                             uint64_t kmin, uint64_t kmax, uint32_t nmax, pps_hit* hits,
                                             uint32_t* hit_count, uint32_t hit_cap, uint32_t step = 32u) {
  const uint32_t i = klo ? (uint32_t)(__ffs(klo) - 1) : (uint32_t)(31 + __ffs(khi));
  const uint64_t k = mk64(klo, khi) >> (i & 63u);
  const bool hit = (i < step) && (k <= kmax) && (k >= kmin) && (n + i < nmax);
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
        h.idx = idx;
        hits[pos] = h;
      }
    }
  }
}

// The queued walk step: FORM 0 is the REDC by 2^32 (s = 32) in the form without
// low-word carries (step_neg32); FORM 1 walks s < 32 through the same step on
// K * 2^(32-s), exact while p <= 2^(32+s)
// ((K + m p) / 2^s == (K 2^(32-s) + m 2^(32-s) p) / 2^32).
// pinv is lo32(-p^-1) for FORM 0 and that << sh for FORM 1 (q_pinv).
template <int FORM>
__device__ __forceinline__ void q_step(uint32_t& klo, uint32_t& khi, uint32_t plon, uint32_t phi1, uint32_t pinv,
                                       uint32_t sh) {
  if (FORM == 0)
    step_neg32(klo, khi, plon, phi1, pinv);
  else
    step_neg32s(klo, khi, plon, phi1, pinv, sh);
}

template <int FORM>
__device__ __forceinline__ uint32_t q_pinv(uint64_t ps, uint32_t sh) {
  return FORM == 0 ? lo32(ps) : lo32(ps) << sh;
}

// A twin job's candidates carry their side in idx bit 31 (set: k*2^n+1).
constexpr uint32_t HIT_SIDE_PROTH = 0x80000000u;

// SH: the small-p window (K < 2^sh_t or the low bits in sh_mask zero) in place
// of the hi-word window, for p far below 2^(64 - bits(kmax)).
// TW: a twin job: the walk holds K = 2^-n, the -1 side's value, and tests
// p - K, the +1 side's, at the same step (the reference's twin build walks
// once for both sides too, pps/app.c:1071-1107).
template <int TEST, int U, int MINB, int FORM = 0, bool SH = false, bool TW = false>
__global__ void __launch_bounds__(256, MINB) k_walk32q(WalkArgs a) {
  __shared__ uint32_t q_ent[WQ_WARPS][WQ_CAP];
  __shared__ uint64_t q_p[WQ_WARPS][32];
  __shared__ uint64_t q_k[WQ_WARPS][32];  // start value of each lane's partial last block
  __shared__ uint32_t q_cnt[WQ_WARPS];
  const uint64_t np = a.d_np ? *a.d_np : a.np;
  const uint32_t win_hi = a.win_hi, win_mask = SH ? a.sh_mask : a.win_mask, bound_hi = a.bound_hi;
  const uint32_t sh_t = a.sh_t, sw_mask = a.sw_mask;
  const uint32_t s = FORM == 0 ? 32u : a.step, sh = 32u - s;
  const uint32_t nsteps = a.nsteps, nmin = a.nmin;
  const uint32_t full = nsteps / (uint32_t)U;  // whole blocks of U steps
  const uint32_t nsplit = a.nsplit > 1u ? a.nsplit : 1u;
  const uint32_t part = (full + nsplit - 1u) / nsplit;  // blocks per part
  const uint64_t npad = (np + 31ull) & ~31ull;
  const uint64_t nvirt = npad * nsplit;
  const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
  const uint64_t wstride = (uint64_t)gridDim.x * blockDim.x;
  const uint32_t qcap = min(a.qcap, (uint32_t)WQ_CAP);  // entries used (a test hook lowers it)
  if (lane == 0) q_cnt[wib] = 0;
  __syncwarp();
  for (uint64_t vbase = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); vbase < nvirt;
       vbase += wstride) {
    const uint32_t j = nsplit > 1u ? (uint32_t)(vbase / npad) : 0u;  // the part, warp-uniform
    const uint64_t base = vbase - (uint64_t)j * npad;                // first prime of the warp
    // (parts past the last whole block start at it: the last part then
    // holds just the partial block, whose start value is computed at `full`)
    const uint32_t b_lo = min(full, j * part), b_hi = min(full, b_lo + part);
    const bool last_part = j == nsplit - 1u;
    const uint64_t pi = base + lane;
    const bool valid = pi < np;
    const uint64_t p = a.P[valid ? pi : (base < np ? base : 0)];
    q_p[wib][lane] = p;
    if (valid) {
      const uint64_t ps = a.Pinv ? a.Pinv[pi] : neg_inv64(p);
      const uint32_t plon = neg_lo(p), phi1 = neg_hi(p), pinv = q_pinv<FORM>(ps, sh);
      const uint64_t x = inv_pow2(nmin + s * (uint32_t)U * b_lo, p, ps);
      const uint64_t K = a.proth ? p - x : x;
      uint32_t klo = lo32(K), khi = hi32(K);
      // twin: p - K is below the window bound `lim` iff K > p - lim, and its low
      // bits are zero iff K's equal p's (lim = 0 stands for 2^64)
      uint64_t tw_above = 0;
      uint32_t tw_low = 0;
      if (TW) {
        const uint64_t lim = SH ? (1ull << sh_t) : (win_hi == 0xffffffffu ? 0ull : ((uint64_t)win_hi + 1ull) << 32);
        tw_above = (lim != 0ull && p > lim) ? p - lim : 0ull;
        tw_low = lo32(p) & win_mask;
      }
      for (uint32_t b = b_lo; b < b_hi; ++b) {
        uint32_t acc = 0xffffffffu;
        bool f = false;
#pragma unroll
        for (int u = 0; u < U; ++u) {
          if (TEST == 3) {
            // walk form 1: the window K < 2^s is the step's own high word
            // (K >> s) being zero; otherwise the low s+1-kb bits of K are zero
            const uint32_t hi = __funnelshift_l(klo, khi, sh);
            acc = min(acc, min(hi, klo & sw_mask));
            neg_sum(klo * pinv, hi, plon, phi1, klo, khi);
            continue;
          }
          if (TEST == 0) acc = min(acc, min(SH ? __funnelshift_rc(klo, khi, sh_t) : khi, klo & win_mask));
          else if (TEST == 1) f |= (SH ? __funnelshift_rc(klo, khi, sh_t) == 0u : khi <= win_hi) | ((klo & win_mask) == 0u);
          else f |= khi <= bound_hi;
          if (TW) f |= (mk64(klo, khi) > tw_above) | ((klo & win_mask) == tw_low);
          q_step<FORM>(klo, khi, plon, phi1, pinv, sh);
        }
        if (TEST == 0 || TEST == 3) f |= acc == 0u;
        if (f) {
          const uint32_t pos = atomicAdd(&q_cnt[wib], 1u);
          if (pos < qcap) q_ent[wib][pos] = (lane << 27) | b;
        }
      }
      // the last partial block (fewer than U steps) always goes to the queue,
      // with its start value, which is at hand (in the last part)
      if (last_part && full * (uint32_t)U < nsteps) {
        q_k[wib][lane] = mk64(klo, khi);
        const uint32_t pos = atomicAdd(&q_cnt[wib], 1u);
        if (pos < qcap) q_ent[wib][pos] = (lane << 27) | full;
      }
    }
    __syncwarp();
    const uint32_t cnt = q_cnt[wib];
    if (cnt <= qcap) {
      // re-check the queued blocks exactly, one block per lane
      for (uint32_t e = lane; e < cnt; e += 32u) {
        const uint32_t ent = q_ent[wib][e];
        const uint32_t owner = ent >> 27, blk = ent & ((1u << 27) - 1u);
        const uint64_t op = q_p[wib][owner];
        const uint64_t ops = neg_inv64(op);
        const uint32_t t0 = (uint32_t)U * blk;
        const uint32_t nblk = min((uint32_t)U, nsteps - t0);
        const uint32_t n0 = nmin + s * t0;
        uint64_t K;
        if (blk == full) {
          K = q_k[wib][owner];
        } else {
          const uint64_t x = inv_pow2(n0, op, ops);
          K = a.proth ? op - x : x;
        }
        uint32_t klo = lo32(K), khi = hi32(K);
        const uint32_t oplon = neg_lo(op), ophi1 = neg_hi(op), opinv = q_pinv<FORM>(ops, sh);
#pragma unroll 1
        for (uint32_t u = 0; u < nblk; ++u) {
          const uint32_t idx = a.idx_base + (uint32_t)(base + owner);
          record_exact(klo, khi, n0 + s * u, op, idx, a.kmin, a.kmax, a.nmax, a.hits, a.hit_count, a.hit_cap, s);
          if (TW) {
            const uint64_t v = op - mk64(klo, khi);
            record_exact(lo32(v), hi32(v), n0 + s * u, op, idx | HIT_SIDE_PROTH, a.kmin, a.kmax, a.nmax, a.hits,
                         a.hit_count, a.hit_cap, s);
          }
          q_step<FORM>(klo, khi, oplon, ophi1, opinv, sh);
        }
      }
    } else if (valid) {
      // queue overflow (not expected at the designed false-pass rates): each
      // lane re-walks its own part of its prime with the exact test at every step
      const uint64_t p = q_p[wib][lane];
      const uint64_t ps = neg_inv64(p);
      const uint32_t t_lo = (uint32_t)U * b_lo, t_hi = last_part ? nsteps : (uint32_t)U * b_hi;
      const uint64_t x = inv_pow2(nmin + s * t_lo, p, ps);
      const uint64_t K = a.proth ? p - x : x;
      uint32_t klo = lo32(K), khi = hi32(K);
      const uint32_t plon = neg_lo(p), phi1 = neg_hi(p), pinv = q_pinv<FORM>(ps, sh);
#pragma unroll 1
      for (uint32_t t = t_lo; t < t_hi; ++t) {
        const uint32_t idx = a.idx_base + (uint32_t)pi;
        record_exact(klo, khi, nmin + s * t, p, idx, a.kmin, a.kmax, a.nmax, a.hits, a.hit_count, a.hit_cap, s);
        if (TW) {
          const uint64_t v = p - mk64(klo, khi);
          record_exact(lo32(v), hi32(v), nmin + s * t, p, idx | HIT_SIDE_PROTH, a.kmin, a.kmax, a.nmax, a.hits,
                       a.hit_count, a.hit_cap, s);
        }
        q_step<FORM>(klo, khi, plon, phi1, pinv, sh);
      }
    }
    __syncwarp();
    if (lane == 0) q_cnt[wib] = 0;
    __syncwarp();
  }
}

// ---- queued walk, two primes per thread.  The same walk as k_walk32q for
// 32-bit steps (window as a running minimum, TEST 0, or the single bound,
// TEST 2), with lane l of a warp walking primes base + l and base + 32 + l
// side by side, so that each thread holds two independent step chains (their
// multiplies interleave).  A warp covers 64 primes of one n part; queue
// entries carry the prime's slot (0..63) in their top 6 bits.
template <int TEST, int U, int MINB>
__global__ void __launch_bounds__(256, MINB) k_walk32q2(WalkArgs a) {
  __shared__ uint32_t q_ent[WQ_WARPS][WQ_CAP];
  __shared__ uint64_t q_p[WQ_WARPS][64];
  __shared__ uint64_t q_k[WQ_WARPS][64];
  __shared__ uint32_t q_cnt[WQ_WARPS];
  const uint64_t np = a.d_np ? *a.d_np : a.np;
  const uint32_t win_mask = a.win_mask, bound_hi = a.bound_hi;
  const uint32_t nsteps = a.nsteps, nmin = a.nmin;
  const uint32_t full = nsteps / (uint32_t)U;
  const uint32_t nsplit = a.nsplit > 1u ? a.nsplit : 1u;
  const uint32_t part = (full + nsplit - 1u) / nsplit;
  const uint64_t npad = (np + 63ull) & ~63ull;  // primes, rounded to whole warps of 64
  const uint64_t nwarps = npad / 64 * nsplit;
  const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
  const uint64_t wstride = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const uint32_t qcap = min(a.qcap, (uint32_t)WQ_CAP);
  if (lane == 0) q_cnt[wib] = 0;
  __syncwarp();
  for (uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nwarps; w += wstride) {
    const uint64_t wpp = npad / 64;  // warps per part
    const uint32_t j = (uint32_t)(w / wpp);
    const uint64_t base = (w - (uint64_t)j * wpp) * 64;
    const uint32_t b_lo = min(full, j * part), b_hi = min(full, b_lo + part);
    const bool last_part = j == nsplit - 1u;
    const uint64_t pi0 = base + lane, pi1 = base + 32 + lane;
    const bool v0 = pi0 < np, v1 = pi1 < np;
    const uint64_t p0 = a.P[v0 ? pi0 : base], p1 = a.P[v1 ? pi1 : base];
    q_p[wib][lane] = p0;
    q_p[wib][32 + lane] = p1;
    if (v0) {
      const uint64_t ps0 = a.Pinv ? a.Pinv[pi0] : neg_inv64(p0);
      const uint64_t ps1 = v1 ? (a.Pinv ? a.Pinv[pi1] : neg_inv64(p1)) : ps0;
      const uint32_t plon0 = neg_lo(p0), phi10 = neg_hi(p0), pinv0 = lo32(ps0);
      const uint32_t plon1 = neg_lo(p1), phi11 = neg_hi(p1), pinv1 = lo32(ps1);
      const uint32_t n0 = nmin + 32u * (uint32_t)U * b_lo;
      const uint64_t x0 = inv_pow2(n0, p0, ps0), x1 = inv_pow2(n0, p1, ps1);
      const uint64_t K0 = a.proth ? p0 - x0 : x0, K1 = a.proth ? p1 - x1 : x1;
      uint32_t klo0 = lo32(K0), khi0 = hi32(K0), klo1 = lo32(K1), khi1 = hi32(K1);
      for (uint32_t b = b_lo; b < b_hi; ++b) {
        uint32_t acc0 = 0xffffffffu, acc1 = 0xffffffffu;
#pragma unroll
        for (int u = 0; u < U; ++u) {
          if (TEST == 0) {
            acc0 = min(acc0, min(khi0, klo0 & win_mask));
            acc1 = min(acc1, min(khi1, klo1 & win_mask));
          } else {
            acc0 = min(acc0, khi0);
            acc1 = min(acc1, khi1);
          }
          step_neg32(klo0, khi0, plon0, phi10, pinv0);
          step_neg32(klo1, khi1, plon1, phi11, pinv1);
        }
        const bool f0 = TEST == 2 ? acc0 <= bound_hi : acc0 == 0u;
        const bool f1 = v1 && (TEST == 2 ? acc1 <= bound_hi : acc1 == 0u);
        if (f0 | f1) {
          const uint32_t pos = atomicAdd(&q_cnt[wib], (uint32_t)f0 + (uint32_t)f1);
          if (f0 && pos < qcap) q_ent[wib][pos] = (lane << 26) | b;
          if (f1 && pos + (uint32_t)f0 < qcap) q_ent[wib][pos + (uint32_t)f0] = ((32u + lane) << 26) | b;
        }
      }
      if (last_part && full * (uint32_t)U < nsteps) {
        q_k[wib][lane] = mk64(klo0, khi0);
        q_k[wib][32 + lane] = mk64(klo1, khi1);
        const uint32_t pos = atomicAdd(&q_cnt[wib], 1u + (uint32_t)v1);
        if (pos < qcap) q_ent[wib][pos] = (lane << 26) | full;
        if (v1 && pos + 1u < qcap) q_ent[wib][pos + 1u] = ((32u + lane) << 26) | full;
      }
    }
    __syncwarp();
    const uint32_t cnt = q_cnt[wib];
    if (cnt <= qcap) {
      for (uint32_t e = lane; e < cnt; e += 32u) {
        const uint32_t ent = q_ent[wib][e];
        const uint32_t owner = ent >> 26, blk = ent & ((1u << 26) - 1u);
        const uint64_t op = q_p[wib][owner];
        const uint64_t ops = neg_inv64(op);
        const uint32_t t0 = (uint32_t)U * blk;
        const uint32_t nblk = min((uint32_t)U, nsteps - t0);
        const uint32_t n0 = nmin + 32u * t0;
        uint64_t K;
        if (blk == full) {
          K = q_k[wib][owner];
        } else {
          const uint64_t x = inv_pow2(n0, op, ops);
          K = a.proth ? op - x : x;
        }
        uint32_t klo = lo32(K), khi = hi32(K);
        const uint32_t oplon = neg_lo(op), ophi1 = neg_hi(op), opinv = lo32(ops);
        const uint32_t idx = a.idx_base + (uint32_t)(base + owner);
#pragma unroll 1
        for (uint32_t u = 0; u < nblk; ++u) {
          record_exact(klo, khi, n0 + 32u * u, op, idx, a.kmin, a.kmax, a.nmax, a.hits, a.hit_count, a.hit_cap);
          step_neg32(klo, khi, oplon, ophi1, opinv);
        }
      }
    } else {
      // queue overflow: each lane re-walks its part of its two primes with the
      // exact test at every step
      for (int which = 0; which < 2; ++which) {
        const uint64_t pi = which ? pi1 : pi0;
        if (pi >= np) continue;
        const uint64_t p = q_p[wib][which * 32 + lane];
        const uint64_t ps = neg_inv64(p);
        const uint32_t t_lo = (uint32_t)U * b_lo, t_hi = last_part ? nsteps : (uint32_t)U * b_hi;
        const uint64_t x = inv_pow2(nmin + 32u * t_lo, p, ps);
        const uint64_t K = a.proth ? p - x : x;
        uint32_t klo = lo32(K), khi = hi32(K);
        const uint32_t plon = neg_lo(p), phi1 = neg_hi(p), pinv = lo32(ps);
        const uint32_t idx = a.idx_base + (uint32_t)pi;
#pragma unroll 1
        for (uint32_t t = t_lo; t < t_hi; ++t) {
          record_exact(klo, khi, nmin + 32u * t, p, idx, a.kmin, a.kmax, a.nmax, a.hits, a.hit_count, a.hit_cap);
          step_neg32(klo, khi, plon, phi1, pinv);
        }
      }
    }
    __syncwarp();
    if (lane == 0) q_cnt[wib] = 0;
    __syncwarp();
  }
}

// name, queued, twin, s32, shifted, smallp, min_window, bound, lowbit, stepwin, unroll, per_thread
static const VariantTraits kVariants[PPS_NUM_VARIANTS] = {
    {"form0-window-u4-step", false, false, false, false, false, false, false, false, false, 4, 1},
    {"chain-window-u4-step", false, false, false, false, false, false, false, false, false, 4, 1},
    {"chain-window-u8-block", false, false, false, false, false, false, false, false, false, 8, 1},
    {"form2-window-u8-block", false, false, false, false, false, false, false, false, false, 8, 1},
    {"form0-window-u8-block", false, false, false, false, false, false, false, false, false, 8, 1},
    {"chain-window-u8-block-ilp2", false, false, false, false, false, false, false, false, false, 8, 1},
    {"form2-window-u8-block-ilp2", false, false, false, false, false, false, false, false, false, 8, 1},
    {"chain-lowbit-u8-block", false, false, false, false, false, false, false, true, false, 8, 1},
    {"form0-lowbit-u8-block", false, false, false, false, false, false, false, true, false, 8, 1},
    {"chain-window-u16-block", false, false, false, false, false, false, false, false, false, 16, 1},
    {"queue-min-u8", true, false, true, false, false, true, false, false, false, 8, 1},
    {"queue-window-u8", true, false, true, false, false, false, false, false, false, 8, 1},
    {"queue-bound-u8", true, false, true, false, false, false, true, false, false, 8, 1},
    {"queue-min-u16", true, false, true, false, false, true, false, false, false, 16, 1},
    {"queue-bound-u16", true, false, true, false, false, false, true, false, false, 16, 1},
    {"queue-min-u8-r40", true, false, true, false, false, true, false, false, false, 8, 1},
    {"queue-bound-u8-r40", true, false, true, false, false, false, true, false, false, 8, 1},
    {"queue-window-u8-r40", true, false, true, false, false, false, false, false, false, 8, 1},
    {"queue-smallp-u8", true, false, true, false, true, false, false, false, false, 8, 1},
    {"queue-shift-hiwin-u8", true, false, false, true, false, false, false, false, true, 8, 1},
    {"queue-shift-smallp-u8", true, false, false, true, true, false, false, false, false, 8, 1},
    {"queue-shift-hiwin-u8-r40", true, false, false, true, false, false, false, false, true, 8, 1},
    {"twin-window-u8", true, true, true, false, false, false, false, false, false, 8, 1},
    {"twin-smallp-u8", true, true, true, false, true, false, false, false, false, 8, 1},
    {"twin-shift-window-u8", true, true, false, true, false, false, false, false, false, 8, 1},
    {"twin-shift-smallp-u8", true, true, false, true, true, false, false, false, false, 8, 1},
    {"queue2-min-u8", true, false, true, false, false, true, false, false, false, 8, 2},
    {"queue2-bound-u8", true, false, true, false, false, false, true, false, false, 8, 2},
    {"queue-min-u16-r40", true, false, true, false, false, true, false, false, false, 16, 1},
    {"queue-bound-u16-r40", true, false, true, false, false, false, true, false, false, 16, 1},
    {"queue2-bound-u16", true, false, true, false, false, false, true, false, false, 16, 2},
};

const VariantTraits& walk_variant_traits(int v) {
  static const VariantTraits none = {"?", false, false, false, false, false, false, false, false, false, 8, 1};
  return (v >= 0 && v < PPS_NUM_VARIANTS) ? kVariants[v] : none;
}

const char* walk_variant_name(int v) { return walk_variant_traits(v).name; }

typedef void (*walk_fn)(WalkArgs);

template <bool S32>
static walk_fn pick(int v) {
  switch (v) {
    case 0: return k_walk<0, 0, 4, S32, 1, false>;
    case 1: return k_walk<1, 0, 4, S32, 1, false>;
    case 2: return k_walk<1, 0, 8, S32, 1, true>;
    case 3: return k_walk<2, 0, 8, S32, 1, true>;
    case 4: return k_walk<0, 0, 8, S32, 1, true>;
    case 5: return k_walk<1, 0, 8, S32, 2, true>;
    case 6: return k_walk<2, 0, 8, S32, 2, true>;
    case 7: return k_walk<1, 1, 8, S32, 1, true>;
    case 8: return k_walk<0, 1, 8, S32, 1, true>;
    case 9: return k_walk<1, 0, 16, S32, 1, true>;
    case 10: return S32 ? k_walk32q<0, 8, 8> : nullptr;
    case 11: return S32 ? k_walk32q<1, 8, 8> : nullptr;
    case 12: return S32 ? k_walk32q<2, 8, 8> : nullptr;
    case 13: return S32 ? k_walk32q<0, 16, 8> : nullptr;
    case 14: return S32 ? k_walk32q<2, 16, 8> : nullptr;
    case 15: return S32 ? k_walk32q<0, 8, 6> : nullptr;
    case 16: return S32 ? k_walk32q<2, 8, 6> : nullptr;
    case 17: return S32 ? k_walk32q<1, 8, 6> : nullptr;
    case 18: return S32 ? k_walk32q<0, 8, 8, 0, true> : nullptr;
    case 19: return S32 ? nullptr : k_walk32q<3, 8, 8, 1, false>;
    case 20: return S32 ? nullptr : k_walk32q<0, 8, 8, 1, true>;
    case 21: return S32 ? nullptr : k_walk32q<3, 8, 6, 1, false>;
    case 22: return S32 ? k_walk32q<1, 8, 8, 0, false, true> : nullptr;
    case 23: return S32 ? k_walk32q<1, 8, 8, 0, true, true> : nullptr;
    case 24: return S32 ? nullptr : k_walk32q<1, 8, 8, 1, false, true>;
    case 25: return S32 ? nullptr : k_walk32q<1, 8, 8, 1, true, true>;
    case 26: return S32 ? k_walk32q2<0, 8, 5> : nullptr;
    case 27: return S32 ? k_walk32q2<2, 8, 5> : nullptr;
    case 28: return S32 ? k_walk32q<0, 16, 6> : nullptr;
    case 29: return S32 ? k_walk32q<2, 16, 6> : nullptr;
    case 30: return S32 ? k_walk32q2<2, 16, 5> : nullptr;
  }
  return nullptr;
}

int walk_block_threads(int v) {
  (void)v;
  return 256;
}

int walk_max_blocks(int v, int threads, uint32_t step, int num_sms) {
  walk_fn f = step == 32 ? pick<true>(v) : pick<false>(v);
  if (!f) return 0;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, threads, 0) != cudaSuccess) return 0;
  return per_sm * num_sms;
}

cudaError_t launch_walk(int v, const WalkArgs& a, int blocks, int threads, cudaStream_t st) {
  walk_fn f = a.step == 32 ? pick<true>(v) : pick<false>(v);
  if (!f || blocks <= 0) return cudaErrorInvalidValue;
  f<<<blocks, threads, 0, st>>>(a);
  return cudaGetLastError();
}

// ==================================================================== filter

// The output rule on the raw candidates, one CTA per candidate (its threads
// share the trial division, so that a candidate that survives it, the one
// that takes all 3,512 primes, costs 14 rounds of 256 instead of 110 of 32).
__global__ void __launch_bounds__(FILTER_THREADS) k_filter(FilterArgs a) {
  uint32_t nh = *a.d_nhits;
  if (nh > a.hit_cap) nh = a.hit_cap;
  for (uint32_t h = blockIdx.x; h < nh; h += gridDim.x) {
    const pps_hit x = a.hits[h];
    // a twin job's candidates say their side; every other job has one
    const int32_t c = a.sign == PPS_SIGN_TWIN ? ((x.idx & HIT_SIDE_PROTH) ? 1 : -1) : a.sign;
    bool ok = (x.k == a.kstep * (x.k / a.kstep) + a.koffset) && x.n >= a.nmin && x.n < a.nmax;
    if (ok && a.in_keys) {
      // the input file's bit of (k, n), every thread the same search
      ok = x.k >= a.kmin && x.k <= a.kmax;
      if (ok) {
        const uint64_t key = (uint64_t)(x.n - a.nmin) * a.in_width + (x.k - a.kmin) / a.kstep;
        uint64_t lo = 0, hi = a.in_n;
        while (lo < hi) {
          const uint64_t mid = lo + (hi - lo) / 2;
          if (a.in_keys[mid] < key) lo = mid + 1; else hi = mid;
        }
        ok = lo < a.in_n && a.in_keys[lo] == key;
      }
    } else if (ok) {
      ok = !cta_small_factor(x.k, x.n, c, a.small_q, a.nsmall);  // ok is the same in every thread
    }
    if (ok && threadIdx.x == 0) {
      const uint32_t pos = atomicAdd(a.out_count, 1u);
      if (pos < a.out_cap) {
        pps_factor f;
        f.p = x.p;
        f.k = x.k;
        f.n = x.n;
        f.c = c;
        a.out[pos] = f;
      }
    }
  }
}

cudaError_t launch_filter(const FilterArgs& a, uint32_t max_hits, cudaStream_t st) {
  const uint32_t blocks = filter_blocks(max_hits);
  k_filter<<<blocks, FILTER_THREADS, 0, st>>>(a);
  return cudaGetLastError();
}

// ============================================================ multiply probe
// Four independent chains per thread, each iteration one lo multiply, one
// high multiply and one wide multiply-add (the walk step's mix) plus one xor.
__global__ void __launch_bounds__(256) k_imad_probe(uint32_t* sink, uint32_t iters) {
  uint32_t x0 = threadIdx.x * 2654435761u + 1u, x1 = x0 ^ 0x85ebca6bu, x2 = x0 ^ 0xc2b2ae35u,
           x3 = x0 ^ 0x27d4eb2fu;
  const uint32_t c1 = 0x9e3779b1u + blockIdx.x, c2 = 0x7f4a7c15u ^ blockIdx.x, c3 = 0x165667b1u;
  uint64_t w0 = x0, w1 = x1, w2 = x2, w3 = x3;
  for (uint32_t i = 0; i < iters; ++i) {
#define PPS_PROBE_CHAIN(X, W)                      \
  {                                                \
    const uint32_t m = X * c1;                     \
    const uint32_t h = __umulhi(m, c2);            \
    W = (uint64_t)m * c3 + W;                      \
    X = h ^ (uint32_t)(W >> 32);                   \
  }
    PPS_PROBE_CHAIN(x0, w0)
    PPS_PROBE_CHAIN(x1, w1)
    PPS_PROBE_CHAIN(x2, w2)
    PPS_PROBE_CHAIN(x3, w3)
#undef PPS_PROBE_CHAIN
  }
  const uint32_t r = x0 ^ x1 ^ x2 ^ x3 ^ (uint32_t)(w0 ^ w1 ^ w2 ^ w3);
  if (r == 0x12345678u) sink[blockIdx.x * blockDim.x + threadIdx.x] = r;
}

cudaError_t launch_imad_probe(uint32_t* sink, uint32_t iters, int blocks, int threads,
                              cudaStream_t st) {
  k_imad_probe<<<blocks, threads, 0, st>>>(sink, iters);
  return cudaGetLastError();
}

}  // namespace pps
