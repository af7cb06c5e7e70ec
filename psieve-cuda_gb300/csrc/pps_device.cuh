// pps_device.cuh -- device integer arithmetic for the PPSieve walk (sm_103a).
//
// Everything is exact 64-bit modular arithmetic built from 32-bit multiplies.
// Conventions: p is an odd prime, 2^32 < p < 2^62; ps = -p^-1 mod 2^64.
//
// Reference counterparts (file:line in Ken-g6/PSieve-CUDA):
//   neg_inv64      pps/appcu.cu:491-511 invmod2pow_ul (Newton lifting of p^-1)
//   mont_mul       pps/appcu.cu:513-546 mulmod_REDC (R = 2^64 Montgomery product)
//   inv_pow2       pps/appcu.cu:710-736 invpowmod_REDClr (2^-e mod p, left to right)
//   step_*         pps/appcu.cu:591-707 shiftmod_REDC* (k <- k * 2^-s mod p)
#pragma once
#include <stdint.h>

namespace pps {

__device__ __forceinline__ uint32_t lo32(uint64_t x) { return (uint32_t)x; }
__device__ __forceinline__ uint32_t hi32(uint64_t x) { return (uint32_t)(x >> 32); }
__device__ __forceinline__ uint64_t mk64(uint32_t lo, uint32_t hi) {
  return ((uint64_t)hi << 32) | lo;
}

// -p^-1 mod 2^64.  (3p) xor 2 inverts p modulo 2^5; each Newton step
// x <- x(2 - p x) doubles the number of correct low bits: 5, 10, 20, 40 (so 32)
// in 32-bit arithmetic, then one 64-bit step gives 64.
__device__ __forceinline__ uint64_t neg_inv64(uint64_t p) {
  const uint32_t p32 = (uint32_t)p;
  uint32_t x = (3u * p32) ^ 2u;
  x *= 2u - p32 * x;
  x *= 2u - p32 * x;
  x *= 2u - p32 * x;
  uint64_t y = x;
  y *= 2ull - p * y;
  return 0ull - y;
}

// Montgomery product a*b*2^-64 mod p for a, b < p.  T = a*b < p^2, so
// (T + m p) / 2^64 < p^2/2^64 + p < 2p and one conditional subtraction suffices.
__device__ __forceinline__ uint64_t mont_mul(uint64_t a, uint64_t b, uint64_t p, uint64_t ps) {
  const uint64_t tlo = a * b;
  const uint64_t thi = __umul64hi(a, b);
  const uint64_t m = tlo * ps;
  const uint64_t r = thi + __umul64hi(m, p) + (tlo != 0ull ? 1ull : 0ull);
  return r >= p ? r - p : r;
}

// x*2^-64 mod p (leaves Montgomery form).
__device__ __forceinline__ uint64_t mont_out(uint64_t x, uint64_t p, uint64_t ps) {
  const uint64_t m = x * ps;
  const uint64_t r = __umul64hi(m, p) + (x != 0ull ? 1ull : 0ull);
  return r >= p ? r - p : r;
}

// 2^-e mod p for e >= 32, p > 2^32.
// Left to right over the bits of e.  The six leading bits t (32 <= t < 64) give
// the Montgomery form of 2^-t directly as 2^(64-t) (< 2^32 < p, already
// reduced); each further bit squares (doubling the exponent) and, for a 1 bit,
// halves mod p (2^-1 factor).  Leaves Montgomery form at the end.
__device__ __forceinline__ uint64_t inv_pow2(uint32_t e, uint64_t p, uint64_t ps) {
  const int len = 32 - __clz(e);       // bit length, >= 6 because e >= 32
  int b = len - 6;
  uint64_t r = 1ull << (64 - (e >> b));
  for (--b; b >= 0; --b) {
    r = mont_mul(r, r, p, ps);
    if ((e >> b) & 1u) r = (r & 1ull) ? ((r >> 1) + (p >> 1) + 1ull) : (r >> 1);
  }
  return mont_out(r, p, ps);
}

// ---------------------------------------------------------------- the walk step
// K <- K * 2^-s mod p for K < p, 1 <= s <= 32, as (K + m p) / 2^s with
// m = (-K p^-1) mod 2^s.  Because K < p (not K < p 2^s as in a full product
// reduction), (K + m p)/2^s <= (p - 1 + (2^s - 1) p)/2^s < p: the result is
// already reduced and no final subtraction is needed.
//
// With m' = m * 2^(32-s) = (Klo * pinv_s) mod 2^32, pinv_s = (ps mod 2^32) << (32-s):
//   (K + m p)/2^s = (K >> s) + m' * phi + hi32(m' * plo) + [m' != 0]
// (the low words of (K mod 2^s) 2^(32-s) and m' plo sum to 0 or 2^32).
//
// Four formulations of the same arithmetic.  Forms 0-2 serve the older walk
// kernels (the autotuner times them); the queued and batched walks use form 3
// (step_neg32), the one without low-word carries, for s = 32 and, on
// K * 2^(32-s), for s < 32.

// Form 0: one lo multiply, one hi multiply, one wide multiply-add.
template <bool S32>
__device__ __forceinline__ void step_form0(uint32_t& klo, uint32_t& khi, uint32_t plo, uint32_t phi,
                                           uint32_t pinv_s, uint32_t s) {
  const uint32_t m = klo * pinv_s;
  uint64_t base;
  if (S32) {
    base = (uint64_t)khi;
  } else {
    base = mk64(__funnelshift_r(klo, khi, s), khi >> s);
  }
  const uint64_t r = base + __umulhi(m, plo) + (m != 0u ? 1u : 0u) + (uint64_t)m * phi;
  klo = lo32(r);
  khi = hi32(r);
}

// Form 1 (s = 32 only): 32-bit multiply-add carry chain over the 96-bit sum
// K + m p, keeping words 1 and 2.
__device__ __forceinline__ void step_chain32(uint32_t& klo, uint32_t& khi, uint32_t plo, uint32_t phi,
                                             uint32_t pinv) {
  const uint32_t m = klo * pinv;
  uint32_t w1, w2;
  asm("{\n\t"
      ".reg .u32 w0;\n\t"
      "mad.lo.cc.u32  w0, %2, %3, %4;\n\t"   // w0 = lo(m plo) + klo  (== 0), carry
      "madc.hi.cc.u32 %0, %2, %3, %5;\n\t"   // w1 = hi(m plo) + khi + carry
      "madc.hi.u32    %1, %2, %6, 0;\n\t"    // w2 = hi(m phi) + carry
      "mad.lo.cc.u32  %0, %2, %6, %0;\n\t"   // w1 += lo(m phi)
      "addc.u32       %1, %1, 0;\n\t"        // w2 += carry
      "}"
      : "=r"(w1), "=r"(w2)
      : "r"(m), "r"(plo), "r"(klo), "r"(khi), "r"(phi));
  klo = w1;
  khi = w2;
}

// Form 3 (s = 32): no carry out of the low words.  Write p = phi1 2^32 - plon
// with phi1 = phi + 1 and plon = -plo mod 2^32 (plo is odd, so plon = 2^32 - plo).
// Since m p == -K (mod 2^32), lo32(m plon) == klo, and
//   K + m p = (khi + m phi1 - hi32(m plon)) 2^32 + (klo - lo32(m plon)),
// whose low word is exactly zero: K' = khi + m phi1 - hi32(m plon).  The three
// multiplies are the same as the chain's (m, one high product, one wide
// product), but the sum needs no [klo != 0] carry and no carry between the
// hi(m plo) + khi and lo(m phi) words, which lets the compiler keep the
// remaining 64-bit add/subtract on the integer ALU instead of the multiply pipe.
__device__ __forceinline__ uint32_t neg_lo(uint64_t p) { return 0u - lo32(p); }  // plon
__device__ __forceinline__ uint32_t neg_hi(uint64_t p) { return hi32(p) + 1u; }  // phi1 (p < 2^62)
// (The sum is written as one 64-bit add and subtract in PTX: the compiler then
// forms m phi1 as one wide multiply and the add/subtract as a carry pair on
// the integer ALU, with no register moves on the multiply pipe.)
// (khi_in + m phi1 - hi32(m plon)) into (lo, hi): the carry-free sum.
__device__ __forceinline__ void neg_sum(uint32_t m, uint32_t khi_in, uint32_t plon, uint32_t phi1, uint32_t& lo,
                                        uint32_t& hi) {
  asm("{\n\t"
      ".reg .u32 h, l2, g2;\n\t"
      ".reg .u64 t, k, hh;\n\t"
      "mul.hi.u32 h, %2, %3;\n\t"   // hi(m plon)
      "mul.lo.u32 l2, %2, %4;\n\t"  // m phi1, low word
      "mul.hi.u32 g2, %2, %4;\n\t"  // m phi1, high word
      "mov.b64 t, {l2, g2};\n\t"
      "cvt.u64.u32 k, %5;\n\t"
      "cvt.u64.u32 hh, h;\n\t"
      "add.u64 t, t, k;\n\t"        // + khi_in
      "sub.u64 t, t, hh;\n\t"       // - hi(m plon)
      "mov.b64 {%0, %1}, t;\n\t"
      "}"
      : "=r"(lo), "=r"(hi)
      : "r"(m), "r"(plon), "r"(phi1), "r"(khi_in));
}

__device__ __forceinline__ void step_neg32(uint32_t& klo, uint32_t& khi, uint32_t plon, uint32_t phi1,
                                           uint32_t pinv) {
  const uint32_t m = klo * pinv;
  neg_sum(m, khi, plon, phi1, klo, khi);
}

// Form 3 for s < 32 with p <= 2^(32+s): the same reduction applied to
// K 2^(32-s) (< 2^64).  Its high word is the funnel shift of K, and its low word
// enters only through m = lo32(K 2^(32-s)) (-p^-1) = klo (pinv << (32-s)) mod
// 2^32, so the shifted low word is never formed: pass pinv_sh = pinv << sh,
// sh = 32 - s.  (K 2^(32-s) + m p) / 2^32 = (K + (m / 2^(32-s)) p) / 2^s.
__device__ __forceinline__ void step_neg32s(uint32_t& klo, uint32_t& khi, uint32_t plon, uint32_t phi1,
                                            uint32_t pinv_sh, uint32_t sh) {
  const uint32_t hi = __funnelshift_l(klo, khi, sh);
  const uint32_t m = klo * pinv_sh;
  neg_sum(m, hi, plon, phi1, klo, khi);
}

// Form 2: the low product m' plo + (K mod 2^s) 2^(32-s) as one wide
// multiply-add whose high word is hi32(m' plo) + [m' != 0], then a second wide
// multiply-add by phi.
template <bool S32>
__device__ __forceinline__ void step_form2(uint32_t& klo, uint32_t& khi, uint32_t plo, uint32_t phi,
                                           uint32_t pinv_s, uint32_t s) {
  const uint32_t m = klo * pinv_s;
  uint64_t x, base;
  if (S32) {
    x = (uint64_t)m * plo + klo;
    base = (uint64_t)khi;
  } else {
    x = (uint64_t)m * plo + (klo << (32u - s));
    base = mk64(__funnelshift_r(klo, khi, s), khi >> s);
  }
  const uint64_t r = (uint64_t)m * phi + (base + (x >> 32));
  klo = lo32(r);
  khi = hi32(r);
}

// ---------------------------------------------------------------- output rule
// Whether the odd prime q < 2^16 divides k 2^n + c (c = +-1): the trial
// division of pps/factor_proth.c:247-253 by the primes below 32768, in 32-bit
// arithmetic (every product of two residues stays below 2^32).
__device__ __forceinline__ bool small_divides(uint64_t k, uint32_t n, int32_t c, uint32_t q) {
  const uint32_t t32 = (0xffffffffu % q + 1u) % q;  // 2^32 mod q
  const uint32_t kr = ((hi32(k) % q) * t32 + lo32(k) % q) % q;
  uint32_t r = 1u, b = 2u;
  for (uint32_t e = n; e; e >>= 1) {
    if (e & 1u) r = r * b % q;
    b = b * b % q;
  }
  return (kr * r + (uint32_t)((int32_t)q + c)) % q == 0u;
}

// Whether k 2^n + c has a factor among small_q[0, nsmall), tested by all the
// threads of a CTA together: rounds of blockDim.x primes, ending with the
// first round that finds one.  Every thread of the CTA calls it with the same
// arguments.
__device__ __forceinline__ bool cta_small_factor(uint64_t k, uint32_t n, int32_t c, const uint16_t* small_q,
                                                 uint32_t nsmall) {
  for (uint32_t base = 0; base < nsmall; base += blockDim.x) {
    const uint32_t i = base + threadIdx.x;
    const bool d = i < nsmall && small_divides(k, n, c, small_q[i]);
    if (__syncthreads_or(d)) return true;
  }
  return false;
}

}  // namespace pps
