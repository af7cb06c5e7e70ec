/* pps_oracle.h -- CPU restatement of PPSieve's hot path.

   ORACLE / TEST INFRASTRUCTURE ONLY.  Used by tests/, by __graft_entry__.smoke()
   as the checker, and by bench.py's CPU-baseline leg.  The shipped library never
   links, loads or calls this code.

   What it restates (file:line in the reference project):
     ppo_normalize    main.c:916-931 (pmin/pmax defaults), pps/app.c:649-712
                      (kmin/kmax rounding, nmin auto, nstep), pps/appcu.cu:155-209
                      (nstep clamp, 32-forcing, nmin >= 64), pps/appcu.cu:236
                      (pmin > 2^32), main.c:971-972 (qmax default)
     ppo_sieve_range  sieve.c:168-608 + main.c:750-777: odd p, pmin|1 <= p < pmax|1,
                      with no prime factor q <= qmax (q itself survives)
     ppo_walk_prime   pps/app.c:1037-1121 (test_one_p): Montgomery inverse,
                      2^-nmin mod p, walk by 2^-nstep with count-trailing-zeros
     ppo_test_factor  pps/app.c:159-186 (test_factor) + pps/factor_proth.c:247-253
                      (try_all_factors): k == kstep*(k/kstep)+koffset, nmin <= n <
                      nmax, and k*2^n+c has no odd prime factor below 32768
   Arithmetic is plain 128-bit integer math (unsigned __int128), kept independent
   of the device kernels it checks.
*/
#ifndef PPS_ORACLE_H
#define PPS_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Error codes of the reference (pps/app.h:64-71). */
#define PPO_OK 0
#define PPO_ERR_INVALID_PARAM (-178)
#define PPO_ERR_INSUFFICIENT_RESOURCE (-198)

/* c of a twin job: both sides in one walk (the reference's SEARCH_TWIN build,
   tpsieve); each reported factor carries its own c = +1 or -1. */
#define PPO_TWIN 2

typedef struct {
  uint64_t pmin, pmax;   /* primes p: pmin <= p < pmax */
  uint64_t kmin, kmax;   /* rounded to kstep*b+koffset */
  uint32_t nmin, nmax;   /* n in [nmin, nmax) */
  int32_t  c;            /* +1 Proth (k*2^n+1), -1 Riesel (k*2^n-1), PPO_TWIN both */
  uint32_t kstep, koffset;
  uint32_t qmax;         /* largest sieving prime bound actually used */
  uint32_t nstep;        /* n values covered per walk step */
  /* Input sieve file (-i) as the output rule (pps/app.c:180-183): when
     input_keys is set, a line is printed iff its (k, n) is in the file, with
     no small-prime filter.  Keys (n - nmin) * input_width + (k - kmin) / kstep,
     ascending; input_width = (kmax - kmin) / kstep + 1. */
  uint32_t pad0;
  const uint64_t *input_keys;
  uint64_t ninput, input_width;
} ppo_params;

typedef struct {
  uint64_t p, k;
  uint32_t n;
  int32_t  c;
} ppo_factor;

/* Inputs as the user gives them (0 = "not given", as in the reference). */
int ppo_normalize(ppo_params *out, uint64_t pmin, uint64_t pmax, uint64_t kmin,
                  uint64_t kmax, uint32_t nmin, uint32_t nmax, int32_t c,
                  uint32_t kstep, uint32_t koffset, uint32_t qmax);

/* Walk one prime; found factors are appended to out (up to cap); returns the
   number of factors found (may exceed cap). */
size_t ppo_walk_prime(const ppo_params *pp, uint64_t p, ppo_factor *out, size_t cap);

/* Raw candidates of one prime before the output filter (k in range, n < nmax). */
size_t ppo_walk_prime_raw(const ppo_params *pp, uint64_t p, ppo_factor *out, size_t cap);

/* The output filter alone (test_factor): 1 if the line would be printed. */
int ppo_test_factor(const ppo_params *pp, uint64_t k, uint32_t n, int32_t c);

/* Smallest odd prime q < 32768 dividing k*2^n+c, or 0. */
uint32_t ppo_small_factor(uint64_t k, uint32_t n, int32_t c);
/* Same, only primes q >= qmin (pps/factor_proth.c:247 starts at 11). */
uint32_t ppo_small_factor_from(uint64_t k, uint32_t n, int32_t c, uint32_t qmin);

/* Sieve primes in [lo, hi) (lo, hi already inside [pmin, pmax)), qmax bound. */
size_t ppo_sieve_range(uint64_t lo, uint64_t hi, uint32_t qmax, uint64_t *out, size_t cap);

/* Whole job over [pp->pmin, pp->pmax) with nthreads host threads.
   Factors sorted by (p, k, n).  count and sum receive the number and 64-bit wrapping sum of
   the primes processed (the reference's count=/sum= fingerprint, main.c:1232).
   Returns the total number of factors (may exceed cap) or a negative error. */
long ppo_run(const ppo_params *pp, int nthreads, ppo_factor *out, size_t cap,
             uint64_t *count, uint64_t *sum);

/* Walk a given list of primes with nthreads threads (no sieve). */
long ppo_walk_list(const ppo_params *pp, const uint64_t *P, size_t np, int nthreads,
                   ppo_factor *out, size_t cap);

/* Count and 64-bit wrapping sum of the primes in [lo, hi) under the sieve rule
   (odd p, no prime factor q <= qmax other than p), with nthreads threads: the
   reference's count=/sum= fingerprint (main.c:1232) of a whole job's range. */
int ppo_sieve_fingerprint(uint64_t lo, uint64_t hi, uint32_t qmax, int nthreads, uint64_t *count,
                          uint64_t *sum);

/* Per-line verification of reported factors: line i belongs to
   jobs[job_of[i]] (jobs[0] when job_of is NULL) and must have p prime
   (deterministic Miller-Rabin), pmin <= p < pmax, k in [kmin, kmax] with
   k == koffset (mod kstep), nmin <= n < nmax, c the job's side (+1 or -1 for
   a twin job), k*2^n + c == 0 (mod p), and pass the job's output rule
   (ppo_test_factor: pps/app.c:159-186, pps/factor_proth.c:247-253).  bad[i]
   (optional) receives the PPO_BAD_* bits of the failed checks.  Returns the
   number of failed lines. */
#define PPO_BAD_NOT_PRIME 1
#define PPO_BAD_P_RANGE 2
#define PPO_BAD_K 4
#define PPO_BAD_N 8
#define PPO_BAD_C 16
#define PPO_BAD_NOT_DIVISOR 32
#define PPO_BAD_RULE 64
long ppo_verify_factors(const ppo_params *jobs, const uint32_t *job_of, const ppo_factor *f, size_t n,
                        int nthreads, uint8_t *bad);

/* Primality (deterministic Miller-Rabin for 64-bit) and k*2^n+c mod p. */
int ppo_is_prime(uint64_t n);
uint64_t ppo_kpow_mod(uint64_t k, uint32_t n, int32_t c, uint64_t p);

#ifdef __cplusplus
}
#endif
#endif
