/* ref_appcu_stub.c -- CPU stand-in for the reference's GPU C ABI (pps/appcu.h:27-37).

   ORACLE / TEST INFRASTRUCTURE ONLY.  Linked with the reference's own C sources
   (main.c, sieve.c, putil.c, clock.c, pps/app.c, pps/factor_proth.c), compiled
   where they lie, this turns the reference into its own CPU-only build: a prime
   is flagged, as the GPU would flag it, when any step of its walk holds a k in
   range (the twin build flags every prime), and the reference's CPU re-walk
   (pps/app.c:1037-1121 test_one_p, 1197-1219 check_factors_found) and output
   filter (pps/app.c:159-186 test_factor, pps/factor_proth.c:247 try_all_factors)
   examine the whole [nmin, nmax) range of every flagged prime.  Nothing here is
   part of the shipped library.

   With -DPPS_STUB_FLAG_ALL every prime is flagged, so that the reference's own
   CPU re-walk runs over every prime and the stand-in does no walking of its
   own: the reference's CPU path as a timed baseline (each prime without a
   candidate makes the re-walk print "Computation Error: no candidates found"
   on stderr, pps/app.c:1116-1120).

   Parameter handling restates pps/appcu.cu:155-209 (cuda_init): nstep clamp to
   nmax-nmin+1, the 2^(64-nstep) <= pmin requirement, forcing nstep to 32 when
   32 <= nstep < 48 and pmin >= 2^32, and the r0 / bbits constants that
   pps/app.c reads through ld_r0 / ld_bbits.  One subsection [nmin, nmax) is
   published per thread (pps/appcu.cu:366-393 fills up to eight; the re-walk of
   one whole range visits the same n grid, so the found set is the same).
*/
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include "main.h"
#include "app.h"
#include "appcu.h"

unsigned int ld_nstep;
int ld_bbits;
uint64_t ld_r0;

static int stub_lg2(uint64_t v)
{
  int r = 0;
  while (v >>= 1) r++;
  return r;
}

void cuda_finalize(void) {}

void cuda_init(void)
{
  if (ld_nstep > (nmax - nmin + 1))
    ld_nstep = nmax - nmin + 1;
  if ((((uint64_t)1) << (64 - ld_nstep)) > pmin) {
    bmsg("Error: pmin is not large enough (or nmax is close to nmin).\n");
    bexit(ERR_INVALID_PARAM);
  }
#ifdef SEARCH_TWIN
  ld_nstep--; /* pps/appcu.cu:177-180 */
#endif
  if (ld_nstep >= 32 && ld_nstep < 48 && (((uint64_t)1) << 32) <= pmin)
    ld_nstep = 32;
  ld_bbits = stub_lg2(nmin);
  if (ld_bbits < 6) {
    fprintf(stderr, "Error: nmin too small at %u (must be at least 64).\n", nmin);
    bexit(ERR_INVALID_PARAM);
  }
  ld_r0 = ((uint64_t)1) << (64 - (nmin >> (ld_bbits - 5)));
  ld_bbits = ld_bbits - 6;
}

unsigned int cuda_app_init(int gpuno, int th, unsigned int cthread_count)
{
  int j;
  struct n_subsection *s = &thread_subsections[th];
  (void)gpuno;
  if (pmin <= ((uint64_t)1) << 32) {
    bmsg("Error: PMin is too small, <= 2^32!\n");
    bexit(ERR_INVALID_PARAM);
  }
  /* One subsection [nmin, nmax) in bit 0; the unused slots repeat nmin so the
     per-subsection constants computed by app_thread_init stay defined. */
  for (j = 1; j <= 8; j++) s->n_subsection_start[j] = nmin;
  s->n_subsection_start[0] = nmax;
  s->first_n_subsection = &s->n_subsection_start[0];
  if (cthread_count == 0) cthread_count = 1024;
  return cthread_count;
}

/* A copy of the primes of the calling thread's last check_ns, taken at the
   call as the device copy is (pps/app.c:1224-1250 refills P before it asks for
   the previous batch's flags); P == NULL keeps them. */
static __thread uint64_t *t_P;
static __thread unsigned int t_cap;

void check_ns(const uint64_t *P, const unsigned int cthread_count, const int th)
{
  (void)th;
  if (!P) return;
  if (t_cap < cthread_count) {
    free(t_P);
    t_P = malloc(cthread_count * sizeof *t_P);
    t_cap = t_P ? cthread_count : 0;
  }
  if (t_P) memcpy(t_P, P, cthread_count * sizeof *t_P);
}

#ifndef SEARCH_TWIN
static uint64_t stub_mulmod(uint64_t a, uint64_t b, uint64_t m)
{
  return (uint64_t)(((unsigned __int128)a * b) % m);
}

/* The device flag of one prime (pps/appcu.cu:779-1115 TEST_SHIFT_SMALL_KMAX):
   does any step of the walk hold k = K >> ctz(K) in [kmin, kmax] with
   ctz(K) < nstep and n + ctz(K) < nmax?  Only flagged primes are re-walked by
   pps/app.c, as with the GPU; a prime with no candidate is never re-walked (its
   re-walk would print "no candidates found"). */
static int stub_has_candidate(uint64_t p)
{
  if (p < 3 || !(p & 1)) return 1;
  uint64_t k = 1, b = (p + 1) / 2;  /* 2^-1 mod p */
  for (uint32_t e = nmin; e; e >>= 1) {
    if (e & 1) k = stub_mulmod(k, b, p);
    b = stub_mulmod(b, b, p);
  }
  if (search_proth == 1) k = p - k;
  uint64_t inv2s = 1, h = (p + 1) / 2;  /* 2^-nstep mod p */
  for (unsigned i = 0; i < ld_nstep; i++) inv2s = stub_mulmod(inv2s, h, p);
  for (uint32_t n = nmin; n < nmax; n += ld_nstep) {
    const int i = __builtin_ctzll(k);
    const uint64_t kk = k >> i;
    if (kk <= kmax && kk >= kmin && (unsigned)i < ld_nstep && n + (uint32_t)i < nmax) return 1;
    k = stub_mulmod(k, inv2s, p);
  }
  return 0;
}
#endif

void get_factors_found(unsigned char *factor_found, const unsigned int cthread_count,
                       const uint64_t start_t, int *check_ns_delay)
{
  (void)start_t; (void)check_ns_delay;
#if defined(SEARCH_TWIN) || defined(PPS_STUB_FLAG_ALL)
  memset(factor_found, 1, cthread_count);
#else
  for (unsigned int i = 0; i < cthread_count; i++)
    factor_found[i] = t_P ? (unsigned char)stub_has_candidate(t_P[i]) : 1;
#endif
}
