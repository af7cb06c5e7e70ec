/* ref_appcu_stub.c -- CPU stand-in for the reference's GPU C ABI (pps/appcu.h:27-37).

   ORACLE / TEST INFRASTRUCTURE ONLY.  Linked with the reference's own C sources
   (main.c, sieve.c, putil.c, clock.c, pps/app.c, pps/factor_proth.c), compiled
   where they lie, this turns the reference into its own CPU-only build: every
   n-subsection of every prime is flagged, so the reference's CPU re-walk
   (pps/app.c:1037-1121 test_one_p, 1197-1219 check_factors_found) and output
   filter (pps/app.c:159-186 test_factor, pps/factor_proth.c:247 try_all_factors)
   examine the whole [nmin, nmax) range for every prime.  Nothing here is part of
   the shipped library.

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

void check_ns(const uint64_t *P, const unsigned int cthread_count, const int th)
{
  (void)P; (void)cthread_count; (void)th;
}

void get_factors_found(unsigned char *factor_found, const unsigned int cthread_count,
                       const uint64_t start_t, int *check_ns_delay)
{
  (void)start_t; (void)check_ns_delay;
  memset(factor_found, 1, cthread_count);
}
