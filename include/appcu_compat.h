/* appcu_compat.h -- the reference's GPU C ABI, served by libppsgpu_appcu.so.

   Same names, arguments and meaning as pps/appcu.h:27-37 of Ken-g6/PSieve-CUDA,
   so the reference's unmodified pps/app.c (and main.c, sieve.c) link against
   this library instead of pps/appcu.cu.  The library reads the globals that
   app.c / main.c define (pps/app.h:88-96: nmin, nmax, search_proth, kmin, kmax,
   thread_subsections; main.h:57-60: pmin, pmax, num_threads) and reports fatal
   errors through main.c's bmsg()/bexit() exactly as the reference does.

   Differences from the reference, none visible to app.c:
     - per-thread device state (the reference keeps one set of device buffers
       in file-scope globals shared by all host threads, pps/appcu.cu:67-70);
     - the walk produces exact candidates on the device; the per-prime flag byte
       that get_factors_found() returns is derived from them (bit j set when a
       candidate lies in [start[j+1], start[j]) of thread_subsections[th]).
*/
#ifndef APPCU_COMPAT_H
#define APPCU_COMPAT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* pps/appcu.h:27: per-thread device setup; returns the batch size (primes per
   check_ns call, a multiple of 128 times the SM count) or 0 if the thread has
   no usable device.  Fills thread_subsections[th]. */
unsigned int cuda_app_init(int gpuno, int th, unsigned int cthread_count);

/* pps/appcu.h:29: start the walk of cthread_count primes P (host memory) for
   thread th; P == NULL re-walks the primes passed last time. */
void check_ns(const uint64_t *P, const unsigned int cthread_count, const int th);

/* pps/appcu.h:30: wait for the walk started by the last check_ns of the
   calling thread and write one flag byte per prime.  start_t and
   check_ns_delay are accepted for ABI compatibility (the wait blocks). */
void get_factors_found(unsigned char *factor_found, const unsigned int cthread_count,
                       const uint64_t start_t, int *check_ns_delay);

/* pps/appcu.h:31: once, before threads start: nstep rules of
   pps/appcu.cu:158-204 (may change ld_nstep); exits through bexit() on the
   reference's invalid-parameter conditions. */
void cuda_init(void);

/* pps/appcu.h:32: release the calling thread's device state. */
void cuda_finalize(void);

/* pps/appcu.h:35-37 */
extern unsigned int ld_nstep;
extern int ld_bbits;
extern uint64_t ld_r0;

#ifdef __cplusplus
}
#endif
#endif
