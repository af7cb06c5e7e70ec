/* pps_app.h -- the application plugin hooks served by the GPU plugin
   (psieve-cuda_gb300/host/app_gpu.c, built as _build/libppsgpu_app.so; its twin
   build, the reference's tpsieve, as _build/libppsgpu_app_twin.so).

   Same names, arguments, return values and error behaviour as the reference's
   plugin interface pps/app.h:73-96 (Ken-g6/PSieve-CUDA), so the reference's
   main.c and sieve.c link against this plugin in place of pps/app.c +
   pps/appcu.cu + pps/factor_proth.c.  The plugin reads main.c's globals
   (main.h:57-60), parses option values with main.c's parse_uint64 / parse_uint
   (putil.h:36-39) and reports fatal errors through main.c's bexit(); an
   executable that links it provides those symbols, as main.c + putil.c do.

   Behaviour differences (by design; outputs are the same lines):
     - the device returns exact (p, k, n) and applies the output rule of
       pps/app.c:159-186 itself, so there is no CPU re-walk of flagged primes;
     - app_thread_fun1() does not pad a partial batch with composites;
     - -i (input sieve file, NewPGen or ABCD) is read on the host and becomes
       the output rule on the device (pps/app.c:180-183), as in the reference.
*/
#ifndef PPS_APP_H
#define PPS_APP_H

#include <stdint.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifdef PPS_TWIN
/* the twin build (tpsieve, pps/app.h:35): no -R, both sides at once */
#define PPS_APP_SHORT_OPTS "k:K:n:N:i:f:b:d:m:M:s:T"
#else
#define PPS_APP_SHORT_OPTS "k:K:n:N:i:f:b:d:m:M:s:R"
#endif

/* pps/app.h:73-84 */
void app_banner(void);
int app_parse_option(int opt, char *arg, const char *source);
void app_help(void);
void app_init(void);
unsigned int app_thread_init(int th);
void app_thread_fun(int th, const uint64_t *P, uint64_t *lastP, const unsigned int cthread_count);
void app_thread_fun1(int th, uint64_t *P, uint64_t *lastP, const unsigned int cthread_count,
                     unsigned int len);
void app_thread_fini(int th);
int app_read_checkpoint(FILE *f);
void app_write_checkpoint(FILE *f);
void app_fini(uint64_t pstop);

/* pps/app.h:85-96 */
struct n_subsection {
  unsigned int n_subsection_start[9];
  unsigned int *first_n_subsection;
};
extern struct n_subsection *thread_subsections;
extern unsigned int nmin, nmax;
extern int search_proth;
extern uint64_t kmax, kmin;

#ifdef __cplusplus
}
#endif
#endif
