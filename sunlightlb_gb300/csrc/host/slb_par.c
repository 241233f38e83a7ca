/*
 * A parallel loop over node ranges for the host side of uploads and
 * downloads (the reference does these loops on one core; a 512^3 lattice
 * has 134M nodes, and one Grace core streams its ~6 GB of host arrays in
 * about 0.8 s).  fn(lo, hi, ctx) runs on contiguous ranges that cover
 * [0, n) once; with fewer than two ranges worth it runs inline.
 */
#include <pthread.h>
#include <stdlib.h>
#include <unistd.h>
#include "slb_private.h"

#define SLB_PAR_MAX 32

typedef struct {
  slb_range_fn fn;
  void *ctx;
  long lo, hi;
} slb_range;

static void *run_range(void *arg) {
  slb_range *r = (slb_range *)arg;
  r->fn(r->lo, r->hi, r->ctx);
  return NULL;
}

int slb_par_threads(long n, long grain) {
  long cores = sysconf(_SC_NPROCESSORS_ONLN), t;
  if (cores < 1) cores = 1;
  if (cores > SLB_PAR_MAX) cores = SLB_PAR_MAX;
  t = grain > 0 ? n / grain : cores;
  if (t > cores) t = cores;
  return t < 1 ? 1 : (int)t;
}

void slb_parallel_for(long n, long grain, slb_range_fn fn, void *ctx) {
  int t = slb_par_threads(n, grain), i;
  slb_range r[SLB_PAR_MAX];
  pthread_t th[SLB_PAR_MAX];
  int started[SLB_PAR_MAX];
  if (t <= 1) {
    fn(0, n, ctx);
    return;
  }
  for (i = 0; i < t; i++) {
    r[i].fn = fn; r[i].ctx = ctx;
    r[i].lo = n * i / t; r[i].hi = n * (i + 1) / t;
  }
  /* ranges 1..t-1 on threads, range 0 here; a range whose thread could not
   * start runs here too */
  for (i = 1; i < t; i++) {
    started[i] = pthread_create(&th[i], NULL, run_range, &r[i]) == 0;
    if (!started[i]) run_range(&r[i]);
  }
  run_range(&r[0]);
  for (i = 1; i < t; i++)
    if (started[i]) pthread_join(th[i], NULL);
}
