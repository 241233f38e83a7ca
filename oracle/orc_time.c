/*
 * ORACLE -- test infrastructure only.
 *
 * Timing entry for the CPU baselines of bench.py: a lattice of the oracle
 * (the C restatement of the reference's update path, orc_lb.c) built from a
 * solid-node mask and advanced by lbstep, the reference's own update cycle
 * (src/lbkernel.c:49-51: bounce-back, three streaming sweeps, collision).
 * oracle/Makefile compiles it with orc_lb.c under the reference's shipped
 * flags (src/Makefile:39: -O3 -ffast-math), once with LBReal = double (the
 * reference's default) and once with -D_SINGLE (the reference's
 * single-precision build).  The same file linked with the reference's own
 * sources (oracle/Makefile ref) checks that these builds step like the
 * reference's.  Never part of the GPU library.
 */
#include <stdio.h>
#include <stdlib.h>
#include <time.h>
#include "sunlightlb.h"

/* the oracle's destructor; absent from a build of the reference's own
 * sources (which has none), where the lattice is left allocated */
extern void freelb(LBSys) __attribute__((weak));

static double now(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/* sizeof(LBReal) of this build: 8 (double) or 4 (-D_SINGLE) */
int orc_real_size(void) { return (int)sizeof(LBReal); }

/* Lattice ni x nj x nk whose nodes with mask[inode] != 0 (inode =
 * nk*(nj*i + j) + k) form one object; tau, Stokes or Navier-Stokes
 * collision, uniform body force fx along x on the fluid nodes.  Runs
 * `warmup` update steps, then `steps` timed ones; returns their wall
 * seconds, and in *checksum the sum of the squared populations (so the work
 * cannot be skipped).  Returns -1 when the lattice cannot be built. */
double orc_time_steps(const unsigned char *mask, int ni, int nj, int nk, double tau, int stokes, double fx,
                      int warmup, int steps, double *checksum) {
  LBSys lb = newlb(ni, nj, nk, "null");
  LBObj p;
  long n, nn = (long)ni * nj * nk;
  int s;
  double t0, dt, sum = 0.0;
  if (lb == NULL) return -1.0;
  lb->tau = tau;
  lb->stokes_flow = stokes;
  p = addobj(lb);
  zeroobj(p);
  for (n = 0; n < nn; n++)
    if (mask[n]) lb->obj[n] = p;
  lb->changed_objects = 1;
  syncobjs(lb);
  addbf(lb, fx, 0.0, 0.0);
  for (s = 0; s < warmup; s++) lbstep(lb);
  t0 = now();
  for (s = 0; s < steps; s++) lbstep(lb);
  dt = now() - t0;
  for (n = 0; n < 15 * nn; n++) sum += (double)lb->a[n] * (double)lb->a[n];
  if (checksum) *checksum = sum;
  if (freelb) freelb(lb);
  return dt;
}
