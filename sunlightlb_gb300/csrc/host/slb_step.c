/*
 * Update step and measurement (host side of reference src/lbkernel.c and
 * src/lbmeasure.c).  Every computation on populations runs on the GPU
 * (slb_device.h); this file keeps the reference's call sequence, status
 * state machine, warnings, step counter and signal polling.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "slb_private.h"

static void out_of_position(LBSys lb, const char *what) {
  printf("%s apparently out of position\n", what);
  wrstatus(lb, stdout);
}

static void after_collide(LBSys lb) {
  lb->status = POST_COLLIDE;
#ifdef SIGNAL
  if (slb_signal_flag) sighandle(lb);
#endif
}

/* reference src/lbkernel.c:35-45: bounce-back as a separate phase */
static void bounce(LBSys lb, int with_force) {
  slbc_lattice *d;
  slb_need_populations(lb, "A separate bounce-back phase");
  if (lb->changed_objects) syncobjs(lb);
  d = slb_device(lb);
  if (lb->status != POST_COLLIDE) out_of_position(lb, "Bounceback");
  slb_check(slbc_bbl(d, with_force), "bounce-back");
  slb_device_changed(lb);
  if (with_force) slb_forces_changed(lb);
  lb->status = POST_BBL;
}

void bbl(LBSys lb) {
  bounce(lb, 0);
  slb_trace(lb, lb->objects_moving ? "bbl (MOV)" : "bbl (STAT)");
}

void bblforce(LBSys lb) {
  bounce(lb, 1);
  slb_trace(lb, lb->objects_moving ? "bblforce (MOV)" : "bblforce (STAT)");
}

/* reference src/lbkernel.c:623-762 */
void propagate(LBSys lb) {
  slbc_lattice *d;
  slb_need_populations(lb, "A separate propagation phase");
  d = slb_device(lb);
  if (lb->status != POST_BBL) out_of_position(lb, "Propagation");
  slb_check(slbc_propagate(d), "propagation");
  slb_device_changed(lb);
  lb->status = POST_PROPAGATE;
  slb_trace(lb, "propagate");
}

/* reference src/lbkernel.c:769-877 */
void collide(LBSys lb) {
  slbc_lattice *d;
  slb_need_relaxed_solids(lb);
  d = slb_device(lb);
  if (lb->status != POST_PROPAGATE) out_of_position(lb, "Collision");
  slb_check(slbc_collide(d), "collision");
  slb_device_changed(lb);
  lb->step += 1;
  after_collide(lb);
  slb_trace(lb, "collide");
}

/* One fused update (bounce-back, streaming, collision) from the
 * post-collision state; with_force also accumulates the node forces of
 * that bounce-back (reference src/lbkernel.c:41-51). */
static void fused_step(LBSys lb, int with_force) {
  slbc_lattice *d;
  slb_need_relaxed_solids(lb);
  if (lb->changed_objects) syncobjs(lb);
  d = slb_device(lb);
  if (with_force) {
    slb_check(slbc_force_step(d), "force step");
    slb_forces_changed(lb);
  } else {
    slb_check(slbc_step(d, 1, 0), "update step");
  }
  slb_device_changed(lb);
  lb->step += 1;
  after_collide(lb);
}

/* reference src/lbkernel.c:49-51 */
void lbstep(LBSys lb) {
  if (lb->status != POST_COLLIDE) {
    /* out of cycle: run the phases one by one, as the reference does */
    bbl(lb); propagate(lb); collide(lb);
    return;
  }
  fused_step(lb, 0);
  if (slb_verbosity & TRACE_ROUTINE_EXITS) {
    printf("LB %i : bbl done\nLB %i : propagate done\nLB %i : collide done\n", lb->step, lb->step, lb->step);
  }
}

/* appended: n update steps, replayed from a CUDA graph */
void lbsteps(LBSys lb, int n) {
  slbc_lattice *d;
  if (n <= 0) return;
  if (lb->status != POST_COLLIDE) { lbstep(lb); n--; if (n <= 0) return; }
  slb_need_relaxed_solids(lb);
  if (lb->changed_objects) syncobjs(lb);
  d = slb_device(lb);
  slb_check(slbc_step(d, n, 1), "update steps");
  slb_device_changed(lb);
  lb->step += n;
  after_collide(lb);
}

/* ---- batches (appended API) -------------------------------------------- */

struct LBBatch_struct {
  int n, cap;
  int mode;
  LBSys *lbs;
  slbc_batch *dev;          /* device batch of ... */
  slbc_lattice **dev_lats;  /* ... these device lattices */
  int dev_n;
};

LBBatch newbatch(void) {
  LBBatch b = (LBBatch)calloc(1, sizeof(struct LBBatch_struct));
  if (b == NULL) error("No room for a batch");
  return b;
}

void batchadd(LBBatch b, LBSys lb) {
  int k;
  for (k = 0; k < b->n; k++) if (b->lbs[k] == lb) return;
  if (b->n == b->cap) {
    b->cap = b->cap ? 2 * b->cap : 16;
    b->lbs = (LBSys *)realloc(b->lbs, b->cap * sizeof(LBSys));
    if (b->lbs == NULL) error("No room for a batch");
  }
  b->lbs[b->n++] = lb;
}

int batchsize(LBBatch b) { return b->n; }

void batchmode(LBBatch b, int mode) {
  if (mode != 0 && mode != 1) { printf("Batch mode is 0 (packed tiles) or 1 (persistent)\n"); return; }
  b->mode = mode;
}

void freebatch(LBBatch b) {
  if (b == NULL) return;
  if (b->dev) slbc_batch_destroy(b->dev);
  free(b->dev_lats);
  free(b->lbs);
  free(b);
}

/* every member by n update steps: members out of the collide-stream cycle,
 * or whose precision differs from the first member's, step on their own */
void batchsteps(LBBatch b, int n) {
  slbc_lattice **devs;
  LBSys *members;
  int k, m = 0, prec = -1;
  if (n <= 0 || b->n == 0) return;
  devs = (slbc_lattice **)malloc(b->n * sizeof(slbc_lattice *));
  members = (LBSys *)malloc(b->n * sizeof(LBSys));
  if (devs == NULL || members == NULL) error("No room for a batch");
  for (k = 0; k < b->n; k++) {
    LBSys lb = b->lbs[k];
    if (lb->changed_objects) syncobjs(lb);
    if (lb->status != POST_COLLIDE || lb->precision == SLB_BF16 || (prec >= 0 && lb->precision != prec)) {
      lbsteps(lb, n);
      continue;
    }
    prec = lb->precision;
    devs[m] = slb_device(lb);
    members[m++] = lb;
  }
  if (m > 0) {
    /* a new device batch when the device lattices changed */
    int same = b->dev != NULL && b->dev_n == m && memcmp(b->dev_lats, devs, m * sizeof(slbc_lattice *)) == 0;
    if (!same) {
      if (b->dev) slbc_batch_destroy(b->dev);
      b->dev = NULL;
      slb_check(slbc_batch_create(&b->dev, devs, m), "batch set-up");
      free(b->dev_lats);
      b->dev_lats = (slbc_lattice **)malloc(m * sizeof(slbc_lattice *));
      if (b->dev_lats == NULL) error("No room for a batch");
      memcpy(b->dev_lats, devs, m * sizeof(slbc_lattice *));
      b->dev_n = m;
    }
    slb_check(slbc_batch_set_mode(b->dev, b->mode), "batch mode");
    slb_check(slbc_batch_step(b->dev, n), "batch steps");
    for (k = 0; k < m; k++) {
      slb_device_changed(members[k]);
      members[k]->step += n;
      after_collide(members[k]);
    }
  }
  free(devs);
  free(members);
}

/* ---- measurement: reference src/lbmeasure.c ------------------------------ */

/* reference src/lbmeasure.c:58-106 */
void accvmean(LBSys lb, LBReal prefac) {
  double s[5];
  LBReal fac = 0.0, wfac, uxtot, uytot, uztot;
  int nfluid;
  if (lb->vel_corrected) switch (lb->status) {
    case POST_PROPAGATE: fac = 0.5; break;
    case POST_COLLIDE: fac = -0.5; break;
    default: printf("Accvmean apparently of position\n"); wrstatus(lb, stdout); break;
  }
  slb_check(slbc_vsum(slb_device(lb), fac, lb->psi, s), "mean velocity");
  nfluid = (int)s[4];
  wfac = nfluid / s[3];
  uxtot = s[0] * wfac; uytot = s[1] * wfac; uztot = s[2] * wfac;
  lb->vmeanx += prefac * uxtot / (lb->nnodes);
  lb->vmeany += prefac * uytot / (lb->nnodes);
  lb->vmeanz += prefac * uztot / (lb->nnodes);
  slb_trace(lb, "accvmean");
}

/* reference src/lbmeasure.c:208-216 */
void zeroforce(LBSys lb) {
  long x;
  for (x = 0; x < lb->nnodes; x++) lb->fx[x] = lb->fy[x] = lb->fz[x] = 0.0;
  slb_check(slbc_zero_force(slb_device(lb)), "force reset");
  slb_state(lb)->host_f_valid = 1;
  slb_trace(lb, "zeroforce");
}

/* reference src/lbmeasure.c:221-231 */
void normforce(LBSys lb, LBReal fac) {
  slb_check(slbc_scale_force(slb_device(lb), fac), "force scaling");
  slb_forces_changed(lb);
  if (slb_verbosity & TRACE_ROUTINE_EXITS) printf("LB %i : normforce(%f) done\n", lb->step, fac);
}

/* reference src/lbmeasure.c:236-263 */
void distribf(LBSys lb) {
  slb_priv *st;
  slbc_lattice *d = slb_device(lb);
  double *pos, *ft;
  int o;
  LBObj p;
  st = slb_state(lb);
  for (p = lb->obj_head; p != NULL; p = p->next_obj) {
    p->frcx = p->frcy = p->frcz = 0.0;
    p->trqx = p->trqy = p->trqz = 0.0;
  }
  if (st->nobj > 0) {
    pos = (double *)malloc(3 * (size_t)st->nobj * sizeof(double));
    ft = (double *)malloc(6 * (size_t)st->nobj * sizeof(double));
    if (pos == NULL || ft == NULL) error("No room for object table");
    for (o = 0; o < st->nobj; o++) {
      pos[3 * o] = st->objs[o]->posx; pos[3 * o + 1] = st->objs[o]->posy; pos[3 * o + 2] = st->objs[o]->posz;
    }
    slb_check(slbc_distribf(d, pos, ft), "object forces");
    for (o = 0; o < st->nobj; o++) {
      p = st->objs[o];
      p->frcx += ft[6 * o]; p->frcy += ft[6 * o + 1]; p->frcz += ft[6 * o + 2];
      p->trqx += ft[6 * o + 3]; p->trqy += ft[6 * o + 4]; p->trqz += ft[6 * o + 5];
    }
    free(pos); free(ft);
  }
  slb_trace(lb, "distribf");
}

/* reference src/lbmeasure.c:30-49: forces and mean flow averaged over two
 * update steps (the lattice advances two steps). */
void measure(LBSys lb) {
  int fused = lb->status == POST_COLLIDE;
  if (!fused) out_of_position(lb, "Measurements");
  /* zeroforce on the device only: the force steps below change the node
   * forces at once, so the host arrays are refreshed by lbpull on demand */
  slb_check(slbc_zero_force(slb_device(lb)), "force reset");
  slb_forces_changed(lb);
  slb_trace(lb, "zeroforce");
  lb->vmeanx = lb->vmeany = lb->vmeanz = 0.0;
  accvmean(lb, 0.25);
  if (fused) fused_step(lb, 1); else { bblforce(lb); propagate(lb); collide(lb); }
  accvmean(lb, 0.5);
  if (fused) fused_step(lb, 1); else { bblforce(lb); propagate(lb); collide(lb); }
  accvmean(lb, 0.25);
  normforce(lb, 0.5);
  distribf(lb);
  slb_trace(lb, "measure");
}

/* appended: check intervals of (interval-2) lbsteps + measure until the
 * relative change of vmeanx between intervals is below tol */
int lbconverge(LBSys lb, int interval, LBReal tol, int maxsteps) {
  int steps = 0, have = 0;
  LBReal last = 0.0;
  if (interval < 3) interval = 3;
  while (steps < maxsteps) {
    lbsteps(lb, interval - 2);
    measure(lb);
    steps += interval;
    if (have && lb->vmeanx != 0.0 && fabs(lb->vmeanx - last) < tol * fabs(lb->vmeanx)) break;
    last = lb->vmeanx;
    have = 1;
  }
  return steps;
}

/* reference src/lbmeasure.c:268-301 */
void wrmeas(LBSys lb) {
  long x;
  double dx, dy, dz, discr, norm, fxt = 0.0, fyt = 0.0, fzt = 0.0, fxs = 0.0, fys = 0.0, fzs = 0.0;
  LBObj p;
  printf("\n\nProperties at lb steps %i to %i\n", lb->step - 2, lb->step);
  printf(" mean flow rate = %0.6f %0.6f %0.6f\n", lb->vmeanx, lb->vmeany, lb->vmeanz);
  for (p = lb->obj_head; p != NULL; p = p->next_obj) {
    if (slb_verbosity & FORCE_DETAILS) {
      printf(" object id %3i (base id %3i), force = %8.3f %8.3f %8.3f\n", p->id, p->base_obj->id, p->frcx, p->frcy, p->frcz);
      printf("                             torque = %8.3f %8.3f %8.3f\n", p->trqx, p->trqy, p->trqz);
    }
    fxt += p->frcx; fyt += p->frcy; fzt += p->frcz;
  }
  printf("            total force = %8.3f %8.3f %8.3f\n", fxt, fyt, fzt);
  for (x = 0; x < lb->nnodes; x++)
    if (lb->obj[x] == NULL) { fxs += lb->bx[x]; fys += lb->by[x]; fzs += lb->bz[x]; }
  printf("  total force should be = %8.3f %8.3f %8.3f\n", fxs, fys, fzs);
  dx = fxt - fxs; dy = fyt - fys; dz = fzt - fzs;
  discr = sqrt(dx * dx + dy * dy + dz * dz);
  norm = sqrt(fxs * fxs + fys * fys + fzs * fzs);
  if (norm != 0.0) discr = discr / norm;
  printf(" force discrepancy = %0.4f (norm = %0.4f)\n", discr, norm);
  slb_trace(lb, "wrforce");
}

/* reference src/lbmeasure.c:308-332 */
LBReal discrf(LBSys lb) {
  long x;
  double dx, dy, dz, norm, fxt = 0.0, fyt = 0.0, fzt = 0.0, fxs = 0.0, fys = 0.0, fzs = 0.0;
  LBReal discr;
  LBObj p;
  for (p = lb->obj_head; p != NULL; p = p->next_obj) { fxt += p->frcx; fyt += p->frcy; fzt += p->frcz; }
  for (x = 0; x < lb->nnodes; x++)
    if (lb->obj[x] == NULL) { fxs += lb->bx[x]; fys += lb->by[x]; fzs += lb->bz[x]; }
  dx = fxt - fxs; dy = fyt - fys; dz = fzt - fzs;
  discr = sqrt(dx * dx + dy * dy + dz * dz);
  norm = sqrt(fxs * fxs + fys * fys + fzs * fzs);
  if (norm != 0.0) discr = discr / norm;
  if (slb_verbosity & TRACE_ROUTINE_EXITS) printf("LB %i : wrforce done, discr = %0.4f\n", lb->step, discr);
  return discr;
}

/* reference src/lbmeasure.c:110-121 */
void vzero(LBSys lb) {
  long x;
  for (x = 0; x < lb->nnodes; x++)
    if (lb->obj[x] == NULL) lb->ux[x] = lb->uy[x] = lb->uz[x] = 0.0;
  slb_trace(lb, "vzero");
}

/* reference src/lbmeasure.c:129-166: velocity field of the fluid nodes from
 * the populations (read back from the GPU), accumulated into ux, uy, uz. */
void vgrab(LBSys lb, LBReal prefac) {
  long x;
  LBReal fac = 0.0;
  if (lb->vel_corrected) switch (lb->status) {
    case POST_PROPAGATE: fac = 0.5; break;
    case POST_COLLIDE: fac = -0.5; break;
    default: printf("vgrab apparently of position\n"); wrstatus(lb, stdout); break;
  }
  lbpull(lb);
  for (x = 0; x < lb->nnodes; x++) {
    const LBReal *t = lb->a + 15 * x;
    LBReal rho;
    if (lb->obj[x] != NULL) continue;
    rho = lb->rho0 + t[0] + t[1] + t[2] + t[3] + t[4] + t[5] + t[6] + t[7] + t[8] + t[9] + t[10] +
          t[11] + t[12] + t[13] + t[14];
    lb->ux[x] += prefac * (t[1] - t[2] + t[7] - t[8] + t[9] - t[10] + t[11] - t[12] + t[13] - t[14] + fac * lb->bx[x]) / rho;
    lb->uy[x] += prefac * (t[3] - t[4] + t[7] + t[8] - t[9] - t[10] + t[11] + t[12] - t[13] - t[14] + fac * lb->by[x]) / rho;
    lb->uz[x] += prefac * (t[5] - t[6] + t[7] + t[8] + t[9] + t[10] - t[11] - t[12] - t[13] - t[14] + fac * lb->bz[x]) / rho;
  }
  slb_trace(lb, "vgrab");
}

/* reference src/lbmeasure.c:173-203 */
void vsave(LBSys lb, char *savefile) {
  int i, j, k;
  LBReal ux, uy, uz, fac = 12.0 / lb->rho0;
  FILE *fp;
  if ((fp = fopen(savefile, "w")) == NULL) { printf("savefile: %s could not be opened\n", savefile); return; }
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    long x = slb_node(lb, i, j, k);
    if (lb->obj[x] != NULL) {
      if (lb->skip_solid) ux = uy = uz = 0.0;
      else { ux = fac * lb->ux[x]; uy = fac * lb->uy[x]; uz = fac * lb->uz[x]; }
    } else { ux = lb->ux[x]; uy = lb->uy[x]; uz = lb->uz[x]; }
    fprintf(fp, "%g %g %g %i %i %i\n", ux, uy, uz, i, j, k);
  }
  fclose(fp);
  slb_trace(lb, "lbsavevel");
}
