/*
 * ORACLE -- test infrastructure only.
 *
 * CPU restatement of the SunlightLB reference algorithm for the lattice
 * Boltzmann update path (setup, link bounce-back, streaming, collision,
 * measurement).  The GPU library is tested against it; it is never part of it:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs load
 * it.  It exports the same C API names and struct layout as the library
 * (include/sunlightlb.h), so one ctypes driver runs the library, this oracle
 * and (where it is available) a build of the reference side by side.
 *
 * Storage follows the reference: AoS populations a[15*inode + q] in double,
 * inode = esk*(esj*i + j) + k.  Loop structure (full-lattice mask scan for
 * bounce-back, three periodic sweeps for streaming, per-node collision) and
 * floating-point association are those of the reference, so results agree
 * bit for bit with a strict (no fast-math, no FMA contraction) build of it.
 * Each routine names the reference file:line it restates.
 *
 * Build: oracle/Makefile (-O2 -fno-fast-math -ffp-contract=off).
 */

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "sunlightlb.h"

int slb_verbosity = 0;
int slb_signal_flag = 0;

/* D3Q15 link table: reference src/lbmisc.c:87-104 */
static const int CX[15] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1};
static const int CY[15] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
static const int CZ[15] = {0, 0, 0, 0, 0, 1, -1, 1, 1, 1, 1, -1, -1, -1, -1};
static const int WQ[15] = {16, 8, 8, 8, 8, 8, 8, 1, 1, 1, 1, 1, 1, 1, 1};
static const int OPP[15] = {0, 2, 1, 4, 3, 6, 5, 14, 13, 12, 11, 10, 9, 8, 7};

/* ------------------------------------------------------------------------
 * small utilities (reference src/lbmisc.c:39-42, 361-378, 414-428)
 * ---------------------------------------------------------------------- */

void error(char *s) { fprintf(stderr, "Opps!  %s\n", s); exit(EXIT_FAILURE); }

static void *zalloc(size_t n) {
  void *p = calloc(n ? n : 1, 1);
  if (p == NULL) error("oracle: out of memory");
  return p;
}

char *mycat(char *s, char *t) {
  char *v = (char *)zalloc(strlen(s) + strlen(t) + 1);
  strcpy(v, s); strcat(v, t);
  return v;
}
char *mycopy(char *s) { return mycat(s, ""); }
int myscmp(char *s, char *t) { return strncmp(t, s, strlen(s)) == 0; }

void set_verbosity(int what) { slb_verbosity |= what; }
void unset_verbosity(int what) { if (slb_verbosity & what) slb_verbosity -= what; }

static long node(const LBSys lb, int i, int j, int k) {
  return (long)lb->esk * ((long)lb->esj * i + j) + k;
}

/* periodic neighbour of (i,j,k) along link q */
static long nbr(const LBSys lb, int i, int j, int k, int q) {
  int ii = i + CX[q], jj = j + CY[q], kk = k + CZ[q];
  if (ii < 0) ii = lb->esi - 1; else if (ii >= lb->esi) ii = 0;
  if (jj < 0) jj = lb->esj - 1; else if (jj >= lb->esj) jj = 0;
  if (kk < 0) kk = lb->esk - 1; else if (kk >= lb->esk) kk = 0;
  return node(lb, ii, jj, kk);
}

/* ------------------------------------------------------------------------
 * lattice construction: reference src/lbmisc.c:81-152
 * ---------------------------------------------------------------------- */

LBSys newlb(int esi, int esj, int esk, char *name) {
  LBSys lb = (LBSys)zalloc(sizeof(LBSys_type));
  long n = (long)esi * esj * esk, q;
  lb->c = (int *)zalloc(45 * sizeof(int));
  lb->w = (int *)zalloc(15 * sizeof(int));
  for (q = 0; q < 15; q++) {
    lb->c[3 * q] = CX[q]; lb->c[3 * q + 1] = CY[q]; lb->c[3 * q + 2] = CZ[q];
    lb->w[q] = WQ[q];
  }
  lb->esi = esi; lb->esj = esj; lb->esk = esk; lb->nnodes = (int)n;
  lb->a = (LBReal *)zalloc(15 * n * sizeof(LBReal));
  lb->mask = (int *)zalloc(n * sizeof(int));
  lb->obj = (LBObj *)zalloc(n * sizeof(LBObj));
  lb->ux = (LBReal *)zalloc(n * sizeof(LBReal));
  lb->uy = (LBReal *)zalloc(n * sizeof(LBReal));
  lb->uz = (LBReal *)zalloc(n * sizeof(LBReal));
  lb->fx = (LBReal *)zalloc(n * sizeof(LBReal));
  lb->fy = (LBReal *)zalloc(n * sizeof(LBReal));
  lb->fz = (LBReal *)zalloc(n * sizeof(LBReal));
  lb->bx = (LBReal *)zalloc(n * sizeof(LBReal));
  lb->by = (LBReal *)zalloc(n * sizeof(LBReal));
  lb->bz = (LBReal *)zalloc(n * sizeof(LBReal));
  lb->tau = 0.75;
  lb->rho0 = 0.0;
  for (q = 0; q < 15; q++) lb->rho0 += lb->w[q];
  lb->objects_moving = 0; lb->skip_solid = 0; lb->stokes_flow = 0;
  lb->vel_corrected = 1; lb->step = 0; lb->next_id = 0; lb->obj_head = NULL;
  lb->status = POST_COLLIDE; lb->changed_objects = 0;
  lb->rescale = 1.0; lb->load_average = 0; lb->psi = NULL; lb->rho = NULL;
  slb_verbosity = 0;
  if (myscmp("null", name)) lb->name = NULL; else lb->name = mycopy(name);
  lb->monitoring = (lb->name == NULL) ? 0 : 1;
  lb->precision = SLB_FP64; lb->priv = NULL;
  return lb;
}

/* ------------------------------------------------------------------------
 * objects: reference src/lbobjs.c:33-72
 * ---------------------------------------------------------------------- */

LBObj addobj(LBSys lb) {
  LBObj p = (LBObj)zalloc(sizeof(LBObj_type));
  p->base_obj = p;
  p->id = lb->next_id++;
  p->next_obj = lb->obj_head; lb->obj_head = p;
  return p;
}

void zeroobj(LBObj p) {
  p->posx = p->posy = p->posz = 0.0;
  p->velx = p->vely = p->velz = 0.0;
  p->angx = p->angy = p->angz = 0.0;
  p->frcx = p->frcy = p->frcz = 0.0;
  p->trqx = p->trqy = p->trqz = 0.0;
}

LBObj lookupobj(LBSys lb, int tid) {
  LBObj p;
  for (p = lb->obj_head; p != NULL; p = p->next_obj) if (p->id == tid) return p;
  return NULL;
}

/* drop the head object that was just added (insert* with no node set) */
static void drop_head(LBSys lb, LBObj p, int undo_id) {
  lb->obj_head = p->next_obj; free(p);
  if (undo_id) lb->next_id--;
}

static void free_objects(LBSys lb) {
  LBObj p = lb->obj_head, pp;
  while (p != NULL) { pp = p; p = p->next_obj; free(pp); }
  lb->next_id = 0; lb->obj_head = NULL;
}

/* reference src/lbobjs.c:128-165 */
LBObj insertlist(LBSys lb, char *listfile) {
  int i, j, k, ns = 0;
  FILE *fp;
  LBObj p;
  if ((fp = fopen(listfile, "r")) == NULL) return NULL;
  p = addobj(lb); zeroobj(p);
  while (fscanf(fp, "%i%i%i", &i, &j, &k) == 3) {
    if (i >= 0 && i < lb->esi && j >= 0 && j < lb->esj && k >= 0 && k < lb->esk) {
      lb->obj[node(lb, i, j, k)] = p; ns++;
    }
  }
  if (ns == 0) { drop_head(lb, p, 0); return NULL; }
  lb->changed_objects = 1;
  fclose(fp);
  return p;
}

/* reference src/lbobjs.c:170-199 */
LBObj insertslab(LBSys lb, LBReal x1, LBReal x2, LBReal y1, LBReal y2, LBReal z1, LBReal z2) {
  int i, j, k, ns = 0;
  LBObj p = addobj(lb);
  zeroobj(p);
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++)
    if (i > x1 && i < x2 && j > y1 && j < y2 && k > z1 && k < z2) {
      lb->obj[node(lb, i, j, k)] = p; ns++;
    }
  if (ns == 0) { drop_head(lb, p, 0); return NULL; }
  lb->changed_objects = 1;
  p->posx = 0.5 * (x1 + x2 - 1); p->posy = 0.5 * (y1 + y2 - 1); p->posz = 0.5 * (z1 + z2 - 1);
  return p;
}

/* reference src/lbobjs.c:204-232 */
LBObj insertsph(LBSys lb, LBReal rad, LBReal ox, LBReal oy, LBReal oz) {
  int i, j, k, ns = 0;
  LBReal rsq, radsq = rad * rad;
  LBObj p = addobj(lb);
  zeroobj(p);
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    rsq = (i - ox) * (i - ox) + (j - oy) * (j - oy) + (k - oz) * (k - oz);
    if (rsq < radsq) { lb->obj[node(lb, i, j, k)] = p; ns++; }
  }
  if (ns == 0) { drop_head(lb, p, 1); return NULL; }
  lb->changed_objects = 1;
  p->posx = ox; p->posy = oy; p->posz = oz;
  return p;
}

/* reference src/lbobjs.c:241-287 */
LBObj insertcyl(LBSys lb, char *type, LBReal rad, LBReal a, LBReal b) {
  int i, j, k, ns = 0, within;
  LBReal rsq = 0.0, radsq = rad * rad;
  LBObj p = addobj(lb);
  zeroobj(p);
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    switch (type[0]) {
      case 'x': case 'i': rsq = (j - a) * (j - a) + (k - b) * (k - b); break;
      case 'y': case 'j': rsq = (i - a) * (i - a) + (k - b) * (k - b); break;
      case 'z': case 'k': rsq = (i - a) * (i - a) + (j - b) * (j - b); break;
      default: error("Unrecognised cylinder direction"); return NULL;
    }
    within = (rsq < radsq);
    if (type[1] != '\0') within = !within;
    if (within) { lb->obj[node(lb, i, j, k)] = p; ns++; }
  }
  if (ns == 0) { drop_head(lb, p, 1); return NULL; }
  lb->changed_objects = 1;
  switch (type[0]) {
    case 'x': case 'i': p->posx = 0.5 * (lb->esi - 1); p->posy = a; p->posz = b; break;
    case 'y': case 'j': p->posx = a; p->posy = 0.5 * (lb->esj - 1); p->posz = b; break;
    default:            p->posx = a; p->posy = b; p->posz = 0.5 * (lb->esk - 1); break;
  }
  return p;
}

/* reference src/lbobjs.c:294-357 (an out-of-range wall leaves the freshly
 * added, empty object in the list, as the reference does) */
LBObj insertwall(LBSys lb, char *type, int wallpos) {
  int i, j, k, ns = 0, axis;
  int lim[3];
  LBObj p = addobj(lb);
  zeroobj(p);
  lim[0] = lb->esi; lim[1] = lb->esj; lim[2] = lb->esk;
  switch (type[0]) {
    case 'x': case 'i': axis = 0; break;
    case 'y': case 'j': axis = 1; break;
    case 'z': case 'k': axis = 2; break;
    default: return NULL;
  }
  if (wallpos < 0 || wallpos > lim[axis] - 1) return NULL;
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    int c = (axis == 0) ? i : (axis == 1) ? j : k;
    if (c == wallpos) { lb->obj[node(lb, i, j, k)] = p; ns++; }
  }
  p->posx = (axis == 0) ? wallpos : 0.5 * (lb->esi - 1);
  p->posy = (axis == 1) ? wallpos : 0.5 * (lb->esj - 1);
  p->posz = (axis == 2) ? wallpos : 0.5 * (lb->esk - 1);
  if (ns == 0) { drop_head(lb, p, 0); return NULL; }
  lb->changed_objects = 1;
  return p;
}

/* reference src/lbobjs.c:362-392 (mode 0) and 397-428 (mode 1) */
static LBObj merge_objects(LBSys lb, int invert) {
  int i, j, k, ns = 0;
  LBReal ox = 0.0, oy = 0.0, oz = 0.0;
  LBObj p;
  free_objects(lb);
  p = addobj(lb); zeroobj(p);
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    long n = node(lb, i, j, k);
    int solid = lb->obj[n] != NULL;
    if (invert) {
      if (solid) { lb->obj[n] = NULL; continue; }
    } else if (!solid) continue;
    ox += (double)i; oy += (double)j; oz += (double)k; ns++; lb->obj[n] = p;
  }
  if (ns == 0) { drop_head(lb, p, 0); return NULL; }
  lb->changed_objects = 1;
  p->posx = ox / ns; p->posy = oy / ns; p->posz = oz / ns;
  return p;
}
LBObj flattenobj(LBSys lb) { return merge_objects(lb, 0); }
LBObj invertobj(LBSys lb) { return merge_objects(lb, 1); }

/* reference src/lbobjs.c:433-453 */
void removeobjs(LBSys lb) {
  long n;
  free_objects(lb);
  for (n = 0; n < lb->nnodes; n++) {
    lb->obj[n] = NULL;
    lb->ux[n] = lb->uy[n] = lb->uz[n] = 0.0;
    lb->fx[n] = lb->fy[n] = lb->fz[n] = 0.0;
  }
  memset(lb->a, 0, 15 * (size_t)lb->nnodes * sizeof(LBReal));
  lb->changed_objects = 1;
}

/* reference src/lbobjs.c:526-560 */
void makemask(LBSys lb) {
  int i, j, k, q;
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    long n = node(lb, i, j, k);
    int val = 0;
    if (lb->obj[n] != NULL)
      for (q = 1; q < 15; q++)
        if (lb->obj[nbr(lb, i, j, k, q)] == NULL) val |= 1 << (q - 1);
    lb->mask[n] = val;
  }
}

/* wall velocity of object p at node (i,j,k), times rho0/12:
 * reference src/lbobjs.c:582-585 (also src/mpkernel.c:264-267) */
static void wall_velocity(LBSys lb, LBObj p, int i, int j, int k, LBReal *u) {
  LBReal rx = i - p->posx, ry = j - p->posy, rz = k - p->posz, rho0 = lb->rho0;
  u[0] = rho0 * ((p->velx) + (p->angy) * rz - (p->angz) * ry) / 12.0;
  u[1] = rho0 * ((p->vely) + (p->angz) * rx - (p->angx) * rz) / 12.0;
  u[2] = rho0 * ((p->velz) + (p->angx) * ry - (p->angy) * rx) / 12.0;
}

/* reference src/lbobjs.c:565-589 */
void vspread(LBSys lb) {
  int i, j, k;
  LBReal u[3];
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    long n = node(lb, i, j, k);
    LBObj p = lb->obj[n];
    if (p == NULL) { lb->ux[n] = lb->uy[n] = lb->uz[n] = 0.0; continue; }
    wall_velocity(lb, p, i, j, k, u);
    lb->ux[n] = u[0]; lb->uy[n] = u[1]; lb->uz[n] = u[2];
  }
}

/* reference src/lbobjs.c:593-619 */
void zerobf(LBSys lb) {
  long n;
  for (n = 0; n < lb->nnodes; n++)
    if (lb->obj[n] == NULL) lb->bx[n] = lb->by[n] = lb->bz[n] = 0.0;
}
void addbf(LBSys lb, double fx, double fy, double fz) {
  long n;
  for (n = 0; n < lb->nnodes; n++)
    if (lb->obj[n] == NULL) {
      lb->bx[n] += (LBReal)fx; lb->by[n] += (LBReal)fy; lb->bz[n] += (LBReal)fz;
    }
}

/* reference src/lbobjs.c:623-643 */
void vset(LBSys lb, int i, int j, int k, LBReal vx, LBReal vy, LBReal vz) {
  long n;
  if (i < 0 || i >= lb->esi || j < 0 || j >= lb->esj || k < 0 || k >= lb->esk) return;
  n = node(lb, i, j, k);
  if (lb->obj[n] == NULL) return;
  lb->ux[n] = lb->rho0 * vx / 12.0;
  lb->uy[n] = lb->rho0 * vy / 12.0;
  lb->uz[n] = lb->rho0 * vz / 12.0;
}

/* reference src/lbobjs.c:648-663 */
int countfluid(LBSys lb) {
  long n;
  int count = 0;
  for (n = 0; n < lb->nnodes; n++) if (lb->obj[n] == NULL) count++;
  return count;
}
void syncobjs(LBSys lb) { makemask(lb); countfluid(lb); lb->changed_objects = 0; }

/* reference src/lbobjs.c:671-714 */
int countmask(LBSys lb, char *type) {
  long n;
  int q, count = 0, faces;
  switch (type[0]) {
    case 'a': case 'l': faces = 0; break;
    case 'f': case 's': faces = 1; break;
    default: printf("countmask: expected 'links' or 'faces'\n"); return 0;
  }
  for (n = 0; n < lb->nnodes; n++) {
    int m = lb->mask[n];
    if (m <= 0) continue;
    for (q = 1; q < (faces ? 7 : 15); q++)
      if (m & (1 << (q - 1))) count += faces ? 1 : lb->w[q];
  }
  return count;
}

/* ------------------------------------------------------------------------
 * link bounce-back: reference src/lbkernel.c:58-618
 * ---------------------------------------------------------------------- */

/* moving-wall momentum term of link q at a solid node with velocity u
 * (ux,uy,uz already carry rho0/12): reference src/lbkernel.c:360-446 */
static LBReal link_term(int q, LBReal ux, LBReal uy, LBReal uz) {
  if (q <= 6) {
    LBReal u = (q <= 2) ? ux : (q <= 4) ? uy : uz;
    return (q & 1) ? 8.0 * u : -8.0 * u;
  }
  return ((CX[q] > 0 ? ux : -ux) + (CY[q] > 0 ? uy : -uy)) + (CZ[q] > 0 ? uz : -uz);
}

static void bounce(LBSys lb, int with_force) {
  int i, j, k, q;
  LBReal *aa = lb->a;
  if (lb->status != POST_COLLIDE) printf("Bounceback apparently out of position\n");
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    long s = node(lb, i, j, k);
    int m = lb->mask[s];
    if (m <= 0) continue;
    for (q = 1; q < 15; q++) {
      long f;
      LBReal a, b, term = 0.0, dp;
      if (!(m & (1 << (q - 1)))) continue;
      f = nbr(lb, i, j, k, q);
      a = aa[q + 15 * s]; b = aa[OPP[q] + 15 * f];
      if (lb->objects_moving) {
        term = link_term(q, lb->ux[s], lb->uy[s], lb->uz[s]);
        aa[OPP[q] + 15 * f] = a - term; aa[q + 15 * s] = b + term;
        dp = 2.0 * (a - b - term);
      } else {
        aa[q + 15 * s] = b; aa[OPP[q] + 15 * f] = a;
        dp = 2.0 * (a - b);
      }
      if (!with_force) continue;
      if (CX[q] > 0) lb->fx[s] += dp; else if (CX[q] < 0) lb->fx[s] -= dp;
      if (CY[q] > 0) lb->fy[s] += dp; else if (CY[q] < 0) lb->fy[s] -= dp;
      if (CZ[q] > 0) lb->fz[s] += dp; else if (CZ[q] < 0) lb->fz[s] -= dp;
    }
  }
  lb->status = POST_BBL;
}

/* reference src/lbkernel.c:35-45 */
void bbl(LBSys lb) { if (lb->changed_objects) syncobjs(lb); bounce(lb, 0); }
void bblforce(LBSys lb) { if (lb->changed_objects) syncobjs(lb); bounce(lb, 1); }

/* ------------------------------------------------------------------------
 * streaming: reference src/lbkernel.c:623-762.  Three periodic sweeps; in
 * each, the five populations moving up the axis shift by +1 and the five
 * moving down shift by -1, with wrap-around through a saved end value.
 * ---------------------------------------------------------------------- */

static const int UP[3][5] = {{1, 7, 9, 11, 13}, {3, 7, 8, 11, 12}, {5, 7, 8, 9, 10}};
static const int DN[3][5] = {{2, 8, 10, 12, 14}, {4, 9, 10, 13, 14}, {6, 11, 12, 13, 14}};

static void sweep_line(LBReal *aa, long first, long stride, int len, int axis) {
  LBReal keep_up[5], keep_dn[5];
  int m, p;
  long last = first + (long)(len - 1) * stride;
  for (p = 0; p < 5; p++) {
    keep_up[p] = aa[UP[axis][p] + 15 * last];
    keep_dn[p] = aa[DN[axis][p] + 15 * first];
  }
  for (m = len - 1; m > 0; m--) {
    long to = first + m * stride, from = to - stride;
    for (p = 0; p < 5; p++) aa[UP[axis][p] + 15 * to] = aa[UP[axis][p] + 15 * from];
  }
  for (m = 0; m < len - 1; m++) {
    long to = first + m * stride, from = to + stride;
    for (p = 0; p < 5; p++) aa[DN[axis][p] + 15 * to] = aa[DN[axis][p] + 15 * from];
  }
  for (p = 0; p < 5; p++) {
    aa[UP[axis][p] + 15 * first] = keep_up[p];
    aa[DN[axis][p] + 15 * last] = keep_dn[p];
  }
}

void propagate(LBSys lb) {
  int i, j, k;
  long sj = lb->esk, si = (long)lb->esj * lb->esk;
  if (lb->status != POST_BBL) printf("Propagation apparently out of position\n");
  for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++)
    sweep_line(lb->a, node(lb, 0, j, k), si, lb->esi, 0);
  for (i = 0; i < lb->esi; i++) for (k = 0; k < lb->esk; k++)
    sweep_line(lb->a, node(lb, i, 0, k), sj, lb->esj, 1);
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++)
    sweep_line(lb->a, node(lb, i, j, 0), 1, lb->esk, 2);
  lb->status = POST_PROPAGATE;
}

/* ------------------------------------------------------------------------
 * collision: reference src/lbkernel.c:769-877.  The moments drho, ru and
 * the stress are formed from partial sums, the stress relaxes by
 * comega = 1 - 1/tau (plus the rho u u term for Navier-Stokes), and the 15
 * populations are rebuilt from these moments alone.  The evaluation order
 * below is the reference's.
 * ---------------------------------------------------------------------- */

/* rebuild the 15 populations from drho, ru and the stress:
 * reference src/lbkernel.c:838-865 (also src/lbstore.c:362-389) */
static void rebuild(LBReal *t, LBReal drho, LBReal rux, LBReal ruy, LBReal ruz,
                    LBReal sxx, LBReal syy, LBReal szz, LBReal sxy, LBReal sxz, LBReal syz) {
  const LBReal b = 72.0, dbybc2 = 1.0 / 24.0, dd2bybc4 = 1.0 / 8.0;
  const LBReal fdd2bybc4 = 4.0 * dd2bybc4, edbybc2 = 8.0 * dbybc2;
  LBReal rhobyb = drho / b, erhobyb = 8.0 * rhobyb;
  LBReal trsby3 = (sxx + syy + szz) / 3.0, ru, st;
  t[0] = 2.0 * erhobyb - 2.0 * fdd2bybc4 * trsby3;
  ru = edbybc2 * rux; st = fdd2bybc4 * (sxx - trsby3);
  t[1] = erhobyb + ru + st; t[2] = erhobyb - ru + st;
  ru = edbybc2 * ruy; st = fdd2bybc4 * (syy - trsby3);
  t[3] = erhobyb + ru + st; t[4] = erhobyb - ru + st;
  ru = edbybc2 * ruz; st = fdd2bybc4 * (szz - trsby3);
  t[5] = erhobyb + ru + st; t[6] = erhobyb - ru + st;
  ru = dbybc2 * (rux + ruy + ruz); st = dd2bybc4 * (trsby3 + sxy + sxz + syz);
  t[7] = rhobyb + ru + st; t[14] = rhobyb - ru + st;
  ru = dbybc2 * (rux - ruy - ruz); st = dd2bybc4 * (trsby3 - sxy - sxz + syz);
  t[8] = rhobyb - ru + st; t[13] = rhobyb + ru + st;
  ru = dbybc2 * (rux - ruy + ruz); st = dd2bybc4 * (trsby3 - sxy + sxz - syz);
  t[9] = rhobyb + ru + st; t[12] = rhobyb - ru + st;
  ru = dbybc2 * (rux + ruy - ruz); st = dd2bybc4 * (trsby3 + sxy - sxz - syz);
  t[10] = rhobyb - ru + st; t[11] = rhobyb + ru + st;
}

void collide(LBSys lb) {
  long n;
  LBReal omega = 1.0 / lb->tau, comega = 1.0 - omega, twoby3 = 2.0 / 3.0;
  LBReal rho0 = lb->rho0;
  if (lb->status != POST_PROPAGATE) printf("Collision apparently out of position\n");
  for (n = 0; n < lb->nnodes; n++) {
    LBReal *t = lb->a + 15 * n;
    LBReal p12, p34, p56, lo_sum, hi_sum, lo_x, hi_x, lo_y, hi_y, lo_xy, hi_xy;
    LBReal p06, drho, rux, ruy, ruz, sdiag, sxx, syy, szz, sxy, sxz, syz;
    int fluid = lb->obj[n] == NULL;
    if (lb->skip_solid && !fluid) continue;
    p12 = t[1] + t[2]; p34 = t[3] + t[4]; p56 = t[5] + t[6];
    lo_sum = t[7] + t[8] + t[9] + t[10]; hi_sum = t[11] + t[12] + t[13] + t[14];
    lo_x = t[7] - t[8] + t[9] - t[10];   hi_x = t[11] - t[12] + t[13] - t[14];
    lo_y = t[7] + t[8] - t[9] - t[10];   hi_y = t[11] + t[12] - t[13] - t[14];
    lo_xy = t[7] - t[8] - t[9] + t[10];  hi_xy = t[11] - t[12] - t[13] + t[14];
    p06 = t[0] + p12 + p34 + p56;
    drho = p06 + (lo_sum + hi_sum);
    rux = t[1] - t[2] + lo_x + hi_x;
    ruy = t[3] - t[4] + lo_y + hi_y;
    ruz = t[5] - t[6] + lo_sum - hi_sum;
    if (fluid) { rux += lb->bx[n]; ruy += lb->by[n]; ruz += lb->bz[n]; }
    sdiag = twoby3 * drho - p06;
    sxx = sdiag + p12; syy = sdiag + p34; szz = sdiag + p56;
    sxy = lo_xy + hi_xy; sxz = lo_x - hi_x; syz = lo_y - hi_y;
    if (lb->stokes_flow) {
      sxx = comega * sxx; sxy = comega * sxy; sxz = comega * sxz;
      syy = comega * syy; syz = comega * syz; szz = comega * szz;
    } else {
      LBReal obyr = omega / (rho0 + drho);
      sxx = comega * sxx + obyr * rux * rux;
      sxy = comega * sxy + obyr * rux * ruy;
      sxz = comega * sxz + obyr * rux * ruz;
      syy = comega * syy + obyr * ruy * ruy;
      syz = comega * syz + obyr * ruy * ruz;
      szz = comega * szz + obyr * ruz * ruz;
    }
    rebuild(t, drho, rux, ruy, ruz, sxx, syy, szz, sxy, sxz, syz);
  }
  lb->step += 1;
  lb->status = POST_COLLIDE;
}

/* reference src/lbkernel.c:49-51 */
void lbstep(LBSys lb) { bbl(lb); propagate(lb); collide(lb); }

/* ------------------------------------------------------------------------
 * measurement: reference src/lbmeasure.c
 * ---------------------------------------------------------------------- */

/* reference src/lbmeasure.c:58-106 */
void accvmean(LBSys lb, LBReal prefac) {
  long n;
  int nfluid = 0;
  LBReal fac = 0.0, uxtot = 0.0, uytot = 0.0, uztot = 0.0, wnorm = 0.0, wfac = 1.0;
  if (lb->vel_corrected) {
    if (lb->status == POST_PROPAGATE) fac = 0.5;
    else if (lb->status == POST_COLLIDE) fac = -0.5;
    else printf("Accvmean apparently of position\n");
  }
  for (n = 0; n < lb->nnodes; n++) {
    const LBReal *t = lb->a + 15 * n;
    LBReal rho, ux, uy, uz;
    if (lb->obj[n] != NULL) continue;
    rho = lb->rho0 + t[0] + t[1] + t[2] + t[3] + t[4] + t[5] + t[6]
          + t[7] + t[8] + t[9] + t[10] + t[11] + t[12] + t[13] + t[14];
    ux = (t[1] - t[2] + t[7] - t[8] + t[9] - t[10] + t[11] - t[12] + t[13] - t[14] + fac * lb->bx[n]) / rho;
    uy = (t[3] - t[4] + t[7] + t[8] - t[9] - t[10] + t[11] + t[12] - t[13] - t[14] + fac * lb->by[n]) / rho;
    uz = (t[5] - t[6] + t[7] + t[8] + t[9] + t[10] - t[11] - t[12] - t[13] - t[14] + fac * lb->bz[n]) / rho;
    if (lb->psi != NULL) { wfac = lb->psi[n]; wfac = wfac * wfac; }
    uxtot += wfac * ux; uytot += wfac * uy; uztot += wfac * uz; wnorm += wfac;
    nfluid++;
  }
  wfac = nfluid / wnorm;
  uxtot *= wfac; uytot *= wfac; uztot *= wfac;
  lb->vmeanx += prefac * uxtot / (lb->nnodes);
  lb->vmeany += prefac * uytot / (lb->nnodes);
  lb->vmeanz += prefac * uztot / (lb->nnodes);
}

/* reference src/lbmeasure.c:110-121 */
void vzero(LBSys lb) {
  long n;
  for (n = 0; n < lb->nnodes; n++)
    if (lb->obj[n] == NULL) lb->ux[n] = lb->uy[n] = lb->uz[n] = 0.0;
}

/* reference src/lbmeasure.c:129-166 */
void vgrab(LBSys lb, LBReal prefac) {
  long n;
  LBReal fac = 0.0;
  if (lb->vel_corrected) {
    if (lb->status == POST_PROPAGATE) fac = 0.5;
    else if (lb->status == POST_COLLIDE) fac = -0.5;
  }
  for (n = 0; n < lb->nnodes; n++) {
    const LBReal *t = lb->a + 15 * n;
    LBReal rho;
    if (lb->obj[n] != NULL) continue;
    rho = lb->rho0 + t[0] + t[1] + t[2] + t[3] + t[4] + t[5] + t[6]
          + t[7] + t[8] + t[9] + t[10] + t[11] + t[12] + t[13] + t[14];
    lb->ux[n] += prefac * (t[1] - t[2] + t[7] - t[8] + t[9] - t[10] + t[11] - t[12] + t[13] - t[14] + fac * lb->bx[n]) / rho;
    lb->uy[n] += prefac * (t[3] - t[4] + t[7] + t[8] - t[9] - t[10] + t[11] + t[12] - t[13] - t[14] + fac * lb->by[n]) / rho;
    lb->uz[n] += prefac * (t[5] - t[6] + t[7] + t[8] + t[9] + t[10] - t[11] - t[12] - t[13] - t[14] + fac * lb->bz[n]) / rho;
  }
}

/* reference src/lbmeasure.c:208-231 */
void zeroforce(LBSys lb) {
  long n;
  for (n = 0; n < lb->nnodes; n++) lb->fx[n] = lb->fy[n] = lb->fz[n] = 0.0;
}
void normforce(LBSys lb, LBReal fac) {
  long n;
  for (n = 0; n < lb->nnodes; n++) { lb->fx[n] *= fac; lb->fy[n] *= fac; lb->fz[n] *= fac; }
}

/* reference src/lbmeasure.c:236-263 */
void distribf(LBSys lb) {
  int i, j, k;
  LBObj p;
  for (p = lb->obj_head; p != NULL; p = p->next_obj) {
    p->frcx = p->frcy = p->frcz = 0.0;
    p->trqx = p->trqy = p->trqz = 0.0;
  }
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    long n = node(lb, i, j, k);
    LBReal rx, ry, rz, fx, fy, fz;
    if ((p = lb->obj[n]) == NULL) continue;
    rx = i - p->posx; ry = j - p->posy; rz = k - p->posz;
    fx = lb->fx[n]; fy = lb->fy[n]; fz = lb->fz[n];
    p->frcx += fx; p->frcy += fy; p->frcz += fz;
    p->trqx += ry * fz - rz * fy;
    p->trqy += rz * fx - rx * fz;
    p->trqz += rx * fy - ry * fx;
  }
}

/* reference src/lbmeasure.c:30-49 */
void measure(LBSys lb) {
  if (lb->status != POST_COLLIDE) printf("Measurements apparently out of position\n");
  zeroforce(lb);
  lb->vmeanx = lb->vmeany = lb->vmeanz = 0.0;
  accvmean(lb, 0.25);
  bblforce(lb); propagate(lb); collide(lb);
  accvmean(lb, 0.5);
  bblforce(lb); propagate(lb); collide(lb);
  accvmean(lb, 0.25);
  normforce(lb, 0.5);
  distribf(lb);
}

/* reference src/lbmeasure.c:308-332 */
LBReal discrf(LBSys lb) {
  long n;
  double fxt = 0.0, fyt = 0.0, fzt = 0.0, fxs = 0.0, fys = 0.0, fzs = 0.0, dx, dy, dz, nrm;
  LBReal d;
  LBObj p;
  for (p = lb->obj_head; p != NULL; p = p->next_obj) { fxt += p->frcx; fyt += p->frcy; fzt += p->frcz; }
  for (n = 0; n < lb->nnodes; n++)
    if (lb->obj[n] == NULL) { fxs += lb->bx[n]; fys += lb->by[n]; fzs += lb->bz[n]; }
  dx = fxt - fxs; dy = fyt - fys; dz = fzt - fzs;
  d = sqrt(dx * dx + dy * dy + dz * dz);
  nrm = sqrt(fxs * fxs + fys * fys + fzs * fzs);
  if (nrm != 0.0) d = d / nrm;
  return d;
}

/* ------------------------------------------------------------------------
 * warm start from a velocity field: the rebuild of reference
 * src/lbstore.c:340-401 (lbloadvel), applied to arrays instead of a file.
 * rho may be NULL (then rho = rho0 everywhere).
 * ---------------------------------------------------------------------- */
void lbsetvel(LBSys lb, LBReal *rho, LBReal *ux, LBReal *uy, LBReal *uz) {
  long n;
  int q;
  if (lb->changed_objects) syncobjs(lb);
  for (n = 0; n < lb->nnodes; n++) {
    LBReal r = rho ? rho[n] : lb->rho0;
    LBReal vx = lb->rescale * ux[n], vy = lb->rescale * uy[n], vz = lb->rescale * uz[n];
    LBReal drho = r - lb->rho0, rux = r * vx, ruy = r * vy, ruz = r * vz;
    LBReal sxx = 0.0, syy = 0.0, szz = 0.0, sxy = 0.0, sxz = 0.0, syz = 0.0;
    if (!lb->stokes_flow) {
      sxx = vx * rux; sxy = vx * ruy; sxz = vx * ruz;
      syy = vy * ruy; syz = vy * ruz; szz = vz * ruz;
    }
    rebuild(lb->a + 15 * n, drho, rux, ruy, ruz, sxx, syy, szz, sxy, sxz, syz);
  }
  if (lb->skip_solid)
    for (n = 0; n < lb->nnodes; n++)
      if (lb->obj[n] != NULL) for (q = 0; q < 15; q++) lb->a[q + 15 * n] = 0.0;
  lb->status = POST_PROPAGATE;
  collide(lb);
  lb->rescale = 1.0;
}

/* reference src/lbstore.c:305-404: velocity file -> lbsetvel */
void lbloadvel(LBSys lb, char *loadfile, char *type) {
  long n, N = lb->nnodes;
  int binary = (type[0] == 'b' || type[0] == 'B'), i, j, k;
  LBReal *r, *vx, *vy, *vz;
  FILE *fp;
  if (lb->changed_objects) syncobjs(lb);
  if (myscmp("null", loadfile)) return;
  if ((fp = fopen(loadfile, "r")) == NULL) { printf("lbloadvel: %s could not be opened\n", loadfile); exit(EXIT_FAILURE); }
  r = (LBReal *)zalloc(N * sizeof(LBReal)); vx = (LBReal *)zalloc(N * sizeof(LBReal));
  vy = (LBReal *)zalloc(N * sizeof(LBReal)); vz = (LBReal *)zalloc(N * sizeof(LBReal));
  for (n = 0; n < N; n++) {
    if (binary) {
      if (fread(&r[n], sizeof(LBReal), 1, fp) != 1 || fread(&vx[n], sizeof(LBReal), 1, fp) != 1 ||
          fread(&vy[n], sizeof(LBReal), 1, fp) != 1 || fread(&vz[n], sizeof(LBReal), 1, fp) != 1) break;
    } else {
      float tr, tx, ty, tz;
      if (fscanf(fp, "%f%f%f%f%i%i%i", &tr, &tx, &ty, &tz, &i, &j, &k) != 7) break;
      r[n] = tr; vx[n] = tx; vy[n] = ty; vz[n] = tz;
    }
  }
  fclose(fp);
  lbsetvel(lb, r, vx, vy, vz);
  free(r); free(vx); free(vy); free(vz);
}


/* ------------------------------------------------------------------------
 * moment checkpoint: reference src/lbstore.c:36-218.  drho and the momenta
 * are LBStoreReal (float) variables in the reference, so the stress uses the
 * rounded drho and some of the rebuild sums run in float; kept here.
 * ---------------------------------------------------------------------- */
void lbsave(LBSys lb, char *savefile) {
  long n;
  FILE *fp;
  const LBReal twoby3 = 2.0 / 3.0;
  if ((fp = fopen(savefile, "wb")) == NULL) { printf("savefile: %s could not be opened\n", savefile); return; }
  bbl(lb); propagate(lb);
  for (n = 0; n < lb->nnodes; n++) {
    const LBReal *t = lb->a + 15 * n;
    LBReal p12 = t[1] + t[2], p34 = t[3] + t[4], p56 = t[5] + t[6];
    LBReal lo_sum = t[7] + t[8] + t[9] + t[10], hi_sum = t[11] + t[12] + t[13] + t[14];
    LBReal lo_x = t[7] - t[8] + t[9] - t[10], hi_x = t[11] - t[12] + t[13] - t[14];
    LBReal lo_y = t[7] + t[8] - t[9] - t[10], hi_y = t[11] + t[12] - t[13] - t[14];
    LBReal lo_xy = t[7] - t[8] - t[9] + t[10], hi_xy = t[11] - t[12] - t[13] + t[14];
    LBReal p06 = t[0] + p12 + p34 + p56, sd;
    LBStoreReal m[10];
    m[0] = p06 + (lo_sum + hi_sum);
    m[1] = t[1] - t[2] + lo_x + hi_x;
    m[2] = t[3] - t[4] + lo_y + hi_y;
    m[3] = t[5] - t[6] + lo_sum - hi_sum;
    sd = twoby3 * m[0] - p06;
    m[4] = sd + p12; m[5] = sd + p34; m[6] = sd + p56;
    m[7] = lo_xy + hi_xy; m[8] = lo_x - hi_x; m[9] = lo_y - hi_y;
    fwrite(m, sizeof(LBStoreReal), 10, fp);
  }
  fclose(fp);
  collide(lb);
}

void lbload(LBSys lb, char *loadfile) {
  long n;
  int q;
  FILE *fp;
  LBReal b = 72.0, dbybc2 = 1.0 / 24.0, dd2bybc4 = 1.0 / 8.0;
  LBReal fdd2bybc4 = 4.0 * dd2bybc4, edbybc2 = 8.0 * dbybc2;
  if (lb->changed_objects) syncobjs(lb);
  if ((fp = fopen(loadfile, "r")) == NULL) { printf("lbload: %s could not be opened\n", loadfile); exit(EXIT_FAILURE); }
  for (n = 0; n < lb->nnodes; n++) {
    LBStoreReal s[10], drho, rux, ruy, ruz, sxx, syy, szz, sxy, sxz, syz;
    LBReal rhobyb, erhobyb, trsby3, ru, st, v[15];
    if (fread(s, sizeof(LBStoreReal), 10, fp) != 10) memset(s, 0, sizeof s);
    drho = s[0];
    rux = (lb->rescale) * s[1]; ruy = (lb->rescale) * s[2]; ruz = (lb->rescale) * s[3];
    sxx = s[4]; syy = s[5]; szz = s[6]; sxy = s[7]; sxz = s[8]; syz = s[9];
    rhobyb = drho / b; erhobyb = 8.0 * rhobyb;
    trsby3 = (sxx + syy + szz) / 3.0;
    v[0] = 2.0 * erhobyb - 2.0 * fdd2bybc4 * trsby3;
    ru = edbybc2 * rux; st = fdd2bybc4 * (sxx - trsby3);
    v[1] = erhobyb + ru + st; v[2] = erhobyb - ru + st;
    ru = edbybc2 * ruy; st = fdd2bybc4 * (syy - trsby3);
    v[3] = erhobyb + ru + st; v[4] = erhobyb - ru + st;
    ru = edbybc2 * ruz; st = fdd2bybc4 * (szz - trsby3);
    v[5] = erhobyb + ru + st; v[6] = erhobyb - ru + st;
    ru = dbybc2 * (rux + ruy + ruz); st = dd2bybc4 * (trsby3 + sxy + sxz + syz);
    v[7] = rhobyb + ru + st; v[14] = rhobyb - ru + st;
    ru = dbybc2 * (rux - ruy - ruz); st = dd2bybc4 * (trsby3 - sxy - sxz + syz);
    v[8] = rhobyb - ru + st; v[13] = rhobyb + ru + st;
    ru = dbybc2 * (rux - ruy + ruz); st = dd2bybc4 * (trsby3 - sxy + sxz - syz);
    v[9] = rhobyb + ru + st; v[12] = rhobyb - ru + st;
    ru = dbybc2 * (rux + ruy - ruz); st = dd2bybc4 * (trsby3 + sxy - sxz - syz);
    v[10] = rhobyb - ru + st; v[11] = rhobyb + ru + st;
    for (q = 0; q < 15; q++) {
      if (lb->load_average) lb->a[q + 15 * n] += 0.5 * v[q];
      else lb->a[q + 15 * n] = v[q];
    }
  }
  fclose(fp);
  if (lb->skip_solid)
    for (n = 0; n < lb->nnodes; n++)
      if (lb->obj[n] != NULL) for (q = 0; q < 15; q++) lb->a[q + 15 * n] = 0.0;
  lb->status = POST_PROPAGATE;
  collide(lb);
  lb->rescale = 1.0;
}

/* ------------------------------------------------------------------------
 * field and object files: reference src/lbstore.c:227-296, 412-678 and
 * src/lbmeasure.c:173-203.  Byte layouts and printf formats are the
 * reference's (they define the file formats); the arithmetic of each value
 * follows the reference's association.
 * ---------------------------------------------------------------------- */

/* fluid velocity of one node's populations plus fac times a force, with the
 * density: reference src/lbstore.c:277-283 */
static LBReal node_velocity(const LBSys lb, const LBReal *t, LBReal fac, LBReal gx, LBReal gy,
                            LBReal gz, LBReal u[3]) {
  LBReal rho = lb->rho0 + t[0] + t[1] + t[2] + t[3] + t[4] + t[5] + t[6] + t[7] + t[8] + t[9]
               + t[10] + t[11] + t[12] + t[13] + t[14];
  u[0] = (t[1] - t[2] + t[7] - t[8] + t[9] - t[10] + t[11] - t[12] + t[13] - t[14] + fac * gx) / rho;
  u[1] = (t[3] - t[4] + t[7] + t[8] - t[9] - t[10] + t[11] + t[12] - t[13] - t[14] + fac * gy) / rho;
  u[2] = (t[5] - t[6] + t[7] + t[8] + t[9] + t[10] - t[11] - t[12] - t[13] - t[14] + fac * gz) / rho;
  return rho;
}

/* reference src/lbstore.c:227-296: the correction uses the node force
 * arrays fx, fy, fz (as the reference does), and a solid node of a
 * skip_solid lattice repeats the density of the node written before it */
void lbsavevel(LBSys lb, char *savefile, char *type) {
  int i, j, k, binary = (type[0] == 'b' || type[0] == 'B');
  LBReal fac = 0.0, rho = 0.0, u[3];
  FILE *fp = fopen(savefile, "w");
  if (fp == NULL) { printf("savefile: %s could not be opened\n", savefile); return; }
  if (lb->vel_corrected) {
    if (lb->status == POST_PROPAGATE) fac = 0.5;
    else if (lb->status == POST_COLLIDE) fac = -0.5;
  }
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    long n = node(lb, i, j, k);
    if (lb->obj[n] != NULL && lb->skip_solid) u[0] = u[1] = u[2] = 0.0;
    else rho = node_velocity(lb, lb->a + 15 * n, fac, lb->fx[n], lb->fy[n], lb->fz[n], u);
    if (binary) {
      fwrite(&rho, sizeof(LBReal), 1, fp);
      fwrite(u, sizeof(LBReal), 3, fp);
    } else {
      fprintf(fp, "%g %g %g %g %i %i %i\n", rho, u[0], u[1], u[2], i, j, k);
    }
  }
  fclose(fp);
}

/* reference src/lbmeasure.c:173-203 */
void vsave(LBSys lb, char *savefile) {
  int i, j, k;
  LBReal scale = 12.0 / lb->rho0, v[3];
  FILE *fp = fopen(savefile, "w");
  if (fp == NULL) { printf("savefile: %s could not be opened\n", savefile); return; }
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    long n = node(lb, i, j, k);
    if (lb->obj[n] == NULL) { v[0] = lb->ux[n]; v[1] = lb->uy[n]; v[2] = lb->uz[n]; }
    else if (lb->skip_solid) v[0] = v[1] = v[2] = 0.0;
    else { v[0] = scale * lb->ux[n]; v[1] = scale * lb->uy[n]; v[2] = scale * lb->uz[n]; }
    fprintf(fp, "%g %g %g %i %i %i\n", v[0], v[1], v[2], i, j, k);
  }
  fclose(fp);
}

/* the six stress moments of one node's populations: reference
 * src/lbstore.c:446-458 */
static void node_stress(const LBReal *t, LBReal s[6]) {
  LBReal p12 = t[1] + t[2], p34 = t[3] + t[4], p56 = t[5] + t[6];
  LBReal lo_sum = t[7] + t[8] + t[9] + t[10], hi_sum = t[11] + t[12] + t[13] + t[14];
  LBReal lo_x = t[7] - t[8] + t[9] - t[10], hi_x = t[11] - t[12] + t[13] - t[14];
  LBReal lo_y = t[7] + t[8] - t[9] - t[10], hi_y = t[11] + t[12] - t[13] - t[14];
  LBReal lo_xy = t[7] - t[8] - t[9] + t[10], hi_xy = t[11] - t[12] - t[13] + t[14];
  LBReal p06 = t[0] + p12 + p34 + p56, drho = p06 + (lo_sum + hi_sum);
  LBReal sd = (2.0 / 3.0) * drho - p06;
  s[0] = sd + p12; s[1] = sd + p34; s[2] = sd + p56;
  s[3] = lo_xy + hi_xy; s[4] = lo_x - hi_x; s[5] = lo_y - hi_y;
}

/* reference src/lbstore.c:412-515: mean of the post-propagation and
 * post-collision stress (one update step).  The binary form writes each
 * LBReal with sizeof(LBStoreReal) bytes, as the reference does. */
void lbsavestr(LBSys lb, char *savefile, char *type) {
  long n, N = lb->nnodes;
  int c, binary = (type[0] == 'b' || type[0] == 'B');
  LBReal *acc = (LBReal *)zalloc(6 * N * sizeof(LBReal)), s[6];
  FILE *fp;
  bbl(lb); propagate(lb);
  for (n = 0; n < N; n++) {
    node_stress(lb->a + 15 * n, s);
    for (c = 0; c < 6; c++) acc[6 * n + c] = s[c];
  }
  collide(lb);
  for (n = 0; n < N; n++) {
    node_stress(lb->a + 15 * n, s);
    for (c = 0; c < 6; c++) acc[6 * n + c] += s[c];
  }
  if ((fp = fopen(savefile, "wb")) == NULL) { printf("savefile: %s could not be opened\n", savefile); free(acc); return; }
  for (n = 0; n < N; n++) {
    int fluid = lb->obj[n] == NULL;
    for (c = 0; c < 6; c++) s[c] = (!fluid && lb->skip_solid) ? 0.0 : 0.5 * acc[6 * n + c];
    if (binary) {
      for (c = 0; c < 6; c++) fwrite(&s[c], sizeof(LBStoreReal), 1, fp);
      fwrite(&fluid, sizeof(int), 1, fp);
    } else {
      fprintf(fp, "%f\t%f\t%f\t%f\t%f\t%f\t%i\n", s[0], s[1], s[2], s[3], s[4], s[5], fluid);
    }
  }
  fclose(fp);
  free(acc);
}

/* reference src/lbstore.c:523-545 */
void lbsaveobj(LBSys lb, char *savefile) {
  static const char *tag[5] = {"POS", "VEL", "ANG", "FRC", "TRQ"};
  int console = myscmp("stdout", savefile) || myscmp("stderr", savefile), r;
  FILE *fp = myscmp("stdout", savefile) ? stdout : myscmp("stderr", savefile) ? stderr : fopen(savefile, "w");
  LBObj p;
  if (fp == NULL) { printf("lbsaveobj: %s could not be opened\n", savefile); return; }
  if (console) fprintf(fp, "START of particle data: TYPE, id, base id, x, y, z\n\n");
  for (p = lb->obj_head; p != NULL; p = p->next_obj) {
    LBReal v[5][3] = {{p->posx, p->posy, p->posz}, {p->velx, p->vely, p->velz},
                      {p->angx, p->angy, p->angz}, {p->frcx, p->frcy, p->frcz},
                      {p->trqx, p->trqy, p->trqz}};
    for (r = 0; r < 5; r++)
      fprintf(fp, "%s %3i %3i %f %f %f\n", tag[r], p->id, p->base_obj->id, v[r][0], v[r][1], v[r][2]);
    if (console) fprintf(fp, "\n");
  }
  if (console) fprintf(fp, "END of particle data\n");
  if (!console) fclose(fp);
}

/* reference src/lbstore.c:554-586: five records per object; positions as
 * read, velocities and angular velocities times rescale (then reset) */
void lbloadobj(LBSys lb, char *loadfile) {
  int id, base, r;
  float v[3];
  FILE *fp = fopen(loadfile, "r");
  LBObj p;
  if (fp == NULL) { printf("lbloadobj: %s could not be opened\n", loadfile); return; }
  while (fscanf(fp, "%*s%i%i%f%f%f", &id, &base, &v[0], &v[1], &v[2]) == 5) {
    if ((p = lookupobj(lb, id)) == NULL) break;
    if (base != id) {
      if (lookupobj(lb, base) == NULL) break;
      p->base_obj->id = base;
    }
    p->posx = v[0]; p->posy = v[1]; p->posz = v[2];
    for (r = 1; r < 5; r++) {
      if (fscanf(fp, "%*s%i%i%f%f%f", &id, &base, &v[0], &v[1], &v[2]) != 5) break;
      if (r == 1) { p->velx = lb->rescale * v[0]; p->vely = lb->rescale * v[1]; p->velz = lb->rescale * v[2]; }
      if (r == 2) { p->angx = lb->rescale * v[0]; p->angy = lb->rescale * v[1]; p->angz = lb->rescale * v[2]; }
    }
    if (r < 5) break;
  }
  fclose(fp);
  lb->rescale = 1.0;
}

/* reference src/lbstore.c:595-640 */
void lbsavefrc(LBSys lb, char *frcfile, char *type) {
  int i, j, k;
  FILE *fp = fopen(frcfile, "w");
  if (fp == NULL) { printf("lbsavefrc: %s could not be opened\n", frcfile); exit(EXIT_FAILURE); }
  if (type[0] == 'l' || type[0] == 'L') {
    for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
      long n = node(lb, i, j, k);
      LBObj p = lb->obj[n];
      if (lb->mask[n] <= 0) continue;
      fprintf(fp, "%i %i %i %f %f %f %i %f %f %f\n", i, j, k, lb->fx[n], lb->fy[n], lb->fz[n],
              p->id, p->posx, p->posy, p->posz);
    }
  } else {
    long n;
    int binary = (type[0] == 'b' || type[0] == 'B');
    for (n = 0; n < lb->nnodes; n++) {
      LBStoreReal f[3];
      f[0] = (LBStoreReal)lb->fx[n]; f[1] = (LBStoreReal)lb->fy[n]; f[2] = (LBStoreReal)lb->fz[n];
      if (binary) fwrite(f, sizeof(LBStoreReal), 3, fp);
      else fprintf(fp, "%f %f %f\n", f[0], f[1], f[2]);
    }
  }
  fclose(fp);
}

/* reference src/lbstore.c:647-678 */
void lbsavemap(LBSys lb, char *mapfile, char *type) {
  FILE *fp = fopen(mapfile, "w");
  if (fp == NULL) { printf("lbsavemap: %s could not be opened\n", mapfile); exit(EXIT_FAILURE); }
  if (type[0] == 'l' || type[0] == 'L') {
    int i, j, k;
    for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++)
      if (lb->obj[node(lb, i, j, k)] != NULL) fprintf(fp, "%i %i %i\n", i, j, k);
  } else {
    long n;
    for (n = 0; n < lb->nnodes; n++) fputc(lb->obj[n] == NULL ? 0 : 255, fp);
  }
  fclose(fp);
}

/* ------------------------------------------------------------------------
 * translating a spherical object -- an extension of the GPU library with no
 * counterpart in the reference (which can only remove objects and insert
 * new ones, src/lbobjs.c:433-453); this is the rule the library's
 * lbtranslate implements, written plainly:
 *  - nodes examined: the box around the old and the new sphere (one node of
 *    margin), taken modulo the lattice;
 *  - a node is inside when rsq < rad^2 for the new centre or one of its 26
 *    periodic images (insertsph's test, src/lbobjs.c:214-215);
 *  - a node of the object that is no longer inside becomes fluid with the
 *    equilibrium populations of density rho0 and velocity v + w x r
 *    (r = node - new centre, the vspread convention), rebuilt as lbloadvel
 *    does (src/lbstore.c:352-389); with a uniform body force it gets that
 *    force;
 *  - a fluid node now inside joins the object (populations unchanged, body
 *    force removed when uniform); other objects' nodes are left alone;
 *  - the mask of the changed nodes and their neighbours is rebuilt (their
 *    adsorption bits cleared), the object's wall velocities recomputed when
 *    objects move, pos set to the new centre.
 * ---------------------------------------------------------------------- */
void lbtranslate(LBSys lb, LBObj p, LBReal rad, LBReal x, LBReal y, LBReal z) {
  int dims[3] = {lb->esi, lb->esj, lb->esk}, lo[3], len[3], a, ia, ib, ic, uniform = 1, found = 0;
  double c[3] = {x, y, z}, oc[3] = {p->posx, p->posy, p->posz}, b[3] = {0.0, 0.0, 0.0}, rr = rad * rad;
  long n, nn = lb->nnodes;
  unsigned char *touched = (unsigned char *)zalloc(nn);
  for (n = 0; n < nn && uniform; n++) {
    if (lb->obj[n] != NULL) continue;
    if (!found) { b[0] = lb->bx[n]; b[1] = lb->by[n]; b[2] = lb->bz[n]; found = 1; }
    else if (lb->bx[n] != b[0] || lb->by[n] != b[1] || lb->bz[n] != b[2]) uniform = 0;
  }
  for (a = 0; a < 3; a++) {
    double l0 = floor((oc[a] < c[a] ? oc[a] : c[a]) - rad - 1.0);
    double l1 = ceil((oc[a] > c[a] ? oc[a] : c[a]) + rad + 1.0);
    long s0 = (long)l0, ln = (long)l1 - s0 + 1;
    if (ln >= dims[a] || !(ln > 0)) { s0 = 0; ln = dims[a]; }
    s0 %= dims[a];
    if (s0 < 0) s0 += dims[a];
    lo[a] = (int)s0; len[a] = (int)ln;
  }
  for (ia = 0; ia < len[0]; ia++) for (ib = 0; ib < len[1]; ib++) for (ic = 0; ic < len[2]; ic++) {
    int node3[3] = {(lo[0] + ia) % dims[0], (lo[1] + ib) % dims[1], (lo[2] + ic) % dims[2]}, di, dj, dk, inside = 0;
    double r[3], v[3];
    for (di = -1; di <= 1; di++) for (dj = -1; dj <= 1; dj++) for (dk = -1; dk <= 1; dk++) {
      double ic0 = c[0] + di * dims[0], ic1 = c[1] + dj * dims[1], ic2 = c[2] + dk * dims[2];
      double rsq = (node3[0] - ic0) * (node3[0] - ic0) + (node3[1] - ic1) * (node3[1] - ic1)
                   + (node3[2] - ic2) * (node3[2] - ic2);
      if (rsq < rr) inside = 1;
    }
    n = node(lb, node3[0], node3[1], node3[2]);
    if (lb->obj[n] == p && !inside) {
      LBReal rux, ruy, ruz, sxx = 0.0, syy = 0.0, szz = 0.0, sxy = 0.0, sxz = 0.0, syz = 0.0;
      for (a = 0; a < 3; a++) r[a] = node3[a] - c[a];
      v[0] = p->velx + p->angy * r[2] - p->angz * r[1];
      v[1] = p->vely + p->angz * r[0] - p->angx * r[2];
      v[2] = p->velz + p->angx * r[1] - p->angy * r[0];
      rux = lb->rho0 * v[0]; ruy = lb->rho0 * v[1]; ruz = lb->rho0 * v[2];
      if (!lb->stokes_flow) {
        sxx = v[0] * rux; sxy = v[0] * ruy; sxz = v[0] * ruz;
        syy = v[1] * ruy; syz = v[1] * ruz; szz = v[2] * ruz;
      }
      rebuild(lb->a + 15 * n, 0.0, rux, ruy, ruz, sxx, syy, szz, sxy, sxz, syz);
      lb->obj[n] = NULL;
      if (uniform) { lb->bx[n] = b[0]; lb->by[n] = b[1]; lb->bz[n] = b[2]; }
      touched[n] = 1;
    } else if (lb->obj[n] == NULL && inside) {
      lb->obj[n] = p;
      if (uniform) lb->bx[n] = lb->by[n] = lb->bz[n] = 0.0;
      touched[n] = 1;
    }
  }
  p->posx = x; p->posy = y; p->posz = z;
  /* mask of the changed nodes and their neighbours (reference makemask rule) */
  for (n = 0; n < nn; n++) {
    int i, j, k, q;
    if (!touched[n]) continue;
    k = (int)(n % lb->esk); j = (int)((n / lb->esk) % lb->esj); i = (int)(n / ((long)lb->esk * lb->esj));
    for (q = 0; q < 15; q++) {
      int ii = (i + CX[q] + lb->esi) % lb->esi, jj = (j + CY[q] + lb->esj) % lb->esj;
      int kk = (k + CZ[q] + lb->esk) % lb->esk, r2, val = 0;
      long m = node(lb, ii, jj, kk);
      if (lb->obj[m] != NULL)
        for (r2 = 1; r2 < 15; r2++)
          if (lb->obj[nbr(lb, ii, jj, kk, r2)] == NULL) val |= 1 << (r2 - 1);
      lb->mask[m] = val;
    }
  }
  free(touched);
  if (lb->objects_moving) vspread(lb);
}

/* ------------------------------------------------------------------------
 * appended helpers so drivers written for the GPU library run unchanged
 * ---------------------------------------------------------------------- */

void lbpull(LBSys lb) { (void)lb; }
void lbpush(LBSys lb) { (void)lb; }
void lbsteps(LBSys lb, int n) { int s; for (s = 0; s < n; s++) lbstep(lb); }
long lbkernelcount(void) { return 0; }
int lbtuning(LBSys lb, int *cfg) { (void)lb; cfg[0] = cfg[1] = cfg[2] = cfg[3] = 0; return 0; }

int lbconverge(LBSys lb, int interval, LBReal tol, int maxsteps) {
  int steps = 0, have = 0;
  LBReal last = 0.0;
  if (interval < 3) interval = 3;
  while (steps < maxsteps) {
    lbsteps(lb, interval - 2);
    measure(lb);
    steps += interval;
    if (have && lb->vmeanx != 0.0 && fabs(lb->vmeanx - last) < tol * fabs(lb->vmeanx)) break;
    last = lb->vmeanx; have = 1;
  }
  return steps;
}

void freelb(LBSys lb) {
  if (lb == NULL) return;
  free_objects(lb);
  free(lb->a); free(lb->mask); free(lb->obj);
  free(lb->ux); free(lb->uy); free(lb->uz);
  free(lb->fx); free(lb->fy); free(lb->fz);
  free(lb->bx); free(lb->by); free(lb->bz);
  free(lb->rho); free(lb->name); free(lb->c); free(lb->w);
  free(lb);
}
