/*
 * ORACLE -- test infrastructure only (see orc_lb.c for the rules).
 *
 * CPU restatement of the SunlightLB moment-propagation (passive scalar)
 * path: system set-up, the scatter update with link bounce-back, adsorption
 * and moving walls, tracer injection and diagnostics.  Same AoS layout, loop
 * order and floating-point association as the reference; each routine names
 * the reference file:line it restates.
 *
 * Extension (no reference counterpart): mp->adprob = P in [0,1] makes an
 * adsorbing boundary node take a fraction P of what reaches it along each
 * link and bounce the fraction (1-P) back.  P = 1 (the default) reproduces
 * the reference's all-or-nothing adsorption bit for bit.
 */

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "sunlightlb.h"

static const int CX[15] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1};
static const int CY[15] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
static const int CZ[15] = {0, 0, 0, 0, 0, 1, -1, 1, 1, 1, 1, -1, -1, -1, -1};
static const int OPP[15] = {0, 2, 1, 4, 3, 6, 5, 14, 13, 12, 11, 10, 9, 8, 7};

#define ADSORB 0x4000

static void *zalloc(size_t n) {
  void *p = calloc(n ? n : 1, 1);
  if (p == NULL) error("oracle: out of memory");
  return p;
}

static long node(const LBSys lb, int i, int j, int k) {
  return (long)lb->esk * ((long)lb->esj * i + j) + k;
}
static long nbr(const LBSys lb, int i, int j, int k, int q) {
  int ii = i + CX[q], jj = j + CY[q], kk = k + CZ[q];
  if (ii < 0) ii = lb->esi - 1; else if (ii >= lb->esi) ii = 0;
  if (jj < 0) jj = lb->esj - 1; else if (jj >= lb->esj) jj = 0;
  if (kk < 0) kk = lb->esk - 1; else if (kk >= lb->esk) kk = 0;
  return node(lb, ii, jj, kk);
}

/* reference src/mpmisc.c:38-59 */
MPSys newmp(LBSys lb, char *name) {
  long n;
  MPSys mp = (MPSys)zalloc(sizeof(MPSys_type));
  mp->lb = lb;
  mp->p = (LBReal *)zalloc(lb->nnodes * sizeof(LBReal));
  mp->newp = (LBReal *)zalloc(lb->nnodes * sizeof(LBReal));
  free(lb->rho);
  lb->rho = (LBReal *)zalloc(lb->nnodes * sizeof(LBReal));
  for (n = 0; n < lb->nnodes; n++) lb->rho[n] = lb->rho0;
  mp->objects_moving = lb->objects_moving;
  mp->to_be_initialised = 1;
  mp->name = myscmp("null", name) ? NULL : mycopy(name);
  mp->adprob = 1.0;
  mp->precision = lb->precision;
  mp->priv = zalloc(sizeof(double));  /* tracer added by the fills (extension) */
  return mp;
}

/* p = pval on a fluid node, counting what the fill adds (extension: the
 * GB300 library's injected-tracer count, not in the reference) */
static void set_p(MPSys mp, long n, LBReal pval) {
  *(double *)mp->priv += pval - mp->p[n];
  mp->p[n] = pval;
}

/* reference src/mpmisc.c:64-79 */
void mprhoinit(MPSys mp) {
  LBSys lb = mp->lb;
  long n;
  int q;
  for (n = 0; n < lb->nnodes; n++) {
    lb->rho[n] = lb->rho0;
    if (lb->obj[n] == NULL) for (q = 0; q < 15; q++) lb->rho[n] += lb->a[q + 15 * n];
  }
}

/* reference src/mpmisc.c:83-99 */
void mpinit(MPSys mp) {
  mprhoinit(mp);
  memset(mp->p, 0, mp->lb->nnodes * sizeof(LBReal));
  *(double *)mp->priv = 0.0;
  mp->step = 0; mp->to_be_initialised = 0;
}

/* moving-wall tracer term for boundary link q (as seen from the solid node,
 * u carrying rho0/12): reference src/mpkernel.c:272-350 */
static LBReal mp_wall_term(int q, LBReal fac, const LBReal *u) {
  if (q <= 6) {
    LBReal uu = (q <= 2) ? u[0] : (q <= 4) ? u[1] : u[2];
    return (q & 1) ? 8.0 * fac * uu : -(8.0 * fac * uu);
  }
  {
    /* the reference writes sign(cx) * fac * (ux + (cx*cy) uy + (cx*cz) uz) */
    LBReal inner = (u[0] + (CX[q] * CY[q] > 0 ? u[1] : -u[1])) + (CX[q] * CZ[q] > 0 ? u[2] : -u[2]);
    return CX[q] > 0 ? fac * inner : -(fac * inner);
  }
}

/* reference src/mpkernel.c:47-201 (stationary) and 206-368 (moving) */
static void mp_update(MPSys mp, int moving) {
  LBSys lb = mp->lb;
  const LBReal onebyb = 1.0 / 72.0, eightbyb = 8.0 / 72.0;
  LBReal *a = lb->a, *p = mp->p, *newp = mp->newp, *rho = lb->rho;
  LBReal rho0 = lb->rho0, alpha = mp->alpha, P = mp->adprob;
  int i, j, k, q;
  long n;
  if (lb->status != POST_COLLIDE) printf("Moment propagation apparently out of position\n");
  for (n = 0; n < lb->nnodes; n++) newp[n] = 0.0;
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    long s = node(lb, i, j, k);
    int m = lb->mask[s];
    if (lb->obj[s] == NULL) {
      /* fluid node: scatter along every link (src/mpkernel.c:78-96) */
      LBReal rhot = rho[s], pt = p[s];
      LBReal fac = pt / rhot, piece = pt * onebyb * (rho0 / rhot - alpha);
      LBReal piece8 = 8.0 * piece, piece16 = 16.0 * piece;
      newp[s] += fac * a[15 * s] + piece16 + alpha * pt;
      for (q = 1; q < 15; q++) {
        long d = nbr(lb, i, j, k, q);
        LBReal term = fac * a[q + 15 * s] + (q <= 6 ? piece8 : piece);
        /* extension: an adsorbing solid keeps only the fraction P */
        if (P != 1.0 && lb->obj[d] != NULL && (lb->mask[d] & ADSORB)) term = P * term;
        newp[d] += term;
      }
    } else if (m && (!(m & ADSORB) || P != 1.0)) {
      /* boundary solid node: return what came along each link
       * (src/mpkernel.c:97-185, moving-wall terms 263-351) */
      LBReal u[3] = {0.0, 0.0, 0.0};
      LBReal keep = (m & ADSORB) ? 1.0 - P : 1.0;
      if (moving) {
        LBObj lp = lb->obj[s];
        LBReal rx = i - lp->posx, ry = j - lp->posy, rz = k - lp->posz;
        u[0] = rho0 * ((lp->velx) + (lp->angy) * rz - (lp->angz) * ry) / 12.0;
        u[1] = rho0 * ((lp->vely) + (lp->angz) * rx - (lp->angx) * rz) / 12.0;
        u[2] = rho0 * ((lp->velz) + (lp->angx) * ry - (lp->angy) * rx) / 12.0;
      }
      for (q = 1; q < 15; q++) {
        long f;
        LBReal rhot, pt, fac, piece, term;
        if (!(m & (1 << (q - 1)))) continue;
        f = nbr(lb, i, j, k, q);
        rhot = rho[f]; pt = p[f];
        fac = pt / rhot;
        piece = (q <= 6 ? eightbyb : onebyb) * pt * (rho0 / rhot - alpha);
        term = fac * a[OPP[q] + 15 * f] + piece;
        if (moving) term = term + mp_wall_term(q, fac, u);
        if (keep != 1.0) term = keep * term;
        newp[f] += term;
      }
    }
  }
  /* copy back (src/mpkernel.c:190-197) */
  for (n = 0; n < lb->nnodes; n++) {
    LBReal pt = newp[n];
    if (lb->obj[n] == NULL) p[n] = pt;
    else if (lb->mask[n] & ADSORB) p[n] += pt;
    else p[n] = 0.0;
  }
}

/* reference src/mpkernel.c:33-43 */
void mpstep(MPSys mp) {
  if (mp->to_be_initialised) mpinit(mp);
  mp_update(mp, mp->objects_moving);
  mp->step += 1;
}

/* reference src/mpmisc.c:121-136; the totals are also returned */
static void mp_totals(MPSys mp, LBReal *pfl, LBReal *psl) {
  long n;
  *pfl = *psl = 0.0;
  for (n = 0; n < mp->lb->nnodes; n++) {
    if (mp->lb->obj[n] == NULL) *pfl += mp->p[n]; else *psl += mp->p[n];
  }
}
void mpcheck(MPSys mp) {
  LBReal pfl, psl;
  mp_totals(mp, &pfl, &psl);
  printf("MP '%s' %i : fluid + solid scalar = %10.6f + %10.6f = %10.6f\n",
         mp->name, mp->step, pfl, psl, pfl + psl);
}
/* appended: which = "fluid", "solid", "adsorbed" or "all" */
LBReal mptotal(MPSys mp, char *which) {
  LBReal pfl, psl, pad = 0.0;
  long n;
  if (which[0] == 'i') return *(double *)mp->priv;
  mp_totals(mp, &pfl, &psl);
  if (which[0] == 'f') return pfl;
  if (which[0] == 's') return psl;
  if (which[0] == 'a' && which[1] == 'd') {
    for (n = 0; n < mp->lb->nnodes; n++) if (mp->lb->mask[n] & ADSORB) pad += mp->p[n];
    return pad;
  }
  return pfl + psl;
}

/* extension: mean tracer over the fluid nodes of one plane */
LBReal mpplane(MPSys mp, char *type, int pos) {
  LBSys lb = mp->lb;
  int i, j, k, axis, lim[3];
  double sum = 0.0, cnt = 0.0;
  lim[0] = lb->esi; lim[1] = lb->esj; lim[2] = lb->esk;
  switch (type[0]) {
    case 'x': case 'i': axis = 0; break;
    case 'y': case 'j': axis = 1; break;
    case 'z': case 'k': axis = 2; break;
    default: printf("Unrecognised direction for a plane\n"); return 0.0;
  }
  if (pos < 0 || pos > lim[axis] - 1) { printf("plane position out of range\n"); return 0.0; }
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    int c = (axis == 0) ? i : (axis == 1) ? j : k;
    long n = node(lb, i, j, k);
    if (c != pos || lb->obj[n] != NULL) continue;
    sum += mp->p[n];
    cnt += 1.0;
  }
  return cnt > 0.0 ? sum / cnt : 0.0;
}

/* reference src/mpmisc.c:142-158 */
LBReal mpmean(MPSys mp) {
  long n;
  LBReal ptot = 0.0;
  for (n = 0; n < mp->lb->nnodes; n++) if (mp->lb->obj[n] == NULL) ptot += mp->p[n];
  return ptot / (LBReal)(countfluid(mp->lb));
}

/* reference src/mpmisc.c:164-208 */
static LBReal mp_extreme(MPSys mp, int want_max) {
  long n;
  int found = 0;
  LBReal best = 0.0;
  for (n = 0; n < mp->lb->nnodes; n++) {
    LBReal v;
    if (mp->lb->obj[n] != NULL) continue;
    v = mp->p[n];
    if (!found) { best = v; found = 1; }
    else if (want_max ? (best < v) : (best > v)) best = v;
  }
  return best;
}
LBReal mpmax(MPSys mp) { return mp_extreme(mp, 1); }
LBReal mpmin(MPSys mp) { return mp_extreme(mp, 0); }

/* reference src/mpmisc.c:214-246 */
void mprescale(MPSys mp, LBReal fac) {
  long n;
  for (n = 0; n < mp->lb->nnodes; n++) if (mp->lb->obj[n] == NULL) mp->p[n] *= fac;
}
void mpcopy(MPSys mp, MPSys dest) {
  long n;
  for (n = 0; n < mp->lb->nnodes; n++) if (mp->lb->obj[n] == NULL) dest->p[n] += mp->p[n];
}

/* reference src/mpmisc.c:466-499 */
LBReal mpspread(MPSys mp, char *dirn) {
  LBSys lb = mp->lb;
  int i, j, k, fx = 0, fy = 0, fz = 0, pos;
  LBReal tot = 0.0, mean = 0.0, var = 0.0, pt;
  switch (dirn[0]) {
    case 'x': case 'i': fx = 1; break;
    case 'y': case 'j': fy = 1; break;
    case 'z': case 'k': fz = 1; break;
    default: return -1.0;
  }
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    long n = node(lb, i, j, k);
    if (lb->obj[n] != NULL) continue;
    pt = mp->p[n];
    pos = fx * i + fy * j + fz * k;
    tot += pt; mean += pt * pos; var += pt * pos * pos;
  }
  if (tot > 0.0) { mean = mean / tot; var = var / tot - mean * mean; }
  return var;
}

/* ---- tracer injection: reference src/mpobjs.c ---- */

void mpall(MPSys mp, LBReal pval) {
  long n;
  for (n = 0; n < mp->lb->nnodes; n++) if (mp->lb->obj[n] == NULL) set_p(mp, n, pval);
}

void mpslab(MPSys mp, LBReal x1, LBReal x2, LBReal y1, LBReal y2, LBReal z1, LBReal z2, LBReal pval) {
  LBSys lb = mp->lb;
  int i, j, k;
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++)
    if (i > x1 && i < x2 && j > y1 && j < y2 && k > z1 && k < z2) {
      long n = node(lb, i, j, k);
      if (lb->obj[n] == NULL) set_p(mp, n, pval);
    }
}

void mpwall(MPSys mp, char *type, int wallpos, LBReal pval) {
  LBSys lb = mp->lb;
  int i, j, k, axis, lim[3];
  lim[0] = lb->esi; lim[1] = lb->esj; lim[2] = lb->esk;
  switch (type[0]) {
    case 'x': case 'i': axis = 0; break;
    case 'y': case 'j': axis = 1; break;
    case 'z': case 'k': axis = 2; break;
    default: printf("Unrecognised direction for walls\n"); return;
  }
  if (wallpos < 0 || wallpos > lim[axis] - 1) { printf("wallpos out of range\n"); return; }
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    int c = (axis == 0) ? i : (axis == 1) ? j : k;
    long n;
    if (c != wallpos) continue;
    n = node(lb, i, j, k);
    if (lb->obj[n] == NULL) set_p(mp, n, pval);
  }
}

void mpsph(MPSys mp, LBReal rad, LBReal ox, LBReal oy, LBReal oz, LBReal pval) {
  LBSys lb = mp->lb;
  int i, j, k;
  LBReal radsq = rad * rad;
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    LBReal rsq = (i - ox) * (i - ox) + (j - oy) * (j - oy) + (k - oz) * (k - oz);
    long n = node(lb, i, j, k);
    if (rsq < radsq && lb->obj[n] == NULL) set_p(mp, n, pval);
  }
}

void mpcyl(MPSys mp, char *type, LBReal rad, LBReal a, LBReal b, LBReal pval) {
  LBSys lb = mp->lb;
  int i, j, k, within;
  LBReal rsq = 0.0, radsq = rad * rad;
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    long n = node(lb, i, j, k);
    switch (type[0]) {
      case 'x': case 'i': rsq = (j - a) * (j - a) + (k - b) * (k - b); break;
      case 'y': case 'j': rsq = (i - a) * (i - a) + (k - b) * (k - b); break;
      case 'z': case 'k': rsq = (i - a) * (i - a) + (j - b) * (j - b); break;
      default: error("Unrecognised cylinder direction");
    }
    within = (rsq < radsq);
    if (type[1] != '\0') within = !within;
    if (within && lb->obj[n] == NULL) set_p(mp, n, pval);
  }
}

/* reference src/mpobjs.c:188-226: a byte image of the region
 * (ilo..ihi, jlo..jhi, klo..khi) inclusive, k fastest; a fluid node gets
 * pval * byte / 255.  When the data run out, the rest of that k-row is
 * skipped and every later row tries (and fails) again, as in the
 * reference, whose break leaves only the innermost loop. */
void mpsubs(MPSys mp, char *subsfile, int ilo, int ihi, int jlo, int jhi, int klo, int khi, LBReal pval) {
  LBSys lb = mp->lb;
  int i, j, k;
  unsigned char byte;
  FILE *fp = fopen(subsfile, "r");
  if (fp == NULL) { printf("mpsubs: %s could not be opened\n", subsfile); return; }
  for (i = ilo; i <= ihi; i++)
    for (j = jlo; j <= jhi; j++)
      for (k = klo; k <= khi; k++) {
        long n = node(lb, i, j, k);
        if (fscanf(fp, "%c", &byte) != 1) break;
        if (lb->obj[n] == NULL) mp->p[n] = pval * (double)byte / 255.0;
      }
  fclose(fp);
}

void mplist(MPSys mp, char *file, LBReal pval) {
  LBSys lb = mp->lb;
  int i, j, k;
  FILE *fp;
  if ((fp = fopen(file, "r")) == NULL) { printf("mpsubs: %s could not be opened\n", file); return; }
  while (fscanf(fp, "%i%i%i", &i, &j, &k) == 3) {
    long n = node(lb, i, j, k);
    if (lb->obj[n] == NULL) mp->p[n] = pval;
  }
  fclose(fp);
}

/* ---- adsorption sites: reference src/mpads.c ---- */

void adall(MPSys mp) {
  long n;
  for (n = 0; n < mp->lb->nnodes; n++) if (mp->lb->mask[n] != 0) mp->lb->mask[n] |= ADSORB;
}
void adnone(MPSys mp) {
  long n;
  for (n = 0; n < mp->lb->nnodes; n++) mp->lb->mask[n] &= ~ADSORB;
}
void adslab(MPSys mp, LBReal x1, LBReal x2, LBReal y1, LBReal y2, LBReal z1, LBReal z2) {
  LBSys lb = mp->lb;
  int i, j, k;
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++)
    if (i > x1 && i < x2 && j > y1 && j < y2 && k > z1 && k < z2) {
      long n = node(lb, i, j, k);
      if (lb->mask[n] != 0) lb->mask[n] |= ADSORB;
    }
}
void adsph(MPSys mp, LBReal rad, LBReal ox, LBReal oy, LBReal oz) {
  LBSys lb = mp->lb;
  int i, j, k;
  LBReal radsq = rad * rad;
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    LBReal rsq = (i - ox) * (i - ox) + (j - oy) * (j - oy) + (k - oz) * (k - oz);
    long n = node(lb, i, j, k);
    if (rsq < radsq && lb->mask[n] != 0) lb->mask[n] |= ADSORB;
  }
}
void adcyl(MPSys mp, char *type, LBReal rad, LBReal a, LBReal b) {
  LBSys lb = mp->lb;
  int i, j, k, within;
  LBReal rsq = 0.0, radsq = rad * rad;
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    long n = node(lb, i, j, k);
    switch (type[0]) {
      case 'x': case 'i': rsq = (j - a) * (j - a) + (k - b) * (k - b); break;
      case 'y': case 'j': rsq = (i - a) * (i - a) + (k - b) * (k - b); break;
      case 'z': case 'k': rsq = (i - a) * (i - a) + (j - b) * (j - b); break;
      default: error("Unrecognised cylinder direction");
    }
    within = (rsq < radsq);
    if (type[1] != '\0') within = !within;
    if (within && lb->mask[n] != 0) lb->mask[n] |= ADSORB;
  }
}
LBReal adtotal(MPSys mp, char *file, int imult) {
  static int nadt = 0;
  long n;
  LBReal ptot = 0.0;
  for (n = 0; n < mp->lb->nnodes; n++) if (mp->lb->mask[n] & ADSORB) ptot += mp->p[n];
  if (!myscmp("null", file)) {
    FILE *fp = fopen(file, nadt == 0 ? "w" : "a");
    if (fp != NULL) { fprintf(fp, "%8i %f\n", nadt * imult, ptot); fclose(fp); }
  }
  nadt++;
  return ptot;
}
void adzero(MPSys mp) {
  long n;
  for (n = 0; n < mp->lb->nnodes; n++) if (mp->lb->mask[n] & ADSORB) mp->p[n] = 0.0;
}

void mppull(MPSys mp) { (void)mp; }
void mppush(MPSys mp) { (void)mp; }

void freemp(MPSys mp) {
  if (mp == NULL) return;
  free(mp->priv); free(mp->p); free(mp->newp); free(mp->name); free(mp);
}
