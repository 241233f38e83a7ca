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

/* ---- tracer velocity autocorrelation: reference src/mpvacf.c:28-428 ----
 * Two tracer fields: P carries the start-direction velocity of the tagged
 * tracer, P2 counts the tracer.  The reference's arithmetic is kept as it
 * is, including what it does in three places that look unintended and that
 * a driver's numbers depend on: the rest-population term of P2 goes to the
 * +x neighbour (src/mpvacf.c:120-121), the bounce-back term of link 10
 * misses its velocity factor (:211-213), and the zero-time normalisation
 * adds both sum psi P2 and sum psi^2 rho (:277-280).  State is
 * process-wide, as in the reference. */
static int vacf_l1, vacf_l2, vacf_n, vacf_max;
static LBReal *vacf_arr;

static int vacf_axis(char ch) {
  switch (ch) {
    case 'x': case 'i': return 0;
    case 'y': case 'j': return 1;
    case 'z': case 'k': return 2;
  }
  return -1;
}

void mpvacfinit(MPSys mp, MPSys mp2, char *vacfdir, int reqnvacf) {
  LBSys lb = mp->lb;
  int i, j, k, q, m;
  LBReal *a = lb->a, *p = mp->p, *p2 = mp2->p, *rho = lb->rho, *psi = lb->psi;
  LBReal rho0 = lb->rho0, alpha = mp->alpha, wfac = 1.0, vacftot = 0.0, ntracers = 0.0;
  const LBReal onebyb = 1.0 / 72.0, eightbyb = 8.0 / 72.0, css = 1.0 / 3.0;
  long n;
  free(vacf_arr);
  vacf_arr = (LBReal *)malloc((reqnvacf + 1) * sizeof(LBReal));
  if (vacf_arr == NULL) return;
  vacf_max = reqnvacf;
  vacf_l1 = vacf_axis(vacfdir[0]);
  if (vacf_l1 < 0) error("mpvacfinit: unrecognised initial direction");
  vacf_l2 = vacf_axis(vacfdir[1]);
  if (vacf_l2 < 0) error("mpvacfinit: unrecognised final direction");
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    long x = node(lb, i, j, k);
    if (lb->obj[x] == NULL) {
      LBReal piece = onebyb * (rho0 - alpha * rho[x]), piece8 = 8.0 * piece;
      if (psi != NULL) wfac = psi[x];
      for (q = 1; q < 15; q++)
        p[nbr(lb, i, j, k, q)] += wfac * lb->c[3 * q + vacf_l1] * (a[q + 15 * x] + (q < 7 ? piece8 : piece));
      p2[nbr(lb, i, j, k, 1)] += wfac * (a[15 * x] + 16.0 * piece + alpha * rho[x]);
      for (q = 1; q < 15; q++) p2[nbr(lb, i, j, k, q)] += wfac * (a[q + 15 * x] + (q < 7 ? piece8 : piece));
    } else if ((m = lb->mask[x]) && !(m & 0x4000)) {
      for (q = 1; q < 15; q++) {
        long y;
        LBReal pc, term;
        if (!(m & (1 << (q - 1)))) continue;
        y = nbr(lb, i, j, k, q);
        pc = (q < 7 ? eightbyb : onebyb) * (rho0 - alpha * rho[y]);
        if (psi != NULL) wfac = psi[y];
        term = a[OPP[q] + 15 * y] + pc;
        p[y] += q == 10 ? wfac * term : wfac * lb->c[3 * OPP[q] + vacf_l1] * term;
        p2[y] += wfac * term;
      }
    }
  }
  for (n = 0; n < lb->nnodes; n++)
    if (lb->obj[n] != NULL) p[n] = p2[n] = 0.0;
  wfac = 1.0;
  for (n = 0; n < lb->nnodes; n++) {
    const LBReal *t = a + 15 * n;
    LBReal t1p2, t3p4, t5p6, lo_sum, hi_sum, lo_x, hi_x, lo_y, hi_y, lo_xy, hi_xy, t0p6, sd, s[6], piece;
    if (lb->obj[n] != NULL) continue;
    t1p2 = t[1] + t[2]; t3p4 = t[3] + t[4]; t5p6 = t[5] + t[6];
    lo_sum = t[7] + t[8] + t[9] + t[10]; hi_sum = t[11] + t[12] + t[13] + t[14];
    lo_x = t[7] - t[8] + t[9] - t[10]; hi_x = t[11] - t[12] + t[13] - t[14];
    lo_y = t[7] + t[8] - t[9] - t[10]; hi_y = t[11] + t[12] - t[13] - t[14];
    lo_xy = t[7] - t[8] - t[9] + t[10]; hi_xy = t[11] - t[12] - t[13] + t[14];
    t0p6 = t[0] + t1p2 + t3p4 + t5p6;
    sd = 2.0 * (t0p6 + (lo_sum + hi_sum)) / 3.0 - t0p6;
    s[0] = sd + t1p2; s[1] = sd + t3p4; s[2] = sd + t5p6;
    s[3] = lo_xy + hi_xy; s[4] = lo_x - hi_x; s[5] = lo_y - hi_y;
    if (psi != NULL) wfac = psi[n];
    ntracers += wfac * p2[n];
    wfac = wfac * wfac;
    ntracers += wfac * rho[n];
    piece = rho[n] * css * (1.0 - alpha);
    if (vacf_l1 == vacf_l2) vacftot += wfac * (piece + s[vacf_l1]);
    else vacftot += wfac * s[vacf_l1 + vacf_l2 + 2];  /* xy 3, xz 4, yz 5 */
  }
  vacf_arr[0] = vacftot / ntracers;
  vacf_n = 1;
}

void mpvacfinit2(MPSys mp, MPSys mp2) {
  LBSys lb = mp->lb;
  long n;
  LBReal wfac = 1.0;
  for (n = 0; n < lb->nnodes; n++) {
    const LBReal *t = lb->a + 15 * n;
    LBReal u, r;
    if (lb->obj[n] != NULL) continue;
    r = lb->rho[n];
    u = vacf_l1 == 0 ? (t[1] - t[2] + t[7] - t[8] + t[9] - t[10] + t[11] - t[12] + t[13] - t[14]) / r
      : vacf_l1 == 1 ? (t[3] - t[4] + t[7] + t[8] - t[9] - t[10] + t[11] + t[12] - t[13] - t[14]) / r
                     : (t[5] - t[6] + t[7] + t[8] + t[9] + t[10] - t[11] - t[12] - t[13] - t[14]) / r;
    if (lb->psi != NULL) wfac = lb->psi[n];
    mp->p[n] = wfac * u;
    mp2->p[n] = wfac;
  }
  vacf_n = 0;
}

void mpvacf(MPSys mp, MPSys mp2) {
  LBSys lb = mp->lb;
  long n;
  LBReal wfac = 1.0, ptot = 0.0, psitot = 0.0, pmean, vacftot = 0.0, ntracers = 0.0;
  if (vacf_n > vacf_max) { fprintf(stderr, "Ran out of storage after %i vacf values\n", vacf_max); return; }
  for (n = 0; n < lb->nnodes; n++) {
    if (lb->obj[n] != NULL) continue;
    if (lb->psi != NULL) wfac = lb->psi[n];
    ptot += wfac * mp->p[n]; psitot += wfac * wfac;
  }
  pmean = ptot / psitot;
  for (n = 0; n < lb->nnodes; n++) {
    if (lb->obj[n] != NULL) continue;
    if (lb->psi != NULL) wfac = lb->psi[n];
    mp->p[n] -= wfac * pmean;
  }
  wfac = 1.0;
  for (n = 0; n < lb->nnodes; n++) {
    const LBReal *t = lb->a + 15 * n;
    LBReal u, r;
    if (lb->obj[n] != NULL) continue;
    r = lb->rho[n];
    u = vacf_l2 == 0 ? (t[1] - t[2] + t[7] - t[8] + t[9] - t[10] + t[11] - t[12] + t[13] - t[14]) / r
      : vacf_l2 == 1 ? (t[3] - t[4] + t[7] + t[8] - t[9] - t[10] + t[11] + t[12] - t[13] - t[14]) / r
                     : (t[5] - t[6] + t[7] + t[8] + t[9] + t[10] - t[11] - t[12] - t[13] - t[14]) / r;
    if (lb->psi != NULL) wfac = lb->psi[n];
    vacftot += wfac * mp->p[n] * u;
    ntracers += wfac * mp2->p[n];
  }
  vacf_arr[vacf_n++] = vacftot / ntracers;
}

/* reference src/mpvacf.c:391-428: returns the diffusion coefficient
 * 0.5 vacf(0) + sum_{i>0} vacf(i); the file gets every (nvacf / nvals)-th
 * value.  (The reference divides by zero when nvals > nvacf and closes a
 * null file for "null"; both are guarded here.) */
LBReal mpvacfwr(MPSys mp, MPSys mp2, char *vacffile, int nvals) {
  int i, ntrck = nvals > 0 ? vacf_n / nvals : 0;
  LBReal diffcon = 0.5 * vacf_arr[0];
  FILE *fp = NULL;
  (void)mp; (void)mp2;
  if (!myscmp("null", vacffile) && (fp = fopen(vacffile, "w")) == NULL) {
    fprintf(stderr, "%s could not be opened\n", vacffile);
    return 0.0;
  }
  if (ntrck < 1) ntrck = 1;
  for (i = 1; i < vacf_n; i++) {
    diffcon += vacf_arr[i];
    if (fp != NULL && i % ntrck == 0) fprintf(fp, "%6i %g %g\n", i, vacf_arr[i], diffcon);
  }
  if (fp != NULL) fclose(fp);
  return diffcon;
}

void mppull(MPSys mp) { (void)mp; }
void mppush(MPSys mp) { (void)mp; }

void freemp(MPSys mp) {
  if (mp == NULL) return;
  free(mp->priv); free(mp->p); free(mp->newp); free(mp->name); free(mp);
}
