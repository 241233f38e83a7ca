/*
 * Moment propagation (host side of reference src/mpkernel.c, src/mpmisc.c,
 * src/mpobjs.c, src/mpads.c).  The tracer field p of every MPSys and the
 * lattice's density snapshot live on the GPU; mp->p and lb->rho are host
 * mirrors (mppull / mppush keep them coherent for drivers that touch them).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "slb_private.h"

#define ADSORB 0x4000

static mp_priv *mpstate(MPSys mp) { return (mp_priv *)mp->priv; }

static void mptrace(MPSys mp, const char *what) {
  if (slb_verbosity & TRACE_ROUTINE_EXITS) printf("MP '%s' %i : %s done\n", mp->name, mp->step, what);
}

/* device tracer of mp, created on first use; uploads a host-written p */
static slbc_tracer *tracer(MPSys mp) {
  mp_priv *st = mpstate(mp);
  slbc_lattice *d = slb_device(mp->lb);
  if (st->dev == NULL) {
    st->use_f64 = mp->precision == SLB_FP32 ? 0 : 1;
    slb_check(slbc_mp_create(d, &st->dev, st->use_f64), "tracer set-up");
    st->p_sent = 0;
  }
  if (st->p_sent != st->p_gen) {
    slb_check(slbc_mp_put(st->dev, mp->p), "tracer upload");
    st->p_sent = st->p_gen;
  }
  return st->dev;
}

static void p_changed(MPSys mp) { mpstate(mp)->host_p_valid = 0; }

/* appended: host mirror mp->p <-> device */
void mppull(MPSys mp) {
  mp_priv *st = mpstate(mp);
  if (st->dev == NULL || st->host_p_valid) return;
  slb_check(slbc_mp_get(st->dev, mp->p), "tracer download");
  st->host_p_valid = 1;
}
void mppush(MPSys mp) {
  mp_priv *st = mpstate(mp);
  st->p_gen++;
  st->host_p_valid = 1;
}

/* reference src/mpmisc.c:38-59.  alpha starts at 0 (the reference leaves it
 * unset); adprob = 1 gives the reference's adsorption. */
MPSys newmp(LBSys lb, char *name) {
  long x;
  MPSys mp = (MPSys)calloc(1, sizeof(MPSys_type));
  mp_priv *st = (mp_priv *)calloc(1, sizeof(mp_priv));
  if (mp == NULL || st == NULL) error("No room for mpsys structure\n");
  mp->lb = lb;
  mp->p = (LBReal *)calloc((size_t)lb->nnodes, sizeof(LBReal));
  mp->newp = (LBReal *)calloc(1, sizeof(LBReal));  /* unused: the update gathers */
  free(lb->rho);
  lb->rho = (LBReal *)malloc((size_t)lb->nnodes * sizeof(LBReal));
  if (mp->p == NULL || lb->rho == NULL) error("No room at the inn");
  for (x = 0; x < lb->nnodes; x++) lb->rho[x] = lb->rho0;
  mp->objects_moving = lb->objects_moving;
  mp->to_be_initialised = 1;
  mp->adprob = 1.0;
  mp->precision = lb->precision;
  st->host_p_valid = 1;
  mp->priv = st;
  slb_state(lb)->host_rho_valid = 1;
  if (myscmp("null", name)) mp->name = NULL; else mp->name = mycopy(name);
  printf("MP '%s' initialised for %i * %i * %i lattice\n", mp->name, lb->esi, lb->esj, lb->esk);
  return mp;
}

void freemp(MPSys mp) {
  if (mp == NULL) return;
  if (mpstate(mp)->dev) slbc_mp_destroy(mpstate(mp)->dev);
  free(mp->priv); free(mp->p); free(mp->newp); free(mp->name); free(mp);
}

/* reference src/mpmisc.c:64-79 */
void mprhoinit(MPSys mp) {
  slbc_lattice *d = slb_device(mp->lb);
  tracer(mp);  /* makes sure the snapshot buffers exist */
  slb_check(slbc_mp_rhoinit(d), "density snapshot");
  slb_state(mp->lb)->host_rho_valid = 0;
  mptrace(mp, "mprhoinit");
}

/* reference src/mpmisc.c:83-99 */
void mpinit(MPSys mp) {
  mp_priv *st = mpstate(mp);
  mprhoinit(mp);
  memset(mp->p, 0, (size_t)mp->lb->nnodes * sizeof(LBReal));
  st->p_gen++;
  st->host_p_valid = 1;
  slb_check(slbc_mp_injected(tracer(mp), 1, NULL), "injected tracer");
  mp->step = 0;
  mp->to_be_initialised = 0;
  printf("MP '%s' initialised and ready to go.\n", mp->name);
  mptrace(mp, "mpinit");
}

/* reference src/mpmisc.c:104-114 */
void mpwrpars(MPSys mp) {
  LBReal d = (1.0 - mp->alpha) / 6.0;
  printf("\nMP '%s' parameter list\n\n", mp->name);
  printf(" | LB size  = %i * %i * %i = %i\n", mp->lb->esi, mp->lb->esj, mp->lb->esk, mp->lb->nnodes);
  printf(" | alpha, D = %0.4f %0.6f\n", mp->alpha, d);
  printf(mp->objects_moving ? " | Objects allowed to move\n" : " | All objects are stationary\n");
  printf("\n");
}

/* reference src/mpkernel.c:33-43 */
void mpstep(MPSys mp) {
  slbc_tracer *t;
  double *state = NULL;
  int nobj = 0;
  slb_need_populations(mp->lb, "Moment propagation");
  if (mp->to_be_initialised) mpinit(mp);
  t = tracer(mp);
  if (mp->lb->status != POST_COLLIDE) {
    printf("Moment propagation apparently out of position\n");
    wrstatus(mp->lb, stdout);
  }
  if (mp->objects_moving) {
    slb_priv *ls = slb_state(mp->lb);
    int o;
    nobj = ls->nobj;
    state = (double *)malloc(9 * (size_t)(nobj + 1) * sizeof(double));
    if (state == NULL) error("No room for object table");
    for (o = 0; o < nobj; o++) {
      LBObj p = ls->objs[o];
      double *s = state + 9 * o;
      s[0] = p->posx; s[1] = p->posy; s[2] = p->posz;
      s[3] = p->velx; s[4] = p->vely; s[5] = p->velz;
      s[6] = p->angx; s[7] = p->angy; s[8] = p->angz;
    }
  }
  slb_check(slbc_mp_step(t, 1, mp->alpha, mp->adprob, mp->objects_moving, state, nobj), "tracer update");
  free(state);
  p_changed(mp);
#ifdef SIGNAL
  if (slb_signal_flag) sighandle(mp->lb);
#endif
  mp->step += 1;
  mptrace(mp, "mpdo");
}

static void sums(MPSys mp, int axis, double out[5]) {
  slb_check(slbc_mp_sums(tracer(mp), axis, out), "tracer sums");
}

/* reference src/mpmisc.c:121-136 */
void mpcheck(MPSys mp) {
  double s[5];
  sums(mp, -1, s);
  printf("MP '%s' %i : fluid + solid scalar = %10.6f + %10.6f = %10.6f\n", mp->name, mp->step, s[0], s[1], s[0] + s[1]);
  mptrace(mp, "mpcheck");
}

/* appended: tracer totals, which = "fluid", "solid", "adsorbed", "all" or
 * "injected" (added by the device fills since mpinit) */
LBReal mptotal(MPSys mp, char *which) {
  double s[5];
  if (which[0] == 'i') {
    double v = 0.0;
    slb_check(slbc_mp_injected(tracer(mp), 0, &v), "injected tracer");
    return v;
  }
  sums(mp, -1, s);
  if (which[0] == 'f') return s[0];
  if (which[0] == 's') return s[1];
  if (which[0] == 'a' && which[1] == 'd') return s[2];
  return s[0] + s[1];
}

/* appended: mean tracer over the fluid nodes of the plane type = pos */
LBReal mpplane(MPSys mp, char *type, int pos) {
  double s[2];
  int axis, lim;
  switch (type[0]) {
    case 'x': case 'i': axis = 0; lim = mp->lb->esi; break;
    case 'y': case 'j': axis = 1; lim = mp->lb->esj; break;
    case 'z': case 'k': axis = 2; lim = mp->lb->esk; break;
    default: printf("Unrecognised direction for a plane\n"); return 0.0;
  }
  if (pos < 0 || pos > lim - 1) { printf("plane position out of range\n"); return 0.0; }
  slb_check(slbc_mp_plane(tracer(mp), axis, pos, s), "tracer plane");
  return s[1] > 0.0 ? s[0] / s[1] : 0.0;
}

/* reference src/mpmisc.c:142-158 */
LBReal mpmean(MPSys mp) {
  double s[5];
  LBReal pmean;
  sums(mp, -1, s);
  pmean = s[0] / (LBReal)(countfluid(mp->lb));
  if (slb_verbosity & TRACE_ROUTINE_EXITS)
    printf("MP '%s' %i : mpnorm done, ptot = %f, pmean = %f\n", mp->name, mp->step, s[0], pmean);
  return pmean;
}

/* reference src/mpmisc.c:164-208 (0 when there is no fluid node) */
static LBReal extreme(MPSys mp, int want_max) {
  double mm[2];
  if (countfluid(mp->lb) == 0) return 0.0;
  slb_check(slbc_mp_minmax(tracer(mp), mm), "tracer extremes");
  return want_max ? mm[1] : mm[0];
}
LBReal mpmax(MPSys mp) { return extreme(mp, 1); }
LBReal mpmin(MPSys mp) { return extreme(mp, 0); }

/* reference src/mpmisc.c:214-225 */
void mprescale(MPSys mp, LBReal fac) {
  slb_check(slbc_mp_scale(tracer(mp), fac), "tracer rescale");
  p_changed(mp);
  mptrace(mp, "mprescale");
}

/* reference src/mpmisc.c:233-246 */
void mpcopy(MPSys mp, MPSys dest) {
  slbc_tracer *src = tracer(mp);
  slb_check(slbc_mp_add(tracer(dest), src), "tracer copy");
  p_changed(dest);
  mptrace(mp, "mpcopy");
}

/* reference src/mpmisc.c:466-499 */
LBReal mpspread(MPSys mp, char *dirn) {
  double s[5];
  int axis;
  LBReal tot, mean, var = 0.0;
  switch (dirn[0]) {
    case 'x': case 'i': axis = 0; break;
    case 'y': case 'j': axis = 1; break;
    case 'z': case 'k': axis = 2; break;
    default: printf("Unrecognised direction for measuring spread\n"); return -1.0;
  }
  sums(mp, axis, s);
  tot = s[0]; mean = s[3]; var = s[4];
  if (tot > 0.0) { mean = mean / tot; var = var / tot - mean * mean; }
  mptrace(mp, "mpspread");
  return var;
}

/* ---- tracer injection: reference src/mpobjs.c ---------------------------- */

static void fill(MPSys mp, int kind, const double *geo, LBReal pval) {
  slb_check(slbc_mp_fill(tracer(mp), kind, geo, pval), "tracer injection");
  p_changed(mp);
}

void mpall(MPSys mp, LBReal pval) {
  fill(mp, 0, NULL, pval);
  if (slb_verbosity & MP_OBJECT_DETAILS)
    printf("Diffusing material slab inserted everywhere, %i sites set\n", countfluid(mp->lb));
  mptrace(mp, "mpall");
}

void mpslab(MPSys mp, LBReal x1, LBReal x2, LBReal y1, LBReal y2, LBReal z1, LBReal z2, LBReal pval) {
  double g[6];
  g[0] = x1; g[1] = x2; g[2] = y1; g[3] = y2; g[4] = z1; g[5] = z2;
  fill(mp, 1, g, pval);
  mptrace(mp, "mpslab");
}

void mpwall(MPSys mp, char *type, int wallpos, LBReal pval) {
  double g[2];
  int lim;
  switch (type[0]) {
    case 'x': case 'i': g[0] = 0; lim = mp->lb->esi; break;
    case 'y': case 'j': g[0] = 1; lim = mp->lb->esj; break;
    case 'z': case 'k': g[0] = 2; lim = mp->lb->esk; break;
    default: printf("Unrecognised direction for walls\n"); return;
  }
  if (wallpos < 0 || wallpos > lim - 1) { printf("wallpos out of range\n"); return; }
  g[1] = wallpos;
  fill(mp, 2, g, pval);
  mptrace(mp, "mpwall");
}

void mpsph(MPSys mp, LBReal rad, LBReal ox, LBReal oy, LBReal oz, LBReal pval) {
  double g[4];
  g[0] = rad; g[1] = ox; g[2] = oy; g[3] = oz;
  fill(mp, 3, g, pval);
  mptrace(mp, "mpsph");
}

void mpcyl(MPSys mp, char *type, LBReal rad, LBReal a, LBReal b, LBReal pval) {
  double g[5];
  switch (type[0]) {
    case 'x': case 'i': g[0] = 0; break;
    case 'y': case 'j': g[0] = 1; break;
    case 'z': case 'k': g[0] = 2; break;
    default: error("Unrecognised cylinder direction"); return;
  }
  g[1] = type[1] != '\0' ? 1.0 : 0.0; g[2] = rad; g[3] = a; g[4] = b;
  fill(mp, 4, g, pval);
  mptrace(mp, "mpcyl");
}

/* reference src/mpobjs.c:188-226: a byte image of the region (ilo..ihi,
 * jlo..jhi, klo..khi) inclusive, k fastest, read on the host; a fluid node
 * gets pval * byte / 255.  When the data run out the rest of that k-row is
 * skipped and each later row reports it again, as the reference's break
 * (which leaves only the innermost loop) does.  Nodes outside the lattice
 * use up their byte and are left alone. */
void mpsubs(MPSys mp, char *subsfile, int ilo, int ihi, int jlo, int jhi, int klo, int khi, LBReal pval) {
  int i, j, k, ns = 0;
  unsigned char byte;
  LBReal ptot = 0.0, val;
  FILE *fp;
  LBSys lb = mp->lb;
  if ((fp = fopen(subsfile, "r")) == NULL) { printf("mpsubs: %s could not be opened\n", subsfile); return; }
  if (slb_verbosity & MP_OBJECT_DETAILS) {
    printf("\nInserting mp substrate data from %s\n", subsfile);
    printf("Substrate region is (%i-%i,%i-%i,%i-%i) inclusive\n", ilo, ihi, jlo, jhi, klo, khi);
  }
  mppull(mp);
  for (i = ilo; i <= ihi; i++)
    for (j = jlo; j <= jhi; j++)
      for (k = klo; k <= khi; k++) {
        long x = slb_node(lb, i, j, k);
        if (fscanf(fp, "%c", &byte) != 1) { printf("mpsubs: ran out of data in %s\n", subsfile); break; }
        if (i < 0 || i >= lb->esi || j < 0 || j >= lb->esj || k < 0 || k >= lb->esk) continue;
        if (lb->obj[x] == NULL) {
          val = pval * (double)byte / 255.0;
          mp->p[x] = val; ns++; ptot += val;
        }
      }
  fclose(fp);
  mppush(mp);
  if (slb_verbosity & MP_OBJECT_DETAILS) {
    printf("Inserted mp substrate field, %i sites set\n", ns);
    printf("Total amount of added material is %f\n", ptot);
  }
  mptrace(mp, "mpsubs");
}

/* reference src/mpobjs.c:233-261: a node list is read on the host, the
 * field is updated there and sent back. */
void mplist(MPSys mp, char *file, LBReal pval) {
  int i, j, k;
  FILE *fp;
  LBSys lb = mp->lb;
  if ((fp = fopen(file, "r")) == NULL) { printf("mpsubs: %s could not be opened\n", file); return; }
  mppull(mp);
  while (fscanf(fp, "%i%i%i", &i, &j, &k) == 3) {
    long x = slb_node(lb, i, j, k);
    if (x < 0 || x >= lb->nnodes) continue;
    if (lb->obj[x] == NULL) mp->p[x] = pval;
  }
  fclose(fp);
  mppush(mp);
  mptrace(mp, "mplist");
}

/* ---- tracer velocity autocorrelation: reference src/mpvacf.c ------------ */
/* Two tracer fields: P (mp) carries the start-direction velocity of the
 * tagged tracer, P2 (mp2) counts the tracer.  The initialisations run on
 * the host on the mirrors (once per measurement, in the reference's order
 * of summation, so P and P2 equal the reference's bit for bit); every
 * mpvacf call runs on the GPU (FP64 tracers).  The reference's arithmetic
 * is kept as it is in three places that look unintended but that a
 * driver's numbers depend on: the rest-population term of P2 goes to the
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

static const int VX[15] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1};
static const int VY[15] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};
static const int VZ[15] = {0, 0, 0, 0, 0, 1, -1, 1, 1, 1, 1, -1, -1, -1, -1};
static const int VOPP[15] = {0, 2, 1, 4, 3, 6, 5, 14, 13, 12, 11, 10, 9, 8, 7};

static long vnbr(LBSys lb, int i, int j, int k, int q) {
  int ii = i + VX[q], jj = j + VY[q], kk = k + VZ[q];
  if (ii < 0) ii = lb->esi - 1; else if (ii >= lb->esi) ii = 0;
  if (jj < 0) jj = lb->esj - 1; else if (jj >= lb->esj) jj = 0;
  if (kk < 0) kk = lb->esk - 1; else if (kk >= lb->esk) kk = 0;
  return slb_node(lb, ii, jj, kk);
}

static void vacf_mirrors(MPSys mp, MPSys mp2) {
  if (mp->lb != mp2->lb) error("mpvacf: the two tracer fields belong to different lattices");
  lbpull(mp->lb);
  slb_pull_rho(mp->lb);
  if (mp->lb->rho == NULL) error("mpvacf: no density snapshot (call mpinit first)");
  mppull(mp);
  mppull(mp2);
}

/* reference src/mpvacf.c:39-293 */
void mpvacfinit(MPSys mp, MPSys mp2, char *vacfdir, int reqnvacf) {
  LBSys lb = mp->lb;
  int i, j, k, q, m;
  LBReal *a, *p = mp->p, *p2 = mp2->p, *rho, *psi = lb->psi;
  LBReal rho0 = lb->rho0, alpha = mp->alpha, wfac = 1.0, vacftot = 0.0, ntracers = 0.0;
  const LBReal onebyb = 1.0 / 72.0, eightbyb = 8.0 / 72.0, css = 1.0 / 3.0;
  long x;
  free(vacf_arr);
  vacf_arr = (LBReal *)malloc((reqnvacf + 1) * sizeof(LBReal));
  if (vacf_arr == NULL) { fprintf(stderr, "Not enought room at the inn for %i reals\n", reqnvacf + 1); return; }
  vacf_max = reqnvacf;
  if (vacfdir[0] == '\0') error("mpvacfinit: please supply initial direction");
  if ((vacf_l1 = vacf_axis(vacfdir[0])) < 0) error("mpvacfinit: unrecognised initial direction");
  if (vacfdir[1] == '\0') error("mpvacfinit: please supply final direction");
  if ((vacf_l2 = vacf_axis(vacfdir[1])) < 0) error("mpvacfinit: unrecognised final direction");
  if (lb->status != POST_COLLIDE) {
    fprintf(stderr, "vacf initialisation apparently out of position\n");
    wrstatus(lb, stdout);
  }
  vacf_mirrors(mp, mp2);
  a = lb->a; rho = lb->rho;
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    x = slb_node(lb, i, j, k);
    if (lb->obj[x] == NULL) {
      LBReal piece = onebyb * (rho0 - alpha * rho[x]), piece8 = 8.0 * piece;
      if (psi != NULL) wfac = psi[x];
      for (q = 1; q < 15; q++)
        p[vnbr(lb, i, j, k, q)] += wfac * lb->c[3 * q + vacf_l1] * (a[q + 15 * x] + (q < 7 ? piece8 : piece));
      p2[vnbr(lb, i, j, k, 1)] += wfac * (a[15 * x] + 16.0 * piece + alpha * rho[x]);
      for (q = 1; q < 15; q++) p2[vnbr(lb, i, j, k, q)] += wfac * (a[q + 15 * x] + (q < 7 ? piece8 : piece));
    } else if ((m = lb->mask[x]) && !(m & ADSORB)) {
      for (q = 1; q < 15; q++) {
        long y;
        LBReal pc, term;
        if (!(m & (1 << (q - 1)))) continue;
        y = vnbr(lb, i, j, k, q);
        pc = (q < 7 ? eightbyb : onebyb) * (rho0 - alpha * rho[y]);
        if (psi != NULL) wfac = psi[y];
        term = a[VOPP[q] + 15 * y] + pc;
        p[y] += q == 10 ? wfac * term : wfac * lb->c[3 * VOPP[q] + vacf_l1] * term;
        p2[y] += wfac * term;
      }
    }
  }
  for (x = 0; x < lb->nnodes; x++)
    if (lb->obj[x] != NULL) p[x] = p2[x] = 0.0;
  wfac = 1.0;
  for (x = 0; x < lb->nnodes; x++) {
    const LBReal *t = a + 15 * x;
    LBReal t1p2, t3p4, t5p6, lo_sum, hi_sum, lo_x, hi_x, lo_y, hi_y, lo_xy, hi_xy, t0p6, sd, st[6], piece;
    if (lb->obj[x] != NULL) continue;
    t1p2 = t[1] + t[2]; t3p4 = t[3] + t[4]; t5p6 = t[5] + t[6];
    lo_sum = t[7] + t[8] + t[9] + t[10]; hi_sum = t[11] + t[12] + t[13] + t[14];
    lo_x = t[7] - t[8] + t[9] - t[10]; hi_x = t[11] - t[12] + t[13] - t[14];
    lo_y = t[7] + t[8] - t[9] - t[10]; hi_y = t[11] + t[12] - t[13] - t[14];
    lo_xy = t[7] - t[8] - t[9] + t[10]; hi_xy = t[11] - t[12] - t[13] + t[14];
    t0p6 = t[0] + t1p2 + t3p4 + t5p6;
    sd = 2.0 * (t0p6 + (lo_sum + hi_sum)) / 3.0 - t0p6;
    st[0] = sd + t1p2; st[1] = sd + t3p4; st[2] = sd + t5p6;
    st[3] = lo_xy + hi_xy; st[4] = lo_x - hi_x; st[5] = lo_y - hi_y;
    if (psi != NULL) wfac = psi[x];
    ntracers += wfac * p2[x];
    wfac = wfac * wfac;
    ntracers += wfac * rho[x];
    piece = rho[x] * css * (1.0 - alpha);
    if (vacf_l1 == vacf_l2) vacftot += wfac * (piece + st[vacf_l1]);
    else vacftot += wfac * st[vacf_l1 + vacf_l2 + 2];  /* xy, xz, yz */
  }
  mppush(mp);
  mppush(mp2);
  vacf_arr[0] = vacftot / ntracers;
  vacf_n = 1;
  printf("MP '%s' %i : Initialised for vacf, init drn %c, final drn %c\n", mp->name, mp->step, vacfdir[0], vacfdir[1]);
  printf("MP '%s' %i : Initialised storage for %i vacf values\n", mp->name, mp->step, vacf_max);
  printf("MP '%s' %i : ntracers = %f\n", mp->name, mp->step, ntracers);
  printf("MP '%s' %i : vacf(0) = %f\n", mp->name, mp->step, vacf_arr[0]);
  mptrace(mp, "mpvacfinit");
}

/* reference src/mpvacf.c:298-335 */
void mpvacfinit2(MPSys mp, MPSys mp2) {
  LBSys lb = mp->lb;
  long x;
  LBReal wfac = 1.0;
  vacf_mirrors(mp, mp2);
  for (x = 0; x < lb->nnodes; x++) {
    const LBReal *t = lb->a + 15 * x;
    LBReal u, r;
    if (lb->obj[x] != NULL) continue;
    r = lb->rho[x];
    u = vacf_l1 == 0 ? (t[1] - t[2] + t[7] - t[8] + t[9] - t[10] + t[11] - t[12] + t[13] - t[14]) / r
      : vacf_l1 == 1 ? (t[3] - t[4] + t[7] + t[8] - t[9] - t[10] + t[11] + t[12] - t[13] - t[14]) / r
                     : (t[5] - t[6] + t[7] + t[8] + t[9] + t[10] - t[11] - t[12] - t[13] - t[14]) / r;
    if (lb->psi != NULL) wfac = lb->psi[x];
    mp->p[x] = wfac * u;
    mp2->p[x] = wfac;
  }
  mppush(mp);
  mppush(mp2);
  vacf_n = 0;
  printf("MP '%s' %i : Re-initialised vacf calculation\n", mp->name, mp->step);
  mptrace(mp, "mpvacfinit2");
}

/* reference src/mpvacf.c:337-389, on the GPU */
void mpvacf(MPSys mp, MPSys mp2) {
  double out[2];
  slbc_tracer *t, *t2;
  if (vacf_arr == NULL) { fprintf(stderr, "mpvacf: call mpvacfinit first\n"); return; }
  if (vacf_n > vacf_max) { fprintf(stderr, "Ran out of storage after %i vacf values\n", vacf_max); return; }
  if (mp->lb != mp2->lb) error("mpvacf: the two tracer fields belong to different lattices");
  t = tracer(mp);
  t2 = tracer(mp2);
  slb_check(slbc_mp_vacf(t, t2, vacf_l2, mp->lb->psi, out), "tracer velocity autocorrelation");
  p_changed(mp);
  vacf_arr[vacf_n++] = out[0] / out[1];
  mptrace(mp, "mpvacf");
}

/* reference src/mpvacf.c:391-428: the diffusion coefficient
 * 0.5 vacf(0) + sum_{i>0} vacf(i); the file (not "null") gets every
 * (nvacf / nvals)-th value.  The reference divides by zero when
 * nvals > nvacf and closes a null file for "null": both guarded here. */
LBReal mpvacfwr(MPSys mp, MPSys mp2, char *vacffile, int nvals) {
  int i, ntrck;
  LBReal diffcon;
  FILE *fp = NULL;
  (void)mp2;
  if (vacf_arr == NULL) return 0.0;
  if (!myscmp("null", vacffile)) {
    if ((fp = fopen(vacffile, "w")) == NULL) { fprintf(stderr, "%s could not be opened\n", vacffile); return 0.0; }
    printf("MP '%s' %i : Writing vacf data to %s\n", mp->name, mp->step, vacffile);
  } else {
    printf("MP '%s' %i : Analyzing vacf data\n", mp->name, mp->step);
  }
  ntrck = nvals > 0 ? vacf_n / nvals : 0;
  if (ntrck < 1) ntrck = 1;
  diffcon = 0.5 * vacf_arr[0];
  for (i = 1; i < vacf_n; i++) {
    diffcon += vacf_arr[i];
    if (fp != NULL && i % ntrck == 0) fprintf(fp, "%6i %g %g\n", i, vacf_arr[i], diffcon);
    if (i > vacf_n - 4) printf("MP '%s' %i : step, d = %8i %g %g\n", mp->name, mp->step, i, vacf_arr[i], diffcon);
  }
  if (fp != NULL) fclose(fp);
  mptrace(mp, "mpvacfwr");
  return diffcon;
}

/* ---- adsorption sites: reference src/mpads.c ------------------------------ */

void adall(MPSys mp) {
  long x;
  int ns = 0;
  for (x = 0; x < mp->lb->nnodes; x++)
    if (mp->lb->mask[x] != 0) { mp->lb->mask[x] |= ADSORB; ns++; }
  slb_mark_ads(mp->lb);
  printf("All nodes are adsorption sites, %i sites set\n", ns);
  mptrace(mp, "adall");
}

void adnone(MPSys mp) {
  long x;
  int ns = 0;
  for (x = 0; x < mp->lb->nnodes; x++)
    if (mp->lb->mask[x] & ADSORB) { mp->lb->mask[x] &= ~ADSORB; ns++; }
  slb_mark_ads(mp->lb);
  printf("Reset %i adsorption sites to non-adsorbing sites\n", ns);
  mptrace(mp, "adnone");
}

void adslab(MPSys mp, LBReal x1, LBReal x2, LBReal y1, LBReal y2, LBReal z1, LBReal z2) {
  LBSys lb = mp->lb;
  int i, j, k, ns = 0;
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++)
    if (i > x1 && i < x2 && j > y1 && j < y2 && k > z1 && k < z2) {
      long x = slb_node(lb, i, j, k);
      if (lb->mask[x] != 0) { lb->mask[x] |= ADSORB; ns++; }
    }
  slb_mark_ads(lb);
  printf("Adsorption site slab from %5.2f %5.2f %5.2f to %5.2f %5.2f %5.2f, %i sites set\n", x1, y1, z1, x2, y2, z2, ns);
  mptrace(mp, "adslab");
}

void adsph(MPSys mp, LBReal rad, LBReal ox, LBReal oy, LBReal oz) {
  LBSys lb = mp->lb;
  int i, j, k, ns = 0;
  LBReal radsq = rad * rad;
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    LBReal rsq = (i - ox) * (i - ox) + (j - oy) * (j - oy) + (k - oz) * (k - oz);
    long x = slb_node(lb, i, j, k);
    if (rsq < radsq && lb->mask[x] != 0) { lb->mask[x] |= ADSORB; ns++; }
  }
  slb_mark_ads(lb);
  printf("Adsorption site sphere, radius %5.2f at %5.2f %5.2f %5.2f, %i sites set\n", rad, ox, oy, oz, ns);
  mptrace(mp, "adsph");
}

void adcyl(MPSys mp, char *type, LBReal rad, LBReal a, LBReal b) {
  LBSys lb = mp->lb;
  int i, j, k, ns = 0, within;
  LBReal rsq = 0.0, radsq = rad * rad;
  for (i = 0; i < lb->esi; i++) for (j = 0; j < lb->esj; j++) for (k = 0; k < lb->esk; k++) {
    long x = slb_node(lb, i, j, k);
    switch (type[0]) {
      case 'x': case 'i': rsq = (j - a) * (j - a) + (k - b) * (k - b); break;
      case 'y': case 'j': rsq = (i - a) * (i - a) + (k - b) * (k - b); break;
      case 'z': case 'k': rsq = (i - a) * (i - a) + (j - b) * (j - b); break;
      default: error("Unrecognised cylinder direction");
    }
    within = (rsq < radsq);
    if (type[1] != '\0') within = !within;
    if (within && lb->mask[x] != 0) { lb->mask[x] |= ADSORB; ns++; }
  }
  slb_mark_ads(lb);
  printf(type[1] == '\0' ? "Adsorbtion site cylinder, \n" : "Adsorbtion site cylindrical hole, \n");
  printf("radius %5.2f, axis %5.2f %5.2f along %c, %i sites set\n", rad, a, b, type[0], ns);
  mptrace(mp, "adcyl");
}

/* reference src/mpads.c:149-172 */
LBReal adtotal(MPSys mp, char *adtfile, int imult) {
  static int nadt = 0;
  double s[5];
  LBReal ptot;
  sums(mp, -1, s);
  ptot = s[2];
  if (!myscmp("null", adtfile)) {
    FILE *fp = fopen(adtfile, nadt == 0 ? "w" : "a");
    if (fp == NULL) printf("adtotal: %s could not be opened to write/append data\n", adtfile);
    else { fprintf(fp, "%8i %f\n", nadt * imult, ptot); fclose(fp); }
  }
  nadt++;
  mptrace(mp, "adtotal");
  return ptot;
}

/* reference src/mpads.c:177-186 */
void adzero(MPSys mp) {
  slb_check(slbc_mp_zero_ads(tracer(mp)), "adsorbed reset");
  p_changed(mp);
  mptrace(mp, "adzero");
}
