/*
 * Lattice construction, host/device coherence and miscellany of the GB300
 * SunlightLB library (host side of reference src/lbmisc.c).
 *
 * The populations live on the GPU.  The host keeps everything a driver can
 * see in the reference structs (object list and map, mask, wall velocity,
 * body force, force arrays, the population mirror lb->a).  Every routine that
 * changes one of those arrays bumps a generation counter; slb_device()
 * uploads whatever changed before a device call, so drivers keep the
 * reference's calling conventions.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>
#include "slb_private.h"

int slb_verbosity = 0;
static time_t tstart;

/* reference src/lbmisc.c:39-42 */
void error(char *s1) {
  fprintf(stderr, "Opps!  %s\n", s1);
  exit(EXIT_FAILURE);
}

void slb_check(int rc, const char *what) {
  char msg[1024];
  if (rc == 0) return;
  snprintf(msg, sizeof msg, "%s failed: %s", what, slbc_last_error());
  error(msg);
}

static void *xcalloc(size_t n, size_t sz) {
  void *p = calloc(n ? n : 1, sz ? sz : 1);
  if (p == NULL) error("No room for LBReal array");
  return p;
}

/* reference src/lbmisc.c:47-51 */
void startclock() {
  if (tstart == 0) printf("Clock started\n");
  else printf("Clock restarted\n");
  tstart = time(NULL);
}

/* reference src/lbmisc.c:55-75 */
void set_verbosity(int what) { slb_verbosity |= what; report_verbosity(); }
void unset_verbosity(int what) {
  if (slb_verbosity & what) slb_verbosity -= what;
  report_verbosity();
}
void report_verbosity() {
  printf("Verbosity =");
  if (slb_verbosity == 0) { printf(" NONE\n"); return; }
  if (slb_verbosity & TRACE_ROUTINE_EXITS) printf(" TRACE_ROUTINE_EXITS");
  if (slb_verbosity & OBJECT_DETAILS) printf(" OBJECT_DETAILS");
  if (slb_verbosity & FORCE_DETAILS) printf(" FORCE_DETAILS");
  printf("\n");
}

void slb_trace(LBSys lb, const char *what) {
  if (slb_verbosity & TRACE_ROUTINE_EXITS) printf("LB %i : %s done\n", lb->step, what);
}

long slb_node(LBSys lb, int i, int j, int k) {
  return (long)lb->esk * ((long)lb->esj * i + j) + k;
}

/* D3Q15 table of reference src/lbmisc.c:87-104, stored as the reference
 * stores it: c[3*q + axis], w[q] */
static const int LINKS[15][4] = {
    {0, 0, 0, 16}, {1, 0, 0, 8}, {-1, 0, 0, 8}, {0, 1, 0, 8}, {0, -1, 0, 8},
    {0, 0, 1, 8}, {0, 0, -1, 8}, {1, 1, 1, 1}, {-1, 1, 1, 1}, {1, -1, 1, 1},
    {-1, -1, 1, 1}, {1, 1, -1, 1}, {-1, 1, -1, 1}, {1, -1, -1, 1}, {-1, -1, -1, 1}};

/* reference src/lbmisc.c:81-152 */
LBSys newlb(int reqesi, int reqesj, int reqesk, char *name) {
  LBSys lb = (LBSys)xcalloc(1, sizeof(LBSys_type));
  slb_priv *st = (slb_priv *)xcalloc(1, sizeof(slb_priv));
  long n, q;
  if (lb == NULL) error("No room for lbsys structure\n");
  lb->c = (int *)xcalloc(45, sizeof(int));
  lb->w = (int *)xcalloc(15, sizeof(int));
  for (q = 0; q < 15; q++) {
    lb->c[3 * q] = LINKS[q][0]; lb->c[3 * q + 1] = LINKS[q][1]; lb->c[3 * q + 2] = LINKS[q][2];
    lb->w[q] = LINKS[q][3];
  }
  lb->esi = reqesi; lb->esj = reqesj; lb->esk = reqesk;
  n = (long)reqesi * reqesj * reqesk;
  if (n <= 0 || n >= 2147483647L / 15) error("newlb: lattice size out of range");
  lb->nnodes = (int)n;
  lb->a = NULL; /* host mirror, allocated on demand (lbpull / host writes) */
  lb->mask = (int *)xcalloc(n, sizeof(int));
  lb->obj = (LBObj *)xcalloc(n, sizeof(LBObj));
  lb->ux = (LBReal *)xcalloc(n, sizeof(LBReal)); lb->uy = (LBReal *)xcalloc(n, sizeof(LBReal));
  lb->uz = (LBReal *)xcalloc(n, sizeof(LBReal));
  lb->fx = (LBReal *)xcalloc(n, sizeof(LBReal)); lb->fy = (LBReal *)xcalloc(n, sizeof(LBReal));
  lb->fz = (LBReal *)xcalloc(n, sizeof(LBReal));
  lb->bx = (LBReal *)xcalloc(n, sizeof(LBReal)); lb->by = (LBReal *)xcalloc(n, sizeof(LBReal));
  lb->bz = (LBReal *)xcalloc(n, sizeof(LBReal));
  lb->tau = 0.75;
  lb->rho0 = 0.0;
  for (q = 0; q < 15; q++) lb->rho0 += lb->w[q];
  lb->objects_moving = 0; lb->skip_solid = 0; lb->stokes_flow = 0; lb->vel_corrected = 1;
  lb->step = 0; lb->next_id = 0; lb->obj_head = NULL; lb->status = POST_COLLIDE;
  lb->changed_objects = 0; lb->rescale = 1.0; lb->load_average = 0;
  lb->psi = NULL; lb->rho = NULL;
  slb_verbosity = 0;
  tstart = 0;
  if (myscmp("null", name)) lb->name = NULL; else lb->name = mycopy(name);
  lb->monitoring = (lb->name == NULL) ? 0 : 1;
  lb->precision = SLB_FP64;
  /* every host array starts in step with the zeroed device state */
  st->geom_gen = st->ads_gen = st->bf_gen = st->uw_gen = 1;
  st->a_gen = st->a_sent = 0;
  st->host_a_valid = 0; st->host_f_valid = 1;
  lb->priv = st;
  printf("LB system '%s' initialised for %i * %i * %i lattice\n", lb->name, lb->esi, lb->esj, lb->esk);
#ifdef SIGNAL
  siginit();
  printf("Signalling implemented, process id = %i\n", (int)getpid());
#else
  printf("Signalling not implemented\n");
#endif
  return lb;
}

slb_priv *slb_state(LBSys lb) { return (slb_priv *)lb->priv; }

LBReal *slb_host_a(LBSys lb) {
  if (lb->a == NULL) {
    /* page-locked when possible: uploads and downloads then run as DMA */
    lb->a = (LBReal *)slbc_host_alloc(15 * (size_t)lb->nnodes * sizeof(LBReal));
    slb_state(lb)->a_pinned = lb->a != NULL;
    if (lb->a == NULL) lb->a = (LBReal *)xcalloc(15 * (size_t)lb->nnodes, sizeof(LBReal));
  }
  return lb->a;
}

void slb_mark_geometry(LBSys lb) { slb_state(lb)->geom_gen++; }
void slb_mark_ads(LBSys lb) { slb_state(lb)->ads_gen++; }
void slb_mark_bodyforce(LBSys lb) { slb_state(lb)->bf_gen++; }
void slb_mark_wallvel(LBSys lb) { slb_state(lb)->uw_gen++; }
void slb_mark_pops(LBSys lb) { slb_priv *st = slb_state(lb); st->a_gen++; st->host_a_valid = 1; }
void slb_device_changed(LBSys lb) { slb_state(lb)->host_a_valid = 0; }
void slb_forces_changed(LBSys lb) { slb_state(lb)->host_f_valid = 0; }

/* ---- dense object table and boundary list (uploaded with the geometry) --- */

/* open-addressing map object pointer -> dense index */
typedef struct { LBObj *key; int *val; long cap; } objmap_t;

static unsigned long ptr_hash(const void *p) {
  unsigned long h = (unsigned long)(size_t)p;
  h ^= h >> 33; h *= 0xff51afd7ed558ccdUL; h ^= h >> 33;
  return h;
}

static int objmap_get(objmap_t *m, LBObj p, int *next, LBObj **objs, int *cap) {
  unsigned long h = ptr_hash(p) & (unsigned long)(m->cap - 1);
  while (m->key[h] != NULL) {
    if (m->key[h] == p) return m->val[h];
    h = (h + 1) & (unsigned long)(m->cap - 1);
  }
  m->key[h] = p;
  m->val[h] = *next;
  if (*next == *cap) {
    *cap *= 2;
    *objs = (LBObj *)realloc(*objs, (size_t)*cap * sizeof(LBObj));
    if (*objs == NULL) error("No room for object table");
  }
  (*objs)[*next] = p;
  return (*next)++;
}

static int objmap_find(const objmap_t *m, LBObj p) {
  unsigned long h = ptr_hash(p) & (unsigned long)(m->cap - 1);
  while (m->key[h] != NULL) {
    if (m->key[h] == p) return m->val[h];
    h = (h + 1) & (unsigned long)(m->cap - 1);
  }
  return -1;
}

/* distinct objects of one range of the map, in first-seen order */
typedef struct {
  LBObj *key;     /* open-addressing set */
  long cap;
  LBObj *list;    /* first-seen order */
  long count, list_cap;
} objseen_t;

typedef struct {
  LBSys lb;
  long n;
  int chunks;
  objseen_t *seen;
  const objmap_t *map;
  int *objidx;
} objscan_t;

static void seen_add(objseen_t *s, LBObj p) {
  unsigned long h;
  if (2 * (s->count + 1) > s->cap) {  /* grow and rehash */
    long cap = s->cap ? 4 * s->cap : 64, e;
    LBObj *key = (LBObj *)xcalloc(cap, sizeof(LBObj));
    for (e = 0; e < s->count; e++) {
      h = ptr_hash(s->list[e]) & (unsigned long)(cap - 1);
      while (key[h] != NULL) h = (h + 1) & (unsigned long)(cap - 1);
      key[h] = s->list[e];
    }
    free(s->key);
    s->key = key;
    s->cap = cap;
  }
  h = ptr_hash(p) & (unsigned long)(s->cap - 1);
  while (s->key[h] != NULL) {
    if (s->key[h] == p) return;
    h = (h + 1) & (unsigned long)(s->cap - 1);
  }
  s->key[h] = p;
  if (s->count == s->list_cap) {
    s->list_cap = s->list_cap ? 2 * s->list_cap : 16;
    s->list = (LBObj *)realloc(s->list, (size_t)s->list_cap * sizeof(LBObj));
    if (s->list == NULL) error("No room for the object scan");
  }
  s->list[s->count++] = p;
}

/* tasks [lo, hi) of the first pass: the distinct objects of each range */
static void scan_seen(long lo, long hi, void *ctx) {
  objscan_t *c = (objscan_t *)ctx;
  long t, x;
  for (t = lo; t < hi; t++) {
    const long x0 = c->n * t / c->chunks, x1 = c->n * (t + 1) / c->chunks;
    LBObj last = NULL;
    for (x = x0; x < x1; x++) {
      LBObj p = c->lb->obj[x];
      if (p == NULL || p == last) continue;
      last = p;
      seen_add(&c->seen[t], p);
    }
  }
}

/* tasks of the last pass: the dense index of every node */
static void scan_fill(long lo, long hi, void *ctx) {
  objscan_t *c = (objscan_t *)ctx;
  long t, x;
  for (t = lo; t < hi; t++) {
    const long x0 = c->n * t / c->chunks, x1 = c->n * (t + 1) / c->chunks;
    LBObj last = NULL;
    int idx = -1;
    for (x = x0; x < x1; x++) {
      LBObj p = c->lb->obj[x];
      if (p == NULL) { c->objidx[x] = -1; continue; }
      if (p != last) { last = p; idx = objmap_find(c->map, p); }
      c->objidx[x] = idx;
    }
  }
}

static void upload_geometry(LBSys lb) {
  slb_priv *st = slb_state(lb);
  long n = lb->nnodes, nb = 0;
  int nobj = 0, cap = 16, t;
  int *objidx = (int *)malloc((size_t)n * sizeof(int));
  LBObj *objs = (LBObj *)xcalloc(cap, sizeof(LBObj));
  objmap_t m;
  objscan_t sc;
  if (objidx == NULL) error("No room for the object index");
  /* dense index of every object the map references, in first-seen order:
   * the distinct objects of contiguous ranges in parallel, merged in range
   * order, then every node's index in parallel */
  sc.lb = lb; sc.n = n; sc.objidx = objidx;
  sc.chunks = slb_par_threads(n, 1L << 20);
  sc.seen = (objseen_t *)xcalloc(sc.chunks, sizeof(objseen_t));
  slb_parallel_for(sc.chunks, 1, scan_seen, &sc);
  m.cap = 64;
  {
    long distinct = 16;
    for (t = 0; t < sc.chunks; t++) distinct += sc.seen[t].count;
    while (m.cap < 4 * distinct) m.cap *= 2;
  }
  m.key = (LBObj *)xcalloc(m.cap, sizeof(LBObj));
  m.val = (int *)xcalloc(m.cap, sizeof(int));
  for (t = 0; t < sc.chunks; t++) {
    long e;
    for (e = 0; e < sc.seen[t].count; e++) objmap_get(&m, sc.seen[t].list[e], &nobj, &objs, &cap);
    free(sc.seen[t].key);
    free(sc.seen[t].list);
  }
  free(sc.seen);
  sc.map = &m;
  slb_parallel_for(sc.chunks, 1, scan_fill, &sc);
  free(m.key); free(m.val);
  /* flag words on the GPU, and from them the solid nodes with a fluid
   * neighbour, grouped by object, node order kept */
  free(st->bnd_node); free(st->bnd_obj);
  st->bnd_node = NULL; st->bnd_obj = NULL;
  slb_check(slbc_set_geometry_auto(st->dev, objidx, nobj, &st->bnd_node, &st->bnd_obj, &nb), "geometry upload");
  st->nbnd = nb;
  free(st->objs);
  st->objs = objs;
  st->nobj = nobj;
  free(st->objidx);
  st->objidx = objidx;  /* kept: moves of objects update it in place */
  st->geom_sent = st->geom_gen;
  /* solidity changed: body-force uniformity must be re-checked */
  st->bf_sent = 0;
  st->host_f_valid = 0;
}

typedef struct { const int *mask; unsigned char *ads; } adsfill_t;

static void fill_ads(long lo, long hi, void *ctx) {
  adsfill_t *a = (adsfill_t *)ctx;
  long x;
  for (x = lo; x < hi; x++) a->ads[x] = (a->mask[x] & 0x4000) ? 1 : 0;
}

static void upload_ads(LBSys lb) {
  slb_priv *st = slb_state(lb);
  adsfill_t a;
  unsigned char *ads = (unsigned char *)malloc((size_t)lb->nnodes);
  if (ads == NULL) error("No room for the adsorption bits");
  a.mask = lb->mask; a.ads = ads;
  slb_parallel_for(lb->nnodes, 1L << 20, fill_ads, &a);
  slb_check(slbc_set_adsorption(st->dev, ads), "adsorption upload");
  free(ads);
  st->ads_sent = st->ads_gen;
}

static void sync_params(LBSys lb) {
  slbc_params p;
  memset(&p, 0, sizeof p);
  p.tau = lb->tau; p.rho0 = lb->rho0;
  p.stokes_flow = lb->stokes_flow; p.skip_solid = lb->skip_solid;
  p.objects_moving = lb->objects_moving;
  slb_check(slbc_set_params(slb_state(lb)->dev, &p), "parameter upload");
}

/* Create the device state at the first call, re-create it when lb->precision
 * changed, and upload every host array that changed since the last call. */
slbc_lattice *slb_device(LBSys lb) {
  slb_priv *st = slb_state(lb);
  if (st->dev != NULL && st->dev_precision != lb->precision) {
    /* keep the state across a precision change */
    if (!st->host_a_valid) {
      slb_check(slbc_get_pops(st->dev, slb_host_a(lb)), "population download");
      st->host_a_valid = 1;
    }
    slbc_destroy(st->dev);
    st->dev = NULL;
    st->a_gen++;
  }
  if (st->dev == NULL) {
    if (lb->precision != SLB_FP64 && lb->precision != SLB_FP32 && lb->precision != SLB_BF16)
      error("lb->precision must be SLB_FP64, SLB_FP32 or SLB_BF16");
    slb_check(slbc_create(&st->dev, lb->esi, lb->esj, lb->esk, lb->precision), "device set-up");
    st->dev_precision = lb->precision;
    st->geom_sent = st->ads_sent = st->bf_sent = st->uw_sent = 0;
    st->a_sent = (lb->a == NULL) ? st->a_gen : 0;
  }
  if (st->geom_sent != st->geom_gen) upload_geometry(lb);
  if (st->ads_sent != st->ads_gen) upload_ads(lb);
  if (st->bf_sent != st->bf_gen) {
    slb_check(slbc_set_bodyforce(st->dev, lb->bx, lb->by, lb->bz), "body force upload");
    st->bf_sent = st->bf_gen;
  }
  if (lb->objects_moving && st->uw_sent != st->uw_gen) {
    slb_check(slbc_set_wallvel(st->dev, lb->ux, lb->uy, lb->uz), "wall velocity upload");
    st->uw_sent = st->uw_gen;
  }
  if (st->a_sent != st->a_gen) {
    int rc = slbc_put_pops(st->dev, slb_host_a(lb));
    if (rc == 2 && lb->precision == SLB_BF16) {
      /* the host array stays the state: upload it again in FP32 */
      printf("Populations with unpaired deviations: lb->precision changed from SLB_BF16 to SLB_FP32\n");
      lb->precision = SLB_FP32;
      st->host_a_valid = 1;
      return slb_device(lb);
    }
    slb_check(rc, "population upload");
    st->a_sent = st->a_gen;
  }
  sync_params(lb);
  return st->dev;
}

/* ---- appended API --------------------------------------------------------- */

static void zero_forces(long lo, long hi, void *ctx) {
  LBSys lb = (LBSys)ctx;
  memset(lb->fx + lo, 0, (size_t)(hi - lo) * sizeof(LBReal));
  memset(lb->fy + lo, 0, (size_t)(hi - lo) * sizeof(LBReal));
  memset(lb->fz + lo, 0, (size_t)(hi - lo) * sizeof(LBReal));
}

typedef struct { LBSys lb; const long *node; const double *f3; } fscatter_t;

/* node forces of the boundary list into lb->fx/fy/fz (distinct nodes) */
static void scatter_forces(long lo, long hi, void *ctx) {
  fscatter_t *f = (fscatter_t *)ctx;
  long e;
  for (e = lo; e < hi; e++) {
    const long x = f->node[e];
    f->lb->fx[x] = f->f3[3 * e]; f->lb->fy[x] = f->f3[3 * e + 1]; f->lb->fz[x] = f->f3[3 * e + 2];
  }
}

void lbpull(LBSys lb) {
  slb_priv *st = slb_state(lb);
  if (st->dev == NULL) { slb_host_a(lb); return; }
  if (!st->host_a_valid) {
    slb_check(slbc_get_pops(st->dev, slb_host_a(lb)), "population download");
    st->host_a_valid = 1;
  }
  if (!st->host_f_valid) {
    fscatter_t fs;
    double *f3 = (double *)malloc(3 * (size_t)(st->nbnd + 1) * sizeof(double));
    if (f3 == NULL) error("No room for the node forces");
    slb_check(slbc_get_force(st->dev, f3), "force download");
    slb_parallel_for(lb->nnodes, 1L << 20, zero_forces, lb);
    fs.lb = lb; fs.node = st->bnd_node; fs.f3 = f3;
    slb_parallel_for(st->nbnd, 1L << 18, scatter_forces, &fs);
    free(f3);
    st->host_f_valid = 1;
  }
  slb_pull_rho(lb);
}

/* Deviation storage keeps post-collision states only: a separate bounce-back
 * or propagation phase, or a tracer step, moves the lattice to FP32 first. */
void slb_need_populations(LBSys lb, const char *what) {
  if (lb->precision != SLB_BF16) return;
  printf("%s needs stored populations: lb->precision changed from SLB_BF16 to SLB_FP32\n", what);
  lb->precision = SLB_FP32;
}

/* BF16 storage pairs the deviations of q and opp(q), which a collision makes
 * equal; solid nodes left unrelaxed (skip_solid) keep unpaired streamed
 * populations, so such a lattice steps in FP32. */
void slb_need_relaxed_solids(LBSys lb) {
  if (lb->precision != SLB_BF16 || !lb->skip_solid) return;
  printf("Relaxation only on fluid nodes (skip_solid) needs stored populations: "
         "lb->precision changed from SLB_BF16 to SLB_FP32\n");
  lb->precision = SLB_FP32;
}

void slb_pull_rho(LBSys lb) {
  slb_priv *st = slb_state(lb);
  if (st->dev == NULL || lb->rho == NULL || st->host_rho_valid) return;
  if (slbc_mp_get_rho(st->dev, lb->rho) == 0) st->host_rho_valid = 1;
}

void lbpush(LBSys lb) {
  slb_priv *st = slb_state(lb);
  st->geom_gen++; st->ads_gen++; st->bf_gen++; st->uw_gen++;
  if (lb->a != NULL) { st->a_gen++; st->host_a_valid = 1; }
}

void freelb(LBSys lb) {
  slb_priv *st;
  LBObj p, pp;
  if (lb == NULL) return;
  st = slb_state(lb);
  if (st->dev) slbc_destroy(st->dev);
  if (st->a_pinned) slbc_host_free(lb->a); else free(lb->a);
  free(st->objs); free(st->objidx); free(st->bnd_node); free(st->bnd_obj); free(st);
  p = lb->obj_head;
  while (p != NULL) { pp = p; p = p->next_obj; free(pp); }
  free(lb->mask); free(lb->obj);
  free(lb->ux); free(lb->uy); free(lb->uz); free(lb->fx); free(lb->fy); free(lb->fz);
  free(lb->bx); free(lb->by); free(lb->bz); free(lb->rho); free(lb->name);
  free(lb->c); free(lb->w);
  free(lb);
}

void *lbgetstream(LBSys lb) { return slbc_get_stream(slb_device(lb)); }
void lbsetstream(LBSys lb, void *stream) {
  slb_check(slbc_set_stream(slb_device(lb), stream), "stream change");
}
long lbkernelcount(void) { return slbc_launch_count(); }
int lbtuning(LBSys lb, int *cfg) {
  slb_priv *st = slb_state(lb);
  if (st->dev == NULL) { cfg[0] = cfg[1] = cfg[2] = cfg[3] = 0; return 0; }
  return slbc_get_tuning(st->dev, cfg);
}

int lbsettuning(LBSys lb, int *cfg) {
  int rc = slbc_set_tuning(slb_device(lb), cfg);
  if (rc) printf("lbsettuning: %s\n", slbc_last_error());
  return rc;
}

int lblayout(LBSys lb) {
  slb_priv *st = slb_state(lb);
  return st->dev == NULL ? -1 : slbc_layout(st->dev);
}

/* ---- printing and bookkeeping (reference src/lbmisc.c:156-412) ---------- */

void about() {
  printf("\nSunlightLB - a 3D Lattice Boltzmann code - GB300 library\n");
  printf("Drop-in implementation of the SunlightLB C API; the reference is\n");
  printf("Copyright (C) 2005 Unilever UK Central Resources Ltd., GPL v2 or later.\n\n");
}

void wrlinks(LBSys lb) {
  int q;
  for (q = 0; q < 15; q++)
    printf(" w%02i = %2i  c%02i = (%2i,%2i,%2i)\n", q, lb->w[q], q, lb->c[3 * q], lb->c[3 * q + 1], lb->c[3 * q + 2]);
  printf("\n");
}

void wrpars(LBSys lb) {
  long x;
  int nobjs = 0, nfluid = 0;
  double fxs = 0.0, fys = 0.0, fzs = 0.0, msize;
  LBReal nu, eta;
  LBObj p;
  for (p = lb->obj_head; p != NULL; p = p->next_obj) nobjs++;
  for (x = 0; x < lb->nnodes; x++)
    if (lb->obj[x] == NULL) { fxs += lb->bx[x]; fys += lb->by[x]; fzs += lb->bz[x]; nfluid++; }
  nu = (lb->tau - 0.5) / 3.0; eta = lb->rho0 * nu;
  msize = (lb->precision == SLB_BF16 ? 2 * 16.0 + 2 * 16.0 : 15.0 * (lb->precision == SLB_FP32 ? 4 : 8)) * lb->nnodes + 2.0 * lb->nnodes;
  printf("---------------------------------------------------\n");
  printf(" Operating parameters\n");
  printf("---------------------------------------------------\n");
  printf(" LB size = %i * %i * %i = %i\n", lb->esi, lb->esj, lb->esk, lb->nnodes);
  printf(" Using %s populations on the GPU\n", lb->precision == SLB_FP32 ? "single precision" :
         lb->precision == SLB_BF16 ? "BF16 deviation (FP32 moments)" : "double precision");
  printf(" Device memory requirement approx %0.2f MByte\n", msize / (1024.0 * 1024.0));
  printf(" rho0 = %0.4f\n", lb->rho0);
  printf(" tau, nu, eta = %0.4f %0.4f %0.4f\n", lb->tau, nu, eta);
  printf(" Number of objects = %i\n", nobjs);
  printf(" Number of fluid + solid nodes = %i + %i = %i\n", nfluid, lb->nnodes - nfluid, lb->nnodes);
  printf(" Expected total Fx, y, z = %0.2f %0.2f %0.2f\n", fxs, fys, fzs);
  printf(lb->stokes_flow ? " Stokes equations simulated\n" : " Navier-Stokes equations simulated\n");
  printf(lb->vel_corrected ? " Corrected velocity field used\n" : " Uncorrected velocity field used\n");
  printf(lb->skip_solid ? " Relaxation only on fluid nodes\n" : " Relaxation on fluid and solid nodes\n");
  printf(lb->objects_moving ? " Objects allowed to move\n" : " All objects are stationary\n");
#ifdef SIGNAL
  printf(" Signalling implemented, process id = %i\n", (int)getpid());
#else
  printf(" Signalling not implemented\n");
#endif
  if (lb->monitoring != 0) printf(" Monitoring data will be written to %s.mon\n", lb->name);
  else printf(" No monitoring\n");
  printf("---------------------------------------------------\n");
  slb_trace(lb, "wrpars");
}

void wrstatus(LBSys lb, FILE *fp) {
  fprintf(fp, "Currently at ");
  switch (lb->status) {
    case POST_BBL: fprintf(fp, "post-bounceback"); break;
    case POST_PROPAGATE: fprintf(fp, "post-propagation"); break;
    case POST_COLLIDE: fprintf(fp, "post-collision"); break;
    default: fprintf(fp, "(help, I'm stymied!)"); break;
  }
  fprintf(fp, " stage in the LB update cycle\n");
  slb_trace(lb, "wrstatus");
}

static void wrhms(FILE *fp, const char *fmt, long secs) {
  long hours, mins;
  if (secs < 0) return;
  hours = secs / 3600; secs -= 3600 * hours;
  mins = secs / 60; secs -= 60 * mins;
  if (fmt[0] != 'l') { fprintf(fp, "%li:%02li:%02li", hours, mins, secs); return; }
  if (hours == 0 && mins == 0 && secs == 0) { fprintf(fp, "no time at all"); return; }
  if (hours == 1) fprintf(fp, "1 hour "); else if (hours > 1) fprintf(fp, "%li hours ", hours);
  if (mins == 1) fprintf(fp, "1 min "); else if (mins > 1) fprintf(fp, "%li mins ", mins);
  if (secs == 0) fprintf(fp, "exactly"); else if (secs == 1) fprintf(fp, "1 sec");
  else fprintf(fp, "%li secs", secs);
}

void fwrstats(FILE *fp, int lbstep, int lbsize) {
  double rate = 0.0;
  time_t telapse = time(NULL) - tstart;
  if (telapse > 0) rate = (double)lbstep / (double)telapse;
  fprintf(fp, "LB step %6i: ", lbstep);
  wrhms(fp, "long", (long)telapse);
  fprintf(fp, " elapsed\n");
  fprintf(fp, " %6.2f updates/sec\n", rate);
  fprintf(fp, " %6.1f ksite-updates/sec\n", lbsize * rate / 1000.0);
}

void wrstats(LBSys lb) { fwrstats(stdout, lb->step, lb->nnodes); }

void wrmon(LBSys lb, char *what) {
  double rate = 0.0;
  time_t telapse = 0;
  char *monfile, w0;
  FILE *fp;
  if (lb->monitoring == 0) return;
  w0 = what[0];
  monfile = mycat(lb->name, ".mon");
  if ((fp = fopen(monfile, "w")) == NULL) {
    fprintf(stderr, "wrmon: I couldn't open %s.\n", monfile);
    free(monfile);
    return;
  }
  if (w0 == 'i' || w0 == 's') startclock();
  else if (w0 == 'r' || w0 == 'f' || w0 == 'e') {
    telapse = time(NULL) - tstart;
    if (telapse > 0) rate = (double)lb->step / (double)telapse;
  }
#ifdef SIGNAL
  fprintf(fp, "%i %s ", (int)getpid(), lb->name);
  if (w0 == 'i' || w0 == 's') fprintf(fp, "started 0:00:00 ? ?\n");
  else if (w0 == 'r' || w0 == 'f' || w0 == 'e') {
    fprintf(fp, w0 == 'r' ? "running " : "finished ");
    wrhms(fp, "short", (long)telapse);
    if (telapse > 0) fprintf(fp, " %0.2f %0.2f\n", rate, lb->nnodes * rate / 1000.0);
    else fprintf(fp, " ? ?\n");
  }
#endif
  if (w0 == 'r' || w0 == 'f' || w0 == 'e') {
#ifndef SIGNAL
    fprintf(fp, "%s %s\n", lb->name, w0 == 'r' ? "running" : "finished");
#endif
    fwrstats(fp, lb->step, lb->nnodes);
  }
#ifdef SIGNAL
  if (w0 == 'i' || w0 == 's' || w0 == 'r')
    fprintf(fp, "To update this file type : kill -USR1 %i\n", (int)getpid());
#endif
  if (fclose(fp) != 0) {
    fprintf(stderr, "wrmon: I couldn't close %s.\n", monfile);
    exit(EXIT_FAILURE);
  }
  free(monfile);
  printf("Monitor file %s.mon %s at %i\n", lb->name, what, lb->step);
  slb_trace(lb, "wrmon");
}

/* reference src/lbmisc.c:361-378 */
char *mycat(char *s, char *t) {
  char *v = (char *)malloc(strlen(s) + strlen(t) + 1);
  if (v == NULL) error("No room for string");
  strcpy(v, s);
  strcat(v, t);
  return v;
}
char *mycopy(char *s) { return mycat(s, ""); }
int myscmp(char *s, char *t) { return strncmp(t, s, strlen(s)) == 0; }
