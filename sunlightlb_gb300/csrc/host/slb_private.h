/*
 * Library-private host state of GB300 SunlightLB (hangs off lb->priv and
 * mp->priv).  The public structs of sunlightlb.h stay the reference's; this
 * records which host arrays changed since they were last sent to the GPU,
 * the dense object table the device uses, and the device handles.
 */
#ifndef SLB_PRIVATE_H_INC
#define SLB_PRIVATE_H_INC

#include "sunlightlb.h"
#include "slb_device.h"

typedef struct slb_priv {
  slbc_lattice *dev;        /* device state, created at the first device call */
  int dev_precision;
  /* generation counters of host-side data; *_sent = generation on the GPU */
  long geom_gen, geom_sent;   /* object map (obj[]) */
  long ads_gen, ads_sent;     /* adsorption bits (mask & 0x4000) */
  long bf_gen, bf_sent;       /* body force arrays */
  long uw_gen, uw_sent;       /* wall velocity arrays */
  long a_gen, a_sent;         /* host population mirror lb->a */
  int host_a_valid;           /* lb->a equals the device populations */
  int host_f_valid;           /* lb->fx/fy/fz equal the device node forces */
  int host_rho_valid;         /* lb->rho equals the device density snapshot */
  int a_pinned;               /* lb->a is page-locked (slbc_host_alloc) */
  /* dense object table of the last geometry upload */
  int nobj;
  LBObj *objs;                /* index -> object */
  int *objidx;                /* dense object index per node (-1 fluid), as on the GPU */
  long nbnd;
  long *bnd_node;             /* solid nodes with a fluid neighbour */
  int *bnd_obj;
  int nfluid;
} slb_priv;

typedef struct mp_priv {
  slbc_tracer *dev;
  int use_f64;
  long p_gen, p_sent;         /* host mirror mp->p written since upload */
  int host_p_valid;
} mp_priv;

/* helpers shared by the host translation units (slb_core.c) */
slb_priv *slb_state(LBSys lb);
slbc_lattice *slb_device(LBSys lb);        /* create / refresh the device state */
void slb_check(int rc, const char *what);  /* fatal on a device error */
LBReal *slb_host_a(LBSys lb);              /* lb->a, allocated on demand */
void slb_mark_geometry(LBSys lb);
void slb_mark_ads(LBSys lb);
void slb_mark_bodyforce(LBSys lb);
void slb_mark_wallvel(LBSys lb);
void slb_mark_pops(LBSys lb);              /* host lb->a is authoritative */
void slb_device_changed(LBSys lb);         /* device populations changed */
void slb_forces_changed(LBSys lb);
long slb_node(LBSys lb, int i, int j, int k);
void slb_trace(LBSys lb, const char *what);
void slb_pull_rho(LBSys lb);
void slb_need_populations(LBSys lb, const char *what);
void slb_need_relaxed_solids(LBSys lb);
/* parallel loop over [0, n) in contiguous ranges of at least `grain` (slb_par.c) */
typedef void (*slb_range_fn)(long lo, long hi, void *ctx);
void slb_parallel_for(long n, long grain, slb_range_fn fn, void *ctx);
int slb_par_threads(long n, long grain);

#endif
