/*
 * sunlightlb.h -- public C API of the GB300 SunlightLB library.
 *
 * This header is the drop-in boundary: every type, struct field (names,
 * types and order) and prototype that a SunlightLB C, Perl or Python (SWIG)
 * driver uses is declared here with the same meaning as in the reference
 * header src/sunlightlb.h.  Each prototype names the reference file:line of
 * the routine it replaces.  Fields and functions that the reference does not
 * have are APPENDED at the end of the structs and listed in the last section,
 * so binary layouts of the shared prefix are unchanged and a SWIG wrap of
 * this file (%include sunlightlb.h, as in src/SunlightLB.i:24-30) still
 * exposes every field the reference exposes.
 *
 * Velocity set: D3Q15 with weights w = {16, 8 x 6, 1 x 8}, b = sum w = 72
 * (reference src/lbmisc.c:87-104).  Populations are the deviations
 * a_i = w_i (f_i - rho0/b) (reference src/sunlightlb.h:72).
 *
 * Node index: inode = esk*(esj*i + j) + k, k fastest (reference
 * src/lbkernel.c:72).
 *
 * Population storage lives on the GPU.  lb->a is a HOST MIRROR in the
 * reference AoS order a[15*inode + q]; library routines keep it coherent
 * when they need it, and a driver that reads or writes lb->a directly calls
 * lbpull() before reading and lbpush() after writing (see the appended API).
 */

#ifndef SUNLIGHTLB_H_INC
#define SUNLIGHTLB_H_INC

#include <stdio.h>

/* Precision switches, as in reference src/sunlightlb.h:23-35.  LBReal is the
 * host-side real type of every struct field and API argument; the device
 * population precision is chosen at run time by lb->precision. */
#ifdef _SINGLE
typedef float LBReal;
#else
typedef double LBReal;
#endif

#ifdef _STORE_DOUBLE
typedef double LBStoreReal;
#else
typedef float LBStoreReal;
#endif

/* Verbosity flags (reference src/sunlightlb.h:39-43) */
#define TRACE_ROUTINE_EXITS   0x02
#define TRACING_ROUTINE_EXITS 0x02
#define OBJECT_DETAILS        0x04
#define MP_OBJECT_DETAILS     0x04
#define FORCE_DETAILS         0x08

/* Update-cycle status codes (reference src/sunlightlb.h:47-49) */
#define POST_BBL       42
#define POST_PROPAGATE 47
#define POST_COLLIDE   49

/* Device population precision (appended; value of lb->precision) */
#define SLB_FP64 0   /* FP64 populations, FP64 collision: parity path */
#define SLB_FP32 1   /* FP32 populations, FP32 collision, FP64 reductions */
#define SLB_BF16 2   /* FP32 moments + BF16 paired deviations from their equilibrium;
                        needs skip_solid = 0 (else the lattice moves to FP32) */

/* Lattice object (reference src/sunlightlb.h:53-64) */
typedef struct LBObj_struct {
  int id;
  LBReal posx, posy, posz;
  LBReal velx, vely, velz;
  LBReal angx, angy, angz;
  LBReal frcx, frcy, frcz;
  LBReal trqx, trqy, trqz;
  struct LBObj_struct *next_obj;
  struct LBObj_struct *base_obj;
} LBObj_type;

typedef LBObj_type *LBObj;

/* Lattice Boltzmann system (reference src/sunlightlb.h:68-102).  The fields
 * up to next_id are the reference's, in its order; precision and priv are
 * appended. */
typedef struct LBSys_struct {
  int *w, *c;
  LBReal *a;
  LBReal *ux, *uy, *uz;
  LBReal *fx, *fy, *fz;
  LBReal *bx, *by, *bz;
  int esi, esj, esk, nnodes, step, status, changed_objects;
  int objects_moving, skip_solid, stokes_flow, vel_corrected, monitoring;
  LBReal tau, rho0;
  LBReal vmeanx, vmeany, vmeanz;
  LBReal *psi;
  LBReal *rho;
  char *name;
  LBReal rescale;
  int load_average;
  LBObj *obj;
  LBObj obj_head;
  int *mask;
  int next_id;
  /* --- appended --- */
  int precision;      /* SLB_FP64 (default), SLB_FP32 or SLB_BF16 */
  void *priv;         /* library-private host/device state */
} LBSys_type;

typedef LBSys_type *LBSys;

/* Moment propagation system (reference src/sunlightlb.h:106-121) */
typedef struct MPSys_struct {
  LBSys lb;
  LBReal *p, *newp;
  int step;
  int objects_moving;
  int to_be_initialised;
  LBReal alpha, isoslice, poffset;
  LBReal p2bytemin, p2bytemax;
  char *name;
  /* --- appended --- */
  LBReal adprob;      /* adsorption probability per encounter, default 1.0
                         (1.0 = the reference's all-or-nothing adsorption) */
  int precision;      /* tracer precision SLB_FP64 / SLB_FP32; newmp copies
                         lb->precision, change it before the first mpstep */
  void *priv;         /* library-private host/device state */
} MPSys_type;

typedef MPSys_type *MPSys;

/* Isosurface, colour and image types, kept for source compatibility of
 * drivers (reference src/sunlightlb.h:125-161). */
typedef struct MPIso_struct {
  MPSys mp;
  LBReal val;
  int *count;
} MPIso_type;
typedef MPIso_type *MPIso;

typedef struct LBColour_struct {
  int red, green, blue;
} LBColour_type;
typedef LBColour_type *LBColour;

typedef struct LBColourMap_struct {
  int red_lo, green_lo, blue_lo;
  int red_hi, green_hi, blue_hi;
  LBReal v_lo, v_hi;
} LBColourMap_type;
typedef LBColourMap_type *LBColourMap;

typedef struct LBImage_struct {
  int width, height;
  int *red, *green, *blue;
  int back_red, back_green, back_blue;
  int object_red, object_green, object_blue;
} LBImage_type;
typedef LBImage_type *LBImage;

#ifdef __cplusplus
extern "C" {
#endif

/* Global verbosity (reference src/sunlightlb.h:171, defined in lbmisc.c) */
extern int slb_verbosity;

/* ---- Lattice construction, verbosity, misc (reference src/lbmisc.c) ---- */
LBSys newlb(int, int, int, char *);            /* src/lbmisc.c:81-152  */
void set_verbosity(int);                       /* src/lbmisc.c:55-59   */
void unset_verbosity(int);                     /* src/lbmisc.c:61-65   */
void report_verbosity();                       /* src/lbmisc.c:67-75   */
void error(char *);                            /* src/lbmisc.c:39-42   */
void about();                                  /* src/lbmisc.c:156-167 */
void wrpars(LBSys);                            /* src/lbmisc.c:193-242 */
void wrstatus(LBSys, FILE *);                  /* src/lbmisc.c:247-257 */
void wrlinks(LBSys);                           /* src/lbmisc.c:171-188 */
void wrstats(LBSys);                           /* src/lbmisc.c:278     */
void fwrstats(FILE *, int, int);               /* src/lbmisc.c:264-274 */
void startclock();                             /* src/lbmisc.c:47-51   */
void wrmon(LBSys, char *);                     /* src/lbmisc.c:286-354 */
char *mycat(char *, char *);                   /* src/lbmisc.c:361-366 */
char *mycopy(char *);                          /* src/lbmisc.c:370     */
int myscmp(char *, char *);                    /* src/lbmisc.c:376-378 */

/* ---- Update step (reference src/lbkernel.c) ---- */
void lbstep(LBSys);                            /* src/lbkernel.c:49-51   */
void bbl(LBSys);                               /* src/lbkernel.c:35-39   */
void bblforce(LBSys);                          /* src/lbkernel.c:41-45   */
void propagate(LBSys);                         /* src/lbkernel.c:623-762 */
void collide(LBSys);                           /* src/lbkernel.c:769-877 */

/* ---- Objects and geometry (reference src/lbobjs.c) ---- */
LBObj lookupobj(LBSys, int);                   /* src/lbobjs.c:68-72   */
LBObj addobj(LBSys);                           /* src/lbobjs.c:45-52   */
void zeroobj(LBObj);                           /* src/lbobjs.c:57-63   */
LBObj insertsubs(LBSys, char *, int, int, int, int, int, int); /* src/lbobjs.c:77-123 */
LBObj insertlist(LBSys, char *);               /* src/lbobjs.c:128-165 */
LBObj insertslab(LBSys, LBReal, LBReal, LBReal, LBReal, LBReal, LBReal); /* src/lbobjs.c:170-199 */
LBObj insertsph(LBSys, LBReal, LBReal, LBReal, LBReal); /* src/lbobjs.c:204-232 */
LBObj insertcyl(LBSys, char *, LBReal, LBReal, LBReal); /* src/lbobjs.c:241-287 */
LBObj insertwall(LBSys, char *, int);          /* src/lbobjs.c:294-357 */
LBObj flattenobj(LBSys);                       /* src/lbobjs.c:362-392 */
LBObj invertobj(LBSys);                        /* src/lbobjs.c:397-428 */
void removeobjs(LBSys);                        /* src/lbobjs.c:433-453 */
void wrobjs(LBSys);                            /* src/lbobjs.c:457-467 */
void wrmap(LBSys, char *);                     /* src/lbobjs.c:472-516 */
void makemask(LBSys);                          /* src/lbobjs.c:526-560 */
void vspread(LBSys);                           /* src/lbobjs.c:565-589 */
void zerobf(LBSys);                            /* src/lbobjs.c:593-604 */
void addbf(LBSys, double, double, double);     /* src/lbobjs.c:608-619 */
void vset(LBSys, int, int, int, LBReal, LBReal, LBReal); /* src/lbobjs.c:623-643 */
int countmask(LBSys, char *);                  /* src/lbobjs.c:671-714 */
int countfluid(LBSys);                         /* src/lbobjs.c:648-655 */
void syncobjs(LBSys);                          /* src/lbobjs.c:660-663 */

/* ---- Checkpoint and field I/O (reference src/lbstore.c) ---- */
void lbsave(LBSys, char *);                    /* src/lbstore.c:36-91    */
void lbload(LBSys, char *);                    /* src/lbstore.c:104-218  */
void lbsavevel(LBSys, char *, char *);         /* src/lbstore.c:227-296  */
void lbloadvel(LBSys, char *, char *);         /* src/lbstore.c:305-404  */
void lbsavestr(LBSys, char *, char *);         /* src/lbstore.c:412-515  */
void lbsaveobj(LBSys, char *);                 /* src/lbstore.c:523-545  */
void lbloadobj(LBSys, char *);                 /* src/lbstore.c:554-586  */
void lbsavefrc(LBSys, char *, char *);         /* src/lbstore.c:595-640  */
void lbsavemap(LBSys, char *, char *);         /* src/lbstore.c:647-678  */

/* ---- Measurement (reference src/lbmeasure.c) ---- */
void accvmean(LBSys, LBReal);                  /* src/lbmeasure.c:58-106  */
void vzero(LBSys);                             /* src/lbmeasure.c:110-121 */
void vgrab(LBSys, LBReal);                     /* src/lbmeasure.c:129-166 */
void vsave(LBSys, char *);                     /* src/lbmeasure.c:173-203 */
void measure(LBSys);                           /* src/lbmeasure.c:30-49   */
void zeroforce(LBSys);                         /* src/lbmeasure.c:208-216 */
void normforce(LBSys, LBReal);                 /* src/lbmeasure.c:221-231 */
void distribf(LBSys);                          /* src/lbmeasure.c:236-263 */
void wrmeas(LBSys);                            /* src/lbmeasure.c:268-301 */
LBReal discrf(LBSys);                          /* src/lbmeasure.c:308-332 */

/* ---- Moment propagation (reference src/mpkernel.c, src/mpmisc.c) ---- */
void mpstep(MPSys);                            /* src/mpkernel.c:33-43  */
MPSys newmp(LBSys, char *);                    /* src/mpmisc.c:38-59    */
void mpinit(MPSys);                            /* src/mpmisc.c:83-99    */
void mpwrpars(MPSys);                          /* src/mpmisc.c:104-114  */
void mprhoinit(MPSys);                         /* src/mpmisc.c:64-79    */
void mpcheck(MPSys);                           /* src/mpmisc.c:121-136  */
LBReal mpmean(MPSys);                          /* src/mpmisc.c:142-158  */
LBReal mpmax(MPSys);                           /* src/mpmisc.c:164-183  */
LBReal mpmin(MPSys);                           /* src/mpmisc.c:189-208  */
void mprescale(MPSys, LBReal);                 /* src/mpmisc.c:214-225  */
void mpcopy(MPSys, MPSys);                     /* src/mpmisc.c:233-246  */
LBReal mpspread(MPSys, char *);                /* src/mpmisc.c:466-499  */

/* ---- Tracer velocity autocorrelation (reference src/mpvacf.c) ---- */
void mpvacfinit(MPSys, MPSys, char *, int);    /* src/mpvacf.c:39-293   */
void mpvacfinit2(MPSys, MPSys);                /* src/mpvacf.c:298-335  */
void mpvacf(MPSys, MPSys);                     /* src/mpvacf.c:337-389  */
LBReal mpvacfwr(MPSys, MPSys, char *, int);    /* src/mpvacf.c:391-428  */

/* ---- Tracer injection (reference src/mpobjs.c) ---- */
void mpall(MPSys, LBReal);                     /* src/mpobjs.c:28-43    */
void mpslab(MPSys, LBReal, LBReal, LBReal, LBReal, LBReal, LBReal, LBReal); /* src/mpobjs.c:50-68 */
void mpwall(MPSys, char *, int, LBReal);       /* src/mpobjs.c:75-117   */
void mpsph(MPSys, LBReal, LBReal, LBReal, LBReal, LBReal); /* src/mpobjs.c:122-143 */
void mpcyl(MPSys, char *, LBReal, LBReal, LBReal, LBReal); /* src/mpobjs.c:152-180 */
void mpsubs(MPSys, char *, int, int, int, int, int, int, LBReal); /* src/mpobjs.c:188-226 */
void mplist(MPSys, char *, LBReal);            /* src/mpobjs.c:233-261  */

/* ---- Adsorption (reference src/mpads.c) ---- */
void adall(MPSys);                             /* src/mpads.c:37-46     */
void adnone(MPSys);                            /* src/mpads.c:51-62     */
void adslab(MPSys, LBReal, LBReal, LBReal, LBReal, LBReal, LBReal); /* src/mpads.c:67-82 */
void adsph(MPSys, LBReal, LBReal, LBReal, LBReal); /* src/mpads.c:87-105 */
void adcyl(MPSys, char *, LBReal, LBReal, LBReal); /* src/mpads.c:114-139 */
LBReal adtotal(MPSys, char *, int);            /* src/mpads.c:149-172   */
void adzero(MPSys);                            /* src/mpads.c:177-186   */

/* ---- Signals (reference src/sunlightlb.h:298-314, src/lbsignal.c) ---- */
#ifndef _NO_SIGNALLING
#define SIGNAL
extern int slb_signal_flag;
void sighandle(LBSys);                         /* src/lbsignal.c:40-62  */
void sighook(int);                             /* src/lbsignal.c:72-79  */
void siginit();                                /* src/lbsignal.c:84-88  */
#endif

/* ==========================================================================
 * Appended API (no counterpart in the reference).
 * ========================================================================== */

/* Copy the device state into the host mirrors: lb->a (reference AoS order,
 * FP64 values of the device populations), and lb->fx/fy/fz (node forces of
 * the last measure).  Call before reading these arrays directly. */
void lbpull(LBSys);
/* Mark every host-side array of lb (a, bx/by/bz, ux/uy/uz, mask, obj map)
 * as changed, so the next device call uploads it.  Call after writing these
 * arrays directly (the library's own routines do this themselves). */
void lbpush(LBSys);
/* Advance n update steps; identical to n calls of lbstep but replayed from
 * a captured CUDA graph. */
void lbsteps(LBSys, int);
/* Run n steps of check intervals: repeat (n-2 lbstep + measure) until the
 * relative change of vmeanx between intervals is below tol or maxsteps
 * update steps are done; returns the update steps taken. */
int lbconverge(LBSys, int, LBReal, int);
/* Release every host and device resource of lb. */
void freelb(LBSys);
/* CUDA stream the lattice launches on (cudaStream_t as void*); setting it
 * makes all later launches of lb go to that stream. */
void *lbgetstream(LBSys);
void lbsetstream(LBSys, void *);
/* Number of GPU kernel launches made by the library so far (all lattices). */
long lbkernelcount(void);
/* Launch shape the autotuner chose for the fused step of lb, cfg[4] = {even
 * rows per thread, even threads along k, odd rows per thread, odd threads
 * along k} (BF16 lattices: planes per block in place of rows per thread;
 * rows per thread -4: the 128-bit form, 4 nodes along k per thread, 128
 * threads per block); returns 1 tuned, -1 defaults, 0 not decided yet. */
int lbtuning(LBSys, int *);
/* Set the launch shape of the fused step of lb (same cfg as lbtuning; rows
 * per thread -4 selects the 128-bit form, 4 nodes along k per thread and
 * 128 threads per block, FP32 populations with esk a multiple of 4);
 * returns 0, or non-zero (with a message) for a shape it does not take. */
int lbsettuning(LBSys, int *);
/* Storage layout of the device populations of lb: 0 the reference's order
 * (after an upload), 1 after an even update (the next update is the
 * pull-and-push one), 2 after an odd update; -1 before the first device
 * call. */
int lblayout(LBSys);
/* Release every host and device resource of mp. */
void freemp(MPSys);
/* Host mirror mp->p: mppull copies the device tracer into it, mppush marks
 * it as written so the next device call uploads it. */
void mppull(MPSys);
void mppush(MPSys);
/* Warm start from a velocity field held in arrays (rho may be NULL for
 * rho = rho0): the population rebuild of lbloadvel (reference
 * src/lbstore.c:340-401) followed by a collision. */
void lbsetvel(LBSys, LBReal *, LBReal *, LBReal *, LBReal *);
/* The same from three FP32 device arrays u[0..n), u[n..2n), u[2n..3n) with
 * rho = rho0 (a velocity field computed on the GPU, e.g. a learned
 * prediction, never crosses to the host). */
void lbsetveldev(LBSys, void *);
/* Velocity field (the per-node accvmean term, half-force corrected when
 * lb->vel_corrected) into three FP32 device arrays laid out as above. */
void lbvelocity(LBSys, void *);
/* lbvelocity plus the density deviation rho - rho0 of every fluid node (0 on
 * solid nodes) into one FP32 device array (appended, no counterpart). */
void lbstate(LBSys, void *, void *);
/* lbsetveldev with the density rho0 + drho[x] of every node from an FP32
 * device array of deviations (NULL: rho0) (appended, no counterpart). */
void lbsetstatedev(LBSys, void *, void *);
/* Tracer totals over "fluid", "solid", "adsorbed" or "all" nodes (the sums
 * that mpcheck and adtotal print, reference src/mpmisc.c:121-136), or
 * "injected": the tracer that mpall, mpslab, mpwall, mpsph and mpcyl have
 * added (sum of pval - old p over the nodes they set) since mpinit, for the
 * mass balance of a constant-concentration source. */
LBReal mptotal(MPSys, char *);
/* Mean tracer over the fluid nodes of the plane "x"/"y"/"z" = pos (0 when
 * the plane has no fluid node): the breakthrough curve of a front. */
LBReal mpplane(MPSys, char *, int);

/* One object made of the nodes where mask[inode] != 0, inode =
 * esk*(esj*i+j)+k: the node list of insertlist (reference
 * src/lbobjs.c:128-165) held in memory instead of a file. */
LBObj insertmask(LBSys, unsigned char *);

/* Seeded random sequential addition of spheres in a periodic n^3 box (no
 * counterpart in the reference, whose packings come from files): centres
 * uniform in [0, n)^3 and radii uniform in [rmin, rmax] from splitmix64
 * (four draws per try: x, y, z, r, each (z >> 11) * 2^-53); a try is
 * accepted when its periodic minimum-image distance to every accepted
 * sphere is at least the sum of the radii (always, with overlap != 0); each
 * accepted sphere and its periodic images are stamped into the node mask
 * (rsq < r^2) until the solid fraction reaches phi.  spheres gets
 * (r, x, y, z) for each accepted sphere (room for max_spheres), solid (may
 * be NULL) the n^3 mask, inode = n*(n*i + j) + k.  Returns the number of
 * spheres, -1 when the packing stalls (a sphere would need more than
 * max_tries tries), -2 when max_spheres is too small, -3 on bad arguments. */
int rsapacking(int n, double phi, double rmin, double rmax, unsigned long long seed, int overlap,
               long max_tries, double *spheres, int max_spheres, unsigned char *solid);

/* n calls of insertsph (rad[s], x[s], y[s], z[s]) in order, with the node
 * tests on the GPU: the same objects (one per sphere that covers a node,
 * pos = its centre), the same object map (a later sphere takes a node over)
 * and the same messages.  Returns the number of objects created.  No
 * counterpart in the reference (insertsph, src/lbobjs.c:204-232, one
 * sphere at a time). */
int insertspheres(LBSys, int, LBReal *, LBReal *, LBReal *, LBReal *);
/* Move the spherical object obj of radius rad (a sphere with its periodic
 * images, as insertsph + flattenobj build it) so that its centre is
 * (x, y, z): the node set is re-rasterised on the GPU, nodes the sphere
 * leaves become fluid at the equilibrium of density rho0 and the wall
 * velocity v + w x r there, fluid nodes it reaches join the object, and the
 * flag words, boundary list, mask, a uniform body force, the object's wall
 * velocities (when objects move) and obj->pos follow.  No counterpart in the
 * reference, which can only remove objects and insert new ones
 * (src/lbobjs.c:433-453).  FP32 or FP64 populations. */
void lbtranslate(LBSys, LBObj, LBReal, LBReal, LBReal, LBReal);

/* Batches (no counterpart in the reference): many independent lattices of
 * one precision (FP32 or FP64), each set up as usual, advanced together by
 * batchsteps in one persistent GPU launch; afterwards each lattice is used
 * as before (measure, lbpull, lbsave ...).  batchsteps(b, n) gives every
 * lattice the same state as lbsteps(lb, n).  A lattice must outlive the
 * batches it is in. */
typedef struct LBBatch_struct *LBBatch;
LBBatch newbatch(void);
void batchadd(LBBatch, LBSys);
void batchsteps(LBBatch, int);
int batchsize(LBBatch);
/* 0 (default): one launch per step over the packed cell index of all the
 * lattices, replayed from a CUDA graph; 1: one persistent launch for all
 * the steps, every GPU block owning whole lattices. */
void batchmode(LBBatch, int);
void freebatch(LBBatch);

#ifdef __cplusplus
}
#endif

#endif /* SUNLIGHTLB_H_INC */
