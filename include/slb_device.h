/*
 * slb_device.h -- C ABI of the GB300 device layer of SunlightLB.
 *
 * Plain C types only (pointers, sizes, doubles): this is the thin layer the
 * host C implementation of sunlightlb.h calls to run the update path on one
 * GPU.  Every function returns 0 on success and a non-zero status on error;
 * slbc_last_error() then describes the failure.  The host layer maps a
 * failure to the reference's fatal-error convention (error() -> exit,
 * reference src/lbmisc.c:39-42).
 *
 * Device state of one lattice (an slbc_lattice):
 *   - populations, structure of arrays: pop[q*npad + inode], in FP64, FP32
 *     or BF16 (precision fixed at creation), stored in one of three layouts:
 *       N  : pop[q][x] = a[x][q], the reference's post-phase array;
 *       C0 : post-collision, pop[opp q][x] = a[x][q] (after an even step);
 *       C1 : post-collision, streamed: a[x][q] lives at pop[q][x + c_q], or at
 *            pop[opp q][x] when the link x -> x + c_q is a boundary link
 *            (after an odd step);
 *     the in-place AA update alternates C0 -> C1 -> C0;
 *     BF16 lattices hold each node's post-collision state instead, always in
 *     the reference's layout (N): FP32 moments (drho, ru) and the BF16
 *     deviations of the 8 pairs {q, opp q} from the zero-stress rebuild of
 *     those moments (a collision makes q and opp q deviate equally), two
 *     copies swapped by every step;
 *   - a per-node flag word (solid bit + 14 boundary-link bits);
 *   - the list of solid boundary nodes, sorted by object then node, with
 *     FP64 node forces accumulated during measurement;
 *   - body force (uniform constant or per node) and wall velocities.
 *
 * Node index inode = esk*(esj*i + j) + k; populations q follow the D3Q15
 * link table of reference src/lbmisc.c:87-104.
 */

#ifndef SLB_DEVICE_H_INC
#define SLB_DEVICE_H_INC

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct slbc_lattice slbc_lattice;

/* Run-time scalars of a lattice (fields of LBSys, reference
 * src/sunlightlb.h:81-83) */
typedef struct slbc_params {
  double tau, rho0;
  int stokes_flow, skip_solid, objects_moving;
} slbc_params;

/* Status (reference src/sunlightlb.h:47-49) matching a device layout */
#define SLBC_LAYOUT_N  0
#define SLBC_LAYOUT_C0 1
#define SLBC_LAYOUT_C1 2

const char *slbc_last_error(void);
/* Number of kernel launches made by this library since load. */
long slbc_launch_count(void);
/* Number of CUDA devices visible (0 when none). */
int slbc_device_count(void);

/* Create the device state of an esi*esj*esk lattice with populations in
 * `precision` (0 FP64, 1 FP32, 2 BF16), all populations zero (layout N).
 * Replaces the device side of newlb, reference src/lbmisc.c:81-152. */
int slbc_create(slbc_lattice **out, int esi, int esj, int esk, int precision);
void slbc_destroy(slbc_lattice *h);
int slbc_set_stream(slbc_lattice *h, void *stream);
void *slbc_get_stream(slbc_lattice *h);
int slbc_synchronize(slbc_lattice *h);

/* Geometry: objidx[nnodes] = dense object index of the node (-1 = fluid);
 * bnd_node[nbnd] / bnd_obj[nbnd] = solid nodes with at least one fluid
 * neighbour, sorted by (object, node).  Builds the flag words on the GPU.
 * Replaces the device side of makemask/syncobjs, reference
 * src/lbobjs.c:526-560, 660-663. */
int slbc_set_geometry(slbc_lattice *h, const int *objidx, int nobj,
                      const long *bnd_node, const int *bnd_obj, long nbnd);
/* The same with the boundary list built on the GPU from the flag words
 * (solid nodes with a fluid neighbour, grouped by object, node order kept
 * within an object); the list is returned in *bnd_node / *bnd_obj (malloc'ed,
 * the caller frees them) with its length in *nbnd.  Replaces the device side
 * of makemask/syncobjs like slbc_set_geometry. */
int slbc_set_geometry_auto(slbc_lattice *h, const int *objidx, int nobj,
                           long **bnd_node, int **bnd_obj, long *nbnd);
/* Adsorption bits (0x4000 of the reference mask) of every node, 1 byte per
 * node (reference src/mpads.c:28-44). */
int slbc_set_adsorption(slbc_lattice *h, const unsigned char *ads);
/* Node tests of n insertsph calls at once, on the GPU (reference
 * src/lbobjs.c:204-232 per sphere; no counterpart for many): spheres
 * sph[4s..4s+3] = (r, x, y, z) in insertion order on an esi x esj x esk
 * lattice whose nodes taken[x] != 0 already belong to an object.  Returns
 * last[x] = the highest s whose sphere covers node x (-1 none) -- the
 * sphere that holds the node after the n insertions --, count[s] = the
 * nodes sphere s covers, overlap[s] = 1 when one of them was taken or is
 * covered by an earlier sphere.  Host arrays; blocking. */
int slbc_raster_spheres(int esi, int esj, int esk, int nsph, const double *sph, const unsigned char *taken,
                        int *last, int *count, unsigned char *overlap);
/* 1 when the body force is one constant over the fluid nodes (returned in
 * b), 0 when it is held per node. */
int slbc_bodyforce_uniform(slbc_lattice *h, double b[3]);
/* Translate the spherical object of dense index obj (radius rad, centre
 * oldc, with its periodic images) to the centre newc, on the GPU (no
 * counterpart in the reference, which can only remove and re-insert
 * objects).  Nodes of the object the sphere no longer covers become fluid
 * at the equilibrium of density rho0 and the wall velocity vel + ang x r
 * (r = node - newc); fluid nodes it now covers join the object, their
 * populations unchanged; nodes of other objects are left alone; with
 * with_wallvel the wall velocities of the object's nodes are recomputed
 * (the vspread formula).  The changes come back in changed[2 * e] (node)
 * and changed[2 * e + 1] (new object index or -1), room for cap of them,
 * their number in *nchanged.  The flag words are rebuilt and the boundary
 * list with them, grouped by the caller's host copy of the dense object map
 * objidx_host (nobj objects), which this call updates with the changes; the
 * list comes back as in slbc_set_geometry_auto. */
int slbc_move_sphere(slbc_lattice *h, int obj, double rad, const double oldc[3], const double newc[3],
                     const double vel[3], const double ang[3], int with_wallvel, int *changed, long cap,
                     long *nchanged, int nobj, int *objidx_host, long **bnd_node, int **bnd_obj,
                     long *nbnd);
int slbc_set_params(slbc_lattice *h, const slbc_params *p);
/* Body force per node (NULL = zero); a force uniform over the fluid nodes is
 * detected and kept as a kernel constant (reference src/lbobjs.c:593-619). */
int slbc_set_bodyforce(slbc_lattice *h, const double *bx, const double *by, const double *bz);
/* Wall velocities per node, already scaled by rho0/12 as vspread/vset store
 * them (reference src/lbobjs.c:565-643); NULL releases them. */
int slbc_set_wallvel(slbc_lattice *h, const double *ux, const double *uy, const double *uz);

/* Populations in the reference AoS order a[15*inode + q] (FP64). put sets
 * layout N; get reads from any layout.  On a BF16 lattice put returns 2 when
 * some node's populations deviate unequally within a pair {q, opp q} (more
 * than BF16 rounding): that state needs FP32 or FP64 storage. */
int slbc_put_pops(slbc_lattice *h, const double *a);
/* Page-locked, zero-filled host memory for population mirrors (copies from
 * and to it run as DMA without a staging copy); NULL when it cannot be had,
 * in which case the caller uses ordinary memory.  Free with slbc_host_free. */
void *slbc_host_alloc(size_t bytes);
void slbc_host_free(void *p);
int slbc_get_pops(slbc_lattice *h, double *a);
int slbc_layout(slbc_lattice *h);
/* Launch shape of the fused step per parity, cfg = {even rows per thread,
 * even threads along k, odd rows per thread, odd threads along k}; for BF16
 * lattices the "rows per thread" entries are planes per block (1..64),
 * threads along k is 32, and the even entries serve every step (one update
 * kernel).  The
 * first slbc_step of a lattice of 2^20 nodes or more times the candidate
 * shapes on a copy of the populations and keeps the fastest (environment
 * SLB_AUTOTUNE=0 turns this off); get returns 1 tuned, -1 defaults, 0 not
 * yet decided; set pins a shape. */
int slbc_get_tuning(slbc_lattice *h, int cfg[4]);
int slbc_set_tuning(slbc_lattice *h, const int cfg[4]);

/* Fused update steps from a post-collision state (replaces lbstep,
 * reference src/lbkernel.c:49-51): n in-place AA steps.  use_graph replays
 * the steps from a captured CUDA graph. */
int slbc_step(slbc_lattice *h, int n, int use_graph);
/* Node-force accumulation of one bblforce (reference src/lbkernel.c:179-321
 * and 464-618) on the post-collision state, followed by one fused step. */
int slbc_force_step(slbc_lattice *h);
/* Separate phases on layout N (reference src/lbkernel.c:35-45, 623-762,
 * 769-877).  Any other layout is converted first. */
int slbc_bbl(slbc_lattice *h, int with_force);
int slbc_propagate(slbc_lattice *h);
int slbc_collide(slbc_lattice *h);

/* Node forces of the solid boundary nodes (reference src/lbmeasure.c:208-231) */
int slbc_zero_force(slbc_lattice *h);
int slbc_scale_force(slbc_lattice *h, double fac);
/* Node forces of the boundary list, 3 per entry (x, y, z). */
int slbc_get_force(slbc_lattice *h, double *f3);

/* Sums of accvmean over fluid nodes (reference src/lbmeasure.c:58-106):
 * out[0..2] = sum w*u, out[3] = sum w, out[4] = number of fluid nodes, with
 * u the velocity corrected by fac*b and w = psi^2 (psi NULL: w = 1). */
int slbc_vsum(slbc_lattice *h, double fac, const double *psi, double out[5]);
/* Object force and torque (reference src/lbmeasure.c:236-263):
 * pos[3*nobj] in, ft[6*nobj] out (frc xyz, trq xyz). */
int slbc_distribf(slbc_lattice *h, const double *pos, double *ft);

/* Warm start: populations rebuilt from (rho, u) with the lbloadvel formula
 * (reference src/lbstore.c:340-401), leaving layout N at POST_PROPAGATE.
 * rho may be NULL (rho = rho0). */
int slbc_set_velocity(slbc_lattice *h, const double *rho, const double *ux,
                      const double *uy, const double *uz, int skip_solid);

/* Moment propagation (reference src/mpkernel.c:33-368, src/mpmisc.c:38-246).
 * A tracer holds the scalar p of one MPSys; the density snapshot rho is per
 * lattice (the reference keeps one lb->rho shared by all its MPSys). */
typedef struct slbc_tracer slbc_tracer;
/* New tracer, p = 0, in FP64 (use_f64 = 1) or FP32 (reference
 * src/mpmisc.c:38-59). */
int slbc_mp_create(slbc_lattice *h, slbc_tracer **out, int use_f64);
void slbc_mp_destroy(slbc_tracer *t);
/* Density snapshot rho = rho0 + sum_q a_q on fluid nodes, rho0 on solid
 * nodes (reference src/mpmisc.c:64-79). */
int slbc_mp_rhoinit(slbc_lattice *h);
int slbc_mp_get_rho(slbc_lattice *h, double *rho);
int slbc_mp_put(slbc_tracer *t, const double *p);
int slbc_mp_get(slbc_tracer *t, double *p);
/* n tracer updates (reference src/mpkernel.c:47-368) with diffusion
 * parameter alpha and adsorption probability adprob (1 = the reference's
 * all-or-nothing adsorption).  moving: objstate holds 9 doubles per object
 * (pos xyz, vel xyz, ang xyz) for the moving-wall terms. */
int slbc_mp_step(slbc_tracer *t, int n, double alpha, double adprob, int moving,
                 const double *objstate, int nobj);
/* out[0] = sum p on fluid nodes, out[1] = sum p on solid nodes, out[2] = sum
 * p on adsorbing nodes, out[3] = sum p*pos, out[4] = sum p*pos^2 on fluid
 * nodes along axis (0,1,2; -1 none): reference src/mpmisc.c:121-158,466-499,
 * src/mpads.c:149-172. */
int slbc_mp_sums(slbc_tracer *t, int axis, double out[5]);
/* One step of the tracer velocity autocorrelation (reference
 * src/mpvacf.c:337-389) on FP64 tracers t (P) and t2 (P2) of one lattice:
 * P -= psi * pmean on fluid nodes (pmean = sum psi P / sum psi^2), then
 * out[0] = sum psi P u_axis, out[1] = sum psi P2 over the fluid nodes, u
 * from the populations and the density snapshot; psi_host per-node weights
 * (host) or null. */
int slbc_mp_vacf(slbc_tracer *t, slbc_tracer *t2, int axis, const double *psi_host, double out[2]);
/* Extremes of p over fluid nodes (reference src/mpmisc.c:164-208). */
int slbc_mp_minmax(slbc_tracer *t, double out[2]);
/* Set p = value on the fluid nodes of a region (reference src/mpobjs.c):
 * kind 0 all; 1 slab, geo = x1,x2,y1,y2,z1,z2; 2 wall, geo = axis, pos;
 * 3 sphere, geo = rad, ox, oy, oz; 4 cylinder, geo = axis, hole, rad, a, b. */
int slbc_mp_fill(slbc_tracer *t, int kind, const double *geo, double value);
/* Tracer added by slbc_mp_fill, sum of (value - old p) over the nodes set
 * since the tracer was created or last reset (no counterpart in the
 * reference: the mass balance of a constant-concentration source).  reset
 * = 1 zeroes the count after reading it. */
int slbc_mp_injected(slbc_tracer *t, int reset, double *out);
/* out[0] = sum of p, out[1] = number of fluid nodes on the plane axis = pos
 * (axis 0, 1, 2 for i, j, k; no counterpart in the reference: the
 * breakthrough curve of a tracer front). */
int slbc_mp_plane(slbc_tracer *t, int axis, int pos, double out[2]);
/* p *= fac on fluid nodes (reference src/mpmisc.c:214-225). */
int slbc_mp_scale(slbc_tracer *t, double fac);
/* p = 0 on adsorbing nodes (reference src/mpads.c:177-186). */
int slbc_mp_zero_ads(slbc_tracer *t);
/* dst p += src p on fluid nodes (reference src/mpmisc.c:233-246). */
int slbc_mp_add(slbc_tracer *dst, const slbc_tracer *src);

/* Batches (no counterpart in the reference: its drivers step one lattice at
 * a time).  A batch advances FP32 or FP64 lattices of one precision, each of
 * any size, by n fused steps.  Persistent mode: ONE launch per class for all
 * the steps, every block owns whole lattices (largest first to the least
 * loaded block) and runs all their steps with block barriers only.  Each lattice keeps its own device
 * state, so every other call works on it before and after; its stream waits
 * for the batch.  The lattices must outlive the batch. */
typedef struct slbc_batch slbc_batch;
int slbc_batch_create(slbc_batch **out, slbc_lattice *const *lats, int n);
int slbc_batch_step(slbc_batch *b, int nsteps);
int slbc_batch_workers(const slbc_batch *b);  /* blocks of the last persistent launch */
/* mode 0 (default): each step is one launch per class over the packed cell
 * index of all lattices (tiles of 256 cells), steps replayed from a CUDA
 * graph; mode 1: the persistent launch described above.  A class is the
 * lattices sharing moving walls (or not) and a uniform body force (or not). */
int slbc_batch_set_mode(slbc_batch *b, int mode);
void slbc_batch_destroy(slbc_batch *b);

/* Velocity field of the post-collision state into three device FP32 arrays
 * u[0..n), u[n..2n), u[2n..3n): (sum_q c_q a_q + fac * b) / (rho0 + sum_q a_q)
 * on fluid nodes (the per-node accvmean term, reference
 * src/lbmeasure.c:58-106), 0 on solid nodes.  FP32 and FP64 lattices. */
int slbc_get_velocity_dev(slbc_lattice *h, double fac, float *u);
/* Velocity warm start from three device FP32 arrays (as slbc_set_velocity
 * with rho = rho0; velocities already rescaled): layout N. */
int slbc_set_velocity_dev(slbc_lattice *h, const float *u, int skip_solid);
/* slbc_get_velocity_dev plus, when drho is not null, the density deviation
 * rho - rho0 = sum_q a_q of every fluid node (0 on solid nodes) into one
 * device FP32 array. */
int slbc_get_state_dev(slbc_lattice *h, double fac, float *u, float *drho);
/* slbc_set_velocity_dev with the density of every node rho0 + drho[x]
 * (drho: device FP32 deviations, kept exact; null: rho = rho0). */
int slbc_set_state_dev(slbc_lattice *h, const float *u, const float *drho, int skip_solid);

/* Tensor-core kernels of the learned warm start (no counterpart in the
 * reference).  slbc_tc_gemm: D[M x N] (FP32, row-major, leading dimension
 * ldd) = A[M x K] * B[N x K]^T, A and B BF16 row-major; M and N multiples of
 * 128, K of 64, device pointers 16-byte aligned; launched on `stream`.
 * slbc_tc_status synchronises the device and returns (and clears) the error
 * flag of these kernels: 0 fine, 1 a pipeline wait gave up, 2 a load never
 * landed, -1 the device could not be read. */
int slbc_tc_gemm(const void *A, const void *B, float *D, int M, int N, int K, int ldd, void *stream);
int slbc_tc_status(void);
/* Periodic 3x3x3 convolution (implicit GEMM on the tensor cores).  Buffers
 * are channels-last BF16 with a one-voxel periodic halo,
 * buf[n][z + 1][y + 1][x + 1][c] of B x (D+2) x (H+2) x (W+2) x ctot.
 * Reads input channels [in_coff, in_coff + cin) (cin a multiple of 32),
 * weights w[tap][cin/32][cout][32] (tap = 9 dz + 3 dy + dx for the neighbour
 * offset (dx-1, dy-1, dz-1)), adds bias (or none), applies ReLU if relu,
 * multiplies by (mask > 0) if mask is given (same layout as out), and writes
 * the interior of output channels [out_coff, out_coff + cout) (cout a
 * multiple of 16 up to 256).  D, H, W powers of two with D*H*W >= 128. */
int slbc_tc_conv3d(const void *in, int B, int D, int H, int W, int in_ctot, int in_coff, int cin, const void *wgt,
                   const float *bias, int cout, void *out, int out_ctot, int out_coff, int relu, const void *mask,
                   void *stream);
/* The same with FP32 output (out_ctot a multiple of 4), no ReLU, no mask:
 * the network's last layer. */
int slbc_tc_conv3d_f32(const void *in, int B, int D, int H, int W, int in_ctot, int in_coff, int cin,
                       const void *wgt, const float *bias, int cout, float *out, int out_ctot, int out_coff,
                       void *stream);
/* Fill the periodic halo of channels [coff, coff + nch) of such a buffer. */
int slbc_tc_halo(void *buf, int B, int D, int H, int W, int ctot, int coff, int nch, void *stream);
/* Channel-major flat copy of channels [coff, coff + nch) of such a buffer
 * for the weight gradients: dst[c][n * pstride + (z * (H+2) + y) * Wp + x] =
 * src[n][z][y][x - shift][coff + c] (0 outside; zero_halo keeps interior
 * voxels only).  Wp a multiple of 8 >= W + 2, pstride a multiple of 64 >=
 * (D+2) * (H+2) * Wp, shift -1, 0 or 1. */
int slbc_tc_cmajor(const void *src, int B, int D, int H, int W, int ctot, int coff, int nch, int Wp,
                   long long pstride, int shift, int zero_halo, void *dst, void *stream);
/* Weight gradient of slbc_tc_conv3d: dw[tap][cout][cin] (FP32) = sum over
 * voxels u of dY[u - off(tap)][co] * X[u][ci], from channel-major copies:
 * dy0, dy1, dy2 = dY with its periodic halo at shift -1, 0, 1 (shift =
 * dx - 1 for the taps of dx = 0, 1, 2), xt = X with a zero halo at shift 0.  K is split over `splits`
 * blocks into partial (splits * 27 * cout * cin floats) summed in order.
 * cout 32, 64, 128 or a multiple of 128; cin a multiple of 16.  For cout
 * <= 128 the taps' y/z offsets move to the input (27 taps in one block per
 * K range: dx along M, (dy, dz) taps x input channels along N). */
int slbc_tc_wgrad(const void *dy0, const void *dy1, const void *dy2, const void *xt, int B, int D, int H, int W,
                  int Wp, long long pstride, int cin, int cout, float *partial, long long partial_floats, int splits,
                  float *dw, void *stream);
/* slbc_tc_cmajor's copy (zero_halo 0) written as K-tile blocks for
 * slbc_tc_wgrad_tiles: the 64-position rows of flat tile t = position / 64
 * go to dst[t][copy][c][64] (ncopy copies side by side per tile). */
int slbc_tc_cmajor_tiles(const void *src, int B, int D, int H, int W, int ctot, int coff, int nch, int Wp,
                         long long pstride, int shift, int copy, int ncopy, void *dst, void *stream);
/* slbc_tc_wgrad with dY's three copies as K-tile blocks dyt[t][3][cout][64]
 * (slbc_tc_cmajor_tiles, copy = shift + 1, ncopy 3): one tile's operand is
 * one contiguous block of memory.  cout 32, 64 or 128. */
int slbc_tc_wgrad_tiles(const void *dyt, const void *xt, int B, int D, int H, int W, int Wp, long long pstride,
                        int cin, int cout, float *partial, long long partial_floats, int splits, float *dw,
                        void *stream);
/* K splits for slbc_tc_wgrad that fill the current device once (at most
 * k_tiles / 8 and max_splits; k_tiles = B * pstride / 64). */
int slbc_tc_wgrad_splits(int cin, int cout, long long k_tiles, long long max_splits);

/* Network glue of the learned warm start (same buffers; channel slices
 * [coff, coff + C) with C, coff, ctot multiples of 8; D, H, W the fine grid).
 * pool: 2x2x2 average fine -> coarse interior.  pool_bwd: dfine = (dcoarse
 * / 8 + add) * (mask > 0), add and mask optional.  up: nearest upsampling
 * coarse -> fine interior.  up_bwd: dcoarse = sum of the 8 children *
 * (mask > 0).  bias_grad: db[c] += sum of g over interior voxels (C / 8
 * dividing 256).  wfwd: forward weights w[tap][cin/32][cout][32] from
 * master[tap][cout][cin] (FP32).  wdgrad: weights of the input gradient for
 * input channels [ci0, ci0 + nci): w[t][cout/32][nci][32] =
 * master[26 - t][32 ck + j][ci0 + ci].  adam: Adam step t >= 1.  mse: loss
 * += mean w[n] (pred[0..2] - label)^2 (pred FP32 channels 0..2 of a padded
 * buffer, label [n][D][H][W][3], per-sample weights w or null for 1), grad
 * (BF16, gctot channels) = its derivative in channels 0..2, 0 in the
 * others.  encode: channel 0 = 1 on
 * solid nodes; with features = 1, channels 1 and 2 = d / 5 and (d / 5)^2, d
 * the periodic distance of a fluid node to the nearest solid node (capped
 * at 5); with features = 2, d / 12 and (d / 12)^2 (capped at 12) and
 * min(d, 5) / 5 in channel 3; the rest 0.  decode: scale * pred[0..2] on fluid nodes (0 on
 * solid) into u[c * N + e], the layout of lbsetveldev. */
int slbc_nn_pool(const void *in, int in_ctot, int in_coff, void *out, int out_ctot, int out_coff, int B, int D, int H,
                 int W, int C, void *stream);
int slbc_nn_pool_bwd(const void *dcoarse, int dc_ctot, int dc_coff, void *dfine, int df_ctot, int df_coff,
                     const void *add, int a_ctot, int a_coff, const void *mask, int m_ctot, int m_coff, int B, int D,
                     int H, int W, int C, void *stream);
int slbc_nn_up(const void *in, int in_ctot, int in_coff, void *out, int out_ctot, int out_coff, int B, int D, int H,
               int W, int C, void *stream);
int slbc_nn_up_bwd(const void *dfine, int df_ctot, int df_coff, void *dcoarse, int dc_ctot, int dc_coff,
                   const void *mask, int m_ctot, int m_coff, int B, int D, int H, int W, int C, void *stream);
int slbc_nn_bias_grad(const void *g, int ctot, int coff, int B, int D, int H, int W, int C, float *db, void *stream);
int slbc_nn_wfwd(const float *master, int cout, int cin, void *w, void *stream);
int slbc_nn_wdgrad(const float *master, int cout, int cin, int ci0, int nci, void *w, void *stream);
int slbc_nn_adam(float *p, const float *g, float *m, float *v, long long n, float lr, float b1, float b2, float eps,
                 int t, void *stream);
int slbc_nn_mse(const float *pred, int ctot_p, const float *label, int nch, const float *sample_w, int B, int D, int H,
                int W, void *grad, int gctot, double *loss, void *stream);
/* Projection term of the loss, after slbc_nn_mse on the same buffers: per
 * sample s_n = <label_n, pred_n - label_n> / lab_sq[n] (labels
 * [n][D][H][W][lch], channels [0, nch) taken, lab_sq[n] = <label_n,
 * label_n> over them, device doubles), loss += (weight / B) sum_n s_n^2 and
 * its derivative added to grad; dot: B device doubles of scratch. */
int slbc_nn_proj(const float *pred, int ctot_p, const float *label, int lch, int nch, const double *lab_sq, int B,
                 int D, int H, int W, float weight, void *grad, int gctot, double *dot, double *loss, void *stream);
/* Gradient-norm clipping against a running norm, without a host round
 * trip: slbc_nn_sqsum adds the sum of squares of one gradient tensor to
 * state[0] (call it for every tensor), slbc_nn_clip turns the total into
 * state[2] = min(1, factor * running / norm) and updates the running norm
 * state[1] (0 before the first call) by decay, slbc_nn_scale multiplies a
 * tensor by state[2].  A non-finite norm zeroes the gradients.  state is
 * three device doubles, zero at the start. */
int slbc_nn_sqsum(const float *g, long long n, double *state, void *stream);
int slbc_nn_clip(double *state, float factor, float decay, void *stream);
int slbc_nn_scale(float *g, long long n, const double *state, void *stream);
int slbc_nn_encode(const unsigned char *solid, int B, int D, int H, int W, void *out, int ctot, int features,
                   void *stream);
int slbc_nn_decode(const float *pred, int ctot_p, const unsigned char *solid, int D, int H, int W, float scale,
                   float shift_x, float *u, float drho_scale, float *drho, void *stream);
/* Uniform plane flux of a decoded state (u: 3 x D*H*W FP32, x = the slowest
 * index; drho: D*H*W or null; solid: D*H*W bytes): the x flux q[i] through
 * every x plane becomes the harmonic mean qh of the planes' fluxes (u of
 * plane i times qh / q[i]), and the fluid nodes of plane i get the density
 * deviation 3 p[i], p the pressure that carries the body force `force`
 * through slabs in series (dp/dx = force (1 - qh / q[i]), zero mean).  A
 * converged periodic flow has the same mass flux through every plane.  The
 * whole state (velocity, density deviation, p) is then multiplied by gain
 * (1: none; a calibrated flux gain of the network otherwise).  work: 3 D + 1
 * device doubles (q, scale, p, then the relative spread (max - min) / mean
 * of the fluxes before, -1 when some flux is <= 0 and only the gain was
 * applied). */
int slbc_nn_plane_flux(float *u, float *drho, const unsigned char *solid, int D, int H, int W, float force,
                       float gain, double *work, void *stream);
/* Cross fluxes of the same state made uniform: the flux of u_y through
 * every y plane (u_z through every z plane) set to its mean by adding
 * delta(plane) |u| to the component (|u| of the state before: zero in
 * solids and at walls).  u: 3 x D*H*W, z the fastest index; work: 3 (H + W)
 * doubles. */
int slbc_nn_cross_flux(float *u, int D, int H, int W, double *work, void *stream);

/* Mean-flow sums of slbc_vsum over buffers the caller owns, allocating no
 * device memory.  For callers that cannot call cudaMalloc where they need
 * the result: an application that hands out all device memory from its own
 * pool, or a time-stepping loop that must not allocate (cudaMalloc can
 * synchronise the whole device and can fail under memory pressure in the
 * middle of a run).  No counterpart in the reference.
 *   pop, npad, precision, layout: populations as described at the top of
 *     this header (device memory);
 *   flags: per-node flag words (device, 16 bit: bit 15 = solid node, bit q =
 *     the link between x and x - c_q joins a fluid and a solid node);
 *   bx, by, bz: uniform body force, used when bf is NULL; otherwise bf holds
 *     3*npad per-node values of the population type (device);
 *   psi: per-node weights (device) or NULL; out: 5 doubles (device), written
 *     as out[0..4] of slbc_vsum.
 * Its only intermediate data, one partial sum per reduction block, lives in
 * a static device array of SLBC_VSUM_NOALLOC_MAX_BLOCKS * 5 doubles that
 * every GPU loading the library keeps until the process exits; nblocks (the
 * number of reduction blocks) must lie in 1..SLBC_VSUM_NOALLOC_MAX_BLOCKS
 * and larger values are rejected with an error.  The first call on each
 * device (and the first after a device reset, or with another CUDA context
 * current on that device) looks up the array's device address; make that
 * first call before any stream capture.  Every call shares the array, so calls that overlap on
 * the GPU (on different streams) race.  Work is queued on `stream` and not
 * synchronised. */
#define SLBC_VSUM_NOALLOC_MAX_BLOCKS 1216
int slbc_vsum_noalloc(const void *pop, long long npad, int precision, int layout,
                      const unsigned short *flags, int esi, int esj, int esk,
                      double rho0, double fac, double bx, double by, double bz,
                      const void *bf, const double *psi, int nblocks, double *out,
                      void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SLB_DEVICE_H_INC */
