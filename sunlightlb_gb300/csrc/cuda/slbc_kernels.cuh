// Population kernels of the GB300 SunlightLB device layer, templated on the
// population type T.  Included once per precision (slbc_f64.cu compiles it
// with FMA contraction off so FP64 results equal the reference bit for bit;
// slbc_f32.cu compiles it with FMA on).
//
// Update scheme.  The reference step (src/lbkernel.c:49-51) is link
// bounce-back (swap a_q(solid) <-> a_opp(q)(fluid) on every solid-fluid link,
// plus a wall term for moving objects), periodic streaming, then collision.
// The swaps of different links touch disjoint slots, so the step is exactly
// this pull rule at every node x and population q:
//   link x <- x - c_q joins fluid and solid:  a'_q(x) = a_opp(q)(x) +- wall
//   otherwise:                                a'_q(x) = a_q(x - c_q)
// followed by the local collision.  It is applied in place with the AA
// pattern: an odd step reads C0 (post-collision values kept at the node in
// reversed slots), pulls from the neighbours, collides and pushes to the
// neighbours (C1); an even step reads C1 locally, collides and writes back
// reversed (C0).  Bounce-back values are stored raw and the wall term is
// added when they are read, so C0 and C1 are both exact permutations of the
// reference's post-collision array.  Each thread reads exactly the slots it
// writes, so the in-place update has no races.
#pragma once

#include "slbc_internal.cuh"

namespace slbc {

// Periodic neighbourhood of node (i,j,k).
struct Nbr {
  int I[3], J[3], K[3];
  int esk;
  __device__ __forceinline__ int at(int dx, int dy, int dz) const {
    return (I[dx + 1] + J[dy + 1]) * esk + K[dz + 1];
  }
};

__device__ __forceinline__ Nbr make_nbr(int i, int j, int k, int esi, int esj, int esk) {
  Nbr n;
  const int im = i == 0 ? esi - 1 : i - 1, ip = i == esi - 1 ? 0 : i + 1;
  const int jm = j == 0 ? esj - 1 : j - 1, jp = j == esj - 1 ? 0 : j + 1;
  const int km = k == 0 ? esk - 1 : k - 1, kp = k == esk - 1 ? 0 : k + 1;
  n.I[0] = im * esj; n.I[1] = i * esj; n.I[2] = ip * esj;
  n.J[0] = jm; n.J[1] = j; n.J[2] = jp;
  n.K[0] = km; n.K[1] = k; n.K[2] = kp;
  n.esk = esk;
  return n;
}

// Plane-marching tiles: a block of kTileK (k) x kTileJ (j) threads walks
// along i and keeps per-node values of three consecutive planes, with a
// one-node halo, in shared memory (kPlane entries per plane).
constexpr int kTileK = 32, kTileJ = 8;
constexpr int kHaloK = kTileK + 2, kHaloJ = kTileJ + 2;
constexpr int kPlane = kHaloK * kHaloJ;
constexpr int kTileThreads = kTileK * kTileJ;
constexpr int kPlaneLoads = (kPlane + kTileThreads - 1) / kTileThreads;

__device__ __forceinline__ int wrap_index(int v, int n) {
  v %= n;
  return v < 0 ? v + n : v;
}

__device__ __forceinline__ void decode(int x, int esj, int esk, int &i, int &j, int &k) {
  k = x % esk;
  const int r = x / esk;
  j = r % esj;
  i = r / esj;
}

// Moving-wall momentum term of link q for a solid node whose wall velocity
// (times rho0/12) is u: reference src/lbkernel.c:360-446, same evaluation.
template <typename R>
__device__ __forceinline__ R link_term(int q, R ux, R uy, R uz) {
  switch (q) {
    case 1: return R(8.0) * ux;
    case 2: return R(-8.0) * ux;
    case 3: return R(8.0) * uy;
    case 4: return R(-8.0) * uy;
    case 5: return R(8.0) * uz;
    case 6: return R(-8.0) * uz;
    case 7: return (ux + uy) + uz;
    case 8: return (-ux + uy) + uz;
    case 9: return (ux - uy) + uz;
    case 10: return (-ux - uy) + uz;
    case 11: return (ux + uy) - uz;
    case 12: return (-ux + uy) - uz;
    case 13: return (ux - uy) - uz;
    default: return (-ux - uy) - uz;
  }
}

// Correctly rounded a / b for a constant b with rb = RN(1/b), by Markstein's
// theorem (binary64, round to nearest, no underflow or overflow): q = RN(a rb)
// is within one ulp of a / b, the remainder r = a - b q is exact (one fused
// multiply-add), and RN(q + r rb) = RN(a / b).  Three FP64 operations instead
// of a full division; a = +-0 returns a (keeps the sign of zero).
__device__ __forceinline__ double div_const(double a, double b, double rb) {
  const double q = __dmul_rn(a, rb);
  const double r = __fma_rn(-q, b, a);
  const double q1 = __fma_rn(r, rb, q);
  return a == 0.0 ? a : q1;
}

// Rebuild the 15 populations from density deviation, momentum and stress:
// reference src/lbkernel.c:838-865, same evaluation order.
template <typename T, bool EXACT>
__device__ __forceinline__ void rebuild(T (&t)[15], T drho, T rux, T ruy, T ruz, T sxx,
                                        T syy, T szz, T sxy, T sxz, T syz) {
  const T dbybc2 = T(1.0 / 24.0), dd2bybc4 = T(1.0 / 8.0);
  const T fdd2bybc4 = T(4.0) * dd2bybc4, edbybc2 = T(8.0) * dbybc2;
  T rhobyb, trsby3;
  if (EXACT) {  // the reference's divisions, correctly rounded
    rhobyb = div_const(drho, 72.0, 1.0 / 72.0);
    trsby3 = div_const(sxx + syy + szz, 3.0, 1.0 / 3.0);
  } else {
    rhobyb = drho * T(1.0 / 72.0);
    trsby3 = (sxx + syy + szz) * T(1.0 / 3.0);
  }
  const T erhobyb = T(8.0) * rhobyb;
  T ru, st;
  t[0] = T(2.0) * erhobyb - T(2.0) * fdd2bybc4 * trsby3;
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

// Moments of one node after relaxation: density deviation, momentum (with
// the body force on fluid nodes) and the relaxed stress.
template <typename T>
struct Relaxed {
  T drho, rux, ruy, ruz, sxx, syy, szz, sxy, sxz, syz;
};

// The moment half of the collision: reference src/lbkernel.c:805-836, same
// evaluation order.
template <typename T>
__device__ __forceinline__ Relaxed<T> relax(const T (&t)[15], T omega, T comega, T rho0, int stokes, bool fluid,
                                            T bx, T by, T bz) {
  const T twoby3 = T(2.0 / 3.0);
  const T p12 = t[1] + t[2], p34 = t[3] + t[4], p56 = t[5] + t[6];
  const T lo_sum = t[7] + t[8] + t[9] + t[10], hi_sum = t[11] + t[12] + t[13] + t[14];
  const T lo_x = t[7] - t[8] + t[9] - t[10], hi_x = t[11] - t[12] + t[13] - t[14];
  const T lo_y = t[7] + t[8] - t[9] - t[10], hi_y = t[11] + t[12] - t[13] - t[14];
  const T lo_xy = t[7] - t[8] - t[9] + t[10], hi_xy = t[11] - t[12] - t[13] + t[14];
  const T p06 = t[0] + p12 + p34 + p56;
  Relaxed<T> r;
  r.drho = p06 + (lo_sum + hi_sum);
  r.rux = t[1] - t[2] + lo_x + hi_x;
  r.ruy = t[3] - t[4] + lo_y + hi_y;
  r.ruz = t[5] - t[6] + lo_sum - hi_sum;
  if (fluid) { r.rux += bx; r.ruy += by; r.ruz += bz; }
  const T sdiag = twoby3 * r.drho - p06;
  T sxx = sdiag + p12, syy = sdiag + p34, szz = sdiag + p56;
  T sxy = lo_xy + hi_xy, sxz = lo_x - hi_x, syz = lo_y - hi_y;
  if (stokes) {
    sxx = comega * sxx; sxy = comega * sxy; sxz = comega * sxz;
    syy = comega * syy; syz = comega * syz; szz = comega * szz;
  } else {
    const T obyr = omega / (rho0 + r.drho);
    sxx = comega * sxx + obyr * r.rux * r.rux;
    sxy = comega * sxy + obyr * r.rux * r.ruy;
    sxz = comega * sxz + obyr * r.rux * r.ruz;
    syy = comega * syy + obyr * r.ruy * r.ruy;
    syz = comega * syz + obyr * r.ruy * r.ruz;
    szz = comega * szz + obyr * r.ruz * r.ruz;
  }
  r.sxx = sxx; r.syy = syy; r.szz = szz; r.sxy = sxy; r.sxz = sxz; r.syz = syz;
  return r;
}

// Collision of one node: reference src/lbkernel.c:805-865.
template <typename T, bool EXACT>
__device__ __forceinline__ void collide(T (&t)[15], T omega, T comega, T rho0, int stokes,
                                        bool fluid, T bx, T by, T bz) {
  const Relaxed<T> r = relax<T>(t, omega, comega, rho0, stokes, fluid, bx, by, bz);
  rebuild<T, EXACT>(t, r.drho, r.rux, r.ruy, r.ruz, r.sxx, r.syy, r.szz, r.sxy, r.sxz, r.syz);
}

// Add the moving-wall term to every population that arrived over a
// bounce-back link (bits of fl).  Fluid node: the wall velocity is that of
// the solid upstream node x - c_q and the term is added; solid node: its own
// wall velocity, the term of the opposite link is subtracted.
template <typename T>
__device__ __forceinline__ void apply_wall(T (&t)[15], uint16_t fl, bool solid, const Nbr &nb,
                                           int x, const T *uw, long long S) {
#pragma unroll
  for (int q = 1; q < 15; q++) {
    if (!((fl >> q) & 1)) continue;
    if (solid) {
      t[q] = t[q] - link_term<T>(OPP(q), uw[x], uw[S + x], uw[2 * S + x]);
    } else {
      const int y = nb.at(-CX(q), -CY(q), -CZ(q));
      t[q] = t[q] + link_term<T>(q, uw[y], uw[S + y], uw[2 * S + y]);
    }
  }
}

// Element index of population `slot` of node `node`.  I32: the whole
// population array (15 x S elements) is indexable in 32 unsigned bits, so
// the index is formed and scaled in 32-bit arithmetic (one multiply-add and
// one widening address multiply per access instead of 64-bit products).
template <bool I32>
__device__ __forceinline__ auto pop_index(int slot, long long S, int node) {
  if constexpr (I32) {
    return (unsigned)slot * (unsigned)S + (unsigned)node;
  } else {
    return slot * S + node;
  }
}

// Populations of node x entering a fused update.  ODD = false (C1 -> C0):
// the node's own slots; ODD = true (C0 -> C1): pulled from the upstream
// neighbours x - c_q, or from the node's own slot q across a bounce-back
// link (bit q of fl).
template <typename T, bool ODD, bool I32 = false>
__device__ __forceinline__ void load_pops(const T *__restrict__ P, long long S, const Nbr &nb, int x,
                                          uint16_t fl, T (&t)[15]) {
  if (!ODD) {
#pragma unroll
    for (int q = 0; q < 15; q++) t[q] = P[pop_index<I32>(q, S, x)];
  } else {
    t[0] = P[x];
#pragma unroll
    for (int q = 1; q < 15; q++) {
      const bool bnd = (fl >> q) & 1;
      const int src = bnd ? x : nb.at(-CX(q), -CY(q), -CZ(q));
      const int slot = bnd ? q : OPP(q);
      t[q] = P[pop_index<I32>(slot, S, src)];
    }
  }
}

// Element offsets of the pull-and-push update for nodes away from the
// lattice's faces (no periodic wrap): population q arrives from element
// x + pull_nbr[q] (slot opp(q) of x - c_q) or, over a bounce-back link, from
// x + pull_self[q] (slot q of x); it leaves to x + push_nbr[q] (slot q of
// x + c_q) or x + push_self[q] (slot opp(q) of x).  Unsigned 32-bit: only
// used when 15 x npad elements fit (I32).
struct OddOffsets {
  unsigned pull_self[15], pull_nbr[15], push_self[15], push_nbr[15];
};

// Wall terms and collision of node x.
template <typename T, bool EXACT, bool MOVING, bool BFU>
__device__ __forceinline__ void relax_node(const StepArgs<T> &a, const Nbr &nb, int x, uint16_t fl, T (&t)[15]) {
  const long long S = a.p.npad;
  const bool solid = (fl & FLAG_SOLID) != 0;
  if (MOVING && (fl & FLAG_LINKS)) apply_wall<T>(t, fl, solid, nb, x, a.uw, S);
  if (!(a.skip_solid && solid)) {
    T bx = a.bfx, by = a.bfy, bz = a.bfz;
    if (!BFU) { bx = a.bf[x]; by = a.bf[S + x]; bz = a.bf[2 * S + x]; }
    collide<T, EXACT>(t, a.omega, a.comega, a.rho0, a.stokes, !solid, bx, by, bz);
  }
}

// The pull and push of a node away from the faces through OddOffsets: one
// select between two uniform offsets per access, no neighbour indexing.
template <typename T>
__device__ __forceinline__ void load_pops_inner(const T *__restrict__ P, const OddOffsets &o, int x, uint16_t fl,
                                                T (&t)[15]) {
  t[0] = P[x];
#pragma unroll
  for (int q = 1; q < 15; q++) t[q] = P[(unsigned)x + (((fl >> q) & 1) ? o.pull_self[q] : o.pull_nbr[q])];
}

template <typename T>
__device__ __forceinline__ void store_pops_inner(T *__restrict__ P, const OddOffsets &o, int x, uint16_t fl,
                                                 const T (&t)[15]) {
  P[x] = t[0];
#pragma unroll
  for (int q = 1; q < 15; q++) P[(unsigned)x + (((fl >> OPP(q)) & 1) ? o.push_self[q] : o.push_nbr[q])] = t[q];
}

// Wall terms, collision and the write-back of node x (the slots load_pops
// read: locally reversed for the even step, pushed to the neighbours, or to
// the node's own opposite slot across a bounce-back link, for the odd one).
template <typename T, bool ODD, bool EXACT, bool MOVING, bool BFU, bool I32 = false>
__device__ __forceinline__ void finish_node(const StepArgs<T> &a, const Nbr &nb, int x, uint16_t fl,
                                            T (&t)[15]) {
  T *__restrict__ P = a.p.pop;
  const long long S = a.p.npad;
  relax_node<T, EXACT, MOVING, BFU>(a, nb, x, fl, t);
  if (!ODD) {
#pragma unroll
    for (int q = 0; q < 15; q++) P[pop_index<I32>(OPP(q), S, x)] = t[q];
  } else {
    P[x] = t[0];
#pragma unroll
    for (int q = 1; q < 15; q++) {
      const bool bnd = (fl >> OPP(q)) & 1;
      const int dst = bnd ? x : nb.at(CX(q), CY(q), CZ(q));
      const int slot = bnd ? OPP(q) : q;
      P[pop_index<I32>(slot, S, dst)] = t[q];
    }
  }
}

// Fused update (bounce-back + streaming + collision) of node (i, j, k).
// ODD = false: C1 -> C0 (local), ODD = true: C0 -> C1 (pull and push).
// MOVING compiles the wall terms in, BFU selects a uniform body force (a
// kernel constant) over per-node arrays.
template <typename T, bool ODD, bool EXACT, bool MOVING, bool BFU>
__device__ __forceinline__ void step_node(const StepArgs<T> &a, int i, int j, int k) {
  const Nbr nb = make_nbr(i, j, k, a.p.esi, a.p.esj, a.p.esk);
  const int x = nb.at(0, 0, 0);
  const uint16_t fl = __ldg(a.p.flags + x);
  T t[15];
  load_pops<T, ODD>(a.p.pop, a.p.npad, nb, x, fl, t);
  finish_node<T, ODD, EXACT, MOVING, BFU>(a, nb, x, fl, t);
}

// One fused update step of every node.  A thread updates NPT consecutive
// rows along j at one (i, k), software-pipelined: the flag words of all its
// rows are loaded first, and the populations of row r + 1 are loaded before
// row r is collided and written back.  This is safe in place because, in
// the AA pattern, every node reads exactly the slots it writes, so no two
// nodes' slot sets meet; it keeps about two rows of loads in flight per
// thread and removes the flag-then-populations round trip of the odd step
// from every row but the first.
// Grid: (ceil(esk/blockDim.x), ceil(esj/NPT), esi).  I32: 15 x npad
// elements fit 32 unsigned bits (pop_index); then, in the pull-and-push
// update, a row whose nodes in the whole warp lie away from the lattice's
// faces takes the OddOffsets addressing (a warp-uniform choice, so no warp
// runs both forms).
template <typename T, bool ODD, bool EXACT, bool MOVING, bool BFU, int NPT, bool I32 = false>
__global__ void __launch_bounds__(256) k_step(StepArgs<T> a, OddOffsets off) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.z;
  if (k >= a.p.esk) return;
  const int j0 = blockIdx.y * NPT;
  const int nrow = min(NPT, a.p.esj - j0);
  T *P = a.p.pop;
  const long long S = a.p.npad;
  uint16_t fl[NPT];
  bool inner[NPT];
  const unsigned warp_mask = __activemask();
  const bool ik_inner = i > 0 && i < a.p.esi - 1 && k > 0 && k < a.p.esk - 1;
#pragma unroll
  for (int r = 0; r < NPT; r++) {
    if (r < nrow) fl[r] = __ldg(a.p.flags + ((i * a.p.esj + j0 + r) * a.p.esk + k));
    const int j = j0 + r;
    inner[r] = ODD && I32 && __all_sync(warp_mask, ik_inner && j > 0 && j < a.p.esj - 1);
  }
  Nbr nb = make_nbr(i, j0, k, a.p.esi, a.p.esj, a.p.esk);
  T cur[15];
  if (inner[0]) load_pops_inner<T>(P, off, nb.at(0, 0, 0), fl[0], cur);
  else load_pops<T, ODD, I32>(P, S, nb, nb.at(0, 0, 0), fl[0], cur);
#pragma unroll
  for (int r = 0; r < NPT; r++) {
    if (r >= nrow) break;
    T nxt[15];
    Nbr nbn = nb;
    const bool more = r + 1 < nrow;
    if (more) {
      nbn = make_nbr(i, j0 + r + 1, k, a.p.esi, a.p.esj, a.p.esk);
      const int rn = r + 1 < NPT ? r + 1 : r;
      if (inner[rn]) load_pops_inner<T>(P, off, nbn.at(0, 0, 0), fl[rn], nxt);
      else load_pops<T, ODD, I32>(P, S, nbn, nbn.at(0, 0, 0), fl[rn], nxt);
    }
    if (inner[r]) {
      relax_node<T, EXACT, MOVING, BFU>(a, nb, nb.at(0, 0, 0), fl[r], cur);
      store_pops_inner<T>(P, off, nb.at(0, 0, 0), fl[r], cur);
    } else {
      finish_node<T, ODD, EXACT, MOVING, BFU, I32>(a, nb, nb.at(0, 0, 0), fl[r], cur);
    }
    if (more) {
#pragma unroll
      for (int q = 0; q < 15; q++) cur[q] = nxt[q];
      nb = nbn;
    }
  }
}

// ---- batches of independent lattices ----------------------------------------
// One persistent launch advances many lattices ("domains") by nsteps fused
// steps each (the parity of each domain's first step follows its layout).  Block b owns the domains
// work[work_off[b] .. work_off[b+1]) outright and runs all their steps, one
// domain after another, with a block barrier between steps: no other block
// touches a domain, so no block ever waits for another.
constexpr int kBatchThreads = 512;

template <typename T, bool ODD, bool EXACT, bool MOVING, bool BFU>
__device__ __forceinline__ void batch_sweep(const StepArgs<T> &a) {
  const int esj = a.p.esj, esk = a.p.esk;
  const int n = a.p.esi * esj * esk;
  for (int e = threadIdx.x; e < n; e += blockDim.x) {
    const int r = e / esk;
    step_node<T, ODD, EXACT, MOVING, BFU>(a, r / esj, r % esj, e - r * esk);
  }
}

// A domain of a batch: its step arguments and the parity of its first step
// (1: the domain starts in C0, 0: in C1).
template <typename T>
struct BatchDom {
  StepArgs<T> a;
  int odd0;
};

template <typename T, bool EXACT, bool MOVING, bool BFU>
__global__ void __launch_bounds__(kBatchThreads, 2) k_batch(const BatchDom<T> *doms, const int *work_off,
                                                            const int *work, int nsteps) {
  for (int w = work_off[blockIdx.x]; w < work_off[blockIdx.x + 1]; w++) {
    const StepArgs<T> a = doms[work[w]].a;
    const int odd0 = doms[work[w]].odd0;
    for (int s = 0; s < nsteps; s++) {
      if (((s + odd0) & 1) == 1) batch_sweep<T, true, EXACT, MOVING, BFU>(a);
      else batch_sweep<T, false, EXACT, MOVING, BFU>(a);
      __syncthreads();
    }
  }
}

// Packed cell index of a batch: every domain is cut into tiles of
// kBatchTile consecutive cells, tile t = (domain, first cell).  One launch
// updates the tiles of one (moving walls, uniform force, parity) group by
// one step: the host groups each class's tiles by the parity of their
// domain's first step, so one launch has one parity (ODD) and carries the
// code of that parity only (64 registers, four blocks per SM).
constexpr int kBatchTile = 256;

template <typename T, bool ODD, bool EXACT, bool MOVING, bool BFU>
__global__ void __launch_bounds__(kBatchTile, 4) k_batch_tiles(const BatchDom<T> *doms, const int2 *tiles) {
  __shared__ BatchDom<T> dom;
  const int2 tile = tiles[blockIdx.x];
  if (threadIdx.x == 0) dom = doms[tile.x];
  __syncthreads();
  const StepArgs<T> &a = dom.a;
  const int esj = a.p.esj, esk = a.p.esk;
  const int e = tile.y + threadIdx.x;
  if (e >= a.p.esi * esj * esk) return;
  const int r = e / esk;
  step_node<T, ODD, EXACT, MOVING, BFU>(a, r / esj, r % esj, e - r * esk);
}

// Explicitly rounded add / multiply: never contracted into FMA, so the
// reduction kernels give the same bits whatever -fmad a translation unit uses.
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }

// Compensated accumulator: FP64 for FP64 data; for FP32 data a float-float
// pair (Knuth's TwoSum keeps the rounding error of every addition), about 48
// significant bits computed on the FP32 pipe, turned into FP64 once.
template <typename T> struct Acc;
template <> struct Acc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double x) { s = radd(s, x); }
  __device__ __forceinline__ double value() const { return s; }
};
template <> struct Acc<float> {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float sum = __fadd_rn(hi, x);
    const float bp = __fsub_rn(sum, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(sum, bp)), __fsub_rn(x, bp));
    hi = sum;
    lo = __fadd_rn(lo, err);
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// Post-collision population q of node x in a given layout (see slb_device.h).
template <typename T>
__device__ __forceinline__ T post_value(const T *P, long long S, int layout, int q, int x,
                                        uint16_t fl, const Nbr &nb) {
  if (layout == SLBC_LAYOUT_N) return P[q * S + x];
  if (layout == SLBC_LAYOUT_C0 || q == 0) return P[OPP(q) * S + x];
  if ((fl >> OPP(q)) & 1) return P[OPP(q) * S + x];
  return P[q * S + nb.at(CX(q), CY(q), CZ(q))];
}

// Node forces of one bblforce (reference src/lbkernel.c:179-321 stationary,
// 464-618 moving) over the solid boundary nodes, accumulated in link order
// into f (x, y, z blocks of nbnd), in FP64.  Reads the post-collision
// state; the links of a solid node s are those whose far end is fluid.
template <typename T>
__global__ void k_force(PopArgs<T> p, int layout, int moving, const T *uw, ForceArgs f) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= f.nbnd) return;
  const int s = f.bnd_node[e];
  int i, j, k;
  decode(s, p.esj, p.esk, i, j, k);
  const Nbr nb = make_nbr(i, j, k, p.esi, p.esj, p.esk);
  const uint16_t fl = p.flags[s];
  const T *P = p.pop;
  const long long S = p.npad;
  if (sizeof(T) == 8) {
    // FP64 populations: the reference's arithmetic, in link order
    double fx = f.f[e], fy = f.f[f.nbnd + e], fz = f.f[2 * f.nbnd + e];
    double ux = 0.0, uy = 0.0, uz = 0.0;
    if (moving) { ux = (double)uw[s]; uy = (double)uw[S + s]; uz = (double)uw[2 * S + s]; }
#pragma unroll
    for (int q = 1; q < 15; q++) {
      if (!((fl >> OPP(q)) & 1)) continue;
      const int n = nb.at(CX(q), CY(q), CZ(q));
      double av, bv;
      if (layout == SLBC_LAYOUT_N) { av = (double)P[q * S + s]; bv = (double)P[OPP(q) * S + n]; }
      else { av = (double)P[OPP(q) * S + s]; bv = (double)P[q * S + n]; }
      const double dp = moving ? 2.0 * (av - bv - link_term<double>(q, ux, uy, uz)) : 2.0 * (av - bv);
      if (CX(q) > 0) fx += dp; else if (CX(q) < 0) fx -= dp;
      if (CY(q) > 0) fy += dp; else if (CY(q) < 0) fy -= dp;
      if (CZ(q) > 0) fz += dp; else if (CZ(q) < 0) fz -= dp;
    }
    f.f[e] = fx; f.f[f.nbnd + e] = fy; f.f[2 * f.nbnd + e] = fz;
  } else {
    // FP32 populations: link terms in FP32 (a - b and the wall term are
    // exact-ish at these magnitudes), sums compensated, stored in FP64
    Acc<float> ax, ay, az;
    float ux = 0.f, uy = 0.f, uz = 0.f;
    if (moving) { ux = (float)uw[s]; uy = (float)uw[S + s]; uz = (float)uw[2 * S + s]; }
#pragma unroll
    for (int q = 1; q < 15; q++) {
      if (!((fl >> OPP(q)) & 1)) continue;
      const int n = nb.at(CX(q), CY(q), CZ(q));
      float av, bv;
      if (layout == SLBC_LAYOUT_N) { av = (float)P[q * S + s]; bv = (float)P[OPP(q) * S + n]; }
      else { av = (float)P[OPP(q) * S + s]; bv = (float)P[q * S + n]; }
      float dp = __fsub_rn(av, bv);
      if (moving) dp = __fsub_rn(dp, link_term<float>(q, ux, uy, uz));
      dp = __fmul_rn(2.f, dp);
      if (CX(q) != 0) ax.add(CX(q) > 0 ? dp : -dp);
      if (CY(q) != 0) ay.add(CY(q) > 0 ? dp : -dp);
      if (CZ(q) != 0) az.add(CZ(q) > 0 ? dp : -dp);
    }
    f.f[e] += ax.value(); f.f[f.nbnd + e] += ay.value(); f.f[2 * f.nbnd + e] += az.value();
  }
}

// Deterministic block reduction of NV doubles; thread 0 gets the totals.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV]) {
  __shared__ double sh[32][NV];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < NV; c++)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[c] += __shfl_down_sync(0xffffffffu, v[c], o);
  if (lane == 0)
#pragma unroll
    for (int c = 0; c < NV; c++) sh[warp][c] = v[c];
  __syncthreads();
  if (warp == 0) {
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int c = 0; c < NV; c++) v[c] = lane < nw ? sh[lane][c] : 0.0;
#pragma unroll
    for (int c = 0; c < NV; c++)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[c] += __shfl_down_sync(0xffffffffu, v[c], o);
  }
}

// Velocity sums of accvmean (reference src/lbmeasure.c:78-97) per block:
// block b reduces the contiguous node range [b*chunk, (b+1)*chunk), its
// threads striding through it; the fixed partition makes the sums
// deterministic.  The per-node velocity is formed in the population type
// (FP64: one reciprocal of rho instead of three divisions) and accumulated
// in FP64.
template <typename T>
__global__ void __launch_bounds__(kReduceThreads)
k_vsum(PopArgs<T> p, int layout, double rho0, double fac, int bf_uniform, double b0, double b1,
       double b2, const T *bf, const double *psi, double *partials) {
  Acc<T> ax, ay, az;
  double wsum = 0.0;
  int count = 0;
  const long long n = (long long)p.esi * p.esj * p.esk;
  const long long chunk = (n + gridDim.x - 1) / gridDim.x;
  const long long lo = (long long)blockIdx.x * chunk;
  const long long hi = lo + chunk < n ? lo + chunk : n;
  const T *P = p.pop;
  const long long S = p.npad;
  const T r0 = (T)rho0, tf = (T)fac;
  for (long long e = lo + threadIdx.x; e < hi; e += blockDim.x) {
    const int x = (int)e;
    const uint16_t fl = p.flags[x];
    if (fl & FLAG_SOLID) continue;
    int i, j, k;
    decode(x, p.esj, p.esk, i, j, k);
    const Nbr nb = make_nbr(i, j, k, p.esi, p.esj, p.esk);
    T t[15];
#pragma unroll
    for (int q = 0; q < 15; q++) t[q] = post_value<T>(P, S, layout, q, x, fl, nb);
    T bx = (T)b0, by = (T)b1, bz = (T)b2;
    if (!bf_uniform) { bx = bf[x]; by = bf[S + x]; bz = bf[2 * S + x]; }
    T rho = r0, nx, ny, nz;
#pragma unroll
    for (int q = 0; q < 15; q++) rho = radd(rho, t[q]);
    nx = radd(radd(radd(radd(radd(radd(radd(radd(radd(radd(t[1], -t[2]), t[7]), -t[8]), t[9]), -t[10]), t[11]), -t[12]), t[13]), -t[14]), rmul(tf, bx));
    ny = radd(radd(radd(radd(radd(radd(radd(radd(radd(radd(t[3], -t[4]), t[7]), t[8]), -t[9]), -t[10]), t[11]), t[12]), -t[13]), -t[14]), rmul(tf, by));
    nz = radd(radd(radd(radd(radd(radd(radd(radd(radd(radd(t[5], -t[6]), t[7]), t[8]), t[9]), t[10]), -t[11]), -t[12]), -t[13]), -t[14]), rmul(tf, bz));
    const T rinv = T(1) / rho;
    T ux = rmul(nx, rinv), uy = rmul(ny, rinv), uz = rmul(nz, rinv);
    if (psi) {
      const double w = rmul(psi[x], psi[x]);
      ax.add((T)rmul(w, (double)ux)); ay.add((T)rmul(w, (double)uy)); az.add((T)rmul(w, (double)uz));
      wsum = radd(wsum, w);
    } else {
      ax.add(ux); ay.add(uy); az.add(uz);
    }
    count++;
  }
  double v[5] = {ax.value(), ay.value(), az.value(), psi ? wsum : (double)count, (double)count};
  block_sum<5>(v);
  if (threadIdx.x == 0)
#pragma unroll
    for (int c = 0; c < 5; c++) partials[5 * blockIdx.x + c] = v[c];
}

// Final sum of nb partial records of NV doubles in one block: each thread
// adds a fixed strided subset in order, then a fixed-shape tree.
template <int NV>
__global__ void __launch_bounds__(256) k_final_sum_tree(const double *partials, int nb, double *out) {
  double v[NV];
#pragma unroll
  for (int c = 0; c < NV; c++) v[c] = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
#pragma unroll
    for (int c = 0; c < NV; c++) v[c] += partials[NV * b + c];
  block_sum<NV>(v);
  if (threadIdx.x == 0)
#pragma unroll
    for (int c = 0; c < NV; c++) out[c] = v[c];
}

// Host AoS staging (FP64, a[15*x + q]) -> layout N.
template <typename T>
__global__ void k_put(PopArgs<T> p, const double *stage, long long x0, long long n) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const long long x = x0 + e;
#pragma unroll
  for (int q = 0; q < 15; q++) p.pop[q * p.npad + x] = (T)stage[15 * e + q];
}

// Any layout -> host AoS staging of the reference's array.
template <typename T>
__global__ void k_get(PopArgs<T> p, int layout, double *stage, long long x0, long long n) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int x = (int)(x0 + e);
  int i, j, k;
  decode(x, p.esj, p.esk, i, j, k);
  const Nbr nb = make_nbr(i, j, k, p.esi, p.esj, p.esk);
  const uint16_t fl = p.flags[x];
#pragma unroll
  for (int q = 0; q < 15; q++) stage[15 * e + q] = (double)post_value<T>(p.pop, p.npad, layout, q, x, fl, nb);
}

// The same two conversions straight from / to a page-locked host array
// the device can address (zero-copy over the host link): a block moves
// kHostTile nodes through shared memory, so that its reads (put) or writes
// (get) of the host array are whole contiguous runs of 15 * kHostTile
// doubles rather than 15 strided 8-byte accesses per node.
constexpr int kHostTile = 128;

template <typename T>
__global__ void __launch_bounds__(kHostTile) k_put_host(PopArgs<T> p, const double *host, long long n) {
  __shared__ double buf[15 * kHostTile];
  for (long long x0 = (long long)blockIdx.x * kHostTile; x0 < n; x0 += (long long)gridDim.x * kHostTile) {
    const int cnt = (int)(n - x0 < kHostTile ? n - x0 : kHostTile);
    for (int e = threadIdx.x; e < 15 * cnt; e += kHostTile) buf[e] = host[15 * x0 + e];
    __syncthreads();
    if (threadIdx.x < cnt) {
      const long long x = x0 + threadIdx.x;
#pragma unroll
      for (int q = 0; q < 15; q++) p.pop[q * p.npad + x] = (T)buf[15 * threadIdx.x + q];
    }
    __syncthreads();
  }
}

template <typename T>
__global__ void __launch_bounds__(kHostTile) k_get_host(PopArgs<T> p, int layout, double *host, long long n) {
  __shared__ double buf[15 * kHostTile];
  for (long long x0 = (long long)blockIdx.x * kHostTile; x0 < n; x0 += (long long)gridDim.x * kHostTile) {
    const int cnt = (int)(n - x0 < kHostTile ? n - x0 : kHostTile);
    if (threadIdx.x < cnt) {
      const int x = (int)(x0 + threadIdx.x);
      int i, j, k;
      decode(x, p.esj, p.esk, i, j, k);
      const Nbr nb = make_nbr(i, j, k, p.esi, p.esj, p.esk);
      const uint16_t fl = p.flags[x];
#pragma unroll
      for (int q = 0; q < 15; q++)
        buf[15 * threadIdx.x + q] = (double)post_value<T>(p.pop, p.npad, layout, q, x, fl, nb);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 15 * cnt; e += kHostTile) host[15 * x0 + e] = buf[e];
    __syncthreads();
  }
}

// N <-> C0: swap the slots of opposite populations at every node.
template <typename T>
__global__ void k_swap(PopArgs<T> p, long long n) {
  const long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= n) return;
  T *P = p.pop;
  const long long S = p.npad;
#pragma unroll
  for (int q = 1; q < 15; q++) {
    if (OPP(q) < q) continue;
    const T a = P[q * S + x], b = P[OPP(q) * S + x];
    P[q * S + x] = b; P[OPP(q) * S + x] = a;
  }
}

// C1 -> N (out of place into dst).
template <typename T>
__global__ void k_c1_to_n(PopArgs<T> p, T *dst) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y, i = blockIdx.z;
  if (k >= p.esk) return;
  const Nbr nb = make_nbr(i, j, k, p.esi, p.esj, p.esk);
  const int x = nb.at(0, 0, 0);
  const uint16_t fl = p.flags[x];
#pragma unroll
  for (int q = 0; q < 15; q++) dst[q * p.npad + x] = post_value<T>(p.pop, p.npad, SLBC_LAYOUT_C1, q, x, fl, nb);
}

// Separate bounce-back on layout N (reference src/lbkernel.c:58-618): every
// solid boundary node swaps each of its fluid links; optional force.
template <typename T>
__global__ void k_bbl_n(PopArgs<T> p, int moving, const T *uw, int with_force, ForceArgs f) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= f.nbnd) return;
  const int s = f.bnd_node[e];
  int i, j, k;
  decode(s, p.esj, p.esk, i, j, k);
  const Nbr nb = make_nbr(i, j, k, p.esi, p.esj, p.esk);
  const uint16_t fl = p.flags[s];
  T *P = p.pop;
  const long long S = p.npad;
  double fx = 0.0, fy = 0.0, fz = 0.0;
  if (with_force) { fx = f.f[e]; fy = f.f[f.nbnd + e]; fz = f.f[2 * f.nbnd + e]; }
#pragma unroll
  for (int q = 1; q < 15; q++) {
    if (!((fl >> OPP(q)) & 1)) continue;
    const int n = nb.at(CX(q), CY(q), CZ(q));
    const T av = P[q * S + s], bv = P[OPP(q) * S + n];
    double dp;
    if (moving) {
      const T term = link_term<T>(q, uw[s], uw[S + s], uw[2 * S + s]);
      P[OPP(q) * S + n] = av - term; P[q * S + s] = bv + term;
      dp = 2.0 * ((double)av - (double)bv - (double)term);
    } else {
      P[q * S + s] = bv; P[OPP(q) * S + n] = av;
      dp = 2.0 * ((double)av - (double)bv);
    }
    if (CX(q) > 0) fx += dp; else if (CX(q) < 0) fx -= dp;
    if (CY(q) > 0) fy += dp; else if (CY(q) < 0) fy -= dp;
    if (CZ(q) > 0) fz += dp; else if (CZ(q) < 0) fz -= dp;
  }
  if (with_force) { f.f[e] = fx; f.f[f.nbnd + e] = fy; f.f[2 * f.nbnd + e] = fz; }
}

// Separate streaming on layout N, out of place: dst[q][x] = pop[q][x - c_q]
// (reference src/lbkernel.c:623-762).
template <typename T>
__global__ void k_propagate_n(PopArgs<T> p, T *dst) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y, i = blockIdx.z;
  if (k >= p.esk) return;
  const Nbr nb = make_nbr(i, j, k, p.esi, p.esj, p.esk);
  const int x = nb.at(0, 0, 0);
#pragma unroll
  for (int q = 0; q < 15; q++) dst[q * p.npad + x] = p.pop[q * p.npad + nb.at(-CX(q), -CY(q), -CZ(q))];
}

// Separate collision on layout N (reference src/lbkernel.c:769-877).
template <typename T, bool EXACT>
__global__ void k_collide_n(StepArgs<T> a) {
  const long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n = (long long)a.p.esi * a.p.esj * a.p.esk;
  if (x >= n) return;
  const bool solid = (a.p.flags[x] & FLAG_SOLID) != 0;
  if (a.skip_solid && solid) return;
  T *P = a.p.pop;
  const long long S = a.p.npad;
  T t[15];
#pragma unroll
  for (int q = 0; q < 15; q++) t[q] = P[q * S + x];
  T bx = a.bfx, by = a.bfy, bz = a.bfz;
  if (!a.bf_uniform) { bx = a.bf[x]; by = a.bf[S + x]; bz = a.bf[2 * S + x]; }
  collide<T, EXACT>(t, a.omega, a.comega, a.rho0, a.stokes, !solid, bx, by, bz);
#pragma unroll
  for (int q = 0; q < 15; q++) P[q * S + x] = t[q];
}

// Populations from (rho, u): the rebuild of lbloadvel (reference
// src/lbstore.c:352-399).  stage holds 4 doubles per node (rho, ux, uy, uz,
// velocities already rescaled); layout N.
template <typename T, bool EXACT>
__global__ void k_setvel(PopArgs<T> p, const double *stage, long long x0, long long n, int has_rho,
                         double rho0, int stokes, int skip_solid) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const long long x = x0 + e;
  // has_rho 1: stage[4e] is the density; 2: it is the deviation rho - rho0
  // (kept exact in FP32, where rho0 + 1e-4 would lose most of it)
  const T r = has_rho == 2 ? (T)rho0 + (T)stage[4 * e] : has_rho ? (T)stage[4 * e] : (T)rho0;
  const T vx = (T)stage[4 * e + 1], vy = (T)stage[4 * e + 2], vz = (T)stage[4 * e + 3];
  T t[15];
  if (skip_solid && (p.flags[x] & FLAG_SOLID)) {
#pragma unroll
    for (int q = 0; q < 15; q++) t[q] = T(0);
  } else {
    const T drho = has_rho == 2 ? (T)stage[4 * e] : r - (T)rho0, rux = r * vx, ruy = r * vy, ruz = r * vz;
    T sxx = T(0), syy = T(0), szz = T(0), sxy = T(0), sxz = T(0), syz = T(0);
    if (!stokes) {
      sxx = vx * rux; sxy = vx * ruy; sxz = vx * ruz;
      syy = vy * ruy; syz = vy * ruz; szz = vz * ruz;
    }
    rebuild<T, EXACT>(t, drho, rux, ruy, ruz, sxx, syy, szz, sxy, sxz, syz);
  }
#pragma unroll
  for (int q = 0; q < 15; q++) p.pop[q * p.npad + x] = t[q];
}

// Tracer velocity autocorrelation (reference src/mpvacf.c:337-389), FP64
// tracer fields P and P2, over the fluid nodes (psi weights or 1):
//   pass 1: sums of psi P and psi^2;
//   pass 2: P -= psi * pmean, then sums of psi P u_axis and psi P2, with
//   u_axis = (sum_q c_q,axis a_q) / rho from the post-collision populations
//   (any layout) and the density snapshot rho of mprhoinit.
template <typename T>
__global__ void __launch_bounds__(kReduceThreads) k_vacf_sums(PopArgs<T> pa, int layout, const double *rho,
                                                            double *p, const double *p2, const double *psi,
                                                            double pmean, int axis, double *partials) {
  const long long n = (long long)pa.esi * pa.esj * pa.esk;
  double v[2] = {0.0, 0.0};
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int x = (int)e;
    const uint16_t fl = pa.flags[x];
    if (fl & FLAG_SOLID) continue;
    const double w = psi ? psi[x] : 1.0;
    const double pv = p[x] - w * pmean;
    p[x] = pv;
    int i, j, k;
    decode(x, pa.esj, pa.esk, i, j, k);
    const Nbr nb = make_nbr(i, j, k, pa.esi, pa.esj, pa.esk);
    double t[15];
#pragma unroll
    for (int q = 0; q < 15; q++) t[q] = (double)post_value<T>(pa.pop, pa.npad, layout, q, x, fl, nb);
    double mom;
    if (axis == 0) mom = t[1] - t[2] + t[7] - t[8] + t[9] - t[10] + t[11] - t[12] + t[13] - t[14];
    else if (axis == 1) mom = t[3] - t[4] + t[7] + t[8] - t[9] - t[10] + t[11] + t[12] - t[13] - t[14];
    else mom = t[5] - t[6] + t[7] + t[8] + t[9] + t[10] - t[11] - t[12] - t[13] - t[14];
    v[0] += w * pv * (mom / rho[x]);
    v[1] += w * p2[x];
  }
  block_sum<2>(v);
  if (threadIdx.x == 0) { partials[2 * blockIdx.x] = v[0]; partials[2 * blockIdx.x + 1] = v[1]; }
}

// Translation of one spherical object (appended operation, no counterpart
// in the reference, which can only remove objects and insert new ones):
// every node of the box `lo`, `len` (indices taken modulo the lattice, so
// the box may wrap) is tested against the sphere of radius rad at the new
// centre and its periodic images -- rsq < rad^2 per image, evaluated like
// insertsph (reference src/lbobjs.c:214-215), without FMA contraction so the
// set is the same as on the host.  A node of the object that the sphere no
// longer covers becomes fluid with the equilibrium populations of density
// rho0 and the wall velocity v + w x r there (r = node - new centre, the
// reference's vspread convention), rebuilt like lbloadvel's
// (src/lbstore.c:352-389); a fluid node it now covers joins the object with
// its populations left as they are.  Nodes of other objects are left alone.
// Wall velocities rho0 (v + w x r) / 12 (src/lbobjs.c:580-582) are written
// for every node of the object in the box when uw is given.  Each change is
// appended to `changed` as (node, new object index or -1), atomically, at
// most `cap` of them (the count keeps going, so the host sees an overflow).
// The state must be in a local layout: N (pop[q][x] = a_q(x)) or C0
// (pop[opp q][x] = a_q(x)).
struct MoveArgs {
  double c[3];
  double rad, rho0;
  double vel[3], ang[3];
  int obj, stokes, layout;
  int lo[3], len[3];
  int *objidx;
  int *changed;
  int *nchanged;
  int cap;
};

template <typename T, bool EXACT>
__global__ void k_move_sphere(PopArgs<T> p, MoveArgs m, T *uw) {
  const long long nbox = (long long)m.len[0] * m.len[1] * m.len[2];
  const double rr = __dmul_rn(m.rad, m.rad);
  const int L3[3] = {p.esi, p.esj, p.esk};
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nbox;
       e += (long long)gridDim.x * blockDim.x) {
    const int a = (int)(e / ((long long)m.len[1] * m.len[2]));
    const int b = (int)((e / m.len[2]) % m.len[1]);
    const int c = (int)(e % m.len[2]);
    const int n3[3] = {wrap_index(m.lo[0] + a, p.esi), wrap_index(m.lo[1] + b, p.esj), wrap_index(m.lo[2] + c, p.esk)};
    bool inside = false;
    for (int di = -1; di <= 1 && !inside; di++)
      for (int dj = -1; dj <= 1 && !inside; dj++)
        for (int dk = -1; dk <= 1 && !inside; dk++) {
          const int d3[3] = {di, dj, dk};
          double sq = 0.0;
#pragma unroll
          for (int q = 0; q < 3; q++) {
            const double cq = __dadd_rn(m.c[q], (double)(d3[q] * L3[q]));
            const double dq = __dsub_rn((double)n3[q], cq);
            sq = q == 0 ? __dmul_rn(dq, dq) : __dadd_rn(sq, __dmul_rn(dq, dq));
          }
          inside = sq < rr;
        }
    const int x = (n3[0] * p.esj + n3[1]) * p.esk + n3[2];
    const int o = m.objidx[x];
    const bool uncovered = o == m.obj && !inside;
    const bool covered = o == -1 && inside;
    // wall velocity at the node (reference vspread: r = node - centre)
    const double rx = __dsub_rn((double)n3[0], m.c[0]);
    const double ry = __dsub_rn((double)n3[1], m.c[1]);
    const double rz = __dsub_rn((double)n3[2], m.c[2]);
    const double vx = __dsub_rn(__dadd_rn(m.vel[0], __dmul_rn(m.ang[1], rz)), __dmul_rn(m.ang[2], ry));
    const double vy = __dsub_rn(__dadd_rn(m.vel[1], __dmul_rn(m.ang[2], rx)), __dmul_rn(m.ang[0], rz));
    const double vz = __dsub_rn(__dadd_rn(m.vel[2], __dmul_rn(m.ang[0], ry)), __dmul_rn(m.ang[1], rx));
    if (uncovered) {
      const T r0 = (T)m.rho0, ux = (T)vx, uy = (T)vy, uz = (T)vz;
      const T rux = r0 * ux, ruy = r0 * uy, ruz = r0 * uz;
      T sxx = T(0), syy = T(0), szz = T(0), sxy = T(0), sxz = T(0), syz = T(0);
      if (!m.stokes) {
        sxx = ux * rux; sxy = ux * ruy; sxz = ux * ruz;
        syy = uy * ruy; syz = uy * ruz; szz = uz * ruz;
      }
      T t[15];
      rebuild<T, EXACT>(t, T(0), rux, ruy, ruz, sxx, syy, szz, sxy, sxz, syz);
#pragma unroll
      for (int q = 0; q < 15; q++) p.pop[(m.layout == SLBC_LAYOUT_C0 ? OPP(q) : q) * p.npad + x] = t[q];
    }
    if (uncovered || covered) {
      m.objidx[x] = covered ? m.obj : -1;
      const int slot = atomicAdd(m.nchanged, 1);
      if (slot < m.cap) {
        m.changed[2 * slot] = x;
        m.changed[2 * slot + 1] = covered ? m.obj : -1;
      }
    }
    if (uw != nullptr && (uncovered || inside && (o == m.obj || o == -1))) {
      const double s = m.rho0;
      uw[x] = uncovered ? T(0) : (T)__ddiv_rn(__dmul_rn(s, vx), 12.0);
      uw[p.npad + x] = uncovered ? T(0) : (T)__ddiv_rn(__dmul_rn(s, vy), 12.0);
      uw[2 * p.npad + x] = uncovered ? T(0) : (T)__ddiv_rn(__dmul_rn(s, vz), 12.0);
    }
  }
}

// Velocity field u = (sum_q c_q a_q + fac * b) / (rho0 + sum_q a_q) of the
// post-collision state (any layout) on fluid nodes, 0 on solid nodes, as
// three FP32 arrays (the per-node form of the accvmean sum).
template <typename T>
__global__ void k_velocity(PopArgs<T> p, int layout, double rho0, double fac, int bf_uniform, double b0, double b1,
                           double b2, const T *bf, float *u, float *drho) {
  const long long n = (long long)p.esi * p.esj * p.esk;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int x = (int)e;
    const uint16_t fl = p.flags[x];
    float ux = 0.f, uy = 0.f, uz = 0.f, dr = 0.f;
    if (!(fl & FLAG_SOLID)) {
      int i, j, k;
      decode(x, p.esj, p.esk, i, j, k);
      const Nbr nb = make_nbr(i, j, k, p.esi, p.esj, p.esk);
      double r = 0.0, mx = 0.0, my = 0.0, mz = 0.0;
#pragma unroll
      for (int q = 0; q < 15; q++) {
        const double v = (double)post_value<T>(p.pop, p.npad, layout, q, x, fl, nb);
        r += v;
        mx += CX(q) * v;
        my += CY(q) * v;
        mz += CZ(q) * v;
      }
      double bx = b0, by = b1, bz = b2;
      if (!bf_uniform) { bx = bf[x]; by = bf[p.npad + x]; bz = bf[2 * p.npad + x]; }
      const double inv = 1.0 / (rho0 + r);
      ux = (float)((mx + fac * bx) * inv);
      uy = (float)((my + fac * by) * inv);
      uz = (float)((mz + fac * bz) * inv);
      dr = (float)r;
    }
    u[x] = ux;
    u[n + x] = uy;
    u[2 * n + x] = uz;
    if (drho) drho[x] = dr;
  }
}

}  // namespace slbc
