// Moment-propagation (passive scalar) kernels, templated on the flow
// population type T and the tracer type TP.
//
// The reference update (src/mpkernel.c:47-201 stationary, 206-368 moving)
// scatters: every fluid node y adds fac*a_q(y) + w_q*piece to the node
// y + c_q, every non-adsorbing solid boundary node returns what its fluid
// neighbours sent along each boundary link, and a copy-back keeps the fluid
// sums, adds to adsorbing solids and zeroes other solids.  Here each node
// GATHERS its 15 incoming terms instead (no atomics, no races) and adds them
// in the order the reference adds them into newp: ascending source node, then
// link.  Away from the periodic wrap that order is fixed; at wrap nodes (and
// in lattices thinner than 3) the terms are ranked by source index first.
#pragma once

#include "slbc_kernels.cuh"

namespace slbc {

struct MpArgs {
  const void *p_in;
  void *p_out;
  const void *rho;  // density snapshot in the tracer type
  const unsigned char *ads;  // adsorbing nodes (0x4000 of the reference mask)
  const uint16_t *ads_links; // per fluid node: links from adsorbing solids
  const int *objidx;         // object of every node (-1 fluid), moving walls
  const double *objstate;    // 9 doubles per object: pos, vel, ang
  int moving;
  double alpha, adprob, rho0;
  // the same in FP32, converted on the host (an FP64 conversion or compare
  // that the compiler re-evaluates inside a loop lands on the narrow FP64
  // pipe), and whether adsorption is partial (adprob != 1)
  float alpha_f, adprob_f, rho0_f;
  int partial;
};

template <typename TP> __device__ __forceinline__ TP mp_param(double d, float f);
template <> __device__ __forceinline__ double mp_param<double>(double d, float) { return d; }
template <> __device__ __forceinline__ float mp_param<float>(double, float f) { return f; }

// Interior accumulation order: links sorted by descending offset
// cx*esj*esk + cy*esk + cz, i.e. ascending source node x - c_q.
__device__ __forceinline__ constexpr int mp_order(int r) {
  return r == 0 ? 7 : r == 1 ? 11 : r == 2 ? 1 : r == 3 ? 9 : r == 4 ? 13 : r == 5 ? 3
       : r == 6 ? 5 : r == 7 ? 0 : r == 8 ? 6 : r == 9 ? 4 : r == 10 ? 8 : r == 11 ? 12
       : r == 12 ? 2 : r == 13 ? 10 : 14;
}

template <typename TP>
__device__ __forceinline__ TP mp_load(const void *p, int x) { return ((const TP *)p)[x]; }

// Wall velocity (times rho0/12) of the object owning solid node (i,j,k):
// reference src/mpkernel.c:263-267.
template <typename R>
__device__ __forceinline__ void mp_wall_u(const double *st, int i, int j, int k, R rho0, R (&u)[3]) {
  const R rx = i - (R)st[0], ry = j - (R)st[1], rz = k - (R)st[2];
  const R vx = (R)st[3], vy = (R)st[4], vz = (R)st[5], ax = (R)st[6], ay = (R)st[7], az = (R)st[8];
  u[0] = rho0 * (vx + ay * rz - az * ry) / R(12.0);
  u[1] = rho0 * (vy + az * rx - ax * rz) / R(12.0);
  u[2] = rho0 * (vz + ax * ry - ay * rx) / R(12.0);
}

// Moving-wall tracer term of link q seen from the solid node: reference
// src/mpkernel.c:272-350 (same evaluation).
template <typename R>
__device__ __forceinline__ R mp_wall_term(int q, R fac, const R (&u)[3]) {
  if (q <= 6) {
    const R uu = q <= 2 ? u[0] : q <= 4 ? u[1] : u[2];
    return (q & 1) ? R(8.0) * fac * uu : -(R(8.0) * fac * uu);
  }
  const R inner = (u[0] + (CX(q) * CY(q) > 0 ? u[1] : -u[1])) + (CX(q) * CZ(q) > 0 ? u[2] : -u[2]);
  return CX(q) > 0 ? fac * inner : -(fac * inner);
}

// fac = p/rho and piece = p/b * (rho0/rho - alpha) of a source node, with
// the reference's operations (src/mpkernel.c:74-76), computed once per node
template <typename TP>
constexpr int mp_bucket_bytes() { return 27 * kTileThreads * (int)sizeof(TP); }

template <typename TP>
struct MpSource {
  TP fac, piece;
};

template <typename TP>
__device__ __forceinline__ MpSource<TP> mp_source(const MpArgs &m, int y, TP rho0, TP alpha) {
  const TP rhot = mp_load<TP>(m.rho, y), pt = mp_load<TP>(m.p_in, y);
  MpSource<TP> r;
  r.fac = pt / rhot;
  r.piece = pt * TP(1.0 / 72.0) * (rho0 / rhot - alpha);
  return r;
}

// One tracer update of every node.  A block of 32 (k) x 8 (j) threads walks
// along i over `planes` planes; fac and piece of every node of three
// consecutive planes (with a one-node halo) sit in shared memory, so each
// node's two divisions are done about 1.7 times per update instead of once
// for each of the up to 15 nodes that gather from it.
template <typename T, typename TP>
__global__ void __launch_bounds__(kTileThreads, sizeof(TP) == 8 ? 2 : 3) k_mp_step(PopArgs<T> p, int layout, MpArgs m, int planes) {
  __shared__ MpSource<TP> ring[3][kPlane];
  // summation order at wrap nodes: 27 x kTileThreads values, dynamic
  // shared memory (mp_bucket_bytes per block)
  extern __shared__ __align__(16) unsigned char mp_dyn[];
  TP(*bucket)[kTileThreads] = reinterpret_cast<TP(*)[kTileThreads]>(mp_dyn);
  const int tk = threadIdx.x, tj = threadIdx.y, tid = tj * kTileK + tk;
  const int k0 = blockIdx.x * kTileK, j0 = blockIdx.y * kTileJ, i0 = blockIdx.z * planes;
  const int np = min(planes, p.esi - i0);
  const int plane_nodes = p.esj * p.esk;
  const TP onebyb = TP(1.0 / 72.0), eightbyb = TP(8.0 / 72.0);
  const TP alpha = mp_param<TP>(m.alpha, m.alpha_f), rho0 = mp_param<TP>(m.rho0, m.rho0_f);
  const TP Pa = mp_param<TP>(m.adprob, m.adprob_f);
  const bool partial = m.partial != 0;
  int off[kPlaneLoads];
#pragma unroll
  for (int e = 0; e < kPlaneLoads; e++) {
    const int c = tid + kTileThreads * e;
    off[e] = c < kPlane ? wrap_index(j0 - 1 + c / kHaloK, p.esj) * p.esk + wrap_index(k0 - 1 + c % kHaloK, p.esk)
                        : -1;
  }
  // plane q sits in ring slot (q - i0 + 1) % 3
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int base = wrap_index(i0 - 1 + h, p.esi) * plane_nodes;
#pragma unroll
    for (int e = 0; e < kPlaneLoads; e++)
      if (off[e] >= 0) ring[h][tid + kTileThreads * e] = mp_source<TP>(m, base + off[e], rho0, alpha);
  }
  // Register prefetch, one plane ahead of use: p and rho of the halo tile
  // of plane i+1 (for the ring) and the flag word, adsorption byte, p and
  // rho of this thread's own node of plane i, so that only the 15
  // population loads stay on a node's critical path.
  TP pre_p[kPlaneLoads], pre_r[kPlaneLoads];
  const int j = j0 + tj, k = k0 + tk;
  const bool mine = j < p.esj && k < p.esk;
  const int own = mine ? j * p.esk + k : 0;
  auto prefetch_ring = [&](int plane) {
    const int base = wrap_index(plane, p.esi) * plane_nodes;
#pragma unroll
    for (int e = 0; e < kPlaneLoads; e++)
      if (off[e] >= 0) { pre_p[e] = mp_load<TP>(m.p_in, base + off[e]); pre_r[e] = mp_load<TP>(m.rho, base + off[e]); }
  };
  uint16_t n_fl = 0, n_al = 0;
  unsigned char n_ads = 0;
  TP n_p = TP(0), n_r = TP(1);
  auto prefetch_node = [&](int plane) {
    const int x = plane * plane_nodes + own;
    n_fl = p.flags[x];
    n_ads = m.ads ? m.ads[x] : 0;
    n_al = m.ads ? m.ads_links[x] : 0;
    n_p = mp_load<TP>(m.p_in, x);
    n_r = mp_load<TP>(m.rho, x);
  };
  prefetch_ring(i0 + 1);
  prefetch_node(i0);
  TP *pout = (TP *)m.p_out;
  const T *P = p.pop;
  const long long S = p.npad;
  for (int ii = 0; ii < np; ii++) {
    const int i = i0 + ii;
    const int sm = ii % 3, s0 = (ii + 1) % 3, sp = (ii + 2) % 3;  // planes i-1, i, i+1
    __syncthreads();  // slot sp held plane i-2, last read in the previous iteration
#pragma unroll
    for (int e = 0; e < kPlaneLoads; e++) {
      if (off[e] < 0) continue;
      MpSource<TP> r;
      r.fac = pre_p[e] / pre_r[e];
      r.piece = pre_p[e] * TP(1.0 / 72.0) * (rho0 / pre_r[e] - alpha);
      ring[sp][tid + kTileThreads * e] = r;
    }
    __syncthreads();
    const uint16_t fl = n_fl, al = n_al;
    const bool ads_x = n_ads != 0;
    const TP pt_x = n_p, r_x = n_r;
    if (ii + 1 < np) {
      prefetch_ring(i + 2);
      prefetch_node(i + 1);
    }
    if (!mine) continue;
    const MpSource<TP> *R[3] = {ring[sm], ring[s0], ring[sp]};
    const int c0 = (tj + 1) * kHaloK + tk + 1;
    const Nbr nb = make_nbr(i, j, k, p.esi, p.esj, p.esk);
    const int x = nb.at(0, 0, 0);
    const bool solid = (fl & FLAG_SOLID) != 0;
    if (solid && !ads_x) { pout[x] = TP(0); continue; }
    // rho0/rho - alpha of x itself, for the axis links that return to x
    TP h_x = TP(0);
    if (!solid && (fl & 0x7Eu)) h_x = rho0 / r_x - alpha;
    const MpSource<TP> ex = R[1][c0];
    // Each link q is one of: A fluid y scatters into fluid x; B fluid y
    // scatters into adsorbing solid x; C solid y returns to fluid x what x
    // sent along opp(q); D solid-solid, nothing flows.  First the population
    // each link reads, selected without branches and loaded together; then
    // the terms; then, on fluid boundary nodes only, the moving-wall and
    // adsorbing-neighbour corrections of case C.
    auto source = [&](int q) { return q == 0 ? x : nb.at(-CX(q), -CY(q), -CZ(q)); };
    TP av[15];
#pragma unroll
    for (int q = 0; q < 15; q++) {
      const int y = source(q);
      const bool bnd = q != 0 && ((fl >> q) & 1);  // y and x differ in solidity
      const bool self_c = bnd && !solid;           // case C
      int slot, node;
      if (layout == SLBC_LAYOUT_N) {
        slot = self_c ? OPP(q) : q;
        node = self_c ? x : y;
      } else if (layout == SLBC_LAYOUT_C0 || q == 0 || bnd) {
        slot = self_c ? q : OPP(q);
        node = self_c ? x : y;
      } else {
        slot = q;  // C1, case A: pushed into x
        node = x;
      }
      av[q] = (TP)P[slot * S + node];
    }
    TP term[15];
#pragma unroll
    for (int q = 0; q < 15; q++) {
      const bool bnd = q != 0 && ((fl >> q) & 1);
      const bool self_c = bnd && !solid;
      const MpSource<TP> e = R[1 - CX(q)][c0 - CY(q) * kHaloK - CZ(q)];
      TP t;
      if (q == 0) {
        t = e.fac * av[q] + TP(16.0) * e.piece + alpha * pt_x;
      } else {
        // (b q-weight * p) * (rho0/rho - alpha) of x in case C: for the
        // diagonals this is the piece of x (the products commute exactly)
        const TP fac = self_c ? ex.fac : e.fac;
        const TP pc = self_c ? (q <= 6 ? (eightbyb * pt_x) * h_x : ex.piece)
                             : (q <= 6 ? TP(8.0) * e.piece : e.piece);
        t = fac * av[q] + pc;
        if (bnd && solid && partial) t = Pa * t;  // case B
        // case C from an adsorbing solid keeps 1 - P (nothing when P = 1);
        // with moving walls this follows the wall term, below
        if (self_c && !m.moving && ((al >> q) & 1)) t = partial ? (TP(1.0) - Pa) * t : TP(0);
      }
      term[q] = (solid && !bnd) ? TP(0) : t;  // case D
    }
    if (m.moving && !solid && (fl & FLAG_LINKS)) {
#pragma unroll
      for (int q = 1; q < 15; q++) {
        if (!((fl >> q) & 1)) continue;
        const int y = source(q);
        TP u[3];
        const int o = m.objidx[y];
        int yi = i - CX(q), yj = j - CY(q), yk = k - CZ(q);
        yi = yi < 0 ? p.esi - 1 : (yi >= p.esi ? 0 : yi);
        yj = yj < 0 ? p.esj - 1 : (yj >= p.esj ? 0 : yj);
        yk = yk < 0 ? p.esk - 1 : (yk >= p.esk ? 0 : yk);
        mp_wall_u<TP>(m.objstate + 9 * o, yi, yj, yk, rho0, u);
        TP t = term[q] + mp_wall_term<TP>(q, ex.fac, u);
        if ((al >> q) & 1) t = partial ? (TP(1.0) - Pa) * t : TP(0);
        term[q] = t;
      }
    }
    TP sum = TP(0);
    const bool interior = i > 0 && i < p.esi - 1 && j > 0 && j < p.esj - 1 && k > 0 &&
                          k < p.esk - 1 && p.esj >= 3 && p.esk >= 3;
    if (interior) {
#pragma unroll
      for (int r = 0; r < 15; r++) sum += term[mp_order(r)];
    } else if (p.esi >= 3 && p.esj >= 3 && p.esk >= 3) {
      // Wrap node of a lattice at least 3 wide: the 15 sources are distinct
      // and ascending index order is lexicographic in (i', j', k'); each
      // coordinate's three values rank as below, so the terms go to 27
      // buckets keyed by (rank i', rank j', rank k') and are added in bucket
      // order (empty buckets add +0, which leaves the sum unchanged).
      auto rnk = [](int c, int n, int d) {  // rank of coordinate c + d, wrapped
        if (c == 0) return d == 0 ? 0 : (d == 1 ? 1 : 2);
        if (c == n - 1) return d == 1 ? 0 : (d == -1 ? 1 : 2);
        return d + 1;
      };
      // (this thread's column of a shared array: an indexed store and load
      // per term, where a runtime index into registers becomes select chains)
#pragma unroll
      for (int c = 0; c < 27; c++) bucket[c][tid] = TP(0);
#pragma unroll
      for (int q = 0; q < 15; q++)
        bucket[9 * rnk(i, p.esi, -CX(q)) + 3 * rnk(j, p.esj, -CY(q)) + rnk(k, p.esk, -CZ(q))][tid] = term[q];
#pragma unroll
      for (int c = 0; c < 27; c++) sum += bucket[c][tid];
    } else {
      // thin lattice (sources can coincide): rank every term by (source
      // node, link) and add in rank order
      int src[15], rank[15];
#pragma unroll
      for (int q = 0; q < 15; q++) src[q] = source(q);
#pragma unroll
      for (int q = 0; q < 15; q++) {
        int r = 0;
#pragma unroll
        for (int s2 = 0; s2 < 15; s2++)
          r += (src[s2] < src[q]) || (src[s2] == src[q] && s2 < q);
        rank[q] = r;
      }
#pragma unroll
      for (int r = 0; r < 15; r++) {
        TP v = TP(0);
#pragma unroll
        for (int q = 0; q < 15; q++) v = rank[q] == r ? term[q] : v;
        sum += v;
      }
    }
    if (solid) pout[x] = pt_x + sum;
    else pout[x] = sum;
  }
}

// FP32 tracer update: the terms of k_mp_step with TP = float, added in link
// order (the reference's summation order matters for FP64 bit parity only).
// The density snapshot enters as 1/rho (rinv, FP32), so a source node costs
// no division: fac = p/rho and piece = p/72 * (rho0/rho - alpha) are products.
// Each link term is the case-A/B/C expression times a factor that the flag
// word, the adsorbing-link mask and the adsorption probability P decide:
//   fluid x:  1, or over a link from an adsorbing solid (1 - P), 0 when P = 1;
//   solid x (adsorbing): P over boundary links (1 when P = 1), 0 otherwise;
// and on fluid boundary nodes with moving walls the wall term is added first.
// Population indices are 32-bit (15 * npad < 2^32) and the layout is a
// template argument, so a link's load costs a neighbour index, a select and
// one address computation.
template <typename T, int LAYOUT, bool MOVING>
__global__ void __launch_bounds__(kTileThreads, 3)
k_mp_step_f32(PopArgs<T> p, MpArgs m, const float *rinv, int planes) {
  __shared__ MpSource<float> ring[3][kPlane];
  const int tk = threadIdx.x, tj = threadIdx.y, tid = tj * kTileK + tk;
  const int k0 = blockIdx.x * kTileK, j0 = blockIdx.y * kTileJ, i0 = blockIdx.z * planes;
  const int np = min(planes, p.esi - i0);
  const int plane_nodes = p.esj * p.esk;
  const float alpha = m.alpha_f, rho0 = m.rho0_f, Pa = m.adprob_f;
  const float cB = m.partial ? Pa : 1.0f;         // link into an adsorbing solid
  const float cC = m.partial ? 1.0f - Pa : 0.0f;  // link from an adsorbing solid
  const unsigned npad = (unsigned)p.npad;
  int off[kPlaneLoads];
#pragma unroll
  for (int e = 0; e < kPlaneLoads; e++) {
    const int c = tid + kTileThreads * e;
    off[e] = c < kPlane ? wrap_index(j0 - 1 + c / kHaloK, p.esj) * p.esk + wrap_index(k0 - 1 + c % kHaloK, p.esk)
                        : -1;
  }
  const float *pin = (const float *)m.p_in;
  auto source_of = [&](float pt, float ri) {
    MpSource<float> r;
    r.fac = pt * ri;
    r.piece = pt * (1.0f / 72.0f) * (rho0 * ri - alpha);
    return r;
  };
  // plane q sits in ring slot (q - i0 + 1) % 3
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int base = wrap_index(i0 - 1 + h, p.esi) * plane_nodes;
#pragma unroll
    for (int e = 0; e < kPlaneLoads; e++)
      if (off[e] >= 0) ring[h][tid + kTileThreads * e] = source_of(pin[base + off[e]], rinv[base + off[e]]);
  }
  // register prefetch one plane ahead: p and 1/rho of the halo tile of
  // plane i+1, and the flag word, adsorption byte, adsorbing links and p of
  // this thread's node of plane i
  float pre_p[kPlaneLoads], pre_r[kPlaneLoads];
  const int j = j0 + tj, k = k0 + tk;
  const bool mine = j < p.esj && k < p.esk;
  const int own = mine ? j * p.esk + k : 0;
  auto prefetch_ring = [&](int plane) {
    const int base = wrap_index(plane, p.esi) * plane_nodes;
#pragma unroll
    for (int e = 0; e < kPlaneLoads; e++)
      if (off[e] >= 0) { pre_p[e] = pin[base + off[e]]; pre_r[e] = rinv[base + off[e]]; }
  };
  uint16_t n_fl = 0, n_al = 0;
  unsigned char n_ads = 0;
  float n_p = 0.0f;
  auto prefetch_node = [&](int plane) {
    const int x = plane * plane_nodes + own;
    n_fl = p.flags[x];
    n_ads = m.ads ? m.ads[x] : 0;
    n_al = m.ads ? m.ads_links[x] : 0;
    n_p = pin[x];
  };
  prefetch_ring(i0 + 1);
  prefetch_node(i0);
  float *pout = (float *)m.p_out;
  const T *P = p.pop;
  const int c0 = (tj + 1) * kHaloK + tk + 1;
  for (int ii = 0; ii < np; ii++) {
    const int i = i0 + ii;
    const int sm = ii % 3, s0 = (ii + 1) % 3, sp = (ii + 2) % 3;  // planes i-1, i, i+1
    __syncthreads();  // slot sp held plane i-2, last read in the previous iteration
#pragma unroll
    for (int e = 0; e < kPlaneLoads; e++)
      if (off[e] >= 0) ring[sp][tid + kTileThreads * e] = source_of(pre_p[e], pre_r[e]);
    __syncthreads();
    const uint16_t fl = n_fl, al = n_al;
    const bool ads_x = n_ads != 0;
    const float pt_x = n_p;
    if (ii + 1 < np) {
      prefetch_ring(i + 2);
      prefetch_node(i + 1);
    }
    if (!mine) continue;
    const MpSource<float> *R[3] = {ring[sm], ring[s0], ring[sp]};
    const Nbr nb = make_nbr(i, j, k, p.esi, p.esj, p.esk);
    const int x = nb.at(0, 0, 0);
    const bool solid = (fl & FLAG_SOLID) != 0;
    if (solid && !ads_x) { pout[x] = 0.0f; continue; }
    const MpSource<float> ex = R[1][c0];
    const unsigned bmask = fl & FLAG_LINKS;
    // factor masks: zero (solid x: links that are not boundary links, and
    // the rest link q = 0) and the adsorption factor cval
    const unsigned zmask = solid ? (~bmask & 0x7FFFu) : 0u;
    const unsigned amask = solid ? bmask : (unsigned)al;
    const float cval = solid ? cB : cC;
    float sum = 0.0f;
#pragma unroll
    for (int q = 0; q < 15; q++) {
      float t;
      if (q == 0) {
        t = ex.fac * (float)P[x] + 16.0f * ex.piece + alpha * pt_x;
      } else {
        const bool bnd = (bmask >> q) & 1u;
        const bool self_c = bnd && !solid;  // solid y returns what x sent along opp(q)
        const int y = nb.at(-CX(q), -CY(q), -CZ(q));
        unsigned idx;
        if (LAYOUT == SLBC_LAYOUT_N) {
          idx = self_c ? OPP(q) * npad + (unsigned)x : q * npad + (unsigned)y;
        } else if (LAYOUT == SLBC_LAYOUT_C0) {
          idx = self_c ? q * npad + (unsigned)x : OPP(q) * npad + (unsigned)y;
        } else {  // C1: pushed into x unless y -> x is a boundary link
          idx = (bnd && solid) ? OPP(q) * npad + (unsigned)y : q * npad + (unsigned)x;
        }
        const float av = (float)P[idx];
        const MpSource<float> e = R[1 - CX(q)][c0 - CY(q) * kHaloK - CZ(q)];
        const float fac = self_c ? ex.fac : e.fac;
        const float pw = self_c ? ex.piece : e.piece;
        t = fac * av + (q <= 6 ? 8.0f : 1.0f) * pw;
        if (MOVING && self_c) {
          float u[3];
          const int o = m.objidx[y];
          int yi = i - CX(q), yj = j - CY(q), yk = k - CZ(q);
          yi = yi < 0 ? p.esi - 1 : (yi >= p.esi ? 0 : yi);
          yj = yj < 0 ? p.esj - 1 : (yj >= p.esj ? 0 : yj);
          yk = yk < 0 ? p.esk - 1 : (yk >= p.esk ? 0 : yk);
          mp_wall_u<float>(m.objstate + 9 * o, yi, yj, yk, rho0, u);
          t += mp_wall_term<float>(q, ex.fac, u);
        }
      }
      const float f = ((zmask >> q) & 1u) ? 0.0f : (((amask >> q) & 1u) ? cval : 1.0f);
      sum += f * t;
    }
    pout[x] = solid ? pt_x + sum : sum;
  }
}

// Stencil coefficients of the FP32 tracer update on a frozen flow.  Every
// term of k_mp_step_f32 is p of one node times a factor that depends only on
// the flow, the density snapshot, alpha, P and the geometry, so one update is
//   p'(x) = C_0(x) p(x) + sum_{q=1..14} C_q(x) p(x - c_q):
// case A (and B) terms from y = x - c_q go to C_q; case C terms (x's own
// populations returned by a solid neighbour, with the moving-wall term) and
// the q = 0 term go to C_0; an adsorbing solid keeps its own p (C_0 += 1); a
// non-adsorbing solid gets all zeros.  coef[q * npad + x], one thread per
// node; the layout is that of the flow when the coefficients were built.
template <typename T, int LAYOUT, bool MOVING>
__global__ void __launch_bounds__(256) k_mp_coef(PopArgs<T> p, MpArgs m, const float *rinv, float *coef) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)p.esi * p.esj * p.esk) return;
  const int x = (int)e;
  int i, j, k;
  decode(x, p.esj, p.esk, i, j, k);
  const Nbr nb = make_nbr(i, j, k, p.esi, p.esj, p.esk);
  const unsigned npad = (unsigned)p.npad;
  const uint16_t fl = p.flags[x];
  const bool solid = (fl & FLAG_SOLID) != 0;
  const bool ads_x = m.ads ? m.ads[x] != 0 : false;
  float c[15];
#pragma unroll
  for (int q = 0; q < 15; q++) c[q] = 0.0f;
  if (!solid || ads_x) {
    const float alpha = m.alpha_f, rho0 = m.rho0_f, Pa = m.adprob_f;
    const float cB = m.partial ? Pa : 1.0f, cC = m.partial ? 1.0f - Pa : 0.0f;
    const T *P = p.pop;
    const float rx = rinv[x];
    const float gx = (1.0f / 72.0f) * (rho0 * rx - alpha);  // piece of x per unit p
    const unsigned bmask = fl & FLAG_LINKS;
    const unsigned zmask = solid ? (~bmask & 0x7FFFu) : 0u;
    const unsigned amask = solid ? bmask : (unsigned)(m.ads ? m.ads_links[x] : 0);
    const float cval = solid ? cB : cC;
    if (!solid) c[0] = rx * (float)P[x] + 16.0f * gx + alpha;
#pragma unroll
    for (int q = 1; q < 15; q++) {
      const bool bnd = (bmask >> q) & 1u;
      const bool self_c = bnd && !solid;
      const int y = nb.at(-CX(q), -CY(q), -CZ(q));
      unsigned idx;
      if (LAYOUT == SLBC_LAYOUT_N) {
        idx = self_c ? OPP(q) * npad + (unsigned)x : q * npad + (unsigned)y;
      } else if (LAYOUT == SLBC_LAYOUT_C0) {
        idx = self_c ? q * npad + (unsigned)x : OPP(q) * npad + (unsigned)y;
      } else {
        idx = (bnd && solid) ? OPP(q) * npad + (unsigned)y : q * npad + (unsigned)x;
      }
      const float av = (float)P[idx];
      const float W = q <= 6 ? 8.0f : 1.0f;
      const float f = ((zmask >> q) & 1u) ? 0.0f : (((amask >> q) & 1u) ? cval : 1.0f);
      if (self_c) {
        float kq = rx * av + W * gx;
        if (MOVING) {
          float u[3];
          const int o = m.objidx[y];
          int yi = i - CX(q), yj = j - CY(q), yk = k - CZ(q);
          yi = yi < 0 ? p.esi - 1 : (yi >= p.esi ? 0 : yi);
          yj = yj < 0 ? p.esj - 1 : (yj >= p.esj ? 0 : yj);
          yk = yk < 0 ? p.esk - 1 : (yk >= p.esk ? 0 : yk);
          mp_wall_u<float>(m.objstate + 9 * o, yi, yj, yk, rho0, u);
          kq += rx * mp_wall_term<float>(q, 1.0f, u);
        }
        c[0] += f * kq;
      } else {
        const float ry = rinv[y];
        c[q] = f * (ry * av + W * (1.0f / 72.0f) * (rho0 * ry - alpha));
      }
    }
    if (solid) c[0] += 1.0f;
  }
#pragma unroll
  for (int q = 0; q < 15; q++) coef[q * npad + (unsigned)x] = c[q];
}

// Density snapshot (reference src/mpmisc.c:64-79), kept in FP64 and, when
// FP32 tracers exist, in FP32.
template <typename T>
__global__ void k_mp_rhoinit(PopArgs<T> p, int layout, double rho0, double *rho64, float *rho32) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n = (long long)p.esi * p.esj * p.esk;
  if (e >= n) return;
  const int x = (int)e;
  const uint16_t fl = p.flags[x];
  double r = rho0;
  float rf = (float)rho0;
  if (!(fl & FLAG_SOLID)) {
    int i, j, k;
    decode(x, p.esj, p.esk, i, j, k);
    const Nbr nb = make_nbr(i, j, k, p.esi, p.esj, p.esk);
#pragma unroll
    for (int q = 0; q < 15; q++) {
      const T v = post_value<T>(p.pop, p.npad, layout, q, x, fl, nb);
      r += (double)v;
      rf += (float)v;
    }
  }
  rho64[x] = r;
  if (rho32) rho32[x] = rf;
}

}  // namespace slbc
