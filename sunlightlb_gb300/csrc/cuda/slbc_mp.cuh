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
  const int *objidx;         // object of every node (-1 fluid), moving walls
  const double *objstate;    // 9 doubles per object: pos, vel, ang
  int moving;
  double alpha, adprob, rho0;
};

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

// One tracer update of every node.  Grid as k_step.
template <typename T, typename TP>
__global__ void __launch_bounds__(256) k_mp_step(PopArgs<T> p, int layout, MpArgs m) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y, i = blockIdx.z;
  if (k >= p.esk) return;
  const Nbr nb = make_nbr(i, j, k, p.esi, p.esj, p.esk);
  const int x = nb.at(0, 0, 0);
  const uint16_t fl = p.flags[x];
  const bool solid = (fl & FLAG_SOLID) != 0;
  const bool ads_x = m.ads && m.ads[x];
  TP *pout = (TP *)m.p_out;
  if (solid && !ads_x) { pout[x] = TP(0); return; }
  const T *P = p.pop;
  const long long S = p.npad;
  const TP onebyb = TP(1.0 / 72.0), eightbyb = TP(8.0 / 72.0);
  const TP alpha = (TP)m.alpha, rho0 = (TP)m.rho0, Pa = (TP)m.adprob;
  const bool partial = m.adprob != 1.0;
  TP term[15];
  int src[15];
#pragma unroll
  for (int q = 0; q < 15; q++) {
    term[q] = TP(0);
    const int y = q == 0 ? x : nb.at(-CX(q), -CY(q), -CZ(q));
    src[q] = y;
    const bool bnd = q != 0 && ((fl >> q) & 1);  // y and x differ in solidity
    if (!bnd) {
      if (solid) continue;  // solid-solid link: nothing flows
      // fluid y scatters along q into x
      const TP rhot = mp_load<TP>(m.rho, y), pt = mp_load<TP>(m.p_in, y);
      const TP fac = pt / rhot, piece = pt * onebyb * (rho0 / rhot - alpha);
      T av;
      if (layout == SLBC_LAYOUT_N) av = P[q * S + y];
      else if (layout == SLBC_LAYOUT_C0 || q == 0) av = P[OPP(q) * S + y];
      else av = P[q * S + x];
      if (q == 0) term[q] = fac * (TP)av + TP(16.0) * piece + alpha * pt;
      else term[q] = fac * (TP)av + (q <= 6 ? TP(8.0) * piece : piece);
    } else if (solid) {
      // fluid y scatters into adsorbing solid x (fraction P when partial)
      const TP rhot = mp_load<TP>(m.rho, y), pt = mp_load<TP>(m.p_in, y);
      const TP fac = pt / rhot, piece = pt * onebyb * (rho0 / rhot - alpha);
      T av;
      if (layout == SLBC_LAYOUT_N) av = P[q * S + y];
      else av = P[OPP(q) * S + y];
      TP t = fac * (TP)av + (q <= 6 ? TP(8.0) * piece : piece);
      if (partial) t = Pa * t;
      term[q] = t;
    } else {
      // solid y returns to fluid x what x sent along opp(q)
      const bool ads_y = m.ads && m.ads[y];
      if (ads_y && !partial) continue;
      const TP rhot = mp_load<TP>(m.rho, x), pt = mp_load<TP>(m.p_in, x);
      const TP fac = pt / rhot;
      const TP piece = (q <= 6 ? eightbyb : onebyb) * pt * (rho0 / rhot - alpha);
      const T av = layout == SLBC_LAYOUT_N ? P[OPP(q) * S + x] : P[q * S + x];
      TP t = fac * (TP)av + piece;
      if (m.moving) {
        TP u[3];
        const int o = m.objidx[y];
        int yi = i - CX(q), yj = j - CY(q), yk = k - CZ(q);
        yi = yi < 0 ? p.esi - 1 : (yi >= p.esi ? 0 : yi);
        yj = yj < 0 ? p.esj - 1 : (yj >= p.esj ? 0 : yj);
        yk = yk < 0 ? p.esk - 1 : (yk >= p.esk ? 0 : yk);
        mp_wall_u<TP>(m.objstate + 9 * o, yi, yj, yk, rho0, u);
        t = t + mp_wall_term<TP>(q, fac, u);
      }
      if (ads_y) t = (TP(1.0) - Pa) * t;
      term[q] = t;
    }
  }
  TP sum = TP(0);
  const bool interior = i > 0 && i < p.esi - 1 && j > 0 && j < p.esj - 1 && k > 0 &&
                        k < p.esk - 1 && p.esj >= 3 && p.esk >= 3;
  if (interior) {
#pragma unroll
    for (int r = 0; r < 15; r++) sum += term[mp_order(r)];
  } else {
    // rank every term by (source node, link) and add in rank order
    int rank[15];
#pragma unroll
    for (int q = 0; q < 15; q++) {
      int r = 0;
#pragma unroll
      for (int s = 0; s < 15; s++)
        r += (src[s] < src[q]) || (src[s] == src[q] && s < q);
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
  if (solid) pout[x] = mp_load<TP>(m.p_in, x) + sum;
  else pout[x] = sum;
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
