// BF16 scaled-deviation populations.
//
// Storage of a lattice in this precision:
//   M[x]   = (drho, rux, ruy, ruz) of node x after its last collision, FP32,
//            one float4 per node, two buffers swapped every step;
//   D[q][x]  BF16 of scale * (a_q - eq_q(M)), the deviation of each
//            post-collision population from the equilibrium built from the
//            node's own moments (eq = the collision's rebuild with zero
//            stress, reference src/lbkernel.c:838-865), in the same AA
//            layouts (N, C0, C1) as the FP32 and FP64 populations.
// A population is reconstructed as eq_q(M[source]) + D / scale, where the
// source is the node that produced it.  The equilibrium part carries FP32
// precision; BF16 rounding touches only the non-equilibrium part, which is
// zero for tau = 1 in Stokes flow (the collision then returns the
// equilibrium exactly).  Collision arithmetic is FP32; sums are FP64.
//
// Traffic per node update: 15 x 2 B deviations read and written, one float4
// of moments read and one written (94 B with the flag word, against 120 B
// for FP32 populations).
#include <cuda_bf16.h>

#include "slbc_internal.cuh"
#include "slbc_kernels.cuh"
#include "slbc_mp.cuh"

namespace slbc {

typedef __nv_bfloat16 bf16;

struct Bf16Args {
  bf16 *D;
  long long npad;
  const uint16_t *flags;
  int esi, esj, esk;
  const float4 *Min;   // moments of the current state
  float4 *Mout;        // moments written by a step
  float scale, inv;    // stored = scale * deviation
};

// equilibrium population q of moments (drho, ru): the rebuild with zero stress
__device__ __forceinline__ float eq_pop(int q, float4 m) {
  const float rhobyb = m.x * (1.0f / 72.0f);
  const float erhobyb = 8.0f * rhobyb;
  switch (q) {
    case 0: return 2.0f * erhobyb;
    case 1: return erhobyb + (8.0f / 24.0f) * m.y;
    case 2: return erhobyb - (8.0f / 24.0f) * m.y;
    case 3: return erhobyb + (8.0f / 24.0f) * m.z;
    case 4: return erhobyb - (8.0f / 24.0f) * m.z;
    case 5: return erhobyb + (8.0f / 24.0f) * m.w;
    case 6: return erhobyb - (8.0f / 24.0f) * m.w;
    default: {
      const float cu = (CX(q) > 0 ? m.y : -m.y) + (CY(q) > 0 ? m.z : -m.z) + (CZ(q) > 0 ? m.w : -m.w);
      return rhobyb + (1.0f / 24.0f) * cu;
    }
  }
}

__device__ __forceinline__ float dev_load(const Bf16Args &a, int slot, int node) {
  return __bfloat162float(a.D[slot * a.npad + node]) * a.inv;
}

// post-collision population q of node x, reconstructed, in a given layout
__device__ __forceinline__ float bf_post(const Bf16Args &a, int layout, int q, int x, uint16_t fl,
                                         const Nbr &nb, float4 mx) {
  float d;
  if (layout == SLBC_LAYOUT_N) d = dev_load(a, q, x);
  else if (layout == SLBC_LAYOUT_C0 || q == 0 || ((fl >> OPP(q)) & 1)) d = dev_load(a, OPP(q), x);
  else d = dev_load(a, q, nb.at(CX(q), CY(q), CZ(q)));
  return eq_pop(q, mx) + d;
}

// The fused step of k_step for deviation storage (same pull rule, same AA
// layouts); also writes the new moments.
//
// Every population is reconstructed with the moments of the node that
// produced it, so a node reads the moments of its 14 neighbours.  A block of
// 32 (k) x 8 (j) threads marches along i over `planes` planes and keeps the
// moments of three consecutive planes, with a one-node halo, in shared
// memory; the plane after next is fetched into registers while the current
// one is updated.  Moments then cross L2 about 1.7 times per node instead of
// 15 times.
template <bool ODD, bool MOVING, bool BFU>
__global__ void __launch_bounds__(kTileThreads, 4) k_step_bf16(Bf16Args a, StepArgs<float> s, int planes) {
  __shared__ float4 ring[3][kPlane];
  const int tk = threadIdx.x, tj = threadIdx.y, tid = tj * kTileK + tk;
  const int k0 = blockIdx.x * kTileK, j0 = blockIdx.y * kTileJ, i0 = blockIdx.z * planes;
  const int np = min(planes, a.esi - i0);
  const int plane_nodes = a.esj * a.esk;
  // offsets within a plane of this thread's share of the halo tile (wrapped)
  int off[kPlaneLoads];
#pragma unroll
  for (int e = 0; e < kPlaneLoads; e++) {
    const int c = tid + kTileThreads * e;
    off[e] = c < kPlane ? wrap_index(j0 - 1 + c / kHaloK, a.esj) * a.esk + wrap_index(k0 - 1 + c % kHaloK, a.esk)
                        : -1;
  }
  // plane p sits in ring slot (p - i0 + 1) % 3
  float4 pre[kPlaneLoads];
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int base = wrap_index(i0 - 1 + h, a.esi) * plane_nodes;
#pragma unroll
    for (int e = 0; e < kPlaneLoads; e++)
      if (off[e] >= 0) ring[h][tid + kTileThreads * e] = __ldg(a.Min + base + off[e]);
  }
  {
    const int base = wrap_index(i0 + 1, a.esi) * plane_nodes;
#pragma unroll
    for (int e = 0; e < kPlaneLoads; e++)
      if (off[e] >= 0) pre[e] = __ldg(a.Min + base + off[e]);
  }
  const long long S = a.npad;
  for (int ii = 0; ii < np; ii++) {
    const int i = i0 + ii;
    const int sm = ii % 3, s0 = (ii + 1) % 3, sp = (ii + 2) % 3;  // planes i-1, i, i+1
    __syncthreads();  // slot sp held plane i-2, last read in the previous iteration
#pragma unroll
    for (int e = 0; e < kPlaneLoads; e++)
      if (off[e] >= 0) ring[sp][tid + kTileThreads * e] = pre[e];
    __syncthreads();
    if (ii + 1 < np) {
      const int base = wrap_index(i + 2, a.esi) * plane_nodes;
#pragma unroll
      for (int e = 0; e < kPlaneLoads; e++)
        if (off[e] >= 0) pre[e] = __ldg(a.Min + base + off[e]);
    }
    const int j = j0 + tj, k = k0 + tk;
    if (j >= a.esj || k >= a.esk) continue;
    const float4 *P[3] = {ring[sm], ring[s0], ring[sp]};
    const int c0 = (tj + 1) * kHaloK + tk + 1;
    const Nbr nb = make_nbr(i, j, k, a.esi, a.esj, a.esk);
    const int x = nb.at(0, 0, 0);
    const uint16_t fl = __ldg(a.flags + x);
    const bool solid = (fl & FLAG_SOLID) != 0;
    const float4 mx = P[1][c0];
    // Branch-free selection of each population's cell and producer moments,
    // so that all 15 loads are in flight together.  A bounce-back link
    // (bit q) returns the node's own post-collision opp(q), held in slot q
    // of x in both C0 and C1; its equilibrium eq_opp(q)(m) is eq_q of m with
    // the momentum negated (exact: only signs change).  Otherwise the
    // population was produced by y = x - c_q.
    const float4 mneg = make_float4(mx.x, -mx.y, -mx.z, -mx.w);
    float t[15];
    t[0] = eq_pop(0, mx) + dev_load(a, 0, x);
#pragma unroll
    for (int q = 1; q < 15; q++) {
      const bool bnd = (fl >> q) & 1;
      const float4 my = P[1 - CX(q)][c0 - CY(q) * kHaloK - CZ(q)];
      const float4 m = bnd ? mneg : my;
      int src = x, slot = q;
      if (ODD) {
        src = bnd ? x : nb.at(-CX(q), -CY(q), -CZ(q));
        slot = bnd ? q : OPP(q);
      }
      t[q] = eq_pop(q, m) + dev_load(a, slot, src);
    }
    if (MOVING && (fl & FLAG_LINKS)) apply_wall<float>(t, fl, solid, nb, x, s.uw, s.p.npad);
    if (!(s.skip_solid && solid)) {
      float bx = s.bfx, by = s.bfy, bz = s.bfz;
      if (!BFU) { bx = s.bf[x]; by = s.bf[s.p.npad + x]; bz = s.bf[2 * s.p.npad + x]; }
      collide<float, false>(t, s.omega, s.comega, s.rho0, s.stokes, !solid, bx, by, bz);
    }
    // moments of the post-collision populations (the collision conserves
    // drho and sets ru; summing keeps skipped solid nodes exact too)
    float4 mo;
    {
      const float p12 = t[1] + t[2], p34 = t[3] + t[4], p56 = t[5] + t[6];
      const float lo = t[7] + t[8] + t[9] + t[10], hi = t[11] + t[12] + t[13] + t[14];
      mo.x = t[0] + p12 + p34 + p56 + lo + hi;
      mo.y = t[1] - t[2] + (t[7] - t[8] + t[9] - t[10]) + (t[11] - t[12] + t[13] - t[14]);
      mo.z = t[3] - t[4] + (t[7] + t[8] - t[9] - t[10]) + (t[11] + t[12] - t[13] - t[14]);
      mo.w = t[5] - t[6] + lo - hi;
    }
    a.Mout[x] = mo;
    if (!ODD) {
#pragma unroll
      for (int q = 0; q < 15; q++)
        a.D[OPP(q) * S + x] = __float2bfloat16_rn((t[q] - eq_pop(q, mo)) * a.scale);
    } else {
      a.D[x] = __float2bfloat16_rn((t[0] - eq_pop(0, mo)) * a.scale);
#pragma unroll
      for (int q = 1; q < 15; q++) {
        const bool bnd = (fl >> OPP(q)) & 1;
        const int dst = bnd ? x : nb.at(CX(q), CY(q), CZ(q));
        const int slot = bnd ? OPP(q) : q;
        a.D[slot * S + dst] = __float2bfloat16_rn((t[q] - eq_pop(q, mo)) * a.scale);
      }
    }
  }
}

// populations (host AoS staging, FP64) -> moments + deviations, layout N
__global__ void k_put_bf16(Bf16Args a, const double *stage, long long x0, long long n) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const long long x = x0 + e;
  float t[15];
#pragma unroll
  for (int q = 0; q < 15; q++) t[q] = (float)stage[15 * e + q];
  float4 m;
  const float lo = t[7] + t[8] + t[9] + t[10], hi = t[11] + t[12] + t[13] + t[14];
  m.x = t[0] + (t[1] + t[2]) + (t[3] + t[4]) + (t[5] + t[6]) + lo + hi;
  m.y = t[1] - t[2] + (t[7] - t[8] + t[9] - t[10]) + (t[11] - t[12] + t[13] - t[14]);
  m.z = t[3] - t[4] + (t[7] + t[8] - t[9] - t[10]) + (t[11] + t[12] - t[13] - t[14]);
  m.w = t[5] - t[6] + lo - hi;
  a.Mout[x] = m;
#pragma unroll
  for (int q = 0; q < 15; q++) a.D[q * a.npad + x] = __float2bfloat16_rn((t[q] - eq_pop(q, m)) * a.scale);
}

// any layout -> host AoS staging of the reference's array
__global__ void k_get_bf16(Bf16Args a, int layout, double *stage, long long x0, long long n) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int x = (int)(x0 + e);
  int i, j, k;
  decode(x, a.esj, a.esk, i, j, k);
  const Nbr nb = make_nbr(i, j, k, a.esi, a.esj, a.esk);
  const uint16_t fl = a.flags[x];
  const float4 mx = a.Min[x];
#pragma unroll
  for (int q = 0; q < 15; q++) stage[15 * e + q] = (double)bf_post(a, layout, q, x, fl, nb, mx);
}

// N <-> C0 slot swap of the deviations
__global__ void k_swap_bf16(Bf16Args a, long long n) {
  const long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= n) return;
#pragma unroll
  for (int q = 1; q < 15; q++) {
    if (OPP(q) < q) continue;
    const bf16 u = a.D[q * a.npad + x], v = a.D[OPP(q) * a.npad + x];
    a.D[q * a.npad + x] = v;
    a.D[OPP(q) * a.npad + x] = u;
  }
}

// mean-flow sums straight from the moments: u = (ru + fac*b) / (rho0 + drho)
__global__ void __launch_bounds__(kReduceThreads)
k_vsum_bf16(Bf16Args a, double rho0, double fac, int bf_uniform, double b0, double b1, double b2,
            const float *bf, const double *psi, double *partials) {
  Acc<float> ax, ay, az;
  double wsum = 0.0;
  int count = 0;
  const long long n = (long long)a.esi * a.esj * a.esk;
  const long long chunk = (n + gridDim.x - 1) / gridDim.x;
  const long long lo = (long long)blockIdx.x * chunk;
  const long long hi = lo + chunk < n ? lo + chunk : n;
  const float tf = (float)fac;
  for (long long e = lo + threadIdx.x; e < hi; e += blockDim.x) {
    const int x = (int)e;
    if (a.flags[x] & FLAG_SOLID) continue;
    const float4 m = a.Min[x];
    float bx = (float)b0, by = (float)b1, bz = (float)b2;
    if (!bf_uniform) { bx = bf[x]; by = bf[a.npad + x]; bz = bf[2 * a.npad + x]; }
    const float rinv = 1.0f / ((float)rho0 + m.x);
    const float ux = (m.y + tf * bx) * rinv, uy = (m.z + tf * by) * rinv, uz = (m.w + tf * bz) * rinv;
    if (psi) {
      const double w = psi[x] * psi[x];
      ax.add((float)(w * ux)); ay.add((float)(w * uy)); az.add((float)(w * uz));
      wsum += w;
    } else {
      ax.add(ux); ay.add(uy); az.add(uz);
    }
    count++;
  }
  double v[5] = {ax.value(), ay.value(), az.value(), psi ? wsum : (double)count, (double)count};
  block_sum<5>(v);
  if (threadIdx.x == 0)
    for (int c = 0; c < 5; c++) partials[5 * blockIdx.x + c] = v[c];
}

// node forces of one bblforce from reconstructed populations (FP32 terms,
// compensated sums, FP64 store)
__global__ void k_force_bf16(Bf16Args a, int layout, int moving, const float *uw, ForceArgs f) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= f.nbnd) return;
  const int s = f.bnd_node[e];
  int i, j, k;
  decode(s, a.esj, a.esk, i, j, k);
  const Nbr nb = make_nbr(i, j, k, a.esi, a.esj, a.esk);
  const uint16_t fl = a.flags[s];
  const float4 ms = a.Min[s];
  Acc<float> ax, ay, az;
  float ux = 0.f, uy = 0.f, uz = 0.f;
  if (moving) { ux = uw[s]; uy = uw[a.npad + s]; uz = uw[2 * a.npad + s]; }
#pragma unroll
  for (int q = 1; q < 15; q++) {
    if (!((fl >> OPP(q)) & 1)) continue;
    const int n = nb.at(CX(q), CY(q), CZ(q));
    const float4 mn = a.Min[n];
    float av, bv;
    if (layout == SLBC_LAYOUT_N) {
      av = eq_pop(q, ms) + dev_load(a, q, s);
      bv = eq_pop(OPP(q), mn) + dev_load(a, OPP(q), n);
    } else {
      av = eq_pop(q, ms) + dev_load(a, OPP(q), s);
      bv = eq_pop(OPP(q), mn) + dev_load(a, q, n);
    }
    float dp = av - bv;
    if (moving) dp -= link_term<float>(q, ux, uy, uz);
    dp *= 2.f;
    if (CX(q) != 0) ax.add(CX(q) > 0 ? dp : -dp);
    if (CY(q) != 0) ay.add(CY(q) > 0 ? dp : -dp);
    if (CZ(q) != 0) az.add(CZ(q) > 0 ? dp : -dp);
  }
  f.f[e] += ax.value(); f.f[f.nbnd + e] += ay.value(); f.f[2 * f.nbnd + e] += az.value();
}

// velocity warm start: rebuild from (rho, u) (reference src/lbstore.c:352-399)
__global__ void k_setvel_bf16(Bf16Args a, const double *stage, long long x0, long long n, int has_rho,
                              double rho0, int stokes, int skip_solid) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const long long x = x0 + e;
  float t[15];
  float4 m = make_float4(0.f, 0.f, 0.f, 0.f);
  if (!(skip_solid && (a.flags[x] & FLAG_SOLID))) {
    const float r = has_rho ? (float)stage[4 * e] : (float)rho0;
    const float vx = (float)stage[4 * e + 1], vy = (float)stage[4 * e + 2], vz = (float)stage[4 * e + 3];
    const float drho = r - (float)rho0, rux = r * vx, ruy = r * vy, ruz = r * vz;
    float sxx = 0.f, syy = 0.f, szz = 0.f, sxy = 0.f, sxz = 0.f, syz = 0.f;
    if (!stokes) {
      sxx = vx * rux; sxy = vx * ruy; sxz = vx * ruz;
      syy = vy * ruy; syz = vy * ruz; szz = vz * ruz;
    }
    rebuild<float, false>(t, drho, rux, ruy, ruz, sxx, syy, szz, sxy, sxz, syz);
    m = make_float4(drho, rux, ruy, ruz);
  } else {
#pragma unroll
    for (int q = 0; q < 15; q++) t[q] = 0.f;
  }
  a.Mout[x] = m;
#pragma unroll
  for (int q = 0; q < 15; q++) a.D[q * a.npad + x] = __float2bfloat16_rn((t[q] - eq_pop(q, m)) * a.scale);
}

// collision of layout N in place (after an upload or a velocity warm start):
// reconstruct, collide, store moments and deviations again
template <bool BFU>
__global__ void k_collide_bf16(Bf16Args a, StepArgs<float> s) {
  const long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= (long long)a.esi * a.esj * a.esk) return;
  const bool solid = (a.flags[x] & FLAG_SOLID) != 0;
  if (s.skip_solid && solid) return;
  float4 m = a.Min[x];
  float t[15];
#pragma unroll
  for (int q = 0; q < 15; q++) t[q] = eq_pop(q, m) + dev_load(a, q, (int)x);
  float bx = s.bfx, by = s.bfy, bz = s.bfz;
  if (!BFU) { bx = s.bf[x]; by = s.bf[s.p.npad + x]; bz = s.bf[2 * s.p.npad + x]; }
  collide<float, false>(t, s.omega, s.comega, s.rho0, s.stokes, !solid, bx, by, bz);
  const float lo = t[7] + t[8] + t[9] + t[10], hi = t[11] + t[12] + t[13] + t[14];
  m.x = t[0] + (t[1] + t[2]) + (t[3] + t[4]) + (t[5] + t[6]) + lo + hi;
  m.y = t[1] - t[2] + (t[7] - t[8] + t[9] - t[10]) + (t[11] - t[12] + t[13] - t[14]);
  m.z = t[3] - t[4] + (t[7] + t[8] - t[9] - t[10]) + (t[11] + t[12] - t[13] - t[14]);
  m.w = t[5] - t[6] + lo - hi;
  ((float4 *)a.Min)[x] = m;
#pragma unroll
  for (int q = 0; q < 15; q++) a.D[q * a.npad + x] = __float2bfloat16_rn((t[q] - eq_pop(q, m)) * a.scale);
}

// density snapshot of the tracer: rho0 + drho on fluid nodes
__global__ void k_mp_rhoinit_bf16(Bf16Args a, double rho0, double *rho64, float *rho32) {
  const long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= (long long)a.esi * a.esj * a.esk) return;
  double r = rho0;
  if (!(a.flags[x] & FLAG_SOLID)) r = rho0 + (double)a.Min[x].x;
  rho64[x] = r;
  if (rho32) rho32[x] = (float)r;
}

// ---- launchers ---------------------------------------------------------------

static Bf16Args bf_args(Lattice &L) {
  Bf16Args a;
  a.D = (bf16 *)L.pop;
  a.npad = L.npad;
  a.flags = L.flags;
  a.esi = L.esi; a.esj = L.esj; a.esk = L.esk;
  a.Min = (const float4 *)L.mom[L.mom_cur];
  a.Mout = (float4 *)L.mom[1 - L.mom_cur];
  a.scale = (float)L.bf16_scale;
  a.inv = (float)(1.0 / L.bf16_scale);
  return a;
}

static StepArgs<float> step_args_f(Lattice &L) {
  StepArgs<float> s;
  s.p.pop = nullptr; s.p.npad = L.npad; s.p.flags = L.flags;
  s.p.esi = L.esi; s.p.esj = L.esj; s.p.esk = L.esk;
  const double omega = 1.0 / L.par.tau;
  s.omega = (float)omega; s.comega = (float)(1.0 - omega); s.rho0 = (float)L.par.rho0;
  s.stokes = L.par.stokes_flow; s.skip_solid = L.par.skip_solid;
  s.moving = L.par.objects_moving && L.uw != nullptr;
  s.bf_uniform = L.bf_uniform;
  s.bfx = (float)L.bf_const[0]; s.bfy = (float)L.bf_const[1]; s.bfz = (float)L.bf_const[2];
  s.bf = (const float *)L.bf; s.uw = (const float *)L.uw;
  return s;
}

static int fblocks(long long n, int bs) { return (int)((n + bs - 1) / bs); }

template <bool ODD>
static void bf_step(Lattice &L, const Bf16Args &a, const StepArgs<float> &s, dim3 g, int planes) {
  const dim3 b(kTileK, kTileJ);
  if (s.moving) {
    if (s.bf_uniform) k_step_bf16<ODD, true, true><<<g, b, 0, L.stream>>>(a, s, planes);
    else k_step_bf16<ODD, true, false><<<g, b, 0, L.stream>>>(a, s, planes);
  } else {
    if (s.bf_uniform) k_step_bf16<ODD, false, true><<<g, b, 0, L.stream>>>(a, s, planes);
    else k_step_bf16<ODD, false, false><<<g, b, 0, L.stream>>>(a, s, planes);
  }
}

// planes per block: the tuned value (npt field of the parity's StepConfig),
// else the largest of 1..8 that still gives about four blocks per SM
int bf16_default_planes(const Lattice &L) {
  const long long tiles = (long long)((L.esk + kTileK - 1) / kTileK) * ((L.esj + kTileJ - 1) / kTileJ);
  int p = 8;
  while (p > 1 && tiles * ((L.esi + p - 1) / p) < 152 * 4) p /= 2;
  return p;
}

cudaError_t launch_step_bf16(Lattice &L, int odd) {
  int planes = L.tuned[odd ? 1 : 0].npt;
  if (planes <= 0) planes = bf16_default_planes(L);
  const dim3 g((unsigned)((L.esk + kTileK - 1) / kTileK), (unsigned)((L.esj + kTileJ - 1) / kTileJ),
               (unsigned)((L.esi + planes - 1) / planes));
  const Bf16Args a = bf_args(L);
  const StepArgs<float> s = step_args_f(L);
  if (odd) bf_step<true>(L, a, s, g, planes);
  else bf_step<false>(L, a, s, g, planes);
  count_launch();
  L.mom_cur = 1 - L.mom_cur;
  return cudaGetLastError();
}

cudaError_t launch_put_bf16(Lattice &L, const double *stage, long long x0, long long n) {
  Bf16Args a = bf_args(L);
  a.Mout = (float4 *)L.mom[L.mom_cur];  // defines the current state
  k_put_bf16<<<fblocks(n, 256), 256, 0, L.stream>>>(a, stage, x0, n);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_get_bf16(Lattice &L, double *stage, long long x0, long long n) {
  k_get_bf16<<<fblocks(n, 256), 256, 0, L.stream>>>(bf_args(L), L.layout, stage, x0, n);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_swap_bf16(Lattice &L) {
  k_swap_bf16<<<fblocks(L.nnodes, 256), 256, 0, L.stream>>>(bf_args(L), L.nnodes);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_vsum_bf16(Lattice &L, double fac, const double *psi, double *partials, int nblocks) {
  k_vsum_bf16<<<nblocks, kReduceThreads, 0, L.stream>>>(bf_args(L), L.par.rho0, fac, L.bf_uniform,
                                                         L.bf_const[0], L.bf_const[1], L.bf_const[2],
                                                         (const float *)L.bf, psi, partials);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_force_bf16(Lattice &L) {
  if (L.nbnd == 0) return cudaSuccess;
  ForceArgs f{L.nbnd, L.bnd_node, L.bnd_f};
  const int moving = L.par.objects_moving && L.uw != nullptr;
  k_force_bf16<<<fblocks(L.nbnd, 128), 128, 0, L.stream>>>(bf_args(L), L.layout, moving,
                                                           (const float *)L.uw, f);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_setvel_bf16(Lattice &L, const double *stage, long long x0, long long n, int has_rho,
                               int skip_solid) {
  Bf16Args a = bf_args(L);
  a.Mout = (float4 *)L.mom[L.mom_cur];
  k_setvel_bf16<<<fblocks(n, 256), 256, 0, L.stream>>>(a, stage, x0, n, has_rho, L.par.rho0,
                                                       L.par.stokes_flow, skip_solid);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_collide_bf16(Lattice &L) {
  const StepArgs<float> s = step_args_f(L);
  if (s.bf_uniform) k_collide_bf16<true><<<fblocks(L.nnodes, 256), 256, 0, L.stream>>>(bf_args(L), s);
  else k_collide_bf16<false><<<fblocks(L.nnodes, 256), 256, 0, L.stream>>>(bf_args(L), s);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_mp_rhoinit_bf16(Lattice &L) {
  k_mp_rhoinit_bf16<<<fblocks(L.nnodes, 256), 256, 0, L.stream>>>(bf_args(L), L.par.rho0, L.mp_rho64,
                                                                  L.mp_rho32);
  count_launch();
  return cudaGetLastError();
}

}  // namespace slbc
