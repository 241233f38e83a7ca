// BF16 paired-deviation populations.
//
// A collision rebuilds the 15 populations of a node from its density
// deviation, momentum and relaxed stress (reference src/lbkernel.c:838-865).
// The rebuild is linear, so a post-collision population a_q minus the
// zero-stress rebuild eq_q of the same (drho, ru) is the stress part of the
// rebuild alone, and that part is even in c_q: a_q and a_opp(q) carry the
// same deviation.  A node's post-collision state is therefore held as
//   M[x]    = (drho, rux, ruy, ruz), FP32, one float4;
//   P[x][p] = BF16 of scale * (a_q - eq_q(M[x])) for the 8 pairs
//             p = pair_of(q): {0}, {1,2}, {3,4}, {5,6}, {7,14}, {8,13},
//             {9,12}, {10,11}; one 16-byte vector;
// 32 bytes per node, in two copies: a step reads one and writes the other.
// A population is a_q(x) = eq_q(M[x]) + P[x][pair_of(q)] / scale.  The
// equilibrium part keeps FP32 precision; BF16 rounding touches only the
// stress part, which is zero at tau = 1 in Stokes flow.
//
// The state is always the reference's post-collision array: a step gathers
// a_q(x) from the state of x - c_q, or of x itself over a bounce-back link,
// and writes the new state of x.  Two kinds of state cannot be held this
// way, and the host moves such a lattice to FP32: solid nodes that are not
// relaxed (skip_solid), whose streamed populations are not paired, and
// uploaded populations whose deviations are not paired.
//
// Traffic per node update: 32 B of state read and 32 B written, plus the
// 2-byte flag word (FP32 populations: 120 B of state).
#include <cuda_bf16.h>

#include "slbc_internal.cuh"
#include "slbc_kernels.cuh"
#include "slbc_mp.cuh"

namespace slbc {

struct PairArgs {
  const uint4 *Pin;    // paired deviations of the current state
  uint4 *Pout;         // ... written by a step
  const float4 *Min;   // moments of the current state
  float4 *Mout;        // ... written by a step
  const uint16_t *flags;
  long long npad;
  int esi, esj, esk;
  float scale, inv;    // stored = scale * deviation
};

// pair of direction q: q and opp(q) share one stored deviation
__host__ __device__ constexpr int pair_of(int q) {
  return q == 0 ? 0 : (q <= 6 ? (q + 1) / 2 : (q <= 10 ? q - 3 : 18 - q));
}
static_assert(pair_of(7) == pair_of(OPP(7)) && pair_of(8) == pair_of(OPP(8)) && pair_of(9) == pair_of(OPP(9)) &&
                  pair_of(10) == pair_of(OPP(10)) && pair_of(1) == pair_of(OPP(1)) &&
                  pair_of(3) == pair_of(OPP(3)) && pair_of(5) == pair_of(OPP(5)),
              "pairs must join opposite directions");

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

// stored deviation of pair p in a packed vector
__device__ __forceinline__ float pair_dev(const uint4 &v, int p) {
  const uint32_t w = p < 2 ? v.x : (p < 4 ? v.y : (p < 6 ? v.z : v.w));
  return (p & 1) ? __uint_as_float(w & 0xffff0000u) : __uint_as_float(w << 16);
}

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&h);
}

// Stored deviations of a collided node: the stress part of the rebuild,
// pair by pair (trace part, then the diagonal and mixed stress terms).
__device__ __forceinline__ uint4 pack_stress(const Relaxed<float> &r, float scale) {
  const float tr = (r.sxx + r.syy + r.szz) * (1.0f / 3.0f);
  const float h = 0.5f * scale, e = 0.125f * scale;
  uint4 v;
  v.x = pack2(-tr * scale, h * (r.sxx - tr));
  v.y = pack2(h * (r.syy - tr), h * (r.szz - tr));
  v.z = pack2(e * (tr + r.sxy + r.sxz + r.syz), e * (tr - r.sxy - r.sxz + r.syz));
  v.w = pack2(e * (tr - r.sxy + r.sxz - r.syz), e * (tr + r.sxy - r.sxz - r.syz));
  return v;
}

// post-collision population q of node x
__device__ __forceinline__ float bf_post(const PairArgs &a, int q, long long x) {
  return eq_pop(q, a.Min[x]) + pair_dev(a.Pin[x], pair_of(q)) * a.inv;
}


// The 15 post-collision populations of a node from its state (the same
// operations as eq_pop, so that every kernel reconstructs the same values).
__device__ __forceinline__ void decode_state(float4 m, uint4 v, float inv, float (&a)[15]) {
  const float rhobyb = m.x * (1.0f / 72.0f);
  const float erhobyb = 8.0f * rhobyb;
  const float d0 = __uint_as_float(v.x << 16) * inv, d1 = __uint_as_float(v.x & 0xffff0000u) * inv;
  const float d2 = __uint_as_float(v.y << 16) * inv, d3 = __uint_as_float(v.y & 0xffff0000u) * inv;
  const float d4 = __uint_as_float(v.z << 16) * inv, d5 = __uint_as_float(v.z & 0xffff0000u) * inv;
  const float d6 = __uint_as_float(v.w << 16) * inv, d7 = __uint_as_float(v.w & 0xffff0000u) * inv;
  a[0] = 2.0f * erhobyb + d0;
  a[1] = (erhobyb + (8.0f / 24.0f) * m.y) + d1;
  a[2] = (erhobyb - (8.0f / 24.0f) * m.y) + d1;
  a[3] = (erhobyb + (8.0f / 24.0f) * m.z) + d2;
  a[4] = (erhobyb - (8.0f / 24.0f) * m.z) + d2;
  a[5] = (erhobyb + (8.0f / 24.0f) * m.w) + d3;
  a[6] = (erhobyb - (8.0f / 24.0f) * m.w) + d3;
#pragma unroll
  for (int q = 7; q < 15; q++) a[q] = eq_pop(q, m) + (q == 7 || q == 14 ? d4 : q == 8 || q == 13 ? d5
                                                           : q == 9 || q == 12 ? d6 : d7);
}

constexpr int kPairSlots = 3;  // decoded planes i-1, i, i+1
constexpr int kPairSmem = kPairSlots * 15 * kPlane * (int)sizeof(float);

// The fused update of k_step (same pull rule) on paired-deviation storage.
// A block of 32 (k) x 8 (j) threads marches along i over `planes` planes.
// The populations of three consecutive planes, with a one-node halo, sit
// decoded (FP32, 15 per node, direction-major) in shared memory; the state
// of the plane after them is loaded into registers one plane ahead and
// decoded into the ring when its slot frees up.  A node gathers each of its
// 15 populations with one 4-byte shared load whose address the bounce-back
// bit selects (upstream node y = x - c_q, direction q; or x itself,
// direction opp(q)), and writes its new state with two 16-byte stores.
template <bool MOVING, bool BFU>
__global__ void __launch_bounds__(kTileThreads, 3) k_step_pair(PairArgs a, StepArgs<float> s, int planes) {
  extern __shared__ __align__(16) float dec[];  // [slot][q][kPlane]
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
  float4 pm[kPlaneLoads];
  uint4 pp[kPlaneLoads];
  auto prefetch = [&](int plane) {
    const long long base = (long long)wrap_index(plane, a.esi) * plane_nodes;
#pragma unroll
    for (int e = 0; e < kPlaneLoads; e++)
      if (off[e] >= 0) { pm[e] = __ldcs(a.Min + base + off[e]); pp[e] = __ldcs(a.Pin + base + off[e]); }
  };
  auto decode_into = [&](int slot) {
#pragma unroll
    for (int e = 0; e < kPlaneLoads; e++) {
      if (off[e] < 0) continue;
      float v[15];
      decode_state(pm[e], pp[e], a.inv, v);
      const int c = tid + kTileThreads * e;
#pragma unroll
      for (int q = 0; q < 15; q++) dec[(slot * 15 + q) * kPlane + c] = v[q];
    }
  };
  // plane p sits in ring slot (p - i0 + 1) % 3
  prefetch(i0 - 1);
  decode_into(0);
  prefetch(i0);
  decode_into(1);
  prefetch(i0 + 1);
  const int j = j0 + tj, k = k0 + tk;
  const bool mine = j < a.esj && k < a.esk;
  const int own = mine ? j * a.esk + k : 0;
  const int c0 = (tj + 1) * kHaloK + tk + 1;
  uint16_t fl_next = __ldg(a.flags + (long long)i0 * plane_nodes + own);  // flag word, one plane ahead
  for (int ii = 0; ii < np; ii++) {
    const int i = i0 + ii;
    const uint16_t fl = fl_next;
    if (ii + 1 < np) fl_next = __ldg(a.flags + (long long)(i + 1) * plane_nodes + own);
    __syncthreads();  // the slot of plane i-2 was last read in the previous iteration
    decode_into((ii + 2) % kPairSlots);
    __syncthreads();
    if (ii + 1 < np) prefetch(i + 2);
    if (!mine) continue;
    const float *D[3] = {dec + (ii % kPairSlots) * 15 * kPlane, dec + ((ii + 1) % kPairSlots) * 15 * kPlane,
                         dec + ((ii + 2) % kPairSlots) * 15 * kPlane};
    const int x = i * plane_nodes + own;
    const bool solid = (fl & FLAG_SOLID) != 0;
    float t[15];
    t[0] = D[1][c0];
#pragma unroll
    for (int q = 1; q < 15; q++) {
      // over a bounce-back link the node's own post-collision opp(q) comes
      // back; otherwise the population q of y = x - c_q arrives
      const bool bnd = (fl >> q) & 1;
      const float *src = bnd ? D[1] + OPP(q) * kPlane + c0
                             : D[1 - CX(q)] + q * kPlane + (c0 - CY(q) * kHaloK - CZ(q));
      t[q] = *src;
    }
    if (MOVING && (fl & FLAG_LINKS)) {
      const Nbr nb = make_nbr(i, j, k, a.esi, a.esj, a.esk);
      apply_wall<float>(t, fl, solid, nb, x, s.uw, s.p.npad);
    }
    float bx = s.bfx, by = s.bfy, bz = s.bfz;
    if (!BFU) { bx = s.bf[x]; by = s.bf[s.p.npad + x]; bz = s.bf[2 * s.p.npad + x]; }
    const Relaxed<float> r = relax<float>(t, s.omega, s.comega, s.rho0, s.stokes, !solid, bx, by, bz);
    a.Mout[x] = make_float4(r.drho, r.rux, r.ruy, r.ruz);
    a.Pout[x] = pack_stress(r, a.scale);
  }
}

// populations (host AoS staging, FP64) -> moments + paired deviations; a
// node whose deviations differ within a pair by more than the BF16
// rounding of the larger, or than 2^-20 of the two populations, is counted
// in *unpaired (the host then keeps the lattice in FP32)
__global__ void k_put_pair(PairArgs a, const double *stage, long long x0, long long n, int *unpaired) {
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
  float d[8];
  d[0] = t[0] - eq_pop(0, m);
  bool paired = true;
#pragma unroll
  for (int q = 1; q < 15; q++) {
    if (OPP(q) < q) continue;
    const float u = t[q] - eq_pop(q, m), v = t[OPP(q)] - eq_pop(OPP(q), m);
    const float tol = fmaxf(0x1p-9f * fmaxf(fabsf(u), fabsf(v)), 0x1p-20f * (fabsf(t[q]) + fabsf(t[OPP(q)])));
    if (fabsf(u - v) > tol) paired = false;
    d[pair_of(q)] = 0.5f * (u + v);
  }
  if (!paired) atomicAdd(unpaired, 1);
  a.Mout[x] = m;
  uint4 v;
  v.x = pack2(d[0] * a.scale, d[1] * a.scale);
  v.y = pack2(d[2] * a.scale, d[3] * a.scale);
  v.z = pack2(d[4] * a.scale, d[5] * a.scale);
  v.w = pack2(d[6] * a.scale, d[7] * a.scale);
  a.Pout[x] = v;
}

// state -> host AoS staging of the reference's array
__global__ void k_get_pair(PairArgs a, double *stage, long long x0, long long n) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const long long x = x0 + e;
#pragma unroll
  for (int q = 0; q < 15; q++) stage[15 * e + q] = (double)bf_post(a, q, x);
}

// mean-flow sums straight from the moments: u = (ru + fac*b) / (rho0 + drho)
__global__ void __launch_bounds__(kReduceThreads)
k_vsum_pair(PairArgs a, double rho0, double fac, int bf_uniform, double b0, double b1, double b2,
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
__global__ void k_force_pair(PairArgs a, int moving, const float *uw, ForceArgs f) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= f.nbnd) return;
  const int s = f.bnd_node[e];
  int i, j, k;
  decode(s, a.esj, a.esk, i, j, k);
  const Nbr nb = make_nbr(i, j, k, a.esi, a.esj, a.esk);
  const uint16_t fl = a.flags[s];
  Acc<float> ax, ay, az;
  float ux = 0.f, uy = 0.f, uz = 0.f;
  if (moving) { ux = uw[s]; uy = uw[a.npad + s]; uz = uw[2 * a.npad + s]; }
#pragma unroll
  for (int q = 1; q < 15; q++) {
    if (!((fl >> OPP(q)) & 1)) continue;
    const int n = nb.at(CX(q), CY(q), CZ(q));
    float dp = bf_post(a, q, s) - bf_post(a, OPP(q), n);
    if (moving) dp -= link_term<float>(q, ux, uy, uz);
    dp *= 2.f;
    if (CX(q) != 0) ax.add(CX(q) > 0 ? dp : -dp);
    if (CY(q) != 0) ay.add(CY(q) > 0 ? dp : -dp);
    if (CZ(q) != 0) az.add(CZ(q) > 0 ? dp : -dp);
  }
  f.f[e] += ax.value(); f.f[f.nbnd + e] += ay.value(); f.f[2 * f.nbnd + e] += az.value();
}

// velocity warm start: the rebuild from (rho, u) of reference
// src/lbstore.c:352-399, as moments and paired stress deviations
__global__ void k_setvel_pair(PairArgs a, const double *stage, long long x0, long long n, int has_rho,
                              double rho0, int stokes, int skip_solid) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const long long x = x0 + e;
  Relaxed<float> r{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (!(skip_solid && (a.flags[x] & FLAG_SOLID))) {  // else all populations zero
    // has_rho 1: stage[4e] is the density; 2: the deviation rho - rho0
    const float rho = has_rho == 2 ? (float)rho0 + (float)stage[4 * e] : has_rho ? (float)stage[4 * e] : (float)rho0;
    const float vx = (float)stage[4 * e + 1], vy = (float)stage[4 * e + 2], vz = (float)stage[4 * e + 3];
    r.drho = has_rho == 2 ? (float)stage[4 * e] : rho - (float)rho0;
    r.rux = rho * vx; r.ruy = rho * vy; r.ruz = rho * vz;
    if (!stokes) {
      r.sxx = vx * r.rux; r.sxy = vx * r.ruy; r.sxz = vx * r.ruz;
      r.syy = vy * r.ruy; r.syz = vy * r.ruz; r.szz = vz * r.ruz;
    }
  }
  a.Mout[x] = make_float4(r.drho, r.rux, r.ruy, r.ruz);
  a.Pout[x] = pack_stress(r, a.scale);
}

// collision of the current state in place (the separate collide phase)
template <bool BFU>
__global__ void k_collide_pair(PairArgs a, StepArgs<float> s) {
  const long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= (long long)a.esi * a.esj * a.esk) return;
  const bool solid = (a.flags[x] & FLAG_SOLID) != 0;
  float t[15];
#pragma unroll
  for (int q = 0; q < 15; q++) t[q] = bf_post(a, q, x);
  float bx = s.bfx, by = s.bfy, bz = s.bfz;
  if (!BFU) { bx = s.bf[x]; by = s.bf[s.p.npad + x]; bz = s.bf[2 * s.p.npad + x]; }
  const Relaxed<float> r = relax<float>(t, s.omega, s.comega, s.rho0, s.stokes, !solid, bx, by, bz);
  a.Mout[x] = make_float4(r.drho, r.rux, r.ruy, r.ruz);
  a.Pout[x] = pack_stress(r, a.scale);
}

// density snapshot of the tracer: rho0 + drho on fluid nodes
__global__ void k_mp_rhoinit_pair(PairArgs a, double rho0, double *rho64, float *rho32) {
  const long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= (long long)a.esi * a.esj * a.esk) return;
  double r = rho0;
  if (!(a.flags[x] & FLAG_SOLID)) r = rho0 + (double)a.Min[x].x;
  rho64[x] = r;
  if (rho32) rho32[x] = (float)r;
}

// ---- launchers ---------------------------------------------------------------

// current state: copy mom_cur; a step writes the other copy
static PairArgs pair_args(Lattice &L) {
  PairArgs a;
  const uint4 *P = (const uint4 *)L.pop;
  a.Pin = P + (size_t)L.mom_cur * L.npad;
  a.Pout = const_cast<uint4 *>(P + (size_t)(1 - L.mom_cur) * L.npad);
  a.Min = (const float4 *)L.mom[L.mom_cur];
  a.Mout = (float4 *)L.mom[1 - L.mom_cur];
  a.flags = L.flags;
  a.npad = L.npad;
  a.esi = L.esi; a.esj = L.esj; a.esk = L.esk;
  a.scale = (float)L.bf16_scale;
  a.inv = (float)(1.0 / L.bf16_scale);
  return a;
}

// the current state as both input and output (node-local kernels)
static PairArgs pair_args_inplace(Lattice &L) {
  PairArgs a = pair_args(L);
  a.Pout = const_cast<uint4 *>(a.Pin);
  a.Mout = const_cast<float4 *>(a.Min);
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

static const char *kSkipSolid =
    "BF16 paired-deviation storage relaxes solid nodes too: set skip_solid = 0 or use FP32 populations";

// planes per block: the largest of 1..8 that still gives about four blocks
// per SM
int bf16_default_planes(const Lattice &L) {
  const long long tiles = (long long)((L.esk + kTileK - 1) / kTileK) * ((L.esj + kTileJ - 1) / kTileJ);
  int p = 8;
  while (p > 1 && tiles * ((L.esi + p - 1) / p) < 152 * 4) p /= 2;
  return p;
}

// One update from the current state into the other copy; the caller swaps
// the copies (mom_cur).
cudaError_t launch_pair_step(Lattice &L, int planes) {
  if (L.par.skip_solid) {
    set_error(kSkipSolid);
    return cudaErrorInvalidValue;
  }
  const dim3 g((unsigned)((L.esk + kTileK - 1) / kTileK), (unsigned)((L.esj + kTileJ - 1) / kTileJ),
               (unsigned)((L.esi + planes - 1) / planes));
  const dim3 b(kTileK, kTileJ);
  const PairArgs a = pair_args(L);
  const StepArgs<float> s = step_args_f(L);
  // the decoded ring needs more than the default 48 KB of dynamic shared
  // memory: opt in once per device
  static unsigned long long attr_set = 0;  // bit = device index
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (!(attr_set >> (dev & 63) & 1ull)) {
    const void *fns[4] = {(const void *)k_step_pair<true, true>, (const void *)k_step_pair<true, false>,
                          (const void *)k_step_pair<false, true>, (const void *)k_step_pair<false, false>};
    for (const void *f : fns) {
      e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, kPairSmem);
      if (e != cudaSuccess) return e;
    }
    attr_set |= 1ull << (dev & 63);
  }
  if (s.moving) {
    if (s.bf_uniform) k_step_pair<true, true><<<g, b, kPairSmem, L.stream>>>(a, s, planes);
    else k_step_pair<true, false><<<g, b, kPairSmem, L.stream>>>(a, s, planes);
  } else {
    if (s.bf_uniform) k_step_pair<false, true><<<g, b, kPairSmem, L.stream>>>(a, s, planes);
    else k_step_pair<false, false><<<g, b, kPairSmem, L.stream>>>(a, s, planes);
  }
  count_launch();
  return cudaGetLastError();
}

// the state has one layout, so both parities run the same update
cudaError_t launch_step_bf16(Lattice &L, int /*odd*/) {
  int planes = L.tuned[0].npt;
  if (planes <= 0) planes = bf16_default_planes(L);
  const cudaError_t e = launch_pair_step(L, planes);
  if (e == cudaSuccess) L.mom_cur = 1 - L.mom_cur;
  return e;
}

cudaError_t launch_put_bf16(Lattice &L, const double *stage, long long x0, long long n, int *unpaired) {
  k_put_pair<<<fblocks(n, 256), 256, 0, L.stream>>>(pair_args_inplace(L), stage, x0, n, unpaired);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_get_bf16(Lattice &L, double *stage, long long x0, long long n) {
  k_get_pair<<<fblocks(n, 256), 256, 0, L.stream>>>(pair_args(L), stage, x0, n);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_vsum_bf16(Lattice &L, double fac, const double *psi, double *partials, int nblocks) {
  k_vsum_pair<<<nblocks, kReduceThreads, 0, L.stream>>>(pair_args(L), L.par.rho0, fac, L.bf_uniform,
                                                         L.bf_const[0], L.bf_const[1], L.bf_const[2],
                                                         (const float *)L.bf, psi, partials);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_force_bf16(Lattice &L) {
  if (L.nbnd == 0) return cudaSuccess;
  ForceArgs f{L.nbnd, L.bnd_node, L.bnd_f};
  const int moving = L.par.objects_moving && L.uw != nullptr;
  k_force_pair<<<fblocks(L.nbnd, 128), 128, 0, L.stream>>>(pair_args(L), moving, (const float *)L.uw, f);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_setvel_bf16(Lattice &L, const double *stage, long long x0, long long n, int has_rho,
                               int skip_solid) {
  k_setvel_pair<<<fblocks(n, 256), 256, 0, L.stream>>>(pair_args_inplace(L), stage, x0, n, has_rho, L.par.rho0,
                                                       L.par.stokes_flow, skip_solid);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_collide_bf16(Lattice &L) {
  if (L.par.skip_solid) {
    set_error(kSkipSolid);
    return cudaErrorInvalidValue;
  }
  const StepArgs<float> s = step_args_f(L);
  if (s.bf_uniform) k_collide_pair<true><<<fblocks(L.nnodes, 256), 256, 0, L.stream>>>(pair_args_inplace(L), s);
  else k_collide_pair<false><<<fblocks(L.nnodes, 256), 256, 0, L.stream>>>(pair_args_inplace(L), s);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_mp_rhoinit_bf16(Lattice &L) {
  k_mp_rhoinit_pair<<<fblocks(L.nnodes, 256), 256, 0, L.stream>>>(pair_args(L), L.par.rho0, L.mp_rho64,
                                                                  L.mp_rho32);
  count_launch();
  return cudaGetLastError();
}

}  // namespace slbc
