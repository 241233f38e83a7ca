// Launchers of the population kernels for one population type.  Included by
// slbc_f64.cu and slbc_f32.cu after defining SLBC_T (the type), SLBC_SUFFIX
// (f64 / f32) and SLBC_EXACT (follow the reference's division forms).
#pragma once

#include <algorithm>
#include <cstring>
#include <vector>

#include <type_traits>

#include "slbc_kernels.cuh"
#include "slbc_mp.cuh"
#include "slbc_step_v4.cuh"

#define SLBC_CAT2(a, b) a##_##b
#define SLBC_CAT(a, b) SLBC_CAT2(a, b)
#define SLBC_FN(name) SLBC_CAT(name, SLBC_SUFFIX)

namespace slbc {

using T_ = SLBC_T;

static PopArgs<T_> pop_args(Lattice &L) {
  PopArgs<T_> p;
  p.pop = (T_ *)L.pop;
  p.npad = L.npad;
  p.flags = L.flags;
  p.esi = L.esi; p.esj = L.esj; p.esk = L.esk;
  return p;
}

static StepArgs<T_> step_args(Lattice &L) {
  StepArgs<T_> a;
  a.p = pop_args(L);
  const double omega = 1.0 / L.par.tau;
  a.omega = (T_)omega;
  a.comega = (T_)(1.0 - omega);
  a.rho0 = (T_)L.par.rho0;
  a.stokes = L.par.stokes_flow;
  a.skip_solid = L.par.skip_solid;
  a.moving = L.par.objects_moving && L.uw != nullptr;
  a.bf_uniform = L.bf_uniform;
  a.bfx = (T_)L.bf_const[0]; a.bfy = (T_)L.bf_const[1]; a.bfz = (T_)L.bf_const[2];
  a.bf = (const T_ *)L.bf;
  a.uw = (const T_ *)L.uw;
  return a;
}

static dim3 row_grid(const Lattice &L, int bx) {
  return dim3((unsigned)((L.esk + bx - 1) / bx), (unsigned)L.esj, (unsigned)L.esi);
}

static int flat_blocks(long long n, int bs) { return (int)((n + bs - 1) / bs); }

// Element offsets of the pull-and-push update away from the faces (k_step):
// the neighbour x + c_q is x + c_q . (esj esk, esk, 1) there.
static OddOffsets odd_offsets(const Lattice &L) {
  OddOffsets o;
  const unsigned S = (unsigned)L.npad;
  for (int q = 0; q < 15; q++) {
    const int d = CX(q) * L.esj * L.esk + CY(q) * L.esk + CZ(q);
    o.pull_self[q] = (unsigned)q * S;
    o.pull_nbr[q] = (unsigned)OPP(q) * S - (unsigned)d;
    o.push_self[q] = (unsigned)OPP(q) * S;
    o.push_nbr[q] = (unsigned)q * S + (unsigned)d;
  }
  return o;
}

template <bool ODD, bool MOVING, bool BFU>
static void step_variant(Lattice &L, const StepArgs<T_> &a, int npt, int bx) {
  if (npt == kStepVec4) {  // 128-bit form: 4 nodes along k per thread, bx threads per block
    if constexpr (std::is_same<T_, float>::value) {
      // lanes along k: a power of two, so a block is whole warps
      int lanes_k = 32;
      while (lanes_k > 1 && lanes_k > L.esk / 4) lanes_k /= 2;
      const dim3 block((unsigned)lanes_k, (unsigned)(kV4Threads / lanes_k));
      const dim3 grid((unsigned)((L.esk / 4 + lanes_k - 1) / lanes_k), (unsigned)((L.esj + block.y - 1) / block.y),
                      (unsigned)L.esi);
      k_step_v4<ODD, MOVING, BFU><<<grid, block, 0, L.stream>>>(a);
    }
    return;
  }
  const dim3 grid((unsigned)((L.esk + bx - 1) / bx), (unsigned)((L.esj + npt - 1) / npt), (unsigned)L.esi);
  // 32-bit population indices whenever all 15 arrays fit (lattices up to
  // about 286 M nodes)
  if (15LL * L.npad <= 0xFFFFFFFFLL) {
    const OddOffsets off = odd_offsets(L);
    if (npt == 4) k_step<T_, ODD, SLBC_EXACT, MOVING, BFU, 4, true><<<grid, bx, 0, L.stream>>>(a, off);
    else if (npt == 2) k_step<T_, ODD, SLBC_EXACT, MOVING, BFU, 2, true><<<grid, bx, 0, L.stream>>>(a, off);
    else k_step<T_, ODD, SLBC_EXACT, MOVING, BFU, 1, true><<<grid, bx, 0, L.stream>>>(a, off);
  } else {
    const OddOffsets off{};
    if (npt == 4) k_step<T_, ODD, SLBC_EXACT, MOVING, BFU, 4, false><<<grid, bx, 0, L.stream>>>(a, off);
    else if (npt == 2) k_step<T_, ODD, SLBC_EXACT, MOVING, BFU, 2, false><<<grid, bx, 0, L.stream>>>(a, off);
    else k_step<T_, ODD, SLBC_EXACT, MOVING, BFU, 1, false><<<grid, bx, 0, L.stream>>>(a, off);
  }
}

template <bool ODD>
static void step_dispatch(Lattice &L, const StepArgs<T_> &a, int npt, int bx) {
  if (a.moving) {
    if (a.bf_uniform) step_variant<ODD, true, true>(L, a, npt, bx);
    else step_variant<ODD, true, false>(L, a, npt, bx);
  } else {
    if (a.bf_uniform) step_variant<ODD, false, true>(L, a, npt, bx);
    else step_variant<ODD, false, false>(L, a, npt, bx);
  }
}

// All lattices of a batch by nsteps steps: descriptors and the block
// assignment are rebuilt per call (parameter changes between calls are
// picked up), one launch per (moving walls, uniform body force) class.
// Assignment: longest processing time first, the largest lattice to the
// least loaded block, at most two blocks per SM.
cudaError_t SLBC_FN(launch_batch)(BatchState &B, int nsteps) {
  const int n = (int)B.lats.size();
  std::vector<BatchDom<T_>> h(n);
  std::vector<int> cls(n);
  for (int d = 0; d < n; d++) {
    h[d].a = step_args(*B.lats[d]);
    h[d].odd0 = B.lats[d]->layout == SLBC_LAYOUT_C0 ? 1 : 0;
    cls[d] = (h[d].a.moving ? 2 : 0) + (h[d].a.bf_uniform ? 1 : 0);
  }
  cudaError_t e = cudaMemcpy(B.doms, h.data(), n * sizeof(BatchDom<T_>), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return e;
  std::vector<int> off, work;
  int base_off = 0, base_work = 0;
  for (int c = 0; c < 4; c++) {
    std::vector<int> order;
    for (int d = 0; d < n; d++) if (cls[d] == c) order.push_back(d);
    if (order.empty()) continue;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return B.lats[a]->nnodes > B.lats[b]->nnodes; });
    const int W = std::max(1, std::min((int)order.size(), 2 * B.sms));
    std::vector<long long> load(W, 0);
    std::vector<std::vector<int>> owned(W);
    for (int d : order) {
      int w = 0;
      for (int v = 1; v < W; v++) if (load[v] < load[w]) w = v;
      load[w] += B.lats[d]->nnodes;
      owned[w].push_back(d);
    }
    std::vector<int> o(W + 1, 0), wk;
    for (int w = 0; w < W; w++) {
      o[w + 1] = o[w] + (int)owned[w].size();
      wk.insert(wk.end(), owned[w].begin(), owned[w].end());
    }
    e = cudaMemcpy(B.work_off + base_off, o.data(), (W + 1) * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(B.work + base_work, wk.data(), wk.size() * sizeof(int), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    const BatchDom<T_> *D = (const BatchDom<T_> *)B.doms;
    const int *O = B.work_off + base_off, *K = B.work + base_work;
    switch (c) {
      case 0: k_batch<T_, SLBC_EXACT, false, false><<<W, kBatchThreads, 0, B.stream>>>(D, O, K, nsteps); break;
      case 1: k_batch<T_, SLBC_EXACT, false, true><<<W, kBatchThreads, 0, B.stream>>>(D, O, K, nsteps); break;
      case 2: k_batch<T_, SLBC_EXACT, true, false><<<W, kBatchThreads, 0, B.stream>>>(D, O, K, nsteps); break;
      default: k_batch<T_, SLBC_EXACT, true, true><<<W, kBatchThreads, 0, B.stream>>>(D, O, K, nsteps); break;
    }
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    B.nworkers = W;
    base_off += W + 1;
    base_work += (int)wk.size();
  }
  return cudaSuccess;
}

// Tiles mode: descriptors and the tile table of every class (rebuilt per
// batch step call).
cudaError_t SLBC_FN(prepare_tiles)(BatchState &B) {
  const int n = (int)B.lats.size();
  std::vector<BatchDom<T_>> h(n);
  std::vector<int2> tiles;
  for (int d = 0; d < n; d++) {
    h[d].a = step_args(*B.lats[d]);
    h[d].odd0 = B.lats[d]->layout == SLBC_LAYOUT_C0 ? 1 : 0;
  }
  for (int c = 0; c < 4; c++) {
    for (int g = 0; g < 2; g++) {
      const size_t first = tiles.size();
      for (int d = 0; d < n; d++) {
        if ((h[d].a.moving ? 2 : 0) + (h[d].a.bf_uniform ? 1 : 0) != c || h[d].odd0 != g) continue;
        for (long long e = 0; e < B.lats[d]->nnodes; e += kBatchTile) tiles.push_back(make_int2(d, (int)e));
      }
      B.class_tiles[c][g] = (int)(tiles.size() - first);
    }
  }
  cudaError_t e = cudaMemcpy(B.doms, h.data(), n * sizeof(BatchDom<T_>), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return e;
  if ((long long)tiles.size() > B.tiles_cap) {
    if (B.tiles) cudaFree(B.tiles);
    B.tiles = nullptr;
    B.tiles_cap = 0;
    e = cudaMalloc(&B.tiles, tiles.size() * sizeof(int2));
    if (e != cudaSuccess) return e;
    B.tiles_cap = (long long)tiles.size();
  }
  return cudaMemcpy(B.tiles, tiles.data(), tiles.size() * sizeof(int2), cudaMemcpyHostToDevice);
}

// Tiles mode: one step (step = position in the sequence, for the parity).
cudaError_t SLBC_FN(launch_tiles)(BatchState &B, int step) {
  const BatchDom<T_> *D = (const BatchDom<T_> *)B.doms;
  const int2 *t = B.tiles;
  for (int c = 0; c < 4; c++) {
    for (int g = 0; g < 2; g++) {
      const int nt = B.class_tiles[c][g];
      if (nt == 0) continue;
      // domains of group g take an odd step when (step + g) is odd
      const bool odd = ((step + g) & 1) == 1;
      switch (c * 2 + (odd ? 1 : 0)) {
        case 0: k_batch_tiles<T_, false, SLBC_EXACT, false, false><<<nt, kBatchTile, 0, B.stream>>>(D, t); break;
        case 1: k_batch_tiles<T_, true, SLBC_EXACT, false, false><<<nt, kBatchTile, 0, B.stream>>>(D, t); break;
        case 2: k_batch_tiles<T_, false, SLBC_EXACT, false, true><<<nt, kBatchTile, 0, B.stream>>>(D, t); break;
        case 3: k_batch_tiles<T_, true, SLBC_EXACT, false, true><<<nt, kBatchTile, 0, B.stream>>>(D, t); break;
        case 4: k_batch_tiles<T_, false, SLBC_EXACT, true, false><<<nt, kBatchTile, 0, B.stream>>>(D, t); break;
        case 5: k_batch_tiles<T_, true, SLBC_EXACT, true, false><<<nt, kBatchTile, 0, B.stream>>>(D, t); break;
        case 6: k_batch_tiles<T_, false, SLBC_EXACT, true, true><<<nt, kBatchTile, 0, B.stream>>>(D, t); break;
        default: k_batch_tiles<T_, true, SLBC_EXACT, true, true><<<nt, kBatchTile, 0, B.stream>>>(D, t); break;
      }
      count_launch();
      t += nt;
      const cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
  }
  return cudaSuccess;
}

// One fused step with the tuned (rows per thread, threads along k) of this
// parity; small lattices use one row per thread and the block width that
// fits esk.
cudaError_t SLBC_FN(launch_step)(Lattice &L, int odd) {
  const StepConfig &c = L.tuned[odd ? 1 : 0];
  int bx = c.block_k, npt = c.npt;
  if (bx <= 0) { bx = 128; npt = 1; }
  if (npt == kStepVec4 && !vec4_ok(L)) npt = 1;
  if (npt != kStepVec4)
    while (bx > 32 && bx / 2 >= L.esk) bx /= 2;
  if (L.esj < 2) npt = 1;
  StepArgs<T_> a = step_args(L);
  if (odd) step_dispatch<true>(L, a, npt, bx);
  else step_dispatch<false>(L, a, npt, bx);
  count_launch();
  return cudaGetLastError();
}

cudaError_t SLBC_FN(launch_force)(Lattice &L) {
  if (L.nbnd == 0) return cudaSuccess;
  ForceArgs f{L.nbnd, L.bnd_node, L.bnd_f};
  const int bs = 128;
  const int moving = L.par.objects_moving && L.uw != nullptr;
  k_force<T_><<<flat_blocks(L.nbnd, bs), bs, 0, L.stream>>>(pop_args(L), L.layout, moving,
                                                           (const T_ *)L.uw, f);
  count_launch();
  return cudaGetLastError();
}

cudaError_t SLBC_FN(launch_vsum)(Lattice &L, double fac, const double *psi, double *partials,
                                 int nblocks) {
  k_vsum<T_><<<nblocks, kReduceThreads, 0, L.stream>>>(
      pop_args(L), L.layout, L.par.rho0, fac, L.bf_uniform, L.bf_const[0], L.bf_const[1],
      L.bf_const[2], (const T_ *)L.bf, psi, partials);
  count_launch();
  return cudaGetLastError();
}

cudaError_t SLBC_FN(launch_put)(Lattice &L, const double *stage, long long x0, long long n) {
  k_put<T_><<<flat_blocks(n, 256), 256, 0, L.stream>>>(pop_args(L), stage, x0, n);
  count_launch();
  return cudaGetLastError();
}

cudaError_t SLBC_FN(launch_get)(Lattice &L, double *stage, long long x0, long long n) {
  k_get<T_><<<flat_blocks(n, 256), 256, 0, L.stream>>>(pop_args(L), L.layout, stage, x0, n);
  count_launch();
  return cudaGetLastError();
}

cudaError_t SLBC_FN(launch_put_host)(Lattice &L, const double *host) {
  const int blocks = (int)std::min<long long>((L.nnodes + kHostTile - 1) / kHostTile, 152LL * 16);
  k_put_host<T_><<<blocks, kHostTile, 0, L.stream>>>(pop_args(L), host, L.nnodes);
  count_launch();
  return cudaGetLastError();
}

cudaError_t SLBC_FN(launch_get_host)(Lattice &L, double *host) {
  const int blocks = (int)std::min<long long>((L.nnodes + kHostTile - 1) / kHostTile, 152LL * 16);
  k_get_host<T_><<<blocks, kHostTile, 0, L.stream>>>(pop_args(L), L.layout, host, L.nnodes);
  count_launch();
  return cudaGetLastError();
}

cudaError_t SLBC_FN(launch_swap)(Lattice &L) {
  k_swap<T_><<<flat_blocks(L.nnodes, 256), 256, 0, L.stream>>>(pop_args(L), L.nnodes);
  count_launch();
  return cudaGetLastError();
}

cudaError_t SLBC_FN(launch_to_natural)(Lattice &L) {
  const int bx = L.esk >= 128 ? 128 : 32;
  k_c1_to_n<T_><<<row_grid(L, bx), bx, 0, L.stream>>>(pop_args(L), (T_ *)L.scratch);
  count_launch();
  return cudaGetLastError();
}

cudaError_t SLBC_FN(launch_bbl)(Lattice &L, int with_force) {
  if (L.nbnd == 0) return cudaSuccess;
  ForceArgs f{L.nbnd, L.bnd_node, L.bnd_f};
  const int moving = L.par.objects_moving && L.uw != nullptr;
  k_bbl_n<T_><<<flat_blocks(L.nbnd, 128), 128, 0, L.stream>>>(pop_args(L), moving,
                                                              (const T_ *)L.uw, with_force, f);
  count_launch();
  return cudaGetLastError();
}

cudaError_t SLBC_FN(launch_propagate)(Lattice &L) {
  const int bx = L.esk >= 128 ? 128 : 32;
  k_propagate_n<T_><<<row_grid(L, bx), bx, 0, L.stream>>>(pop_args(L), (T_ *)L.scratch);
  count_launch();
  return cudaGetLastError();
}

cudaError_t SLBC_FN(launch_collide)(Lattice &L) {
  k_collide_n<T_, SLBC_EXACT><<<flat_blocks(L.nnodes, 256), 256, 0, L.stream>>>(step_args(L));
  count_launch();
  return cudaGetLastError();
}

cudaError_t SLBC_FN(launch_setvel)(Lattice &L, const double *stage, long long x0, long long n,
                                   int has_rho, int skip_solid) {
  k_setvel<T_, SLBC_EXACT><<<flat_blocks(n, 256), 256, 0, L.stream>>>(
      pop_args(L), stage, x0, n, has_rho, L.par.rho0, L.par.stokes_flow, skip_solid);
  count_launch();
  return cudaGetLastError();
}

cudaError_t SLBC_FN(launch_vacf_sums)(Lattice &L, double *p, const double *p2, const double *psi, double pmean,
                                      int axis, double *partials, int nblocks) {
  k_vacf_sums<T_><<<nblocks, kReduceThreads, 0, L.stream>>>(pop_args(L), L.layout, L.mp_rho64, p, p2, psi, pmean,
                                                             axis, partials);
  count_launch();
  return cudaGetLastError();
}

cudaError_t SLBC_FN(launch_move_sphere)(Lattice &L, const MoveArgs &m, int with_uw) {
  const long long nbox = (long long)m.len[0] * m.len[1] * m.len[2];
  const int blocks = (int)std::max<long long>(1, std::min<long long>((nbox + 255) / 256, 152LL * 8));
  k_move_sphere<T_, SLBC_EXACT><<<blocks, 256, 0, L.stream>>>(pop_args(L), m, with_uw ? (T_ *)L.uw : nullptr);
  count_launch();
  return cudaGetLastError();
}

cudaError_t SLBC_FN(launch_velocity)(Lattice &L, double fac, float *u, float *drho) {
  const int blocks = (int)std::min<long long>((L.nnodes + 255) / 256, 152LL * 16);
  k_velocity<T_><<<blocks, 256, 0, L.stream>>>(pop_args(L), L.layout, L.par.rho0, fac, L.bf_uniform, L.bf_const[0],
                                               L.bf_const[1], L.bf_const[2], (const T_ *)L.bf, u, drho);
  count_launch();
  return cudaGetLastError();
}

cudaError_t SLBC_FN(launch_mp_rhoinit)(Lattice &L) {
  k_mp_rhoinit<T_><<<flat_blocks(L.nnodes, 256), 256, 0, L.stream>>>(
      pop_args(L), L.layout, L.par.rho0, L.mp_rho64, L.mp_rho32);
  count_launch();
  return cudaGetLastError();
}

cudaError_t SLBC_FN(launch_mp_step)(Lattice &L, const void *p_in, void *p_out, int tp_f64,
                                    double alpha, double adprob, int moving,
                                    const double *objstate, float *lo_in, float *lo_out, int *lo_live) {
  // planes per block: the largest of 1..8 that still gives about four
  // blocks per SM
  const long long tiles = (long long)((L.esk + kTileK - 1) / kTileK) * ((L.esj + kTileJ - 1) / kTileJ);
  int planes = 8;
  while (planes > 1 && tiles * ((L.esi + planes - 1) / planes) < 152 * 4) planes /= 2;
  const dim3 grid((unsigned)((L.esk + kTileK - 1) / kTileK), (unsigned)((L.esj + kTileJ - 1) / kTileJ),
                  (unsigned)((L.esi + planes - 1) / planes));
  const dim3 block(kTileK, kTileJ);
  MpArgs m;
  m.p_in = p_in; m.p_out = p_out;
  m.rho = tp_f64 ? (const void *)L.mp_rho64 : (const void *)L.mp_rho32;
  m.ads = L.ads; m.ads_links = L.ads_links; m.objidx = L.objidx; m.objstate = objstate; m.moving = moving;
  m.alpha = alpha; m.adprob = adprob; m.rho0 = L.par.rho0;
  m.alpha_f = (float)alpha; m.adprob_f = (float)adprob; m.rho0_f = (float)L.par.rho0;
  m.partial = adprob != 1.0;
  // FP32 tracers: the division-free kernel in link order, while 32-bit
  // population indices reach (15 * npad < 2^32)
  if (!tp_f64 && 15ULL * (unsigned long long)L.npad < (1ULL << 32)) {
    const cudaError_t e = ensure_mp_rinv(L);
    if (e != cudaSuccess) return e;
    const PopArgs<T_> pa = pop_args(L);
    const float *ri = L.mp_rinv32;
    // Frozen flow (fixed walls): once two consecutive updates see the same
    // flow, snapshot, geometry, adsorption and parameters, the terms are
    // built into stencil coefficients and later updates apply those.
    if (!moving) {
      unsigned long long key[8];
      double ad[2] = {alpha, adprob};
      key[0] = L.state_version; key[1] = L.mp_rho_gen; key[2] = L.generation;
      key[3] = (unsigned long long)L.layout; key[4] = L.ads_version;
      memcpy(&key[5], &ad[0], 8); memcpy(&key[6], &ad[1], 8);
      key[7] = (unsigned long long)(uintptr_t)L.pop;
      const bool same_as_last = memcmp(key, L.mp_last_key, sizeof key) == 0;
      memcpy(L.mp_last_key, key, sizeof key);
      bool ready = L.mp_coef_valid && memcmp(key, L.mp_coef_key, sizeof key) == 0;
      if (!ready && same_as_last) {
        if (!L.mp_coef && cudaMalloc(&L.mp_coef, 15 * (size_t)L.npad * sizeof(float)) != cudaSuccess) {
          cudaGetLastError();  // no room: keep the direct update
          L.mp_coef = nullptr;
        }
        if (L.mp_coef) {
          const int nb = (int)((L.nnodes + 255) / 256);
          switch (L.layout) {
            case SLBC_LAYOUT_N: k_mp_coef<T_, SLBC_LAYOUT_N, false><<<nb, 256, 0, L.stream>>>(pa, m, ri, L.mp_coef); break;
            case SLBC_LAYOUT_C0: k_mp_coef<T_, SLBC_LAYOUT_C0, false><<<nb, 256, 0, L.stream>>>(pa, m, ri, L.mp_coef); break;
            default: k_mp_coef<T_, SLBC_LAYOUT_C1, false><<<nb, 256, 0, L.stream>>>(pa, m, ri, L.mp_coef); break;
          }
          count_launch();
          cudaError_t ce = cudaGetLastError();
          if (ce == cudaSuccess) ce = launch_mp_coef_norm(L);
          if (ce != cudaSuccess) return ce;
          memcpy(L.mp_coef_key, key, sizeof key);
          L.mp_coef_valid = true;
          ready = true;
        }
      }
      if (ready && lo_in && lo_out) {
        // the low part of p is zero where the direct update or an upload left p
        if (!*lo_live) {
          const cudaError_t me = cudaMemsetAsync(lo_in, 0, (size_t)L.nnodes * sizeof(float), L.stream);
          if (me != cudaSuccess) return me;
        }
        *lo_live = 1;
        return launch_mp_apply(L, (const float *)p_in, lo_in, (float *)p_out, lo_out, grid, block, planes);
      }
    }
    switch (L.layout * 2 + (moving ? 1 : 0)) {
      case SLBC_LAYOUT_N * 2: k_mp_step_f32<T_, SLBC_LAYOUT_N, false><<<grid, block, 0, L.stream>>>(pa, m, ri, planes); break;
      case SLBC_LAYOUT_N * 2 + 1: k_mp_step_f32<T_, SLBC_LAYOUT_N, true><<<grid, block, 0, L.stream>>>(pa, m, ri, planes); break;
      case SLBC_LAYOUT_C0 * 2: k_mp_step_f32<T_, SLBC_LAYOUT_C0, false><<<grid, block, 0, L.stream>>>(pa, m, ri, planes); break;
      case SLBC_LAYOUT_C0 * 2 + 1: k_mp_step_f32<T_, SLBC_LAYOUT_C0, true><<<grid, block, 0, L.stream>>>(pa, m, ri, planes); break;
      case SLBC_LAYOUT_C1 * 2: k_mp_step_f32<T_, SLBC_LAYOUT_C1, false><<<grid, block, 0, L.stream>>>(pa, m, ri, planes); break;
      default: k_mp_step_f32<T_, SLBC_LAYOUT_C1, true><<<grid, block, 0, L.stream>>>(pa, m, ri, planes); break;
    }
    if (lo_live) *lo_live = 0;  // p alone holds the tracer
    count_launch();
    return cudaGetLastError();
  }
  // the wrap-node buckets need more than the default 48 KB of dynamic
  // shared memory for FP64 tracers
  static unsigned long long attr_set[2] = {0, 0};  // per device, bit = device index
  int dev = 0;
  cudaGetDevice(&dev);
  const unsigned long long bit = 1ULL << (dev & 63);
  if (!(attr_set[tp_f64 ? 1 : 0] & bit)) {
    cudaError_t e = tp_f64
        ? cudaFuncSetAttribute(k_mp_step<T_, double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               mp_bucket_bytes<double>())
        : cudaFuncSetAttribute(k_mp_step<T_, float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               mp_bucket_bytes<float>());
    if (e != cudaSuccess) return e;
    attr_set[tp_f64 ? 1 : 0] |= bit;
  }
  if (tp_f64)
    k_mp_step<T_, double><<<grid, block, mp_bucket_bytes<double>(), L.stream>>>(pop_args(L), L.layout, m, planes);
  else
    k_mp_step<T_, float><<<grid, block, mp_bucket_bytes<float>(), L.stream>>>(pop_args(L), L.layout, m, planes);
  if (lo_live) *lo_live = 0;  // p alone holds the tracer
  count_launch();
  return cudaGetLastError();
}

}  // namespace slbc
