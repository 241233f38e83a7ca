// Fused update with 128-bit population accesses (FP32 populations): every
// thread updates 4 consecutive nodes along k, loading and storing each
// population array as one aligned float4.  Included by slbc_launch.cuh.
//
// The update rule is the one of step_node (slbc_kernels.cuh), node by node,
// with the same arithmetic (to FP32 rounding: the compiler may contract
// multiply-adds differently in the two kernels); only the memory accesses
// are regrouped:
//
//  * local step (C1 -> C0): 15 float4 loads of slots q at x0..x0+3, 15
//    float4 stores to slots opp(q): no neighbour involved.
//  * pull-and-push step (C0 -> C1): population q of node x is pulled from
//    slot opp(q) of x - c_q.  The rows (i - cx, j - cy) are aligned, so only
//    the k offset -cz needs care: each lane loads the aligned float4 of its
//    own k range in the upstream row, and the one value its range lacks (at
//    k0 - 1 or k0 + 4) comes from the neighbouring lane by a warp shuffle,
//    or, at a warp's or row's edge, from a scalar load (with the periodic
//    wrap in k).  The push to slot q of x + c_q is regrouped the same way:
//    each lane stores the aligned float4 of destination positions
//    [k0, k0 + 4), taking the value shifted in from the neighbouring lane,
//    and an edge lane stores the value that leaves its range as a scalar.
//  * bounce-back links (flag bits) are exceptions in both directions: a
//    pulled value then comes from the node's own slot q (one more aligned
//    float4 load, only when one of the 4 nodes has such a link for q), and a
//    pushed value goes to the node's own slot opp(q) (a scalar store) while
//    its destination element is skipped -- that element belongs to the
//    destination node, which writes it itself -- so a vector store is used
//    only when all four elements are regular, and scalar stores otherwise.
//
// Requirements (checked by the launcher): esk a multiple of 4 (then every
// row starts on a 16-byte boundary, npad being a multiple of 64).
#pragma once

namespace slbc {


__device__ __forceinline__ float f4_get(const float4 &v, int n) {
  return n == 0 ? v.x : n == 1 ? v.y : n == 2 ? v.z : v.w;
}

template <bool ODD, bool MOVING, bool BFU>
__global__ void __launch_bounds__(kV4Threads, ODD ? (MOVING ? 2 : 3) : 4) k_step_v4(StepArgs<float> a) {
  float *__restrict__ P = a.p.pop;
  const long long S = a.p.npad;
  const int esi = a.p.esi, esj = a.p.esj, esk = a.p.esk;
  const int lane = (threadIdx.y * blockDim.x + threadIdx.x) & 31;  // a warp may span several rows
  const int kq = blockIdx.x * blockDim.x + threadIdx.x;  // k / 4
  const int k0 = 4 * kq;
  const int j = blockIdx.y * blockDim.y + threadIdx.y;
  const int i = blockIdx.z;
  const bool active = k0 < esk && j < esj;
  // neighbouring lanes that hold the adjacent k ranges of the same row
  const bool left_ok = lane != 0 && threadIdx.x != 0;
  const bool right_ok = lane != 31 && threadIdx.x != blockDim.x - 1 && k0 + 4 < esk;
  const int jj = active ? j : 0, k0c = active ? k0 : 0;
  const Nbr nb = make_nbr(i, jj, k0c, esi, esj, esk);  // K[] is only used through kidx below
  const int row = (i * esj + jj) * esk;
  const int x0 = row + k0c;
  uint16_t fl[4] = {0, 0, 0, 0};
  if (active) {
    const ushort4 f4 = *reinterpret_cast<const ushort4 *>(a.p.flags + x0);
    fl[0] = f4.x; fl[1] = f4.y; fl[2] = f4.z; fl[3] = f4.w;
  }
  const uint16_t fl_or = fl[0] | fl[1] | fl[2] | fl[3];
  float t[4][15];
  // ---- loads ----------------------------------------------------------------
  {
    const float4 v = active ? *reinterpret_cast<const float4 *>(P + x0) : make_float4(0.f, 0.f, 0.f, 0.f);
    t[0][0] = v.x; t[1][0] = v.y; t[2][0] = v.z; t[3][0] = v.w;
  }
#pragma unroll
  for (int q = 1; q < 15; q++) {
    if (!ODD) {
      const float4 v = active ? *reinterpret_cast<const float4 *>(P + q * S + x0) : make_float4(0.f, 0.f, 0.f, 0.f);
      t[0][q] = v.x; t[1][q] = v.y; t[2][q] = v.z; t[3][q] = v.w;
    } else {
      const int srow = (nb.I[1 - CX(q)] + nb.J[1 - CY(q)]) * esk;
      const float *src = P + OPP(q) * S + srow;
      const float4 v = active ? *reinterpret_cast<const float4 *>(src + k0c) : make_float4(0.f, 0.f, 0.f, 0.f);
      float e[4];
      if (CZ(q) == 0) {
        e[0] = v.x; e[1] = v.y; e[2] = v.z; e[3] = v.w;
      } else if (CZ(q) == 1) {  // source k - 1
        float lw = __shfl_up_sync(0xffffffffu, v.w, 1);
        if (!left_ok && active) lw = src[k0c == 0 ? esk - 1 : k0c - 1];
        e[0] = lw; e[1] = v.x; e[2] = v.y; e[3] = v.z;
      } else {  // source k + 1
        float rx = __shfl_down_sync(0xffffffffu, v.x, 1);
        if (!right_ok && active) rx = src[k0c + 4 == esk ? 0 : k0c + 4];
        e[0] = v.y; e[1] = v.z; e[2] = v.w; e[3] = rx;
      }
      if ((fl_or >> q) & 1) {  // bounce-back links: the node's own slot q
        const float4 w = *reinterpret_cast<const float4 *>(P + q * S + x0);
#pragma unroll
        for (int n = 0; n < 4; n++)
          if ((fl[n] >> q) & 1) e[n] = f4_get(w, n);
      }
#pragma unroll
      for (int n = 0; n < 4; n++) t[n][q] = e[n];
    }
  }
  // ---- wall terms and collision, node by node ---------------------------------
#pragma unroll
  for (int n = 0; n < 4; n++) {
    const bool solid = (fl[n] & FLAG_SOLID) != 0;
    const int x = x0 + n;
    if (MOVING && active && (fl[n] & FLAG_LINKS)) {
      const Nbr nbn = make_nbr(i, jj, k0c + n, esi, esj, esk);
      apply_wall<float>(t[n], fl[n], solid, nbn, x, a.uw, S);
    }
    if (!(a.skip_solid && solid)) {
      float bx = a.bfx, by = a.bfy, bz = a.bfz;
      if (!BFU && active) { bx = a.bf[x]; by = a.bf[S + x]; bz = a.bf[2 * S + x]; }
      collide<float, false>(t[n], a.omega, a.comega, a.rho0, a.stokes, !solid, bx, by, bz);
    }
  }
  // ---- stores -----------------------------------------------------------------
  if (active) *reinterpret_cast<float4 *>(P + x0) = make_float4(t[0][0], t[1][0], t[2][0], t[3][0]);
#pragma unroll
  for (int q = 1; q < 15; q++) {
    if (!ODD) {
      if (active)
        *reinterpret_cast<float4 *>(P + OPP(q) * S + x0) = make_float4(t[0][q], t[1][q], t[2][q], t[3][q]);
      continue;
    }
    // a node's value goes to x + c_q unless its link along c_q is a
    // bounce-back link (flag bit opp(q)): then to its own slot opp(q)
    bool reg[4];
#pragma unroll
    for (int n = 0; n < 4; n++) {
      reg[n] = !((fl[n] >> OPP(q)) & 1);
      if (!reg[n] && active) P[OPP(q) * S + x0 + n] = t[n][q];
    }
    const int drow = (nb.I[1 + CX(q)] + nb.J[1 + CY(q)]) * esk;
    float *dst = P + q * S + drow;
    float e[4];
    bool er[4];
    if (CZ(q) == 0) {
#pragma unroll
      for (int n = 0; n < 4; n++) { e[n] = t[n][q]; er[n] = reg[n]; }
    } else if (CZ(q) == 1) {  // node k goes to k + 1
      const float lv = __shfl_up_sync(0xffffffffu, t[3][q], 1);
      const bool lr = __shfl_up_sync(0xffffffffu, (int)reg[3], 1) != 0;
      e[0] = lv; er[0] = left_ok && lr;  // else stored by the lane that owns node k0 - 1
      e[1] = t[0][q]; er[1] = reg[0];
      e[2] = t[1][q]; er[2] = reg[1];
      e[3] = t[2][q]; er[3] = reg[2];
      if (!right_ok && active && reg[3]) dst[k0c + 4 == esk ? 0 : k0c + 4] = t[3][q];
    } else {  // node k goes to k - 1
      const float rv = __shfl_down_sync(0xffffffffu, t[0][q], 1);
      const bool rr = __shfl_down_sync(0xffffffffu, (int)reg[0], 1) != 0;
      e[0] = t[1][q]; er[0] = reg[1];
      e[1] = t[2][q]; er[1] = reg[2];
      e[2] = t[3][q]; er[2] = reg[3];
      e[3] = rv; er[3] = right_ok && rr;  // else stored by the lane that owns node k0 + 4
      if (!left_ok && active && reg[0]) dst[k0c == 0 ? esk - 1 : k0c - 1] = t[0][q];
    }
    if (!active) continue;
    if (er[0] && er[1] && er[2] && er[3]) {
      *reinterpret_cast<float4 *>(dst + k0c) = make_float4(e[0], e[1], e[2], e[3]);
    } else {
#pragma unroll
      for (int n = 0; n < 4; n++)
        if (er[n]) dst[k0c + n] = e[n];
    }
  }
}

}  // namespace slbc
