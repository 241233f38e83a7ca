// Glue kernels of the learned warm start's network: pooling and
// upsampling between resolution levels (with their gradients, the ReLU masks
// and the skip-connection sums fused in), bias gradients, weight layouts for
// the tensor-core convolutions, Adam, the loss and the input encoding.
//
// Activation buffers are channels-last BF16 with a one-voxel periodic halo,
// buf[n][z + 1][y + 1][x + 1][c], total channels ctot, and a kernel works on
// a channel slice [coff, coff + C); C and coff multiples of 8 (16-byte
// vectors of 8 channels).
#include <cuda_bf16.h>

#include <algorithm>
#include <string>

#include "slbc_internal.cuh"

namespace {

typedef __nv_bfloat16 bf16;

struct Slice {
  bf16 *p;
  int ctot, coff;
};

__device__ __forceinline__ long long vox(int n, int z, int y, int x, int D, int H, int W) {
  return (((long long)n * (D + 2) + z + 1) * (H + 2) + y + 1) * (W + 2) + x + 1;
}

__device__ __forceinline__ void load8(const bf16 *p, float (&v)[8]) {
  const uint4 u = *(const uint4 *)p;
  const __nv_bfloat162 *h = (const __nv_bfloat162 *)&u;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const float2 f = __bfloat1622float2(h[i]);
    v[2 * i] = f.x;
    v[2 * i + 1] = f.y;
  }
}

__device__ __forceinline__ void store8(bf16 *p, const float (&v)[8]) {
  uint4 u;
  __nv_bfloat162 *h = (__nv_bfloat162 *)&u;
#pragma unroll
  for (int i = 0; i < 4; i++) h[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
  *(uint4 *)p = u;
}

int grid_for(long long n) { return (int)std::min<long long>((n + 255) / 256, 152LL * 32); }

// 2x2x2 average of the fine interior (D, H, W) into the coarse interior
__global__ void k_pool(Slice in, Slice out, int B, int D, int H, int W, int C) {
  const int Dc = D / 2, Hc = H / 2, Wc = W / 2, nv = C / 8;
  const long long total = (long long)B * Dc * Hc * Wc * nv;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    const int cv = (int)(e % nv);
    long long r = e / nv;
    const int x = (int)(r % Wc); r /= Wc;
    const int y = (int)(r % Hc); r /= Hc;
    const int z = (int)(r % Dc);
    const int n = (int)(r / Dc);
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int c = 0; c < 8; c++) {
      float v[8];
      load8(in.p + vox(n, 2 * z + (c >> 2), 2 * y + ((c >> 1) & 1), 2 * x + (c & 1), D, H, W) * in.ctot + in.coff +
                8 * cv,
            v);
#pragma unroll
      for (int i = 0; i < 8; i++) acc[i] += v[i];
    }
#pragma unroll
    for (int i = 0; i < 8; i++) acc[i] *= 0.125f;
    store8(out.p + vox(n, z, y, x, Dc, Hc, Wc) * out.ctot + out.coff + 8 * cv, acc);
  }
}

// gradient of k_pool: dfine = (dcoarse / 8 + add) * (mask > 0); add and mask
// optional (null pointers)
__global__ void k_pool_bwd(Slice dcoarse, Slice dfine, Slice add, Slice mask, int B, int D, int H, int W, int C) {
  const int nv = C / 8;
  const long long total = (long long)B * D * H * W * nv;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    const int cv = (int)(e % nv);
    long long r = e / nv;
    const int x = (int)(r % W); r /= W;
    const int y = (int)(r % H); r /= H;
    const int z = (int)(r % D);
    const int n = (int)(r / D);
    float g[8];
    load8(dcoarse.p + vox(n, z / 2, y / 2, x / 2, D / 2, H / 2, W / 2) * dcoarse.ctot + dcoarse.coff + 8 * cv, g);
#pragma unroll
    for (int i = 0; i < 8; i++) g[i] *= 0.125f;
    const long long v = vox(n, z, y, x, D, H, W);
    if (add.p) {
      float a[8];
      load8(add.p + v * add.ctot + add.coff + 8 * cv, a);
#pragma unroll
      for (int i = 0; i < 8; i++) g[i] += a[i];
    }
    if (mask.p) {
      float m[8];
      load8(mask.p + v * mask.ctot + mask.coff + 8 * cv, m);
#pragma unroll
      for (int i = 0; i < 8; i++) g[i] = m[i] > 0.0f ? g[i] : 0.0f;
    }
    store8(dfine.p + v * dfine.ctot + dfine.coff + 8 * cv, g);
  }
}

// nearest upsampling: fine (D, H, W) interior = coarse parent
__global__ void k_up(Slice in, Slice out, int B, int D, int H, int W, int C) {
  const int nv = C / 8;
  const long long total = (long long)B * D * H * W * nv;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    const int cv = (int)(e % nv);
    long long r = e / nv;
    const int x = (int)(r % W); r /= W;
    const int y = (int)(r % H); r /= H;
    const int z = (int)(r % D);
    const int n = (int)(r / D);
    *(uint4 *)(out.p + vox(n, z, y, x, D, H, W) * out.ctot + out.coff + 8 * cv) =
        *(const uint4 *)(in.p + vox(n, z / 2, y / 2, x / 2, D / 2, H / 2, W / 2) * in.ctot + in.coff + 8 * cv);
  }
}

// gradient of k_up: dcoarse = sum of the 8 children * (mask > 0) (coarse mask)
__global__ void k_up_bwd(Slice dfine, Slice dcoarse, Slice mask, int B, int D, int H, int W, int C) {
  const int Dc = D / 2, Hc = H / 2, Wc = W / 2, nv = C / 8;
  const long long total = (long long)B * Dc * Hc * Wc * nv;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    const int cv = (int)(e % nv);
    long long r = e / nv;
    const int x = (int)(r % Wc); r /= Wc;
    const int y = (int)(r % Hc); r /= Hc;
    const int z = (int)(r % Dc);
    const int n = (int)(r / Dc);
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int c = 0; c < 8; c++) {
      float v[8];
      load8(dfine.p + vox(n, 2 * z + (c >> 2), 2 * y + ((c >> 1) & 1), 2 * x + (c & 1), D, H, W) * dfine.ctot +
                dfine.coff + 8 * cv,
            v);
#pragma unroll
      for (int i = 0; i < 8; i++) acc[i] += v[i];
    }
    const long long v = vox(n, z, y, x, Dc, Hc, Wc);
    if (mask.p) {
      float m[8];
      load8(mask.p + v * mask.ctot + mask.coff + 8 * cv, m);
#pragma unroll
      for (int i = 0; i < 8; i++) acc[i] = m[i] > 0.0f ? acc[i] : 0.0f;
    }
    store8(dcoarse.p + v * dcoarse.ctot + dcoarse.coff + 8 * cv, acc);
  }
}

// db[c] += sum over interior voxels of g.  The grid stride is a multiple of
// C / 8, so a thread always handles the same 8 channels: it sums in
// registers and adds to the block's shared sums once.
__global__ void k_bias_grad(Slice g, int B, int D, int H, int W, int C, float *db) {
  extern __shared__ float sh[];
  for (int c = threadIdx.x; c < C; c += blockDim.x) sh[c] = 0.0f;
  __syncthreads();
  const int nv = C / 8;
  const long long total = (long long)B * D * H * W * nv;
  const long long start = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int cv = (int)(start % nv);
  float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (long long e = start; e < total; e += (long long)gridDim.x * blockDim.x) {
    long long r = e / nv;
    const int x = (int)(r % W); r /= W;
    const int y = (int)(r % H); r /= H;
    const int z = (int)(r % D);
    const int n = (int)(r / D);
    float v[8];
    load8(g.p + vox(n, z, y, x, D, H, W) * g.ctot + g.coff + 8 * cv, v);
#pragma unroll
    for (int i = 0; i < 8; i++) acc[i] += v[i];
  }
#pragma unroll
  for (int i = 0; i < 8; i++) atomicAdd(&sh[8 * cv + i], acc[i]);
  __syncthreads();
  for (int c = threadIdx.x; c < C; c += blockDim.x) atomicAdd(&db[c], sh[c]);
}

// forward weights: w[tap][cin/32][cout][32] from master m[tap][cout][cin]
__global__ void k_wfwd(const float *m, int cout, int cin, bf16 *w) {
  const long long n = 27LL * cout * cin;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(e % 32);
    long long r = e / 32;
    const int co = (int)(r % cout); r /= cout;
    const int ck = (int)(r % (cin / 32));
    const int tap = (int)(r / (cin / 32));
    w[e] = __float2bfloat16(m[((long long)tap * cout + co) * cin + ck * 32 + j]);
  }
}

// dgrad weights for input channels [ci0, ci0 + nci): the forward kernel with
// these weights maps dY (cout channels) to dX: w[t][cout/32][nci][32] =
// m[26 - t][32 ck + j][ci0 + ci]
__global__ void k_wdgrad(const float *m, int cout, int cin, int ci0, int nci, bf16 *w) {
  const long long n = 27LL * nci * cout;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(e % 32);
    long long r = e / 32;
    const int ci = (int)(r % nci); r /= nci;
    const int ck = (int)(r % (cout / 32));
    const int t = (int)(r / (cout / 32));
    w[e] = __float2bfloat16(m[((long long)(26 - t) * cout + ck * 32 + j) * cin + ci0 + ci]);
  }
}

__global__ void k_adam(float *p, const float *g, float *m, float *v, long long n, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// Gradient-norm clipping against a running norm, all on the device (no
// host round trip per iteration).  state[0]: sum of squares of every
// gradient tensor (k_sqsum adds to it, k_clip_scale resets it); state[1]:
// running norm (0 before the first call); state[2]: the scale to apply.
__global__ void k_sqsum(const float *g, long long n, double *state) {
  __shared__ double sh[256];
  double s = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    s += (double)g[i] * g[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(state, sh[0]);
}

// scale = min(1, factor * running / norm); running <- decay * running +
// (1 - decay) * norm * scale.  A non-finite norm gives scale 0 (the
// gradients are zeroed) and leaves the running norm as it was.
__global__ void k_clip_scale(double *state, float factor, float decay) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double nrm = sqrt(state[0]);
  state[0] = 0.0;
  const double run = state[1] > 0.0 ? state[1] : nrm;
  if (!isfinite(nrm)) {
    state[2] = 0.0;
    return;
  }
  const double sc = nrm > (double)factor * run ? (double)factor * run / nrm : 1.0;
  state[1] = (double)decay * run + (1.0 - (double)decay) * nrm * sc;
  state[2] = sc;
}

__global__ void k_scale(float *g, long long n, const double *state) {
  const float sc = (float)state[2];
  if (sc == 1.0f) return;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    g[i] = sc == 0.0f ? 0.0f : g[i] * sc;
}

// loss = mean over voxels and the nch components of (pred - label)^2, pred
// in FP32 channels 0..nch-1 of a padded buffer (ctot_p channels), label
// [n][D][H][W][nch] FP32; grad (BF16, gctot channels, padded) = d loss /
// d pred in channels 0..nch-1, 0 in the others.  loss[0] += the sum / count.
__global__ void k_mse(const float *pred, int ctot_p, const float *label, int nch, const float *sample_w, int B, int D,
                      int H, int W, bf16 *grad, int gctot, double *loss) {
  __shared__ double sh[256];
  const long long total = (long long)B * D * H * W;
  const double inv = 1.0 / ((double)nch * (double)total);
  double acc = 0.0;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    long long r = e;
    const int x = (int)(r % W); r /= W;
    const int y = (int)(r % H); r /= H;
    const int z = (int)(r % D);
    const int n = (int)(r / D);
    const long long v = vox(n, z, y, x, D, H, W);
    const float sw = sample_w ? sample_w[n] : 1.0f;
    bf16 *gp = grad + v * gctot;
    for (int c = 0; c < gctot; c += 8) *(uint4 *)(gp + c) = make_uint4(0, 0, 0, 0);
    for (int c = 0; c < nch; c++) {
      const float d = pred[v * ctot_p + c] - label[e * nch + c];
      acc += (double)sw * d * d;
      gp[c] = __float2bfloat16((float)(2.0 * inv) * sw * d);
    }
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(loss, sh[0] * inv);
}

// Projection of the prediction error on the label, per sample n:
// s_n = <label_n, pred_n - label_n> / <label_n, label_n> over the interior
// voxels and channels [0, nch) (labels [n][D][H][W][lch]).  k_proj_dot adds <label_n, pred_n> into
// dot[n] (grid.y = sample); k_proj_grad adds the derivative of
// (weight / B) * sum_n s_n^2 to the BF16 gradient and the term to the loss.
__global__ void k_proj_dot(const float *pred, int ctot_p, const float *label, int lch, int nch, int D, int H, int W,
                           double *dot) {
  __shared__ double sh[256];
  const int n = blockIdx.y;
  const long long per = (long long)D * H * W;
  double acc = 0.0;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < per; e += (long long)gridDim.x * blockDim.x) {
    long long r = e;
    const int x = (int)(r % W); r /= W;
    const int y = (int)(r % H);
    const int z = (int)(r / H);
    const long long v = vox(n, z, y, x, D, H, W);
    const float *lb = label + ((long long)n * per + e) * lch;
    for (int c = 0; c < nch; c++) acc += (double)pred[v * ctot_p + c] * (double)lb[c];
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(dot + n, sh[0]);
}

__global__ void k_proj_grad(const float *label, int lch, int nch, const double *lab_sq, const double *dot, int B, int D,
                            int H, int W, float weight, bf16 *grad, int gctot, double *loss) {
  const long long per = (long long)D * H * W, total = (long long)B * per;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    long long r = e;
    const int x = (int)(r % W); r /= W;
    const int y = (int)(r % H); r /= H;
    const int z = (int)(r % D);
    const int n = (int)(r / D);
    const double q = lab_sq[n];
    if (!(q > 0.0)) continue;
    const double sn = (dot[n] - q) / q;
    const float coef = (float)(2.0 * weight * sn / (q * B));
    bf16 *gp = grad + vox(n, z, y, x, D, H, W) * gctot;
    for (int c = 0; c < nch; c++) gp[c] = __float2bfloat16(__bfloat162float(gp[c]) + coef * label[e * lch + c]);
    if (e % per == 0) atomicAdd(loss, (double)weight * sn * sn / B);
  }
}

// input encoding: channel 0 = 1 on solid nodes, 0 on fluid; with
// features = 1, channel 1 = d / R and channel 2 = (d / R)^2 where d is the
// periodic distance from a fluid node to the nearest solid node, searched
// over a cube of half-width R = 5 (d = R when none is that close; 0 on
// solid nodes); with features = 2 the search reaches R = 12 (the pores of
// open packings are wider than 5) and channel 3 carries min(d, 5) / 5, the
// near-wall form of the first encoding; other channels zero (interior; the
// halo is filled afterwards)
constexpr int kDistR1 = 5, kDistR2 = 12;

// The squared distance min over the cube of dx^2 + dy^2 + dz^2 (solid
// nodes, capped at R^2 <= 144, so it fits a byte) separates into three
// one-axis passes (a minimum of sums is the nested minimum), each over
// 2R + 1 neighbours instead of (2R + 1)^3.  Values stay integers, so the
// result equals the cube search.
// Pass 1 (along x, stride 1): nearest solid node on the row.
template <int R>
__global__ void k_dist_x(const unsigned char *solid, long long total, int W, unsigned char *a) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(e % W);
    const unsigned char *row = solid + (e - x);
    int best = R * R;
#pragma unroll
    for (int dx = -R; dx <= R; dx++)
      if (dx * dx < best && row[((x + dx) % W + W) % W]) best = dx * dx;
    a[e] = (unsigned char)best;
  }
}

// Passes 2 and 3 (along y, stride W, extent H; along z, stride W H,
// extent D): b = min over |d| <= R of d^2 + a at the node d steps away.
template <int R>
__global__ void k_dist_min(const unsigned char *a, long long total, int n, long long stride, unsigned char *b) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    const int p = (int)((e / stride) % n);
    const unsigned char *col = a + (e - (long long)p * stride);
    int best = R * R;
#pragma unroll
    for (int d = -R; d <= R; d++) best = min(best, d * d + (int)col[(long long)(((p + d) % n + n) % n) * stride]);
    b[e] = (unsigned char)best;
  }
}

// dist2: the squared distances of the passes above (null without features),
// searched to radius R
__global__ void k_encode(const unsigned char *solid, const unsigned char *dist2, int R, int B, int D, int H, int W,
                         bf16 *out, int ctot) {
  const long long total = (long long)B * D * H * W;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    long long r = e;
    const int x = (int)(r % W); r /= W;
    const int y = (int)(r % H); r /= H;
    const int z = (int)(r % D);
    const int n = (int)(r / D);
    bf16 *p = out + vox(n, z, y, x, D, H, W) * ctot;
    for (int c = 0; c < ctot; c += 8) *(uint4 *)(p + c) = make_uint4(0, 0, 0, 0);
    const bool s = solid[e] != 0;
    p[0] = __float2bfloat16(s ? 1.0f : 0.0f);
    if (dist2 && !s) {
      const float dist = sqrtf((float)dist2[e]);
      const float d = dist * (1.0f / (float)R);
      p[1] = __float2bfloat16(d);
      p[2] = __float2bfloat16(d * d);
      if (R != kDistR1) p[3] = __float2bfloat16(fminf(dist, (float)kDistR1) * (1.0f / kDistR1));
    }
  }
}

// prediction (FP32 channels 0..2 of a padded buffer) * scale on fluid
// nodes into three FP32 arrays u[c * N + e] (0 on solid nodes), the layout
// of lbsetveldev; shift_x is subtracted from u_x on fluid nodes.  With
// drho, channel 3 * drho_scale into drho[e] (0 on solid nodes).
__global__ void k_decode(const float *pred, int ctot_p, const unsigned char *solid, int D, int H, int W, float scale,
                         float shift_x, float *u, float drho_scale, float *drho) {
  const long long total = (long long)D * H * W;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    long long r = e;
    const int x = (int)(r % W); r /= W;
    const int y = (int)(r % H);
    const int z = (int)(r / H);
    const long long v = vox(0, z, y, x, D, H, W);
#pragma unroll
    for (int c = 0; c < 3; c++) u[c * total + e] = solid[e] ? 0.0f : scale * pred[v * ctot_p + c] - (c == 0 ? shift_x : 0.0f);
    if (drho) drho[e] = solid[e] ? 0.0f : drho_scale * pred[v * ctot_p + 3];
  }
}

// Uniform plane flux of a decoded state (u: 3 x D*H*W, x = the slowest
// index; the flux of x through plane i is q[i] = sum over the plane of u_x).
// k_plane_sum: one block per plane, a fixed summation order.
__global__ void __launch_bounds__(256) k_plane_sum(const float *u, int D, long long plane, double *q) {
  __shared__ double sh[256];
  const int i = blockIdx.x;
  double acc = 0.0;
  for (long long e = threadIdx.x; e < plane; e += blockDim.x) acc += (double)u[(long long)i * plane + e];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) q[i] = sh[0];
}

// One thread: the harmonic mean qh of the plane fluxes, the scale qh / q[i]
// of every plane and the pressure p[i] = sum over the planes before i of
// force (1 - qh / q) (midpoint rule, zero mean), both times gain; work =
// [q | scale | p | spread].  Any plane flux <= 0 leaves the planes as they
// are (scale = gain, p 0).
__global__ void k_plane_fix(int D, float force, float gain, double *work) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double *q = work, *scale = work + D, *p = work + 2 * D;
  bool ok = true;
  double inv = 0.0, qmin = q[0], qmax = q[0], qsum = 0.0;
  for (int i = 0; i < D; i++) {
    ok = ok && q[i] > 0.0;
    inv += 1.0 / q[i];
    qmin = fmin(qmin, q[i]);
    qmax = fmax(qmax, q[i]);
    qsum += q[i];
  }
  work[3 * D] = ok ? (qmax - qmin) / (qsum / D) : -1.0;
  const double qh = D / inv;
  double acc = 0.0, mean = 0.0;
  for (int i = 0; i < D; i++) {
    const double g = ok ? (double)force * (1.0 - qh / q[i]) : 0.0;
    scale[i] = (ok ? qh / q[i] : 1.0) * gain;
    p[i] = acc + 0.5 * g;
    acc += g;
    mean += p[i];
  }
  mean /= D;
  for (int i = 0; i < D; i++) p[i] = (p[i] - mean) * gain;
}

// u[c][x] *= scale[i]; drho[x] = gain drho[x] + 3 p[i] on fluid nodes (p = rho / 3)
__global__ void k_plane_apply(float *u, float *drho, const unsigned char *solid, int D, long long plane,
                              float gain, const double *work) {
  const long long total = (long long)D * plane;
  const double *scale = work + D, *p = work + 2 * D;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / plane);
    const float s = (float)scale[i];
    u[e] *= s;
    u[total + e] *= s;
    u[2 * total + e] *= s;
    if (drho) drho[e] = gain * drho[e] + (solid[e] ? 0.0f : (float)(3.0 * p[i]));
  }
}

// Uniform cross fluxes: the flux of u_y through every y plane (and of u_z
// through every z plane) made equal to its mean, as mass conservation
// requires of a steady periodic flow, by adding delta(plane) * |u| to the
// component (|u| taken before: zero at walls and in solids, so no slip is
// made).  u: 3 x D*H*W, x the slowest index, z the fastest.  work: q[H + W]
// (plane fluxes, y planes then z planes), m[H + W] (plane sums of |u|),
// delta[H + W].  One block per plane, a fixed summation order.
__global__ void __launch_bounds__(256) k_cross_sum(const float *u, int D, int H, int W, double *work) {
  __shared__ double sq[256], sm[256];
  const int b = blockIdx.x;
  const bool ydir = b < H;
  const int c = ydir ? b : b - H;
  const long long total = (long long)D * H * W;
  const long long n = ydir ? (long long)D * W : (long long)D * H;
  double aq = 0.0, am = 0.0;
  for (long long t = threadIdx.x; t < n; t += blockDim.x) {
    long long e;
    if (ydir) e = ((t / W) * H + c) * W + t % W;  // t = i * W + k
    else e = t * W + c;                           // t = i * H + j
    const float ux = u[e], uy = u[total + e], uz = u[2 * total + e];
    aq += (double)(ydir ? uy : uz);
    am += sqrt((double)ux * ux + (double)uy * uy + (double)uz * uz);
  }
  sq[threadIdx.x] = aq;
  sm[threadIdx.x] = am;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sq[threadIdx.x] += sq[threadIdx.x + o];
      sm[threadIdx.x] += sm[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    work[b] = sq[0];
    work[H + W + b] = sm[0];
  }
}

__global__ void k_cross_fix(int H, int W, double *work) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double *q = work, *m = work + H + W;
  double *delta = work + 2 * (H + W);
  double my = 0.0, mz = 0.0;
  for (int j = 0; j < H; j++) my += q[j];
  for (int k = 0; k < W; k++) mz += q[H + k];
  my /= H;
  mz /= W;
  for (int b = 0; b < H + W; b++) delta[b] = m[b] > 0.0 ? ((b < H ? my : mz) - q[b]) / m[b] : 0.0;
}

__global__ void k_cross_apply(float *u, int D, int H, int W, const double *work) {
  const long long total = (long long)D * H * W;
  const double *delta = work + 2 * (H + W);
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(e % W), j = (int)((e / W) % H);
    const float ux = u[e], uy = u[total + e], uz = u[2 * total + e];
    const double sp = sqrt((double)ux * ux + (double)uy * uy + (double)uz * uz);
    u[total + e] = (float)(uy + delta[j] * sp);
    u[2 * total + e] = (float)(uz + delta[H + k] * sp);
  }
}

bool ok8(int ctot, int coff, int C) { return ctot % 8 == 0 && coff % 8 == 0 && C % 8 == 0 && C > 0 && coff + C <= ctot; }

int launched(const char *what) {
  slbc::count_launch();
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    slbc::set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return 1;
  }
  return 0;
}

int bad(const char *msg) {
  slbc::set_error(msg);
  return 1;
}

}  // namespace

extern "C" {

int slbc_nn_pool(const void *in, int in_ctot, int in_coff, void *out, int out_ctot, int out_coff, int B, int D, int H,
                 int W, int C, void *stream) {
  if (!ok8(in_ctot, in_coff, C) || !ok8(out_ctot, out_coff, C) || D % 2 || H % 2 || W % 2)
    return bad("slbc_nn_pool: channel slices must be multiples of 8 and the grid even");
  const long long n = (long long)B * (D / 2) * (H / 2) * (W / 2) * (C / 8);
  k_pool<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(Slice{(bf16 *)in, in_ctot, in_coff},
                                                        Slice{(bf16 *)out, out_ctot, out_coff}, B, D, H, W, C);
  return launched("slbc_nn_pool");
}

int slbc_nn_pool_bwd(const void *dcoarse, int dc_ctot, int dc_coff, void *dfine, int df_ctot, int df_coff,
                     const void *add, int a_ctot, int a_coff, const void *mask, int m_ctot, int m_coff, int B, int D,
                     int H, int W, int C, void *stream) {
  if (!ok8(dc_ctot, dc_coff, C) || !ok8(df_ctot, df_coff, C) || (add && !ok8(a_ctot, a_coff, C)) ||
      (mask && !ok8(m_ctot, m_coff, C)) || D % 2 || H % 2 || W % 2)
    return bad("slbc_nn_pool_bwd: channel slices must be multiples of 8 and the grid even");
  const long long n = (long long)B * D * H * W * (C / 8);
  k_pool_bwd<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(
      Slice{(bf16 *)dcoarse, dc_ctot, dc_coff}, Slice{(bf16 *)dfine, df_ctot, df_coff},
      Slice{(bf16 *)add, a_ctot, a_coff}, Slice{(bf16 *)mask, m_ctot, m_coff}, B, D, H, W, C);
  return launched("slbc_nn_pool_bwd");
}

int slbc_nn_up(const void *in, int in_ctot, int in_coff, void *out, int out_ctot, int out_coff, int B, int D, int H,
               int W, int C, void *stream) {
  if (!ok8(in_ctot, in_coff, C) || !ok8(out_ctot, out_coff, C) || D % 2 || H % 2 || W % 2)
    return bad("slbc_nn_up: channel slices must be multiples of 8 and the grid even");
  const long long n = (long long)B * D * H * W * (C / 8);
  k_up<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(Slice{(bf16 *)in, in_ctot, in_coff},
                                                      Slice{(bf16 *)out, out_ctot, out_coff}, B, D, H, W, C);
  return launched("slbc_nn_up");
}

int slbc_nn_up_bwd(const void *dfine, int df_ctot, int df_coff, void *dcoarse, int dc_ctot, int dc_coff,
                   const void *mask, int m_ctot, int m_coff, int B, int D, int H, int W, int C, void *stream) {
  if (!ok8(df_ctot, df_coff, C) || !ok8(dc_ctot, dc_coff, C) || (mask && !ok8(m_ctot, m_coff, C)) || D % 2 ||
      H % 2 || W % 2)
    return bad("slbc_nn_up_bwd: channel slices must be multiples of 8 and the grid even");
  const long long n = (long long)B * (D / 2) * (H / 2) * (W / 2) * (C / 8);
  k_up_bwd<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(Slice{(bf16 *)dfine, df_ctot, df_coff},
                                                          Slice{(bf16 *)dcoarse, dc_ctot, dc_coff},
                                                          Slice{(bf16 *)mask, m_ctot, m_coff}, B, D, H, W, C);
  return launched("slbc_nn_up_bwd");
}

int slbc_nn_bias_grad(const void *g, int ctot, int coff, int B, int D, int H, int W, int C, float *db, void *stream) {
  if (!ok8(ctot, coff, C) || C > 1024 || 256 % (C / 8)) return bad("slbc_nn_bias_grad: bad channel slice");
  const long long n = (long long)B * D * H * W * (C / 8);
  k_bias_grad<<<std::min(grid_for(n), 152 * 4), 256, C * sizeof(float), (cudaStream_t)stream>>>(
      Slice{(bf16 *)g, ctot, coff}, B, D, H, W, C, db);
  return launched("slbc_nn_bias_grad");
}

int slbc_nn_wfwd(const float *master, int cout, int cin, void *w, void *stream) {
  if (cin % 32 || cout < 1) return bad("slbc_nn_wfwd: cin must be a multiple of 32");
  k_wfwd<<<grid_for(27LL * cout * cin), 256, 0, (cudaStream_t)stream>>>(master, cout, cin, (bf16 *)w);
  return launched("slbc_nn_wfwd");
}

int slbc_nn_wdgrad(const float *master, int cout, int cin, int ci0, int nci, void *w, void *stream) {
  if (cout % 32 || ci0 < 0 || nci < 1 || ci0 + nci > cin) return bad("slbc_nn_wdgrad: bad channel range");
  k_wdgrad<<<grid_for(27LL * cout * nci), 256, 0, (cudaStream_t)stream>>>(master, cout, cin, ci0, nci, (bf16 *)w);
  return launched("slbc_nn_wdgrad");
}

int slbc_nn_adam(float *p, const float *g, float *m, float *v, long long n, float lr, float b1, float b2, float eps,
                 int t, void *stream) {
  if (t < 1) return bad("slbc_nn_adam: step count starts at 1");
  const float c1 = 1.0f - powf(b1, (float)t), c2 = 1.0f - powf(b2, (float)t);
  k_adam<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(p, g, m, v, n, lr, b1, b2, eps, c1, c2);
  return launched("slbc_nn_adam");
}

int slbc_nn_sqsum(const float *g, long long n, double *state, void *stream) {
  if (n <= 0) return bad("slbc_nn_sqsum: empty tensor");
  k_sqsum<<<std::min(grid_for(n), 152 * 4), 256, 0, (cudaStream_t)stream>>>(g, n, state);
  return launched("slbc_nn_sqsum");
}

int slbc_nn_clip(double *state, float factor, float decay, void *stream) {
  if (!(factor > 0.0f) || !(decay >= 0.0f && decay < 1.0f)) return bad("slbc_nn_clip: factor > 0, 0 <= decay < 1");
  k_clip_scale<<<1, 32, 0, (cudaStream_t)stream>>>(state, factor, decay);
  return launched("slbc_nn_clip");
}

int slbc_nn_scale(float *g, long long n, const double *state, void *stream) {
  if (n <= 0) return bad("slbc_nn_scale: empty tensor");
  k_scale<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(g, n, state);
  return launched("slbc_nn_scale");
}

int slbc_nn_mse(const float *pred, int ctot_p, const float *label, int nch, const float *sample_w, int B, int D, int H,
                int W, void *grad, int gctot, double *loss, void *stream) {
  if (nch < 1 || ctot_p < nch || gctot % 8 || gctot < 8 || gctot < nch) return bad("slbc_nn_mse: bad channel counts");
  k_mse<<<std::min(grid_for((long long)B * D * H * W), 152 * 4), 256, 0, (cudaStream_t)stream>>>(
      pred, ctot_p, label, nch, sample_w, B, D, H, W, (bf16 *)grad, gctot, loss);
  return launched("slbc_nn_mse");
}

int slbc_nn_proj(const float *pred, int ctot_p, const float *label, int lch, int nch, const double *lab_sq, int B, int D,
                 int H, int W, float weight, void *grad, int gctot, double *dot, double *loss, void *stream) {
  if (nch < 1 || lch < nch || ctot_p < nch || gctot % 8 || gctot < nch || B < 1 || B > 65535)
    return bad("slbc_nn_proj: bad arguments");
  const cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemsetAsync(dot, 0, sizeof(double) * B, st) != cudaSuccess) return bad("slbc_nn_proj: memset");
  const long long per = (long long)D * H * W;
  const dim3 g1((unsigned)std::min<long long>((per + 255) / 256, 152), (unsigned)B);
  k_proj_dot<<<g1, 256, 0, st>>>(pred, ctot_p, label, lch, nch, D, H, W, dot);
  if (launched("slbc_nn_proj")) return 1;
  k_proj_grad<<<std::min(grid_for((long long)B * per), 152 * 4), 256, 0, st>>>(label, lch, nch, lab_sq, dot, B, D, H,
                                                                                W, weight, (bf16 *)grad, gctot, loss);
  return launched("slbc_nn_proj");
}

int slbc_nn_encode(const unsigned char *solid, int B, int D, int H, int W, void *out, int ctot, int features,
                   void *stream) {
  if (ctot % 8 || ctot < 8) return bad("slbc_nn_encode: bad channel count");
  const long long total = (long long)B * D * H * W;
  const cudaStream_t st = (cudaStream_t)stream;
  unsigned char *a = nullptr;
  if (features) {
    // two stream-ordered scratch masks of one byte per voxel
    const cudaError_t e = cudaMallocAsync((void **)&a, 2 * total, st);
    if (e != cudaSuccess) return bad((std::string("slbc_nn_encode scratch: ") + cudaGetErrorString(e)).c_str());
    unsigned char *b = a + total;
    if (features == 2) {
      k_dist_x<kDistR2><<<grid_for(total), 256, 0, st>>>(solid, total, W, a);
      k_dist_min<kDistR2><<<grid_for(total), 256, 0, st>>>(a, total, H, W, b);
      k_dist_min<kDistR2><<<grid_for(total), 256, 0, st>>>(b, total, D, (long long)W * H, a);
    } else {
      k_dist_x<kDistR1><<<grid_for(total), 256, 0, st>>>(solid, total, W, a);
      k_dist_min<kDistR1><<<grid_for(total), 256, 0, st>>>(a, total, H, W, b);
      k_dist_min<kDistR1><<<grid_for(total), 256, 0, st>>>(b, total, D, (long long)W * H, a);
    }
    slbc::count_launch(3);
  }
  k_encode<<<grid_for(total), 256, 0, st>>>(solid, a, features == 2 ? kDistR2 : kDistR1, B, D, H, W, (bf16 *)out,
                                            ctot);
  const int rc = launched("slbc_nn_encode");
  if (a) {
    const cudaError_t e = cudaFreeAsync(a, st);
    if (e != cudaSuccess && rc == 0) return bad((std::string("slbc_nn_encode scratch: ") + cudaGetErrorString(e)).c_str());
  }
  return rc;
}

int slbc_nn_plane_flux(float *u, float *drho, const unsigned char *solid, int D, int H, int W, float force,
                       float gain, double *work, void *stream) {
  if (D < 1 || H < 1 || W < 1 || D > 65535 || !u || !solid || !work) return bad("slbc_nn_plane_flux: bad arguments");
  const cudaStream_t st = (cudaStream_t)stream;
  const long long plane = (long long)H * W;
  k_plane_sum<<<D, 256, 0, st>>>(u, D, plane, work);
  if (launched("slbc_nn_plane_flux")) return 1;
  k_plane_fix<<<1, 32, 0, st>>>(D, force, gain, work);
  if (launched("slbc_nn_plane_flux")) return 1;
  k_plane_apply<<<grid_for((long long)D * plane), 256, 0, st>>>(u, drho, solid, D, plane, gain, work);
  return launched("slbc_nn_plane_flux");
}

int slbc_nn_cross_flux(float *u, int D, int H, int W, double *work, void *stream) {
  if (D < 1 || H < 1 || W < 1 || H + W > 65535 || !u || !work) return bad("slbc_nn_cross_flux: bad arguments");
  const cudaStream_t st = (cudaStream_t)stream;
  k_cross_sum<<<H + W, 256, 0, st>>>(u, D, H, W, work);
  if (launched("slbc_nn_cross_flux")) return 1;
  k_cross_fix<<<1, 32, 0, st>>>(H, W, work);
  if (launched("slbc_nn_cross_flux")) return 1;
  k_cross_apply<<<grid_for((long long)D * H * W), 256, 0, st>>>(u, D, H, W, work);
  return launched("slbc_nn_cross_flux");
}

int slbc_nn_decode(const float *pred, int ctot_p, const unsigned char *solid, int D, int H, int W, float scale,
                   float shift_x, float *u, float drho_scale, float *drho, void *stream) {
  if (ctot_p < (drho ? 4 : 3)) return bad("slbc_nn_decode: bad channel count");
  k_decode<<<grid_for((long long)D * H * W), 256, 0, (cudaStream_t)stream>>>(pred, ctot_p, solid, D, H, W, scale,
                                                                                       shift_x, u, drho_scale, drho);
  return launched("slbc_nn_decode");
}

}  // extern "C"
