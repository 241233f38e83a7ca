#include <mutex>
#include <tuple>
#include <array>
#include <map>
// extern "C" device layer of GB300 SunlightLB (declared in slb_device.h):
// lattice state, geometry, host transfers, layout conversions, dispatch to
// the per-precision kernels, reductions, CUDA-graph replay and tracers.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <atomic>
#include <algorithm>
#include <cmath>
#include <thread>
#include <memory>
#include <new>

#include "slbc_internal.cuh"
#include "slbc_kernels.cuh"

using namespace slbc;

struct slbc_lattice {
  Lattice L;
  std::vector<unsigned char> solid_host;  // solidity per node, for body-force checks
};

struct slbc_tracer {
  slbc_lattice *h = nullptr;
  int f64 = 1;
  void *p = nullptr, *p2 = nullptr;
  double *acc = nullptr;  // tracer added by fills since creation or the last reset
  double *objstate = nullptr;
  int objstate_cap = 0;
  // FP32 tracers: the low part of p (p = hi + lo, |lo| <= half an FP32 ulp
  // of hi) kept by the stencil update on a frozen flow, swapped with p and
  // p2; lo_live says lo holds the low part (else it is taken as zero)
  float *lo = nullptr, *lo2 = nullptr;
  int lo_live = 0;
};

namespace {

thread_local std::string g_err;
std::atomic<long> g_launches{0};

int fail(const char *what, cudaError_t e) {
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return (int)e ? (int)e : 1;
}
int fail_msg(const std::string &m) {
  g_err = m;
  return 1;
}

#define CK(call)                                 \
  do {                                           \
    cudaError_t e_ = (call);                     \
    if (e_ != cudaSuccess) return fail(#call, e_); \
  } while (0)

// bytes of one stored population, and of the side arrays (body force, wall
// velocity) that the kernels read in their arithmetic type
size_t elem_size(int precision) { return precision == 0 ? 8 : precision == 1 ? 4 : 2; }

// bytes of the population array: 15 values per node, or for BF16 two copies
// of 8 paired deviations per node
size_t pop_bytes(int precision, long long npad) {
  return precision == 2 ? 2 * 16 * (size_t)npad : 15 * (size_t)npad * elem_size(precision);
}
size_t side_size(int precision) { return precision == 0 ? 8 : 4; }

// kernels that do not depend on the population type -------------------------

// Flag words from the object map: solid bit, and bit q when x - c_q differs
// in solidity from x.
__global__ void k_flags(const int *objidx, uint16_t *flags, int esi, int esj, int esk) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y, i = blockIdx.z;
  if (k >= esk) return;
  const int im = i == 0 ? esi - 1 : i - 1, ip = i == esi - 1 ? 0 : i + 1;
  const int jm = j == 0 ? esj - 1 : j - 1, jp = j == esj - 1 ? 0 : j + 1;
  const int km = k == 0 ? esk - 1 : k - 1, kp = k == esk - 1 ? 0 : k + 1;
  const int I[3] = {im, i, ip}, J[3] = {jm, j, jp}, K[3] = {km, k, kp};
  const int x = (i * esj + j) * esk + k;
  const bool solid = objidx[x] >= 0;
  uint16_t f = solid ? FLAG_SOLID : 0;
#pragma unroll
  for (int q = 1; q < 15; q++) {
    const int y = (I[1 - CX(q)] * esj + J[1 - CY(q)]) * esk + K[1 - CZ(q)];
    if ((objidx[y] >= 0) != solid) f |= (uint16_t)(1u << q);
  }
  flags[x] = f;
}

// Solid boundary nodes (a solid node with at least one boundary link, i.e. a
// fluid neighbour), compacted in node order.  Block b covers the nodes
// [b * kBndChunk, (b + 1) * kBndChunk): k_bnd_count counts them, the host
// turns the counts into offsets, and k_bnd_write writes each block's nodes
// in order (warp ballots and a running block offset).
constexpr int kBndChunk = 4096;

__device__ __forceinline__ bool boundary_solid(uint16_t f) { return (f & FLAG_SOLID) && (f & FLAG_LINKS); }

__global__ void __launch_bounds__(256) k_bnd_count(const uint16_t *flags, long long n, int *counts) {
  __shared__ int total;
  if (threadIdx.x == 0) total = 0;
  __syncthreads();
  const long long lo = (long long)blockIdx.x * kBndChunk;
  const long long hi = lo + kBndChunk < n ? lo + kBndChunk : n;
  int c = 0;
  for (long long x = lo + threadIdx.x; x < hi; x += blockDim.x) c += boundary_solid(flags[x]);
  atomicAdd(&total, c);
  __syncthreads();
  if (threadIdx.x == 0) counts[blockIdx.x] = total;
}

__global__ void __launch_bounds__(256) k_bnd_write(const uint16_t *flags, long long n, const int *offsets,
                                                   int *out) {
  __shared__ int warp_sum[8];
  __shared__ int base;
  if (threadIdx.x == 0) base = offsets[blockIdx.x];
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long lo = (long long)blockIdx.x * kBndChunk;
  const long long hi = lo + kBndChunk < n ? lo + kBndChunk : n;
  for (long long r = lo; r < hi; r += 256) {
    const long long x = r + threadIdx.x;
    const bool p = x < hi && boundary_solid(flags[x]);
    const unsigned m = __ballot_sync(0xffffffffu, p);
    if (lane == 0) warp_sum[w] = __popc(m);
    __syncthreads();
    int off = base;
    for (int v = 0; v < w; v++) off += warp_sum[v];
    if (p) out[off + __popc(m & ((1u << lane) - 1u))] = (int)x;
    __syncthreads();
    if (threadIdx.x == 0) {
      int t = 0;
      for (int v = 0; v < 8; v++) t += warp_sum[v];
      base += t;
    }
    __syncthreads();
  }
}

__global__ void k_scale(double *v, long long n, double fac) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) v[e] *= fac;
}

// distribf, level 1: one block per work piece (object o, entries lo..hi).
__global__ void k_distrib_piece(const int *bnd_node, const double *f, long long nbnd,
                                const int *piece_obj, const int *piece_lo, const int *piece_hi,
                                const double *pos, int esj, int esk, double *piece_sum) {
  const int pc = blockIdx.x;
  const int o = piece_obj[pc];
  const double px = pos[3 * o], py = pos[3 * o + 1], pz = pos[3 * o + 2];
  double v[6] = {0, 0, 0, 0, 0, 0};
  for (int e = piece_lo[pc] + threadIdx.x; e < piece_hi[pc]; e += blockDim.x) {
    const int x = bnd_node[e];
    const int k = x % esk, r = x / esk, j = r % esj, i = r / esj;
    const double rx = i - px, ry = j - py, rz = k - pz;
    const double fx = f[e], fy = f[nbnd + e], fz = f[2 * nbnd + e];
    v[0] += fx; v[1] += fy; v[2] += fz;
    v[3] += ry * fz - rz * fy;
    v[4] += rz * fx - rx * fz;
    v[5] += rx * fy - ry * fx;
  }
  block_sum<6>(v);
  if (threadIdx.x == 0)
    for (int c = 0; c < 6; c++) piece_sum[6 * pc + c] = v[c];
}

// distribf, level 2: per object, its pieces in order.
__global__ void k_distrib_obj(const int *obj_first_piece, const int *obj_npiece,
                              const double *piece_sum, int nobj, double *ft) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= nobj) return;
  double v[6] = {0, 0, 0, 0, 0, 0};
  for (int pc = obj_first_piece[o]; pc < obj_first_piece[o] + obj_npiece[o]; pc++)
    for (int c = 0; c < 6; c++) v[c] += piece_sum[6 * pc + c];
  for (int c = 0; c < 6; c++) ft[6 * o + c] = v[c];
}

// Per fluid node, the boundary links whose solid end adsorbs (bit q: the
// solid node x - c_q has its adsorption byte set).
__global__ void k_ads_links(const uint16_t *flags, const unsigned char *ads, uint16_t *links, int esi,
                            int esj, int esk) {
  const long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= (long long)esi * esj * esk) return;
  const uint16_t fl = flags[x];
  uint16_t mask = 0;
  if (!(fl & FLAG_SOLID) && (fl & FLAG_LINKS)) {
    int i, j, k;
    decode((int)x, esj, esk, i, j, k);
    const Nbr nb = make_nbr(i, j, k, esi, esj, esk);
#pragma unroll
    for (int q = 1; q < 15; q++)
      if (((fl >> q) & 1) && ads[nb.at(-CX(q), -CY(q), -CZ(q))]) mask |= (uint16_t)(1u << q);
  }
  links[x] = mask;
}

// Staging for k_setvel from three device FP32 velocity arrays and, if
// given, the density deviations rho - rho0 (else rho = rho0).
__global__ void k_stage_velocity(const float *u, const float *drho, long long nnodes, long long x0, long long n,
                                 double *stage) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const long long x = x0 + e;
  stage[4 * e] = drho ? (double)drho[x] : 0.0;
  stage[4 * e + 1] = u[x];
  stage[4 * e + 2] = u[nnodes + x];
  stage[4 * e + 3] = u[2 * nnodes + x];
}

// tracer sums: fluid, solid, adsorbing, first and second moment along axis
template <typename TP>
__global__ void __launch_bounds__(kReduceThreads)
k_mp_sums(const TP *p, const uint16_t *flags, const unsigned char *ads, long long n, int esj,
          int esk, int axis, double *partials) {
  double v[5] = {0, 0, 0, 0, 0};
  for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < n;
       x += (long long)gridDim.x * blockDim.x) {
    const double pv = (double)p[x];
    const bool solid = flags[x] & FLAG_SOLID;
    if (solid) v[1] += pv; else v[0] += pv;
    if (ads && ads[x]) v[2] += pv;
    if (!solid && axis >= 0) {
      const int k = (int)(x % esk), r = (int)(x / esk), j = r % esj, i = r / esj;
      const double pos = axis == 0 ? i : axis == 1 ? j : k;
      v[3] += pv * pos;
      v[4] += pv * pos * pos;
    }
  }
  block_sum<5>(v);
  if (threadIdx.x == 0)
    for (int c = 0; c < 5; c++) partials[5 * blockIdx.x + c] = v[c];
}

template <typename TP>
__global__ void k_mp_minmax(const TP *p, const uint16_t *flags, long long n, double *partials) {
  double lo = 1e300, hi = -1e300;
  for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < n;
       x += (long long)gridDim.x * blockDim.x) {
    if (flags[x] & FLAG_SOLID) continue;
    const double pv = (double)p[x];
    lo = pv < lo ? pv : lo;
    hi = pv > hi ? pv : hi;
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_down_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_down_sync(0xffffffffu, hi, o));
  }
  __shared__ double sl[32], sh[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { sl[warp] = lo; sh[warp] = hi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) { lo = fmin(lo, sl[w]); hi = fmax(hi, sh[w]); }
    partials[2 * blockIdx.x] = lo;
    partials[2 * blockIdx.x + 1] = hi;
  }
}

// Node of entry e of a plane (axis 0: i = pos, 1: j = pos, 2: k = pos).
__device__ __forceinline__ long long plane_node(long long e, int axis, int pos, int esi, int esj, int esk) {
  int i, j, k;
  if (axis == 0) { i = pos; j = (int)(e / esk); k = (int)(e % esk); }
  else if (axis == 1) { j = pos; i = (int)(e / esk); k = (int)(e % esk); }
  else { k = pos; i = (int)(e / esj); j = (int)(e % esj); }
  return ((long long)i * esj + j) * esk + k;
}

// Tracer injection on the fluid nodes of a region (reference src/mpobjs.c).
// Kind 2 (a wall) visits only the nodes of its plane.  Each block also
// writes the sum of (value - old p) over the nodes it set, so the host
// layer can keep count of the tracer the fills have added.
template <typename TP>
__global__ void __launch_bounds__(kReduceThreads)
k_mp_fill(TP *p, float *lo, const uint16_t *flags, int esi, int esj, int esk, int kind, double g0, double g1,
          double g2, double g3, double g4, double g5, double value, long long count, double *partials) {
  double v[1] = {0.0};
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (long long)gridDim.x * blockDim.x) {
    const long long x = kind == 2 ? plane_node(e, (int)g0, (int)g1, esi, esj, esk) : e;
    if (flags[x] & FLAG_SOLID) continue;
    const int k = (int)(x % esk), r = (int)(x / esk), j = r % esj, i = r / esj;
    bool in = false;
    switch (kind) {
      case 0: in = true; break;
      case 1: in = i > g0 && i < g1 && j > g2 && j < g3 && k > g4 && k < g5; break;
      case 2: in = true; break;
      case 3: {
        const double rsq = (i - g1) * (i - g1) + (j - g2) * (j - g2) + (k - g3) * (k - g3);
        in = rsq < g0 * g0;
      } break;
      case 4: {
        const int ax = (int)g0;
        const double u = ax == 0 ? j : i, w = ax == 2 ? j : k;
        const double rsq = (u - g3) * (u - g3) + (w - g4) * (w - g4);
        in = rsq < g2 * g2;
        if (g1 != 0.0) in = !in;
      } break;
    }
    if (in) {
      const TP nv = (TP)value;
      v[0] += (double)nv - (double)p[x] - (lo ? (double)lo[x] : 0.0);
      p[x] = nv;
      if (lo) lo[x] = 0.0f;
    }
  }
  block_sum<1>(v);
  if (threadIdx.x == 0) partials[blockIdx.x] = v[0];
}

// acc[0] += sum of nb partials, in a fixed order
__global__ void __launch_bounds__(256) k_sum_into(const double *partials, int nb, double *acc) {
  double v[1] = {0.0};
  for (int b = threadIdx.x; b < nb; b += blockDim.x) v[0] += partials[b];
  block_sum<1>(v);
  if (threadIdx.x == 0) acc[0] += v[0];
}

// sum of p and number of fluid nodes on one plane
template <typename TP>
__global__ void __launch_bounds__(kReduceThreads)
k_mp_plane(const TP *p, const uint16_t *flags, int esi, int esj, int esk, int axis, int pos,
           long long count, double *partials) {
  double v[2] = {0.0, 0.0};
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < count;
       e += (long long)gridDim.x * blockDim.x) {
    const long long x = plane_node(e, axis, pos, esi, esj, esk);
    if (flags[x] & FLAG_SOLID) continue;
    v[0] += (double)p[x];
    v[1] += 1.0;
  }
  block_sum<2>(v);
  if (threadIdx.x == 0) { partials[2 * blockIdx.x] = v[0]; partials[2 * blockIdx.x + 1] = v[1]; }
}

template <typename TP>
__global__ void k_mp_misc(TP *p, const TP *src, const uint16_t *flags, const unsigned char *ads,
                          long long n, int op, double fac) {
  const long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= n) return;
  const bool solid = flags[x] & FLAG_SOLID;
  if (op == 0) { if (!solid) p[x] = p[x] * (TP)fac; }           // rescale
  else if (op == 1) { if (ads && ads[x]) p[x] = TP(0); }       // adzero
  else if (op == 2) { if (!solid) p[x] = p[x] + src[x]; }      // add
}

template <typename TD, typename TS>
__global__ void k_convert(TD *dst, const TS *src, long long n) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n) dst[e] = (TD)src[e];
}

int blocks_for(long long n, int bs) { return (int)((n + bs - 1) / bs); }

// per-precision dispatch ------------------------------------------------------
#define DISPATCH(L, name, ...)                                               \
  ((L).precision == 0 ? name##_f64(__VA_ARGS__) : name##_f32(__VA_ARGS__))
// operations that also exist for BF16 deviation storage
#define DISPATCH3(L, name, ...)                                              \
  ((L).precision == 2 ? name##_bf16(__VA_ARGS__) : DISPATCH(L, name, __VA_ARGS__))

int no_bf16(const Lattice &L, const char *what) {
  if (L.precision != 2) return 0;
  g_err = std::string(what) + ": not available for BF16 deviation storage (use FP32 or FP64 populations)";
  return 1;
}

int ensure_staging(Lattice &L, long long nodes, int per_node) {
  const long long want = std::min<long long>(nodes, 1 << 20);
  if (L.staging && L.staging_nodes >= want * per_node) return 0;
  if (L.staging) cudaFree(L.staging);
  L.staging = nullptr;
  CK(cudaMalloc(&L.staging, (size_t)want * per_node * sizeof(double)));
  L.staging_nodes = want * per_node;
  return 0;
}

int ensure_scratch(Lattice &L) {
  if (L.scratch) return 0;
  CK(cudaMalloc(&L.scratch, pop_bytes(L.precision, L.npad)));
  return 0;
}

int ensure_partials(Lattice &L, int n) {
  if (L.partials && L.npartials >= n) return 0;
  if (L.partials) cudaFree(L.partials);
  L.partials = nullptr;
  CK(cudaMalloc(&L.partials, (size_t)n * sizeof(double)));
  L.npartials = n;
  return 0;
}

// put the state into a post-collision AA layout (C0 or C1); BF16 storage
// has the reference's layout only
int to_aa(Lattice &L) {
  if (L.precision == 2) return 0;
  if (L.layout == SLBC_LAYOUT_N) {
    CK(DISPATCH(L, launch_swap, L));
    L.layout = SLBC_LAYOUT_C0;
  }
  return 0;
}

// put the state into layout N
int to_natural(Lattice &L) {
  if (L.layout != SLBC_LAYOUT_N && no_bf16(L, "conversion to the reference layout")) return 1;
  if (L.layout == SLBC_LAYOUT_C0) {
    CK(DISPATCH(L, launch_swap, L));
  } else if (L.layout == SLBC_LAYOUT_C1) {
    if (ensure_scratch(L)) return 1;
    CK(DISPATCH(L, launch_to_natural, L));
    std::swap(L.pop, L.scratch);
    L.generation++;  // captured graphs hold the old buffer
  }
  L.layout = SLBC_LAYOUT_N;
  return 0;
}

const char *kPairSkipSolid =
    "BF16 paired-deviation storage relaxes solid nodes too: set skip_solid = 0 or use FP32 populations";

int one_step(Lattice &L) {
  if (L.precision == 2) {
    if (L.par.skip_solid) return fail_msg(kPairSkipSolid);
    CK(launch_step_bf16(L, 0));
    return 0;
  }
  const int odd = L.layout == SLBC_LAYOUT_C0;
  CK(DISPATCH3(L, launch_step, L, odd));
  L.layout = odd ? SLBC_LAYOUT_C1 : SLBC_LAYOUT_C0;
  return 0;
}

// Autotuner of the fused step: for each parity, time every candidate launch
// shape (rows per thread, threads along k) on a copy of the populations --
// the lattice's own state is not touched -- and keep the fastest.  Lattices
// below 2^20 nodes use the default shape; SLB_AUTOTUNE=0 disables tuning.
// Launch shapes chosen so far, per lattice shape and precision: a later
// lattice of the same shape starts from them instead of timing candidates.
struct TuneKey {
  int esi, esj, esk, precision;
  bool operator<(const TuneKey &o) const {
    return std::tie(esi, esj, esk, precision) < std::tie(o.esi, o.esj, o.esk, o.precision);
  }
};
std::map<TuneKey, std::array<StepConfig, 2>> g_tuned;
std::mutex g_tuned_lock;

int autotune_time(Lattice &L);

}  // namespace

namespace slbc {
bool vec4_ok(const Lattice &L) { return L.precision == 1 && L.esk % 4 == 0 && L.npad % 4 == 0; }
}  // namespace slbc

namespace {

int autotune(Lattice &L) {
  {
    std::lock_guard<std::mutex> guard(g_tuned_lock);
    auto it = g_tuned.find(TuneKey{L.esi, L.esj, L.esk, L.precision});
    if (it != g_tuned.end()) {
      L.tuned[0] = it->second[0];
      L.tuned[1] = it->second[1];
      L.tune_state = 1;
      L.generation++;
      return 0;
    }
  }
  return autotune_time(L);
}

int autotune_time(Lattice &L) {
  // FP64/FP32: {rows per thread, threads along k}; BF16: {planes per block, 32}
  static const int cand_fp[][2] = {{1, 64},  {1, 128}, {2, 64}, {2, 128}, {1, 256},
                                   {2, 256}, {4, 64},  {4, 128}, {kStepVec4, kV4Threads}};
  const bool bf = L.precision == 2;
  // BF16: powers of two, and the plane counts that fill one or two waves of
  // three blocks per SM evenly
  int cand_bf[7][2] = {{1, 32}, {2, 32}, {4, 32}, {8, 32}, {16, 32}, {0, 32}, {0, 32}};
  int nbf = 5;
  {
    const long long tiles = (long long)((L.esk + kTileK - 1) / kTileK) * ((L.esj + kTileJ - 1) / kTileJ);
    for (int w = 1; w <= 2; w++) {
      const long long chunks = std::max<long long>(1, (w * 152LL * 3 + tiles - 1) / tiles);
      const int planes = (int)std::min<long long>(64, (L.esi + chunks - 1) / chunks);
      bool dup = false;
      for (int c = 0; c < nbf; c++) dup = dup || cand_bf[c][0] == planes;
      if (!dup) cand_bf[nbf++][0] = planes;
    }
  }
  const int (*cand)[2] = bf ? cand_bf : cand_fp;
  const int ncand = bf ? nbf : (vec4_ok(L) ? 9 : 8);
  const char *env = getenv("SLB_AUTOTUNE");
  for (int p = 0; p < 2; p++) {
    L.tuned[p].npt = bf ? bf16_default_planes(L) : 1;
    L.tuned[p].block_k = bf ? 32 : 128;
  }
  if ((env && env[0] == '0') || L.nnodes < (1LL << 20) || L.esk < 64) {
    L.tune_state = -1;
    return 0;
  }
  // FP64/FP32 candidates run on a copy of the populations; a BF16 update
  // reads the current copy of the state and writes the other one, so it
  // runs on the lattice itself without changing its state
  if (!bf) {
    if (ensure_scratch(L)) return 1;
    CK(cudaMemcpyAsync(L.scratch, L.pop, pop_bytes(L.precision, L.npad), cudaMemcpyDeviceToDevice, L.stream));
    std::swap(L.pop, L.scratch);
  }
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  int rc = 0;
  const int nparity = bf ? 1 : 2;  // BF16: one update kernel for both parities
  for (int parity = 0; parity < nparity && !rc; parity++) {
    float best = 1e30f;
    int besti = 1;
    for (int c = 0; c < ncand && !rc; c++) {
      L.tuned[parity].npt = cand[c][0];
      L.tuned[parity].block_k = cand[c][1];
      float tmin = 1e30f;
      for (int rep = 0; rep < 4 && !rc; rep++) {
        cudaEventRecord(e0, L.stream);
        const cudaError_t le = bf ? launch_pair_step(L, cand[c][0]) : DISPATCH(L, launch_step, L, parity);
        if (le != cudaSuccess) rc = 1;
        cudaEventRecord(e1, L.stream);
        if (cudaEventSynchronize(e1) != cudaSuccess) rc = 1;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < tmin) tmin = ms;
      }
      if (tmin < best) { best = tmin; besti = c; }
    }
    L.tuned[parity].npt = cand[besti][0];
    L.tuned[parity].block_k = cand[besti][1];
  }
  if (bf) L.tuned[1] = L.tuned[0];
  g_launches -= nparity * ncand * 4;  // tuning launches are not part of the simulation
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!bf) std::swap(L.pop, L.scratch);
  if (rc) return fail_msg("autotune: a candidate launch failed");
  L.tune_state = 1;
  L.generation++;
  std::lock_guard<std::mutex> guard(g_tuned_lock);
  g_tuned[TuneKey{L.esi, L.esj, L.esk, L.precision}] = {L.tuned[0], L.tuned[1]};
  return 0;
}

constexpr int kGraphPairs = 25;  // one graph = 50 steps, starting from C0

int ensure_graph(Lattice &L) {
  if (L.graph && L.graph_generation == L.generation && L.graph_mom == L.mom_cur) return 0;
  if (L.graph) { cudaGraphExecDestroy(L.graph); L.graph = nullptr; }
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(L.stream, cudaStreamCaptureModeThreadLocal));
  const int saved = L.layout;
  L.layout = SLBC_LAYOUT_C0;
  int rc = 0;
  for (int s = 0; s < 2 * kGraphPairs && !rc; s++) rc = one_step(L);
  L.layout = saved;
  cudaError_t e = cudaStreamEndCapture(L.stream, &g);
  if (rc) return rc;
  if (e != cudaSuccess) return fail("cudaStreamEndCapture", e);
  // the captured launches were counted at capture time; replays count below
  g_launches -= 2 * kGraphPairs;
  e = cudaGraphInstantiate(&L.graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail("cudaGraphInstantiate", e);
  L.graph_steps = 2 * kGraphPairs;
  L.graph_generation = L.generation;
  L.graph_mom = L.mom_cur;
  return 0;
}

}  // namespace

namespace slbc {

// 1/rho of the FP64 density snapshot, for the FP32 tracer update
__global__ void k_mp_rinv(const double *rho64, float *rinv, long long n) {
  const long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (x < n) rinv[x] = (float)(1.0 / rho64[x]);
}

// One FP32 tracer update from stencil coefficients (k_mp_coef):
// p'(x) = C_0(x) p(x) + sum_q C_q(x) p(x - c_q).  Tiles of 32 (k) x 8 (j)
// nodes march along i with p of three planes (and halo) in shared memory,
// the next plane prefetched into registers; the 15 coefficient loads per
// node are the stream from memory.
//
// p is held as hi + lo (float-float) and the sum is formed with error-free
// products and sums, so the update adds no rounding of its own beyond about
// 2^-44 of p.  A plain FP32 sum stalls once the field is close to steady:
// the remaining change of each node is below half an ulp, rounds away with
// the same sign at every update, and tracer mass drains at a steady rate.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__global__ void __launch_bounds__(kTileThreads, 4)
k_mp_apply(const float *coef, const float *pin, const float *lin, float *pout, float *lout, int esi, int esj,
           int esk, unsigned npad, int planes) {
  __shared__ float2 ring[3][kPlane];
  const int tk = threadIdx.x, tj = threadIdx.y, tid = tj * kTileK + tk;
  const int k0 = blockIdx.x * kTileK, j0 = blockIdx.y * kTileJ, i0 = blockIdx.z * planes;
  const int np = min(planes, esi - i0);
  const int plane_nodes = esj * esk;
  int off[kPlaneLoads];
#pragma unroll
  for (int e = 0; e < kPlaneLoads; e++) {
    const int c = tid + kTileThreads * e;
    off[e] = c < kPlane ? wrap_index(j0 - 1 + c / kHaloK, esj) * esk + wrap_index(k0 - 1 + c % kHaloK, esk) : -1;
  }
#pragma unroll
  for (int h = 0; h < 2; h++) {
    const int base = wrap_index(i0 - 1 + h, esi) * plane_nodes;
#pragma unroll
    for (int e = 0; e < kPlaneLoads; e++)
      if (off[e] >= 0) ring[h][tid + kTileThreads * e] = make_float2(pin[base + off[e]], lin[base + off[e]]);
  }
  float2 pre[kPlaneLoads];
  auto prefetch = [&](int plane) {
    const int base = wrap_index(plane, esi) * plane_nodes;
#pragma unroll
    for (int e = 0; e < kPlaneLoads; e++)
      if (off[e] >= 0) pre[e] = make_float2(pin[base + off[e]], lin[base + off[e]]);
  };
  prefetch(i0 + 1);
  const int j = j0 + tj, k = k0 + tk;
  const bool mine = j < esj && k < esk;
  const int own = mine ? j * esk + k : 0;
  const int c0 = (tj + 1) * kHaloK + tk + 1;
  for (int ii = 0; ii < np; ii++) {
    const int i = i0 + ii;
    const int sm = ii % 3, s0 = (ii + 1) % 3, sp = (ii + 2) % 3;  // planes i-1, i, i+1
    __syncthreads();  // slot sp held plane i-2, last read in the previous iteration
#pragma unroll
    for (int e = 0; e < kPlaneLoads; e++)
      if (off[e] >= 0) ring[sp][tid + kTileThreads * e] = pre[e];
    __syncthreads();
    if (ii + 1 < np) prefetch(i + 2);
    if (!mine) continue;
    const float2 *R[3] = {ring[sm], ring[s0], ring[sp]};
    const unsigned x = (unsigned)(i * plane_nodes + own);
    float cq[15];
#pragma unroll
    for (int q = 0; q < 15; q++) cq[q] = __ldcs(coef + q * npad + x);
    float sh = 0.0f, sl = 0.0f;
#pragma unroll
    for (int q = 0; q < 15; q++) {
      const float2 v = q == 0 ? R[1][c0] : R[1 - CX(q)][c0 - CY(q) * kHaloK - CZ(q)];
      const float ph = __fmul_rn(cq[q], v.x);
      const float pe = __fmaf_rn(cq[q], v.x, -ph);  // exact error of the product
      float s, e;
      two_sum(sh, ph, s, e);
      sh = s;
      sl = __fadd_rn(sl, __fadd_rn(e, __fmaf_rn(cq[q], v.y, pe)));
    }
    const float hi = __fadd_rn(sh, sl);
    pout[x] = hi;
    lout[x] = __fsub_rn(sl, __fsub_rn(hi, sh));
  }
}

// Tracer mass on a frozen flow: what a fluid node y sends to all receivers
// (its column of the stencil: C_0(y) and C_q(y + c_q), q = 1..14) adds up to
// rho(y)/rho(y) = 1 in exact arithmetic.  In FP32 the column misses 1 by the
// rounding of 1/rho and of the terms, with the same sign at every update;
// this pass adds the FP64 residual 1 - sum to C_0(y), so that the stencil
// conserves mass to the rounding of C_0 alone.
__global__ void k_mp_coef_norm(float *coef, const uint16_t *flags, int esi, int esj, int esk, unsigned npad) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)esi * esj * esk) return;
  const int x = (int)e;
  if (flags[x] & FLAG_SOLID) return;
  int i, j, k;
  decode(x, esj, esk, i, j, k);
  const Nbr nb = make_nbr(i, j, k, esi, esj, esk);
  double sum = coef[x];
#pragma unroll
  for (int q = 1; q < 15; q++) sum += (double)coef[q * npad + (unsigned)nb.at(CX(q), CY(q), CZ(q))];
  coef[x] = (float)((double)coef[x] + (1.0 - sum));
}

cudaError_t launch_mp_coef_norm(Lattice &L) {
  k_mp_coef_norm<<<(int)((L.nnodes + 255) / 256), 256, 0, L.stream>>>(L.mp_coef, L.flags, L.esi, L.esj, L.esk,
                                                                      (unsigned)L.npad);
  g_launches += 1;
  return cudaGetLastError();
}

cudaError_t launch_mp_apply(Lattice &L, const float *pin, const float *lin, float *pout, float *lout, dim3 grid,
                            dim3 block, int planes) {
  k_mp_apply<<<grid, block, 0, L.stream>>>(L.mp_coef, pin, lin, pout, lout, L.esi, L.esj, L.esk, (unsigned)L.npad,
                                           planes);
  g_launches += 1;
  return cudaGetLastError();
}

cudaError_t ensure_mp_rinv(Lattice &L) {
  if (L.mp_rinv32 && L.mp_rinv_gen == L.mp_rho_gen) return cudaSuccess;
  if (!L.mp_rho64) return cudaErrorInvalidValue;
  cudaError_t e = cudaSuccess;
  if (!L.mp_rinv32) e = cudaMalloc(&L.mp_rinv32, (size_t)L.nnodes * sizeof(float));
  if (e != cudaSuccess) return e;
  k_mp_rinv<<<(int)((L.nnodes + 255) / 256), 256, 0, L.stream>>>(L.mp_rho64, L.mp_rinv32, L.nnodes);
  g_launches += 1;
  e = cudaGetLastError();
  if (e == cudaSuccess) L.mp_rinv_gen = L.mp_rho_gen;
  return e;
}

void count_launch(int n) { g_launches += n; }
void set_error(const std::string &msg) { g_err = msg; }
int reduction_blocks(const Lattice &L) {
  // 8 blocks of 256 threads per SM, fewer for small lattices
  return (int)std::max<long long>(1, std::min<long long>((L.nnodes + 255) / 256, 152 * 8));
}
}  // namespace slbc

// ============================================================================
// Host loop over [0, n) in contiguous ranges on up to 32 threads (one per
// core), fn(lo, hi) per range; inline below two ranges of `grain`.
template <typename F>
static void host_par_for(long long n, long long grain, F fn) {
  long long t = std::min<long long>(std::max(1u, std::thread::hardware_concurrency()), 32);
  t = std::min(t, grain > 0 ? n / grain : t);
  if (t <= 1) {
    fn(0LL, n);
    return;
  }
  std::vector<std::thread> th;
  for (long long i = 1; i < t; i++) th.emplace_back(fn, n * i / t, n * (i + 1) / t);
  fn(0LL, n / t);
  for (auto &x : th) x.join();
}

extern "C" {

const char *slbc_last_error(void) { return g_err.c_str(); }
long slbc_launch_count(void) { return g_launches.load(); }

int slbc_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
  return n;
}

int slbc_create(slbc_lattice **out, int esi, int esj, int esk, int precision) {
  *out = nullptr;
  if (esi < 1 || esj < 1 || esk < 1) return fail_msg("slbc_create: lattice sides must be >= 1");
  const long long n = (long long)esi * esj * esk;
  if (n >= (1LL << 31)) return fail_msg("slbc_create: lattice has 2^31 nodes or more");
  if (precision < 0 || precision > 2)
    return fail_msg("slbc_create: precision must be 0 (FP64), 1 (FP32) or 2 (BF16 deviations)");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail_msg("slbc_create: no CUDA device is available (the GB300 library has no CPU path)");
  slbc_lattice *h = new slbc_lattice();
  Lattice &L = h->L;
  L.esi = esi; L.esj = esj; L.esk = esk; L.precision = precision;
  L.nnodes = n;
  L.npad = (n + 63) / 64 * 64;
  L.par.tau = 0.75; L.par.rho0 = 72.0;
  h->solid_host.assign((size_t)n, 0);
  cudaError_t e = cudaMalloc(&L.pop, pop_bytes(precision, L.npad));
  if (e == cudaSuccess) e = cudaMemset(L.pop, 0, pop_bytes(precision, L.npad));
  if (e == cudaSuccess) e = cudaMalloc(&L.flags, (size_t)n * sizeof(uint16_t));
  if (e == cudaSuccess) e = cudaMemset(L.flags, 0, (size_t)n * sizeof(uint16_t));
  if (e == cudaSuccess) e = cudaMalloc(&L.objidx, (size_t)n * sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(L.objidx, 0xff, (size_t)n * sizeof(int));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMallocHost(&L.host_out, 64 * sizeof(double));
  for (int b = 0; b < 2 && e == cudaSuccess && precision == 2; b++) {
    e = cudaMalloc(&L.mom[b], (size_t)L.npad * 4 * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(L.mom[b], 0, (size_t)L.npad * 4 * sizeof(float));
  }
  if (e != cudaSuccess) {
    slbc_destroy(h);
    return fail("slbc_create", e);
  }
  L.own_stream = true;
  L.layout = SLBC_LAYOUT_N;
  *out = h;
  return 0;
}

void slbc_destroy(slbc_lattice *h) {
  if (!h) return;
  Lattice &L = h->L;
  if (L.stream) cudaStreamSynchronize(L.stream);
  void *bufs[] = {L.pop, L.scratch, L.flags, L.bnd_node, L.bnd_obj, L.bnd_f, L.piece_obj,
                  L.piece_lo, L.piece_hi, L.piece_sum, L.obj_pos, L.obj_ft, L.ads, L.objidx,
                  L.bf, L.uw, L.partials, L.staging, L.mp_rho64, L.mp_rho32, L.mom[0], L.mom[1],
                  L.ads_links, L.mp_rinv32, L.mp_coef, L.move_buf};
  for (void *b : bufs) if (b) cudaFree(b);
  if (L.host_out) cudaFreeHost(L.host_out);
  if (L.graph) cudaGraphExecDestroy(L.graph);
  if (L.stream && L.own_stream) cudaStreamDestroy(L.stream);
  delete h;
}

int slbc_set_stream(slbc_lattice *h, void *stream) {
  Lattice &L = h->L;
  CK(cudaStreamSynchronize(L.stream));
  if (L.own_stream) cudaStreamDestroy(L.stream);
  L.stream = (cudaStream_t)stream;
  L.own_stream = false;
  L.generation++;
  return 0;
}

void *slbc_get_stream(slbc_lattice *h) { return (void *)h->L.stream; }

int slbc_synchronize(slbc_lattice *h) {
  CK(cudaStreamSynchronize(h->L.stream));
  return 0;
}

int slbc_layout(slbc_lattice *h) { return h->L.layout; }

int slbc_get_tuning(slbc_lattice *h, int cfg[4]) {
  const Lattice &L = h->L;
  cfg[0] = L.tuned[0].npt; cfg[1] = L.tuned[0].block_k;
  cfg[2] = L.tuned[1].npt; cfg[3] = L.tuned[1].block_k;
  return L.tune_state;
}

int slbc_set_tuning(slbc_lattice *h, const int cfg[4]) {
  Lattice &L = h->L;
  for (int p = 0; p < 2; p++) {
    const int npt = cfg[2 * p], bx = cfg[2 * p + 1];
    if (L.precision == 2) {
      if (npt < 1 || npt > 64 || bx != 32)
        return fail_msg("slbc_set_tuning: BF16 lattices take 1 to 64 planes per block and 32 threads along k");
    } else if (npt == kStepVec4) {
      if (!vec4_ok(L) || bx != kV4Threads)
        return fail_msg("slbc_set_tuning: the 4-wide form needs FP32 populations, esk a multiple of 4 and "
                        "128 threads per block");
    } else if ((npt != 1 && npt != 2 && npt != 4) || (bx != 32 && bx != 64 && bx != 128 && bx != 256)) {
      return fail_msg("slbc_set_tuning: rows per thread must be 1, 2 or 4 and threads along k 32, 64, 128 or 256");
    }
    L.tuned[p].npt = npt;
    L.tuned[p].block_k = bx;
  }
  L.tune_state = 1;
  L.generation++;
  return 0;
}

// object map and flag words
static int geometry_flags(Lattice &L, slbc_lattice *h, const int *objidx) {
  L.ads_version++;  // the boundary links change
  const long long n = L.nnodes;
  unsigned char *solid = h->solid_host.data();
  host_par_for(n, 1LL << 20, [&](long long lo, long long hi) {
    for (long long x = lo; x < hi; x++) solid[x] = objidx[x] >= 0;
  });
  CK(cudaMemcpyAsync(L.objidx, objidx, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, L.stream));
  const int bx = L.esk >= 128 ? 128 : 32;
  dim3 grid((L.esk + bx - 1) / bx, L.esj, L.esi);
  k_flags<<<grid, bx, 0, L.stream>>>(L.objidx, L.flags, L.esi, L.esj, L.esk);
  count_launch();
  CK(cudaGetLastError());
  return 0;
}

// boundary list (sorted by object, node order within an object), node
// forces and the distribf pieces
static int geometry_boundary(Lattice &L, int nobj, const long *bnd_node, const int *bnd_obj, long nbnd) {
  void *old[] = {L.bnd_node, L.bnd_obj, L.bnd_f, L.piece_obj, L.piece_lo, L.piece_hi,
                 L.piece_sum, L.obj_pos, L.obj_ft};
  CK(cudaStreamSynchronize(L.stream));
  for (void *b : old) if (b) cudaFree(b);
  L.bnd_node = L.bnd_obj = nullptr; L.bnd_f = nullptr;
  L.piece_obj = L.piece_lo = L.piece_hi = nullptr; L.piece_sum = nullptr;
  L.obj_pos = L.obj_ft = nullptr;
  L.nbnd = nbnd; L.nobj = nobj; L.npiece = 0;
  if (nbnd > 0) {
    std::vector<int> nodes((size_t)nbnd);
    host_par_for(nbnd, 1LL << 20, [&](long long lo, long long hi) {
      for (long long e = lo; e < hi; e++) nodes[e] = (int)bnd_node[e];
    });
    CK(cudaMalloc(&L.bnd_node, nbnd * sizeof(int)));
    CK(cudaMalloc(&L.bnd_obj, nbnd * sizeof(int)));
    CK(cudaMalloc(&L.bnd_f, 3 * nbnd * sizeof(double)));
    CK(cudaMemcpy(L.bnd_node, nodes.data(), nbnd * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(L.bnd_obj, bnd_obj, nbnd * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemset(L.bnd_f, 0, 3 * nbnd * sizeof(double)));
  }
  if (nobj > 0) {
    // distribf pieces: each object's run of the list, split into chunks
    const int chunk = 4096;
    std::vector<int> po, plo, phi, first((size_t)nobj, 0), cnt((size_t)nobj, 0);
    long e = 0;
    for (int o = 0; o < nobj; o++) {
      first[o] = (int)po.size();
      long lo = e;
      while (e < nbnd && bnd_obj[e] == o) e++;
      for (long s = lo; s < e; s += chunk) {
        po.push_back(o); plo.push_back((int)s); phi.push_back((int)std::min<long>(e, s + chunk));
        cnt[o]++;
      }
    }
    if (e != nbnd) return fail_msg("slbc_set_geometry: boundary list not sorted by object");
    L.npiece = (int)po.size();
    CK(cudaMalloc(&L.obj_pos, 3 * nobj * sizeof(double)));
    CK(cudaMalloc(&L.obj_ft, (6 * nobj + 2 * nobj) * sizeof(double)));
    // first/count stored after the 6*nobj results, as ints
    CK(cudaMemcpy((int *)(L.obj_ft + 6 * nobj), first.data(), nobj * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy((int *)(L.obj_ft + 6 * nobj) + nobj, cnt.data(), nobj * sizeof(int), cudaMemcpyHostToDevice));
    if (L.npiece > 0) {
      CK(cudaMalloc(&L.piece_obj, L.npiece * sizeof(int)));
      CK(cudaMalloc(&L.piece_lo, L.npiece * sizeof(int)));
      CK(cudaMalloc(&L.piece_hi, L.npiece * sizeof(int)));
      CK(cudaMalloc(&L.piece_sum, 6 * (size_t)L.npiece * sizeof(double)));
      CK(cudaMemcpy(L.piece_obj, po.data(), L.npiece * sizeof(int), cudaMemcpyHostToDevice));
      CK(cudaMemcpy(L.piece_lo, plo.data(), L.npiece * sizeof(int), cudaMemcpyHostToDevice));
      CK(cudaMemcpy(L.piece_hi, phi.data(), L.npiece * sizeof(int), cudaMemcpyHostToDevice));
    }
  }
  L.generation++;
  return 0;
}

int slbc_set_geometry(slbc_lattice *h, const int *objidx, int nobj, const long *bnd_node,
                      const int *bnd_obj, long nbnd) {
  Lattice &L = h->L;
  if (geometry_flags(L, h, objidx)) return 1;
  return geometry_boundary(L, nobj, bnd_node, bnd_obj, nbnd);
}

// boundary nodes in node order, found on the GPU from the flag words, then
// grouped by object (objidx: the host copy of the object map)
static int boundary_from_flags(Lattice &L, const int *objidx, int nobj, long **bnd_node_out, int **bnd_obj_out,
                               long *nbnd_out);

int slbc_set_geometry_auto(slbc_lattice *h, const int *objidx, int nobj, long **bnd_node_out,
                           int **bnd_obj_out, long *nbnd_out) {
  Lattice &L = h->L;
  *bnd_node_out = nullptr; *bnd_obj_out = nullptr; *nbnd_out = 0;
  if (geometry_flags(L, h, objidx)) return 1;
  return boundary_from_flags(L, objidx, nobj, bnd_node_out, bnd_obj_out, nbnd_out);
}

static int boundary_from_flags(Lattice &L, const int *objidx, int nobj, long **bnd_node_out, int **bnd_obj_out,
                               long *nbnd_out) {
  *bnd_node_out = nullptr; *bnd_obj_out = nullptr; *nbnd_out = 0;
  // boundary nodes in node order, found on the GPU from the flag words
  const int nb = (int)((L.nnodes + kBndChunk - 1) / kBndChunk);
  int *counts = nullptr, *list = nullptr;
  CK(cudaMalloc(&counts, (size_t)nb * sizeof(int)));
  k_bnd_count<<<nb, 256, 0, L.stream>>>(L.flags, L.nnodes, counts);
  count_launch();
  std::vector<int> off((size_t)nb);
  cudaError_t e = cudaMemcpyAsync(off.data(), counts, (size_t)nb * sizeof(int), cudaMemcpyDeviceToHost, L.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(L.stream);
  long total = 0;
  for (int b = 0; b < nb && e == cudaSuccess; b++) {
    const int c = off[b];
    off[b] = (int)total;
    total += c;
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(counts, off.data(), (size_t)nb * sizeof(int), cudaMemcpyHostToDevice, L.stream);
  if (e == cudaSuccess && total > 0) e = cudaMalloc(&list, (size_t)total * sizeof(int));
  std::vector<int> nodes((size_t)total);
  if (e == cudaSuccess && total > 0) {
    k_bnd_write<<<nb, 256, 0, L.stream>>>(L.flags, L.nnodes, counts, list);
    count_launch();
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(nodes.data(), list, (size_t)total * sizeof(int), cudaMemcpyDeviceToHost, L.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(L.stream);
  }
  cudaFree(counts);
  if (list) cudaFree(list);
  if (e != cudaSuccess) return fail("slbc_set_geometry_auto", e);
  // grouped by object, node order kept: a stable counting sort over the
  // list, in parallel ranges (per-range counts, offsets in (object, range)
  // order, each range scattered in its own order)
  long *bn = (long *)malloc((size_t)(total > 0 ? total : 1) * sizeof(long));
  int *bo = (int *)malloc((size_t)(total > 0 ? total : 1) * sizeof(int));
  if (!bn || !bo) { free(bn); free(bo); return fail_msg("slbc_set_geometry_auto: no host memory"); }
  const long long grain = 1LL << 18;
  const int ranges = (int)std::max<long long>(1, std::min<long long>(
      std::min<long long>(std::max(1u, std::thread::hardware_concurrency()), 32), total / grain));
  std::vector<long> start((size_t)ranges * nobj, 0);
  auto range_lo = [&](int r) { return total * r / ranges; };
  host_par_for(ranges, 1, [&](long long r0, long long r1) {
    for (long long r = r0; r < r1; r++) {
      long *cnt = start.data() + (size_t)r * nobj;
      for (long t = range_lo((int)r); t < range_lo((int)r + 1); t++) cnt[objidx[nodes[t]]]++;
    }
  });
  long run = 0;
  for (int o = 0; o < nobj; o++)
    for (int r = 0; r < ranges; r++) {
      long &c = start[(size_t)r * nobj + o];
      const long v = c;
      c = run;
      run += v;
    }
  host_par_for(ranges, 1, [&](long long r0, long long r1) {
    for (long long r = r0; r < r1; r++) {
      long *at = start.data() + (size_t)r * nobj;
      for (long t = range_lo((int)r); t < range_lo((int)r + 1); t++) {
        const int o = objidx[nodes[t]];
        const long slot = at[o]++;
        bn[slot] = nodes[t];
        bo[slot] = o;
      }
    }
  });
  if (geometry_boundary(L, nobj, bn, bo, total)) { free(bn); free(bo); return 1; }
  *bnd_node_out = bn; *bnd_obj_out = bo; *nbnd_out = total;
  return 0;
}

int slbc_bodyforce_uniform(slbc_lattice *h, double b[3]) {
  const Lattice &L = h->L;
  b[0] = L.bf_const[0]; b[1] = L.bf_const[1]; b[2] = L.bf_const[2];
  return L.bf_uniform;
}

int slbc_move_sphere(slbc_lattice *h, int obj, double rad, const double oldc[3], const double newc[3],
                     const double vel[3], const double ang[3], int with_wallvel, int *changed, long cap,
                     long *nchanged, int nobj, int *objidx_host, long **bnd_node_out, int **bnd_obj_out,
                     long *nbnd_out) {
  Lattice &L = h->L;
  *nchanged = 0;
  if (L.precision == 2) return fail_msg("moving a sphere needs FP32 or FP64 populations (lb->precision)");
  if (!(rad > 0.0) || obj < 0 || obj >= nobj) return fail_msg("slbc_move_sphere: bad object or radius");
  if (with_wallvel && L.uw == nullptr) return fail_msg("slbc_move_sphere: no wall velocity arrays");
  if (L.layout == SLBC_LAYOUT_C1 && to_natural(L)) return 1;
  // the box: old and new node sets with a node of margin, at most the lattice
  MoveArgs m;
  const int dims[3] = {L.esi, L.esj, L.esk};
  for (int a = 0; a < 3; a++) {
    const double lo = std::min(oldc[a], newc[a]) - rad - 1.0, hi = std::max(oldc[a], newc[a]) + rad + 1.0;
    long long l0 = (long long)std::floor(lo), len = (long long)std::ceil(hi) - l0 + 1;
    if (len >= dims[a] || !(len > 0)) { l0 = 0; len = dims[a]; }
    l0 %= dims[a];
    if (l0 < 0) l0 += dims[a];
    m.lo[a] = (int)l0;
    m.len[a] = (int)len;
    m.c[a] = newc[a];
    m.vel[a] = vel[a];
    m.ang[a] = ang[a];
  }
  m.rad = rad;
  m.rho0 = L.par.rho0;
  m.obj = obj;
  m.stokes = L.par.stokes_flow;
  m.layout = L.layout;
  m.objidx = L.objidx;
  m.cap = (int)std::min<long>(cap, 1L << 30);
  if (L.move_cap < m.cap) {  // kept with the lattice: moves are repeated
    if (L.move_buf) { CK(cudaStreamSynchronize(L.stream)); cudaFree(L.move_buf); L.move_buf = nullptr; }
    CK(cudaMalloc(&L.move_buf, (size_t)(2 * (long)m.cap + 1) * sizeof(int)));
    L.move_cap = m.cap;
  }
  int *dev_list = L.move_buf;
  m.nchanged = dev_list;
  m.changed = dev_list + 1;
  cudaError_t e = cudaMemsetAsync(dev_list, 0, sizeof(int), L.stream);
  if (e == cudaSuccess) e = DISPATCH(L, launch_move_sphere, L, m, with_wallvel);
  int count = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&count, dev_list, sizeof(int), cudaMemcpyDeviceToHost, L.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(L.stream);
  if (e == cudaSuccess && count > 0)
    e = cudaMemcpyAsync(changed, dev_list + 1, (size_t)2 * std::min(count, m.cap) * sizeof(int),
                        cudaMemcpyDeviceToHost, L.stream);
  if (e == cudaSuccess && count > 0) e = cudaStreamSynchronize(L.stream);
  if (e != cudaSuccess) return fail("slbc_move_sphere", e);
  *nchanged = count;
  if (count > m.cap) return fail_msg("slbc_move_sphere: more changed nodes than the list holds");
  for (int c = 0; c < count; c++) {
    h->solid_host[changed[2 * c]] = changed[2 * c + 1] >= 0;
    objidx_host[changed[2 * c]] = changed[2 * c + 1];
  }
  L.state_version++;
  L.ads_version++;  // the boundary links change
  L.generation++;
  // flag words from the updated map, then the boundary list
  const int bx = L.esk >= 128 ? 128 : 32;
  dim3 grid((L.esk + bx - 1) / bx, L.esj, L.esi);
  k_flags<<<grid, bx, 0, L.stream>>>(L.objidx, L.flags, L.esi, L.esj, L.esk);
  count_launch();
  CK(cudaGetLastError());
  return boundary_from_flags(L, objidx_host, nobj, bnd_node_out, bnd_obj_out, nbnd_out);
}

int slbc_set_adsorption(slbc_lattice *h, const unsigned char *ads) {
  Lattice &L = h->L;
  if (!L.ads) CK(cudaMalloc(&L.ads, (size_t)L.nnodes));
  CK(cudaMemcpyAsync(L.ads, ads, (size_t)L.nnodes, cudaMemcpyHostToDevice, L.stream));
  CK(cudaStreamSynchronize(L.stream));
  L.ads_version++;
  return 0;
}

int slbc_set_params(slbc_lattice *h, const slbc_params *p) {
  Lattice &L = h->L;
  if (memcmp(&L.par, p, sizeof(slbc_params)) != 0) {
    L.par = *p;
    L.generation++;
  }
  return 0;
}

int slbc_set_bodyforce(slbc_lattice *h, const double *bx, const double *by, const double *bz) {
  Lattice &L = h->L;
  const long long n = L.nnodes;
  bool uniform = true;
  double c[3] = {0.0, 0.0, 0.0};
  if (bx && by && bz) {
    // the first fluid node's force, then every fluid node against it (in
    // parallel ranges)
    const unsigned char *solid = h->solid_host.data();
    long long first = 0;
    while (first < n && solid[first]) first++;
    if (first < n) {
      c[0] = bx[first]; c[1] = by[first]; c[2] = bz[first];
      std::atomic<bool> same(true);
      host_par_for(n - first, 1LL << 20, [&](long long lo, long long hi) {
        for (long long x = first + lo; x < first + hi; x++) {
          if (solid[x]) continue;
          if (bx[x] != c[0] || by[x] != c[1] || bz[x] != c[2]) {
            same.store(false, std::memory_order_relaxed);
            return;
          }
          if (((x - first) & 0xFFFF) == 0 && !same.load(std::memory_order_relaxed)) return;
        }
      });
      uniform = same.load();
    }
  }
  if (L.bf) { cudaStreamSynchronize(L.stream); cudaFree(L.bf); L.bf = nullptr; }
  L.bf_uniform = uniform ? 1 : 0;
  L.bf_const[0] = c[0]; L.bf_const[1] = c[1]; L.bf_const[2] = c[2];
  if (!uniform) {
    const size_t es = side_size(L.precision);
    CK(cudaMalloc(&L.bf, 3 * (size_t)L.npad * es));
    std::vector<char> buf((size_t)n * es);
    const double *src[3] = {bx, by, bz};
    for (int c3 = 0; c3 < 3; c3++) {
      for (long long x = 0; x < n; x++) {
        if (L.precision == 0) ((double *)buf.data())[x] = src[c3][x];
        else ((float *)buf.data())[x] = (float)src[c3][x];
      }
      CK(cudaMemcpy((char *)L.bf + c3 * (size_t)L.npad * es, buf.data(), (size_t)n * es,
                    cudaMemcpyHostToDevice));
    }
  }
  L.generation++;
  return 0;
}

int slbc_set_wallvel(slbc_lattice *h, const double *ux, const double *uy, const double *uz) {
  Lattice &L = h->L;
  if (L.uw) { cudaStreamSynchronize(L.stream); cudaFree(L.uw); L.uw = nullptr; }
  if (ux && uy && uz) {
    const long long n = L.nnodes;
    const size_t es = side_size(L.precision);
    CK(cudaMalloc(&L.uw, 3 * (size_t)L.npad * es));
    std::vector<char> buf((size_t)n * es);
    const double *src[3] = {ux, uy, uz};
    for (int c3 = 0; c3 < 3; c3++) {
      for (long long x = 0; x < n; x++) {
        if (L.precision == 0) ((double *)buf.data())[x] = src[c3][x];
        else ((float *)buf.data())[x] = (float)src[c3][x];
      }
      CK(cudaMemcpy((char *)L.uw + c3 * (size_t)L.npad * es, buf.data(), (size_t)n * es,
                    cudaMemcpyHostToDevice));
    }
  }
  L.generation++;
  return 0;
}

// Device address of a page-locked host array the device can reach (so a
// kernel reads or writes it over the host link), else null: pageable
// memory goes through the staging buffer.
static void *mapped_host(const void *p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

int slbc_put_pops(slbc_lattice *h, const double *a) {
  Lattice &L = h->L;
  L.state_version++;
  if (L.precision != 2) {
    if (const double *dev_a = (const double *)mapped_host(a)) {
      CK(DISPATCH(L, launch_put_host, L, dev_a));
      CK(cudaStreamSynchronize(L.stream));
      L.layout = SLBC_LAYOUT_N;
      return 0;
    }
  }
  if (ensure_staging(L, L.nnodes, 15)) return 1;
  if (L.precision == 2) {  // count of unpaired nodes
    if (ensure_partials(L, 1)) return 1;
    CK(cudaMemsetAsync(L.partials, 0, sizeof(double), L.stream));
  }
  const long long chunk = L.staging_nodes / 15;
  for (long long x0 = 0; x0 < L.nnodes; x0 += chunk) {
    const long long n = std::min(chunk, L.nnodes - x0);
    CK(cudaMemcpyAsync(L.staging, a + 15 * x0, (size_t)(15 * n) * sizeof(double),
                       cudaMemcpyHostToDevice, L.stream));
    if (L.precision == 2) {
      CK(launch_put_bf16(L, L.staging, x0, n, (int *)L.partials));
    } else {
      CK(DISPATCH(L, launch_put, L, L.staging, x0, n));
    }
  }
  CK(cudaStreamSynchronize(L.stream));
  L.layout = SLBC_LAYOUT_N;
  if (L.precision == 2) {
    int unpaired = 0;
    CK(cudaMemcpy(&unpaired, L.partials, sizeof(int), cudaMemcpyDeviceToHost));
    if (unpaired > 0) {
      g_err = "slbc_put_pops: " + std::to_string(unpaired) +
              " nodes hold populations whose deviations are not paired (q and opp(q) differ); "
              "BF16 paired-deviation storage cannot hold them";
      return 2;
    }
  }
  return 0;
}

int slbc_get_pops(slbc_lattice *h, double *a) {
  Lattice &L = h->L;
  if (L.precision != 2) {
    if (double *dev_a = (double *)mapped_host(a)) {
      CK(DISPATCH(L, launch_get_host, L, dev_a));
      CK(cudaStreamSynchronize(L.stream));
      return 0;
    }
  }
  if (ensure_staging(L, L.nnodes, 15)) return 1;
  const long long chunk = L.staging_nodes / 15;
  for (long long x0 = 0; x0 < L.nnodes; x0 += chunk) {
    const long long n = std::min(chunk, L.nnodes - x0);
    CK(DISPATCH3(L, launch_get, L, L.staging, x0, n));
    // stream order keeps the next chunk's kernel behind this copy
    CK(cudaMemcpyAsync(a + 15 * x0, L.staging, (size_t)(15 * n) * sizeof(double),
                       cudaMemcpyDeviceToHost, L.stream));
  }
  CK(cudaStreamSynchronize(L.stream));
  return 0;
}

void *slbc_host_alloc(size_t bytes) {
  void *p = nullptr;
  if (cudaMallocHost(&p, bytes) != cudaSuccess) {
    cudaGetLastError();  // clear: the caller falls back to pageable memory
    return nullptr;
  }
  memset(p, 0, bytes);
  return p;
}

void slbc_host_free(void *p) {
  if (p) cudaFreeHost(p);
}

int slbc_step(slbc_lattice *h, int n, int use_graph) {
  Lattice &L = h->L;
  L.state_version++;
  if (to_aa(L)) return 1;
  if (L.tune_state == 0 && autotune(L)) return 1;
  int done = 0;
  if (use_graph && n >= 2 * 2 * kGraphPairs) {
    if (L.layout == SLBC_LAYOUT_C1) { if (one_step(L)) return 1; done++; }
    if (ensure_graph(L)) return 1;
    while (n - done >= L.graph_steps) {
      CK(cudaGraphLaunch(L.graph, L.stream));
      count_launch(L.graph_steps);
      done += L.graph_steps;
    }
    // the graph starts and ends in C0
  }
  for (; done < n; done++)
    if (one_step(L)) return 1;
  return 0;
}

int slbc_force_step(slbc_lattice *h) {
  Lattice &L = h->L;
  L.state_version++;
  if (to_aa(L)) return 1;
  CK(DISPATCH3(L, launch_force, L));
  return one_step(L);
}

int slbc_bbl(slbc_lattice *h, int with_force) {
  Lattice &L = h->L;
  L.state_version++;
  if (no_bf16(L, "slbc_bbl")) return 1;
  if (to_natural(L)) return 1;
  CK(DISPATCH(L, launch_bbl, L, with_force));
  return 0;
}

int slbc_propagate(slbc_lattice *h) {
  Lattice &L = h->L;
  L.state_version++;
  if (no_bf16(L, "slbc_propagate")) return 1;
  if (to_natural(L)) return 1;
  if (ensure_scratch(L)) return 1;
  CK(DISPATCH(L, launch_propagate, L));
  std::swap(L.pop, L.scratch);
  L.generation++;  // captured graphs hold the old buffer
  return 0;
}

int slbc_collide(slbc_lattice *h) {
  Lattice &L = h->L;
  L.state_version++;
  if (L.precision == 2 && L.par.skip_solid) return fail_msg(kPairSkipSolid);
  if (to_natural(L)) return 1;
  CK(DISPATCH3(L, launch_collide, L));
  return 0;
}

int slbc_zero_force(slbc_lattice *h) {
  Lattice &L = h->L;
  if (L.nbnd) CK(cudaMemsetAsync(L.bnd_f, 0, 3 * (size_t)L.nbnd * sizeof(double), L.stream));
  return 0;
}

int slbc_scale_force(slbc_lattice *h, double fac) {
  Lattice &L = h->L;
  if (!L.nbnd) return 0;
  k_scale<<<blocks_for(3 * L.nbnd, 256), 256, 0, L.stream>>>(L.bnd_f, 3 * L.nbnd, fac);
  count_launch();
  CK(cudaGetLastError());
  return 0;
}

int slbc_get_force(slbc_lattice *h, double *f3) {
  Lattice &L = h->L;
  if (!L.nbnd) return 0;
  std::unique_ptr<double[]> tmp(new (std::nothrow) double[3 * (size_t)L.nbnd]);
  if (!tmp) return fail_msg("slbc_get_force: no host memory");
  double *t = tmp.get();
  CK(cudaMemcpyAsync(t, L.bnd_f, 3 * (size_t)L.nbnd * sizeof(double), cudaMemcpyDeviceToHost, L.stream));
  CK(cudaStreamSynchronize(L.stream));
  const long long nb = L.nbnd;
  host_par_for(nb, 1LL << 18, [&](long long lo, long long hi) {
    for (long long e = lo; e < hi; e++) {
      f3[3 * e] = t[e];
      f3[3 * e + 1] = t[nb + e];
      f3[3 * e + 2] = t[2 * nb + e];
    }
  });
  return 0;
}

int slbc_vsum(slbc_lattice *h, double fac, const double *psi, double out[5]) {
  Lattice &L = h->L;
  const int nb = reduction_blocks(L);
  if (ensure_partials(L, 5 * nb + 8)) return 1;
  double *dpsi = nullptr;
  if (psi) {
    CK(cudaMallocAsync(&dpsi, (size_t)L.nnodes * sizeof(double), L.stream));
    CK(cudaMemcpyAsync(dpsi, psi, (size_t)L.nnodes * sizeof(double), cudaMemcpyHostToDevice, L.stream));
  }
  CK(DISPATCH3(L, launch_vsum, L, fac, dpsi, L.partials, nb));
  k_final_sum_tree<5><<<1, 256, 0, L.stream>>>(L.partials, nb, L.partials + 5 * nb);
  count_launch();
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(L.host_out, L.partials + 5 * nb, 5 * sizeof(double), cudaMemcpyDeviceToHost, L.stream));
  if (dpsi) CK(cudaFreeAsync(dpsi, L.stream));
  CK(cudaStreamSynchronize(L.stream));
  for (int c = 0; c < 5; c++) out[c] = L.host_out[c];
  return 0;
}

int slbc_distribf(slbc_lattice *h, const double *pos, double *ft) {
  Lattice &L = h->L;
  if (L.nobj == 0) return 0;
  CK(cudaMemcpyAsync(L.obj_pos, pos, 3 * (size_t)L.nobj * sizeof(double), cudaMemcpyHostToDevice, L.stream));
  if (L.npiece > 0) {
    k_distrib_piece<<<L.npiece, 256, 0, L.stream>>>(L.bnd_node, L.bnd_f, L.nbnd, L.piece_obj,
                                                   L.piece_lo, L.piece_hi, L.obj_pos, L.esj,
                                                   L.esk, L.piece_sum);
    count_launch();
    CK(cudaGetLastError());
  }
  const int *first = (const int *)(L.obj_ft + 6 * L.nobj);
  k_distrib_obj<<<blocks_for(L.nobj, 128), 128, 0, L.stream>>>(first, first + L.nobj, L.piece_sum,
                                                               L.nobj, L.obj_ft);
  count_launch();
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(ft, L.obj_ft, 6 * (size_t)L.nobj * sizeof(double), cudaMemcpyDeviceToHost, L.stream));
  CK(cudaStreamSynchronize(L.stream));
  return 0;
}

int slbc_set_velocity(slbc_lattice *h, const double *rho, const double *ux, const double *uy,
                      const double *uz, int skip_solid) {
  Lattice &L = h->L;
  L.state_version++;
  if (ensure_staging(L, L.nnodes, 4)) return 1;
  const long long chunk = L.staging_nodes / 4;
  std::vector<double> buf((size_t)(4 * std::min(chunk, L.nnodes)));
  for (long long x0 = 0; x0 < L.nnodes; x0 += chunk) {
    const long long n = std::min(chunk, L.nnodes - x0);
    for (long long e = 0; e < n; e++) {
      buf[4 * e] = rho ? rho[x0 + e] : 0.0;
      buf[4 * e + 1] = ux[x0 + e]; buf[4 * e + 2] = uy[x0 + e]; buf[4 * e + 3] = uz[x0 + e];
    }
    CK(cudaMemcpyAsync(L.staging, buf.data(), (size_t)(4 * n) * sizeof(double), cudaMemcpyHostToDevice, L.stream));
    CK(DISPATCH3(L, launch_setvel, L, L.staging, x0, n, rho != nullptr, skip_solid));
    CK(cudaStreamSynchronize(L.stream));
  }
  L.layout = SLBC_LAYOUT_N;
  return 0;
}

int slbc_get_state_dev(slbc_lattice *h, double fac, float *u, float *drho) {
  Lattice &L = h->L;
  if (no_bf16(L, "slbc_get_state_dev")) return 1;
  if (!u) return fail_msg("slbc_get_state_dev: null output");
  CK(DISPATCH(L, launch_velocity, L, fac, u, drho));
  return 0;
}

int slbc_get_velocity_dev(slbc_lattice *h, double fac, float *u) { return slbc_get_state_dev(h, fac, u, nullptr); }

int slbc_set_state_dev(slbc_lattice *h, const float *u, const float *drho, int skip_solid) {
  Lattice &L = h->L;
  L.state_version++;
  if (!u) return fail_msg("slbc_set_state_dev: null input");
  if (ensure_staging(L, L.nnodes, 4)) return 1;
  const long long chunk = L.staging_nodes / 4;
  for (long long x0 = 0; x0 < L.nnodes; x0 += chunk) {
    const long long n = std::min(chunk, L.nnodes - x0);
    k_stage_velocity<<<blocks_for(n, 256), 256, 0, L.stream>>>(u, drho, L.nnodes, x0, n, L.staging);
    count_launch();
    CK(cudaGetLastError());
    CK(DISPATCH3(L, launch_setvel, L, L.staging, x0, n, drho ? 2 : 0, skip_solid));
  }
  L.layout = SLBC_LAYOUT_N;
  return 0;
}

int slbc_set_velocity_dev(slbc_lattice *h, const float *u, int skip_solid) {
  return slbc_set_state_dev(h, u, nullptr, skip_solid);
}

// ---- moment propagation ----------------------------------------------------

int slbc_mp_create(slbc_lattice *h, slbc_tracer **out, int use_f64) {
  Lattice &L = h->L;
  *out = nullptr;
  slbc_tracer *t = new slbc_tracer();
  t->h = h; t->f64 = use_f64 ? 1 : 0;
  const size_t es = use_f64 ? 8 : 4;
  cudaError_t e = cudaMalloc(&t->p, (size_t)L.nnodes * es);
  if (e == cudaSuccess) e = cudaMalloc(&t->p2, (size_t)L.nnodes * es);
  if (e == cudaSuccess) e = cudaMemsetAsync(t->p, 0, (size_t)L.nnodes * es, L.stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(t->p2, 0, (size_t)L.nnodes * es, L.stream);
  if (e == cudaSuccess && !use_f64) e = cudaMalloc(&t->lo, (size_t)L.nnodes * sizeof(float));
  if (e == cudaSuccess && !use_f64) e = cudaMalloc(&t->lo2, (size_t)L.nnodes * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&t->acc, sizeof(double));
  if (e == cudaSuccess) e = cudaMemsetAsync(t->acc, 0, sizeof(double), L.stream);
  if (e == cudaSuccess && !L.mp_rho64) {
    e = cudaMalloc(&L.mp_rho64, (size_t)L.nnodes * sizeof(double));
    if (e == cudaSuccess) {
      // rho = rho0 until the first snapshot (reference src/mpmisc.c:50-52)
      std::vector<double> r0((size_t)L.nnodes, L.par.rho0);
      e = cudaMemcpy(L.mp_rho64, r0.data(), (size_t)L.nnodes * sizeof(double), cudaMemcpyHostToDevice);
    }
  }
  if (e == cudaSuccess && !use_f64 && !L.mp_rho32) {
    e = cudaMalloc(&L.mp_rho32, (size_t)L.nnodes * sizeof(float));
    if (e == cudaSuccess) {
      k_convert<float, double><<<blocks_for(L.nnodes, 256), 256, 0, L.stream>>>(L.mp_rho32, L.mp_rho64, L.nnodes);
      count_launch();
      e = cudaGetLastError();
    }
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(L.stream);
  if (e != cudaSuccess) {
    slbc_mp_destroy(t);
    return fail("slbc_mp_create", e);
  }
  *out = t;
  return 0;
}

void slbc_mp_destroy(slbc_tracer *t) {
  if (!t) return;
  if (t->h) cudaStreamSynchronize(t->h->L.stream);
  if (t->p) cudaFree(t->p);
  if (t->p2) cudaFree(t->p2);
  if (t->acc) cudaFree(t->acc);
  if (t->objstate) cudaFree(t->objstate);
  if (t->lo) cudaFree(t->lo);
  if (t->lo2) cudaFree(t->lo2);
  delete t;
}

int slbc_mp_rhoinit(slbc_lattice *h) {
  Lattice &L = h->L;
  if (!L.mp_rho64) CK(cudaMalloc(&L.mp_rho64, (size_t)L.nnodes * sizeof(double)));
  CK(DISPATCH3(L, launch_mp_rhoinit, L));
  L.mp_rho_gen++;
  return 0;
}

int slbc_mp_get_rho(slbc_lattice *h, double *rho) {
  Lattice &L = h->L;
  if (!L.mp_rho64) return fail_msg("slbc_mp_get_rho: no density snapshot");
  CK(cudaMemcpyAsync(rho, L.mp_rho64, (size_t)L.nnodes * sizeof(double), cudaMemcpyDeviceToHost, L.stream));
  CK(cudaStreamSynchronize(L.stream));
  return 0;
}

int slbc_mp_put(slbc_tracer *t, const double *p) {
  Lattice &L = t->h->L;
  t->lo_live = 0;  // the uploaded values are the whole of p
  if (t->f64) {
    CK(cudaMemcpyAsync(t->p, p, (size_t)L.nnodes * sizeof(double), cudaMemcpyHostToDevice, L.stream));
  } else {
    std::vector<float> buf((size_t)L.nnodes);
    for (long long x = 0; x < L.nnodes; x++) buf[x] = (float)p[x];
    CK(cudaMemcpyAsync(t->p, buf.data(), (size_t)L.nnodes * sizeof(float), cudaMemcpyHostToDevice, L.stream));
  }
  CK(cudaStreamSynchronize(L.stream));
  return 0;
}

int slbc_mp_get(slbc_tracer *t, double *p) {
  Lattice &L = t->h->L;
  if (t->f64) {
    CK(cudaMemcpyAsync(p, t->p, (size_t)L.nnodes * sizeof(double), cudaMemcpyDeviceToHost, L.stream));
    CK(cudaStreamSynchronize(L.stream));
  } else {
    std::vector<float> buf((size_t)L.nnodes);
    CK(cudaMemcpyAsync(buf.data(), t->p, (size_t)L.nnodes * sizeof(float), cudaMemcpyDeviceToHost, L.stream));
    CK(cudaStreamSynchronize(L.stream));
    for (long long x = 0; x < L.nnodes; x++) p[x] = buf[x];
  }
  return 0;
}

int slbc_mp_step(slbc_tracer *t, int n, double alpha, double adprob, int moving,
                 const double *objstate, int nobj) {
  Lattice &L = t->h->L;
  if (no_bf16(L, "slbc_mp_step")) return 1;
  if (L.ads && L.ads_links_version != L.ads_version) {
    if (!L.ads_links) CK(cudaMalloc(&L.ads_links, (size_t)L.nnodes * sizeof(uint16_t)));
    k_ads_links<<<blocks_for(L.nnodes, 256), 256, 0, L.stream>>>(L.flags, L.ads, L.ads_links, L.esi, L.esj, L.esk);
    count_launch();
    CK(cudaGetLastError());
    L.ads_links_version = L.ads_version;
  }
  if (!L.mp_rho64) return fail_msg("slbc_mp_step: density snapshot missing");
  if (!t->f64 && !L.mp_rho32) return fail_msg("slbc_mp_step: FP32 density snapshot missing");
  if (moving) {
    if (nobj > t->objstate_cap) {
      if (t->objstate) { cudaStreamSynchronize(L.stream); cudaFree(t->objstate); }
      CK(cudaMalloc(&t->objstate, 9 * (size_t)nobj * sizeof(double)));
      t->objstate_cap = nobj;
    }
    if (nobj > 0)
      CK(cudaMemcpyAsync(t->objstate, objstate, 9 * (size_t)nobj * sizeof(double), cudaMemcpyHostToDevice, L.stream));
  }
  for (int s = 0; s < n; s++) {
    CK(DISPATCH(L, launch_mp_step, L, t->p, t->p2, t->f64, alpha, adprob, moving, t->objstate, t->lo, t->lo2,
                &t->lo_live));
    std::swap(t->p, t->p2);
    std::swap(t->lo, t->lo2);
  }
  return 0;
}

static int mp_reduce(slbc_tracer *t, int axis, double out[5]) {
  Lattice &L = t->h->L;
  const int nb = 152 * 4;
  if (ensure_partials(L, 5 * nb + 8)) return 1;
  if (t->f64)
    k_mp_sums<double><<<nb, kReduceThreads, 0, L.stream>>>((const double *)t->p, L.flags, L.ads, L.nnodes, L.esj, L.esk, axis, L.partials);
  else
    k_mp_sums<float><<<nb, kReduceThreads, 0, L.stream>>>((const float *)t->p, L.flags, L.ads, L.nnodes, L.esj, L.esk, axis, L.partials);
  count_launch();
  CK(cudaGetLastError());
  k_final_sum_tree<5><<<1, 256, 0, L.stream>>>(L.partials, nb, L.partials + 5 * nb);
  count_launch();
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(L.host_out, L.partials + 5 * nb, 5 * sizeof(double), cudaMemcpyDeviceToHost, L.stream));
  CK(cudaStreamSynchronize(L.stream));
  for (int c = 0; c < 5; c++) out[c] = L.host_out[c];
  return 0;
}

int slbc_mp_sums(slbc_tracer *t, int axis, double out[5]) { return mp_reduce(t, axis, out); }

namespace slbc {
// pass 1 of the tracer velocity autocorrelation: sums of psi P and psi^2
__global__ void __launch_bounds__(kReduceThreads) k_vacf_mean(const double *p, const uint16_t *flags,
                                                            const double *psi, long long n, double *partials) {
  double v[2] = {0.0, 0.0};
  for (long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x; x < n; x += (long long)gridDim.x * blockDim.x) {
    if (flags[x] & FLAG_SOLID) continue;
    const double w = psi ? psi[x] : 1.0;
    v[0] += w * p[x];
    v[1] += w * w;
  }
  block_sum<2>(v);
  if (threadIdx.x == 0) { partials[2 * blockIdx.x] = v[0]; partials[2 * blockIdx.x + 1] = v[1]; }
}

}  // namespace slbc

int slbc_mp_vacf(slbc_tracer *t, slbc_tracer *t2, int axis, const double *psi_host, double out[2]) {
  Lattice &L = t->h->L;
  if (t2->h != t->h) return fail_msg("slbc_mp_vacf: the two tracers belong to different lattices");
  if (!t->f64 || !t2->f64) return fail_msg("the tracer velocity autocorrelation needs FP64 tracers (mp->precision)");
  if (L.precision == 2) return fail_msg("the tracer velocity autocorrelation needs FP32 or FP64 populations");
  if (axis < 0 || axis > 2 || !L.mp_rho64) return fail_msg("slbc_mp_vacf: bad direction or no density snapshot");
  const int nb = 152 * 4;
  if (ensure_partials(L, 2 * nb + 8)) return 1;
  double *psi = nullptr;
  if (psi_host) {
    CK(cudaMalloc(&psi, (size_t)L.nnodes * sizeof(double)));
    CK(cudaMemcpyAsync(psi, psi_host, (size_t)L.nnodes * sizeof(double), cudaMemcpyHostToDevice, L.stream));
  }
  double sums[2];
  cudaError_t e = cudaSuccess;
  k_vacf_mean<<<nb, kReduceThreads, 0, L.stream>>>((const double *)t->p, L.flags, psi, L.nnodes, L.partials);
  count_launch();
  e = cudaGetLastError();
  if (e == cudaSuccess) {
    k_final_sum_tree<2><<<1, 256, 0, L.stream>>>(L.partials, nb, L.partials + 2 * nb);
    count_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(sums, L.partials + 2 * nb, 2 * sizeof(double), cudaMemcpyDeviceToHost, L.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(L.stream);
  if (e == cudaSuccess) e = DISPATCH(L, launch_vacf_sums, L, (double *)t->p, (const double *)t2->p, psi, sums[0] / sums[1],
                                     axis, L.partials, nb);
  if (e == cudaSuccess) {
    k_final_sum_tree<2><<<1, 256, 0, L.stream>>>(L.partials, nb, L.partials + 2 * nb);
    count_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, L.partials + 2 * nb, 2 * sizeof(double), cudaMemcpyDeviceToHost, L.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(L.stream);
  if (psi) cudaFree(psi);
  if (e != cudaSuccess) return fail("slbc_mp_vacf", e);
  L.state_version++;  // the tracer changed
  return 0;
}



int slbc_mp_minmax(slbc_tracer *t, double out[2]) {
  Lattice &L = t->h->L;
  const int nb = 152 * 2;
  if (ensure_partials(L, 2 * nb + 8)) return 1;
  if (t->f64) k_mp_minmax<double><<<nb, 256, 0, L.stream>>>((const double *)t->p, L.flags, L.nnodes, L.partials);
  else k_mp_minmax<float><<<nb, 256, 0, L.stream>>>((const float *)t->p, L.flags, L.nnodes, L.partials);
  count_launch();
  CK(cudaGetLastError());
  std::vector<double> part(2 * nb);
  CK(cudaMemcpyAsync(part.data(), L.partials, 2 * nb * sizeof(double), cudaMemcpyDeviceToHost, L.stream));
  CK(cudaStreamSynchronize(L.stream));
  double lo = 1e300, hi = -1e300;
  for (int b = 0; b < nb; b++) { lo = std::min(lo, part[2 * b]); hi = std::max(hi, part[2 * b + 1]); }
  out[0] = lo; out[1] = hi;
  return 0;
}

static long long plane_size(const Lattice &L, int axis) {
  return axis == 0 ? (long long)L.esj * L.esk : axis == 1 ? (long long)L.esi * L.esk : (long long)L.esi * L.esj;
}

int slbc_mp_fill(slbc_tracer *t, int kind, const double *geo, double value) {
  Lattice &L = t->h->L;
  double g[6] = {0, 0, 0, 0, 0, 0};
  const int ng = kind == 1 ? 6 : kind == 2 ? 2 : kind == 3 ? 4 : kind == 4 ? 5 : 0;
  for (int c = 0; c < ng; c++) g[c] = geo[c];
  long long count = L.nnodes;
  if (kind == 2) {
    const int axis = (int)g[0], pos = (int)g[1];
    const int lim = axis == 0 ? L.esi : axis == 1 ? L.esj : L.esk;
    if (axis < 0 || axis > 2 || pos < 0 || pos >= lim) return fail_msg("slbc_mp_fill: wall outside the lattice");
    count = plane_size(L, axis);
  }
  const int nb = (int)std::max<long long>(1, std::min<long long>(blocks_for(count, kReduceThreads), 152 * 4));
  if (ensure_partials(L, nb + 8)) return 1;
  if (t->f64)
    k_mp_fill<double><<<nb, kReduceThreads, 0, L.stream>>>((double *)t->p, nullptr, L.flags, L.esi, L.esj, L.esk, kind, g[0], g[1], g[2], g[3], g[4], g[5], value, count, L.partials);
  else
    k_mp_fill<float><<<nb, kReduceThreads, 0, L.stream>>>((float *)t->p, t->lo_live ? t->lo : nullptr, L.flags, L.esi, L.esj, L.esk, kind, g[0], g[1], g[2], g[3], g[4], g[5], value, count, L.partials);
  count_launch();
  CK(cudaGetLastError());
  k_sum_into<<<1, 256, 0, L.stream>>>(L.partials, nb, t->acc);
  count_launch();
  CK(cudaGetLastError());
  return 0;
}

int slbc_mp_injected(slbc_tracer *t, int reset, double *out) {
  Lattice &L = t->h->L;
  double v = 0.0;
  CK(cudaMemcpyAsync(&v, t->acc, sizeof(double), cudaMemcpyDeviceToHost, L.stream));
  CK(cudaStreamSynchronize(L.stream));
  if (out) *out = v;
  if (reset) CK(cudaMemsetAsync(t->acc, 0, sizeof(double), L.stream));
  return 0;
}

int slbc_mp_plane(slbc_tracer *t, int axis, int pos, double out[2]) {
  Lattice &L = t->h->L;
  const int lim = axis == 0 ? L.esi : axis == 1 ? L.esj : L.esk;
  if (axis < 0 || axis > 2 || pos < 0 || pos >= lim) return fail_msg("slbc_mp_plane: plane outside the lattice");
  const long long count = plane_size(L, axis);
  const int nb = (int)std::max<long long>(1, std::min<long long>(blocks_for(count, kReduceThreads), 152 * 2));
  if (ensure_partials(L, 2 * nb + 8)) return 1;
  if (t->f64)
    k_mp_plane<double><<<nb, kReduceThreads, 0, L.stream>>>((const double *)t->p, L.flags, L.esi, L.esj, L.esk, axis, pos, count, L.partials);
  else
    k_mp_plane<float><<<nb, kReduceThreads, 0, L.stream>>>((const float *)t->p, L.flags, L.esi, L.esj, L.esk, axis, pos, count, L.partials);
  count_launch();
  CK(cudaGetLastError());
  k_final_sum_tree<2><<<1, 256, 0, L.stream>>>(L.partials, nb, L.partials + 2 * nb);
  count_launch();
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(L.host_out, L.partials + 2 * nb, 2 * sizeof(double), cudaMemcpyDeviceToHost, L.stream));
  CK(cudaStreamSynchronize(L.stream));
  out[0] = L.host_out[0];
  out[1] = L.host_out[1];
  return 0;
}

static int mp_misc(slbc_tracer *t, const slbc_tracer *src, int op, double fac) {
  Lattice &L = t->h->L;
  if (op == 2 && src->f64 != t->f64) return fail_msg("slbc_mp_add: tracers differ in precision");
  // other operations on p act on its high part alone; the low part is dropped
  // (at most half an FP32 ulp per node, once)
  t->lo_live = 0;
  if (t->f64)
    k_mp_misc<double><<<blocks_for(L.nnodes, 256), 256, 0, L.stream>>>((double *)t->p, src ? (const double *)src->p : nullptr, L.flags, L.ads, L.nnodes, op, fac);
  else
    k_mp_misc<float><<<blocks_for(L.nnodes, 256), 256, 0, L.stream>>>((float *)t->p, src ? (const float *)src->p : nullptr, L.flags, L.ads, L.nnodes, op, fac);
  count_launch();
  CK(cudaGetLastError());
  return 0;
}

int slbc_mp_scale(slbc_tracer *t, double fac) { return mp_misc(t, nullptr, 0, fac); }
int slbc_mp_zero_ads(slbc_tracer *t) { return t->h->L.ads ? mp_misc(t, nullptr, 1, 0.0) : 0; }
int slbc_mp_add(slbc_tracer *dst, const slbc_tracer *src) { return mp_misc(dst, src, 2, 0.0); }

// ---- batches of lattices ------------------------------------------------------

struct slbc_batch {
  BatchState B;
};

void slbc_batch_destroy(slbc_batch *b) {
  if (!b) return;
  BatchState &B = b->B;
  if (B.stream) cudaStreamSynchronize(B.stream);
  if (B.doms) cudaFree(B.doms);
  if (B.work_off) cudaFree(B.work_off);
  if (B.work) cudaFree(B.work);
  if (B.tiles) cudaFree(B.tiles);
  if (B.done) cudaEventDestroy(B.done);
  if (B.stream) cudaStreamDestroy(B.stream);
  delete b;
}

int slbc_batch_create(slbc_batch **out, slbc_lattice *const *lats, int n) {
  *out = nullptr;
  if (n < 1 || lats == nullptr) return fail_msg("slbc_batch_create: a batch needs at least one lattice");
  const int prec = lats[0] ? lats[0]->L.precision : -1;
  for (int d = 0; d < n; d++) {
    if (!lats[d]) return fail_msg("slbc_batch_create: null lattice");
    if (lats[d]->L.precision != prec)
      return fail_msg("slbc_batch_create: the lattices of a batch share one precision");
    for (int e = 0; e < d; e++)
      if (lats[e] == lats[d]) return fail_msg("slbc_batch_create: a lattice appears twice");
  }
  if (prec == 2) return fail_msg("slbc_batch_create: BF16 lattices are not batched (FP32 or FP64 only)");
  int dev = 0, sms = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  slbc_batch *b = new slbc_batch();
  BatchState &B = b->B;
  for (int d = 0; d < n; d++) B.lats.push_back(&lats[d]->L);
  B.precision = prec;
  B.sms = sms;
  cudaError_t e = cudaMalloc(&B.doms, (size_t)n * std::max(sizeof(BatchDom<double>), sizeof(BatchDom<float>)));
  // block offsets of up to four launches (n + 4 entries) and the lattices
  if (e == cudaSuccess) e = cudaMalloc(&B.work_off, (n + 4) * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&B.work, n * sizeof(int));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&B.stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&B.done, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    slbc_batch_destroy(b);
    return fail("slbc_batch_create", e);
  }
  *out = b;
  return 0;
}

int slbc_batch_workers(const slbc_batch *b) { return b ? b->B.nworkers : 0; }

int slbc_batch_set_mode(slbc_batch *b, int mode) {
  if (mode != 0 && mode != 1) return fail_msg("slbc_batch_set_mode: mode is 0 (tiles) or 1 (persistent)");
  b->B.mode = mode;
  return 0;
}

int slbc_batch_step(slbc_batch *b, int nsteps) {
  if (nsteps <= 0) return 0;
  BatchState &B = b->B;
  for (Lattice *L : B.lats) {
    L->state_version++;
    if (L->precision != B.precision) return fail_msg("slbc_batch_step: a lattice changed precision");
    if (to_aa(*L)) return 1;
    CK(cudaStreamSynchronize(L->stream));  // the batch stream follows every lattice's work
  }
  if (B.mode == 1) {
    CK(B.precision == 0 ? launch_batch_f64(B, nsteps) : launch_batch_f32(B, nsteps));
  } else {
    CK(B.precision == 0 ? prepare_tiles_f64(B) : prepare_tiles_f32(B));
    auto one = [&](int s) { return B.precision == 0 ? launch_tiles_f64(B, s) : launch_tiles_f32(B, s); };
    // 50 steps (an even number: the parity pattern repeats) per graph replay
    const int G = 50;
    int done = 0;
    if (nsteps >= 2 * G) {
      cudaGraph_t g;
      cudaGraphExec_t ge = nullptr;
      CK(cudaStreamBeginCapture(B.stream, cudaStreamCaptureModeThreadLocal));
      cudaError_t ce = cudaSuccess;
      for (int s = 0; s < G && ce == cudaSuccess; s++) ce = one(s);
      const cudaError_t ee = cudaStreamEndCapture(B.stream, &g);
      if (ce != cudaSuccess) return fail("slbc_batch_step: capture", ce);
      if (ee != cudaSuccess) return fail("slbc_batch_step: cudaStreamEndCapture", ee);
      const cudaError_t ie = cudaGraphInstantiate(&ge, g, 0);
      cudaGraphDestroy(g);
      if (ie != cudaSuccess) return fail("slbc_batch_step: cudaGraphInstantiate", ie);
      int nclass = 0;
      for (int c = 0; c < 4; c++) nclass += (B.class_tiles[c][0] > 0) + (B.class_tiles[c][1] > 0);
      count_launch(-G * nclass);  // the captured launches run only in the replays
      for (; done + G <= nsteps; done += G) {
        const cudaError_t le = cudaGraphLaunch(ge, B.stream);
        if (le != cudaSuccess) { cudaGraphExecDestroy(ge); return fail("slbc_batch_step: cudaGraphLaunch", le); }
        count_launch(G * nclass);
      }
      CK(cudaStreamSynchronize(B.stream));
      cudaGraphExecDestroy(ge);
    }
    for (; done < nsteps; done++) CK(one(done));
  }
  CK(cudaEventRecord(B.done, B.stream));
  for (Lattice *L : B.lats) {
    CK(cudaStreamWaitEvent(L->stream, B.done, 0));  // later work on a lattice follows the batch
    if (nsteps & 1) L->layout = L->layout == SLBC_LAYOUT_C0 ? SLBC_LAYOUT_C1 : SLBC_LAYOUT_C0;
  }
  return 0;
}

}  // extern "C"
