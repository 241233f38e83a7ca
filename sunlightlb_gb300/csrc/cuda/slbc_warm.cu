// Tensor-core kernels of the learned warm start (BF16 inputs, FP32
// accumulation in TMEM, tcgen05.mma issued by one thread, operands staged by
// TMA through a 4-stage mbarrier pipeline).
//
// slbc_tc_gemm: D[M x N] (FP32, row-major, leading dimension ldd) =
// A[M x K] * B[N x K]^T with A and B BF16, row-major (K contiguous).  The
// weight gradients of the network's convolutions are this product.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "slbc_internal.cuh"
#include "slbc_tc.cuh"

#include <cuda_bf16.h>

namespace {

using namespace slbc;

constexpr int kBM = 128, kBN = 128, kBK = 64, kStages = 4;
constexpr int kTileA = kBM * kBK * 2;  // bytes of one A stage (128 rows x 128 B)
constexpr int kTileB = kBN * kBK * 2;
constexpr int kGemmSmem = kStages * (kTileA + kTileB) + 1024;
constexpr uint32_t kWaitLimit = 1u << 20;  // polls before a wait gives up

// error flag of the tensor-core kernels, one per device
int *g_tc_err[64];
std::mutex g_tc_lock;

int *tc_err_flag() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> guard(g_tc_lock);
  if (!g_tc_err[dev]) {
    if (cudaMalloc(&g_tc_err[dev], sizeof(int)) != cudaSuccess) return nullptr;
    if (cudaMemset(g_tc_err[dev], 0, sizeof(int)) != cudaSuccess) return nullptr;
  }
  return g_tc_err[dev];
}

// Opt a kernel into `bytes` of dynamic shared memory on the current device;
// the attribute is per device, so `done` keeps one bit per device index.
cudaError_t smem_opt_in(const void *fn, int bytes, unsigned long long &done) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> guard(g_tc_lock);
  if (done >> dev & 1ull) return cudaSuccess;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) done |= 1ull << dev;
  return e;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point
typedef CUresult (*EncodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
  static EncodeTiled fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiled)p;
  });
  return fn;
}

// 2-D BF16 row-major matrix (rows x cols, cols contiguous), box of
// box_rows x 64 elements (128 bytes, 128-byte swizzle)
bool make_map_2d(CUtensorMap *map, const void *ptr, long long rows, long long cols, int box_rows) {
  EncodeTiled enc = encode_fn();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
  const cuuint32_t box[2] = {64, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// One 128 x 128 output tile per block of 128 threads: thread 0 loads (TMA),
// thread 32 issues the MMAs, all four warps read the accumulator back.
__global__ void __launch_bounds__(128, 1)
k_gemm_bf16(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, float *D, int ldd,
            int K, int *err) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t pad = (1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u;
  uint8_t *tA = smem_raw + pad;
  uint8_t *tB = tA + kStages * kTileA;
  __shared__ uint64_t full[kStages], empty[kStages], done;
  __shared__ uint32_t tmem_base;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
  const int nk = K / kBK;
  if (warp == 0) {
    tc::tmem_alloc(&tmem_base, kBN);
    tc::tmem_relinquish();
  }
  if (threadIdx.x == 32) {
    for (int s = 0; s < kStages; s++) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(&done, 1);
    tc::fence_mbar_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  bool ok = true;
  int issued = 0;
  if (threadIdx.x == 0) {
    for (int kt = 0; kt < nk; kt++) {
      const int s = kt % kStages;
      if (kt >= kStages && !tc::mbar_wait(&empty[s], ((kt / kStages) - 1) & 1, kWaitLimit)) {
        ok = false;
        break;
      }
      tc::mbar_expect_tx(&full[s], kTileA + kTileB);
      tc::tma_load_2d(tA + s * kTileA, &ta, &full[s], kt * kBK, m0);
      tc::tma_load_2d(tB + s * kTileB, &tb, &full[s], kt * kBK, n0);
      issued = kt + 1;
    }
  } else if (threadIdx.x == 32) {
    constexpr uint32_t idesc = tc::idesc_bf16(kBM, kBN);
    for (int kt = 0; kt < nk; kt++) {
      const int s = kt % kStages;
      if (!tc::mbar_wait(&full[s], (kt / kStages) & 1, kWaitLimit)) {
        ok = false;
        break;
      }
      tc::fence_after_sync();
      const uint64_t ad = tc::smem_desc(tA + s * kTileA, tc::kSwizzle128, 128);
      const uint64_t bd = tc::smem_desc(tB + s * kTileB, tc::kSwizzle128, 128);
#pragma unroll
      for (int kk = 0; kk < kBK / 16; kk++)  // 16 BF16 = 32 bytes = 2 descriptor units
        tc::mma_bf16(tmem, ad + 2 * kk, bd + 2 * kk, idesc, (kt | kk) != 0);
      tc::mma_commit(&empty[s]);
    }
    tc::mma_commit(&done);
  }
  __syncwarp();
  const bool okd = __all_sync(0xffffffffu, tc::mbar_wait(&done, 0, kWaitLimit));
  tc::fence_after_sync();
  if (okd) {
    const int row = m0 + warp * 32 + lane;
#pragma unroll 1
    for (int c = 0; c < kBN; c += 8) {
      float v[8];
      tc::tmem_ld8(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
      float4 *dst = (float4 *)(D + (long long)row * ldd + n0 + c);
      dst[0] = make_float4(v[0], v[1], v[2], v[3]);
      dst[1] = make_float4(v[4], v[5], v[6], v[7]);
    }
  }
  if (!ok || !okd) atomicExch(err, 1);
  if (threadIdx.x == 0) {
    // the loads this thread issued have all landed before the block ends
    for (int kt = issued > kStages ? issued - kStages : 0; kt < issued; kt++)
      if (!tc::mbar_wait(&full[kt % kStages], (kt / kStages) & 1, kWaitLimit)) atomicExch(err, 2);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, kBN);
}

bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

// ---- periodic 3x3x3 convolution as an implicit GEMM ---------------------------
// Activations are channels-last BF16 with a one-voxel periodic halo:
// buf[n][z + 1][y + 1][x + 1][c] for z < D, y < H, x < W (the halo holds the
// wrapped neighbours, slbc_tc_halo).  Output tile: 128 voxels (a box of
// wbox x hbox x dbox) x all cout channels.  K runs over the 27 taps x the
// 32-channel chunks of the input: per step one TMA box of the input
// (32 channels x the tile shifted by the tap) and the tap's weights
// (cout x 32), two MMAs of K = 16.  Weights: w[tap][chunk][cout][32].
struct ConvArgs {
  int D, H, W;
  int cin, cout;
  int in_coff;
  int out_ctot, out_coff;
  int wbox, hbox, dbox;
  int relu;
  int tmem_cols;
  const float *bias;         // cout values or null
  const __nv_bfloat16 *mask; // or null: output *= (mask > 0), same layout as out
  __nv_bfloat16 *out;
  float *out_f32;            // or null: FP32 output (same layout) instead of out
};

constexpr int kConvTileA = 128 * 64;       // 128 voxels x 32 channels x 2 B

// Pipeline depth by output width: a stage is one A tile and one B tile of
// cout rows x 64 B, and every depth below keeps the stages within 96 KB, so
// two CTAs share an SM.
__host__ __device__ constexpr int conv_stages(int cout) { return cout <= 64 ? 8 : (cout <= 128 ? 6 : 4); }
__host__ __device__ constexpr int conv_smem(int nst, int cout) { return nst * (kConvTileA + cout * 64) + 1024; }
constexpr int kConvSmemMax = conv_smem(8, 64);
static_assert(conv_smem(6, 128) <= kConvSmemMax && conv_smem(4, 256) <= kConvSmemMax, "stage budget");

// The producer (thread 0) and the MMA issuer (thread 32) step through
// (tap, channel chunk, stage, round) with counters instead of divisions:
// for the narrow layers an MMA pair takes a few tens of cycles, so the
// single-thread loops set the pace.
template <int NST>
__global__ void __launch_bounds__(128, 2)
k_conv_fwd(const __grid_constant__ CUtensorMap tx, const __grid_constant__ CUtensorMap tw, ConvArgs a, int *err) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t pad = (1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u;
  uint8_t *tA = smem_raw + pad;
  const uint32_t tile_b = (uint32_t)a.cout * 64u;
  uint8_t *tB = tA + NST * kConvTileA;
  __shared__ uint64_t full[NST], empty[NST], done;
  __shared__ uint32_t tmem_base;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n = blockIdx.y;
  const int tiles_x = a.W / a.wbox, tiles_y = a.H / a.hbox;
  const int m = blockIdx.x;
  const int x0 = (m % tiles_x) * a.wbox, y0 = ((m / tiles_x) % tiles_y) * a.hbox, z0 = (m / (tiles_x * tiles_y)) * a.dbox;
  const int nck = a.cin / 32;
  const int nk = 27 * nck;
  const uint32_t bytes_b = (uint32_t)a.cout * 64u;
  if (warp == 0) {
    tc::tmem_alloc(&tmem_base, (uint32_t)a.tmem_cols);
    tc::tmem_relinquish();
  }
  if (threadIdx.x == 32) {
    for (int s = 0; s < NST; s++) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(&done, 1);
    tc::fence_mbar_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  bool ok = true;
  int issued = 0;
  if (threadIdx.x == 0) {
    int s = 0, round = 0, ck = 0, dx = 0, dy = 0, dz = 0;
    int c = a.in_coff, wrow = 0;
    for (int kt = 0; kt < nk; kt++) {
      if (round > 0 && !tc::mbar_wait(&empty[s], (uint32_t)(round - 1) & 1u, kWaitLimit)) {
        ok = false;
        break;
      }
      tc::mbar_expect_tx(&full[s], (uint32_t)kConvTileA + bytes_b);
      tc::tma_load_5d(tA + s * kConvTileA, &tx, &full[s], c, x0 + dx, y0 + dy, z0 + dz, n);
      tc::tma_load_2d(tB + s * tile_b, &tw, &full[s], 0, wrow);
      issued = kt + 1;
      wrow += a.cout;
      c += 32;
      if (++ck == nck) {
        ck = 0;
        c = a.in_coff;
        if (++dx == 3) {
          dx = 0;
          if (++dy == 3) {
            dy = 0;
            ++dz;
          }
        }
      }
      if (++s == NST) {
        s = 0;
        ++round;
      }
    }
  } else if (threadIdx.x == 32) {
    const uint32_t idesc = tc::idesc_bf16(128, a.cout);
    const uint64_t ad0 = tc::smem_desc(tA, tc::kSwizzle64, 64);
    const uint64_t bd0 = tc::smem_desc(tB, tc::kSwizzle64, 64);
    int s = 0, round = 0;
    for (int kt = 0; kt < nk; kt++) {
      if (!tc::mbar_wait(&full[s], (uint32_t)round & 1u, kWaitLimit)) {
        ok = false;
        break;
      }
      tc::fence_after_sync();
      // the start-address field counts 16-byte units
      const uint64_t ad = ad0 + (uint64_t)(s * (kConvTileA >> 4));
      const uint64_t bd = bd0 + (uint64_t)(s * (tile_b >> 4));
      tc::mma_bf16(tmem, ad, bd, idesc, kt != 0);
      tc::mma_bf16(tmem, ad + 2, bd + 2, idesc, 1);
      tc::mma_commit(&empty[s]);
      if (++s == NST) {
        s = 0;
        ++round;
      }
    }
    tc::mma_commit(&done);
  }
  __syncwarp();
  const bool okd = __all_sync(0xffffffffu, tc::mbar_wait(&done, 0, kWaitLimit));
  tc::fence_after_sync();
  if (okd) {
    const int r = warp * 32 + lane;
    const int vx = x0 + r % a.wbox, vy = y0 + (r / a.wbox) % a.hbox, vz = z0 + r / (a.wbox * a.hbox);
    const long long vox = (((long long)n * (a.D + 2) + vz + 1) * (a.H + 2) + vy + 1) * (a.W + 2) + vx + 1;
    __nv_bfloat16 *dst = a.out + vox * a.out_ctot + a.out_coff;
    const __nv_bfloat16 *msk = a.mask ? a.mask + vox * a.out_ctot + a.out_coff : nullptr;
#pragma unroll 1
    for (int c = 0; c < a.cout; c += 8) {
      float v[8];
      tc::tmem_ld8(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
      if (a.bias) {
#pragma unroll
        for (int i = 0; i < 8; i++) v[i] += a.bias[c + i];
      }
      if (a.relu) {
#pragma unroll
        for (int i = 0; i < 8; i++) v[i] = fmaxf(v[i], 0.0f);
      }
      if (msk) {
        const uint4 mv = *(const uint4 *)(msk + c);
        const __nv_bfloat16 *mb = (const __nv_bfloat16 *)&mv;
#pragma unroll
        for (int i = 0; i < 8; i++) v[i] = __bfloat162float(mb[i]) > 0.0f ? v[i] : 0.0f;
      }
      if (a.out_f32) {
        float4 *fd = (float4 *)(a.out_f32 + vox * a.out_ctot + a.out_coff + c);
        fd[0] = make_float4(v[0], v[1], v[2], v[3]);
        fd[1] = make_float4(v[4], v[5], v[6], v[7]);
      } else {
        uint4 o;
        __nv_bfloat162 *ob = (__nv_bfloat162 *)&o;
#pragma unroll
        for (int i = 0; i < 4; i++) ob[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
        *(uint4 *)(dst + c) = o;
      }
    }
  }
  if (!ok || !okd) atomicExch(err, 1);
  if (threadIdx.x == 0) {
    for (int kt = issued > NST ? issued - NST : 0; kt < issued; kt++)
      if (!tc::mbar_wait(&full[kt % NST], (kt / NST) & 1, kWaitLimit)) atomicExch(err, 2);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, (uint32_t)a.tmem_cols);
}

// Convolution of the narrower layers (32, 64 or 128 output channels) with input
// reuse.  An output tile is 16 (x) x 8 (y) x 2 (z) voxels.  For each
// 32-channel chunk and each x-shift dx, one 5-D TMA box brings the input
// block x0+dx .. x0+dx+15, y0-1 .. y0+8, z0-1 .. z0+2 (rows of 64 B,
// x fastest) into shared memory, with the weights of the nine taps of that
// dx.  The A operand of tap (dy, dz) for output slice s is then the 128
// consecutive rows starting at row ((s + dz) * 10 + dy) * 16, a multiple of
// 16 rows (1024 B, whole 64-byte swizzle atoms), so each input voxel crosses
// from L2 three times per chunk instead of 27.  Slices s = 0, 1 accumulate
// in TMEM columns [s * cout, (s + 1) * cout).
constexpr int kHzSlices = 2;
constexpr int kHzRows = (kHzSlices + 2) * 10 * 16;  // rows of one input block
constexpr int kHzTileA = kHzRows * 64;              // 40 KB
__host__ __device__ constexpr int hz_stages(int cout) { return cout <= 32 ? 3 : 2; }  // 32: 3, 64 / 128: 2
__host__ __device__ constexpr int hz_smem(int cout) { return hz_stages(cout) * (kHzTileA + 9 * cout * 64) + 1024; }
static_assert(hz_smem(32) <= 227 * 1024 && hz_smem(64) <= 227 * 1024 && hz_smem(128) <= 227 * 1024,
              "stage budget");

template <int NST>
__global__ void __launch_bounds__(128, 1)
k_conv_halo(const __grid_constant__ CUtensorMap tx, const __grid_constant__ CUtensorMap tw, ConvArgs a, int *err) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t pad = (1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u;
  uint8_t *tA = smem_raw + pad;
  const uint32_t tile_b = (uint32_t)a.cout * 64u;  // one tap's weights
  uint8_t *tB = tA + NST * kHzTileA;
  __shared__ uint64_t full[NST], empty[NST], done;
  __shared__ uint32_t tmem_base;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n = blockIdx.y;
  const int tiles_x = a.W / 16, tiles_y = a.H / 8;
  const int m = blockIdx.x;
  const int x0 = (m % tiles_x) * 16, y0 = ((m / tiles_x) % tiles_y) * 8, z0 = (m / (tiles_x * tiles_y)) * kHzSlices;
  const int nck = a.cin / 32;
  const int nk = 3 * nck;  // stages: (chunk, dx)
  if (warp == 0) {
    tc::tmem_alloc(&tmem_base, (uint32_t)a.tmem_cols);
    tc::tmem_relinquish();
  }
  if (threadIdx.x == 32) {
    for (int s = 0; s < NST; s++) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(&done, 1);
    tc::fence_mbar_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  bool ok = true;
  int issued = 0;
  if (threadIdx.x == 0) {
    int s = 0, round = 0, ck = 0, dx = 0;
    for (int kt = 0; kt < nk; kt++) {
      if (round > 0 && !tc::mbar_wait(&empty[s], (uint32_t)(round - 1) & 1u, kWaitLimit)) {
        ok = false;
        break;
      }
      tc::mbar_expect_tx(&full[s], (uint32_t)kHzTileA + 9u * tile_b);
      // padded coordinates: interior voxel v is v + 1, so x0 + dx is x0 + dx - 1 inside
      tc::tma_load_5d(tA + s * kHzTileA, &tx, &full[s], a.in_coff + ck * 32, x0 + dx, y0, z0, n);
      uint8_t *bs = tB + s * 9 * tile_b;
      for (int dz = 0; dz < 3; dz++)
        for (int dy = 0; dy < 3; dy++) {
          const int tap = dz * 9 + dy * 3 + dx;
          tc::tma_load_2d(bs + (dz * 3 + dy) * tile_b, &tw, &full[s], 0, (tap * nck + ck) * a.cout);
        }
      issued = kt + 1;
      if (++dx == 3) { dx = 0; ++ck; }
      if (++s == NST) { s = 0; ++round; }
    }
  } else if (threadIdx.x == 32) {
    const uint32_t idesc = tc::idesc_bf16(128, a.cout);
    int s = 0, round = 0;
    for (int kt = 0; kt < nk; kt++) {
      if (!tc::mbar_wait(&full[s], (uint32_t)round & 1u, kWaitLimit)) {
        ok = false;
        break;
      }
      tc::fence_after_sync();
      const uint64_t a0 = tc::smem_desc(tA + s * kHzTileA, tc::kSwizzle64, 64);
      const uint64_t b0 = tc::smem_desc(tB + s * 9 * tile_b, tc::kSwizzle64, 64);
      for (int dz = 0; dz < 3; dz++)
        for (int dy = 0; dy < 3; dy++) {
          const uint64_t bd = b0 + (uint64_t)((dz * 3 + dy) * (tile_b >> 4));
#pragma unroll
          for (int sl = 0; sl < kHzSlices; sl++) {
            // rows ((sl + dz) * 10 + dy) * 16 of 64 B; the start field counts 16-byte units
            const uint64_t ad = a0 + (uint64_t)(((sl + dz) * 10 + dy) * 16 * 4);
            const uint32_t d = tmem + (uint32_t)(sl * a.cout);
            const uint32_t acc = (kt != 0 || dz != 0 || dy != 0) ? 1u : 0u;
            tc::mma_bf16(d, ad, bd, idesc, acc);
            tc::mma_bf16(d, ad + 2, bd + 2, idesc, 1);
          }
        }
      tc::mma_commit(&empty[s]);
      if (++s == NST) { s = 0; ++round; }
    }
    tc::mma_commit(&done);
  }
  __syncwarp();
  const bool okd = __all_sync(0xffffffffu, tc::mbar_wait(&done, 0, kWaitLimit));
  tc::fence_after_sync();
  if (okd) {
    const int r = warp * 32 + lane;
    const int vx = x0 + r % 16, vy = y0 + r / 16;
#pragma unroll 1
    for (int sl = 0; sl < kHzSlices; sl++) {
      const int vz = z0 + sl;
      const long long vox = (((long long)n * (a.D + 2) + vz + 1) * (a.H + 2) + vy + 1) * (a.W + 2) + vx + 1;
      __nv_bfloat16 *dst = a.out ? a.out + vox * a.out_ctot + a.out_coff : nullptr;
      const __nv_bfloat16 *msk = a.mask ? a.mask + vox * a.out_ctot + a.out_coff : nullptr;
#pragma unroll 1
      for (int c = 0; c < a.cout; c += 8) {
        float v[8];
        tc::tmem_ld8(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(sl * a.cout + c), v);
        if (a.bias) {
#pragma unroll
          for (int i = 0; i < 8; i++) v[i] += a.bias[c + i];
        }
        if (a.relu) {
#pragma unroll
          for (int i = 0; i < 8; i++) v[i] = fmaxf(v[i], 0.0f);
        }
        if (msk) {
          const uint4 mv = *(const uint4 *)(msk + c);
          const __nv_bfloat16 *mb = (const __nv_bfloat16 *)&mv;
#pragma unroll
          for (int i = 0; i < 8; i++) v[i] = __bfloat162float(mb[i]) > 0.0f ? v[i] : 0.0f;
        }
        if (a.out_f32) {
          float4 *fd = (float4 *)(a.out_f32 + vox * a.out_ctot + a.out_coff + c);
          fd[0] = make_float4(v[0], v[1], v[2], v[3]);
          fd[1] = make_float4(v[4], v[5], v[6], v[7]);
        } else {
          uint4 o;
          __nv_bfloat162 *ob = (__nv_bfloat162 *)&o;
#pragma unroll
          for (int i = 0; i < 4; i++) ob[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
          *(uint4 *)(dst + c) = o;
        }
      }
    }
  }
  if (!ok || !okd) atomicExch(err, 1);
  if (threadIdx.x == 0) {
    for (int kt = issued > NST ? issued - NST : 0; kt < issued; kt++)
      if (!tc::mbar_wait(&full[kt % NST], (kt / NST) & 1, kWaitLimit)) atomicExch(err, 2);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, (uint32_t)a.tmem_cols);
}

// Periodic halo of channels [coff, coff + nch) (nch a multiple of 8): every
// halo voxel gets its wrapped interior voxel.  The halo voxels of a sample
// are enumerated face by face: the planes z = 0 and z = D + 1 whole, then
// for interior z the rows y = 0 and y = H + 1, then for interior z, y the
// columns x = 0 and x = W + 1.
__global__ void k_halo(__nv_bfloat16 *buf, int B, int D, int H, int W, int ctot, int coff, int nch) {
  const long long Pz = 2LL * (H + 2) * (W + 2), Py = 2LL * D * (W + 2), Px = 2LL * D * H;
  const long long per = Pz + Py + Px;
  const int nv = nch / 8;
  const long long total = (long long)B * per * nv;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int cv = (int)(e % nv);
    const long long h = e / nv;
    const int n = (int)(h / per);
    long long r = h % per;
    int x, y, z;
    if (r < Pz) {
      z = r < Pz / 2 ? 0 : D + 1;
      r %= Pz / 2;
      y = (int)(r / (W + 2));
      x = (int)(r % (W + 2));
    } else if ((r -= Pz) < Py) {
      y = r < Py / 2 ? 0 : H + 1;
      r %= Py / 2;
      z = 1 + (int)(r / (W + 2));
      x = (int)(r % (W + 2));
    } else {
      r -= Py;
      x = r < Px / 2 ? 0 : W + 1;
      r %= Px / 2;
      z = 1 + (int)(r / H);
      y = 1 + (int)(r % H);
    }
    const int sx = x == 0 ? W : (x == W + 1 ? 1 : x);
    const int sy = y == 0 ? H : (y == H + 1 ? 1 : y);
    const int sz = z == 0 ? D : (z == D + 1 ? 1 : z);
    const long long src = (((long long)n * (D + 2) + sz) * (H + 2) + sy) * (W + 2) + sx;
    const long long dst = (((long long)n * (D + 2) + z) * (H + 2) + y) * (W + 2) + x;
    *(uint4 *)(buf + dst * ctot + coff + 8 * cv) = *(const uint4 *)(buf + src * ctot + coff + 8 * cv);
  }
}

// 5-D map of a padded channels-last buffer: box of 32 channels x wbox x
// hbox x dbox x 1 (64-byte rows, 64-byte swizzle)
bool make_map_act(CUtensorMap *map, const void *ptr, int B, int D, int H, int W, int ctot, int wbox, int hbox,
                  int dbox) {
  EncodeTiled enc = encode_fn();
  if (!enc) return false;
  const cuuint64_t dims[5] = {(cuuint64_t)ctot, (cuuint64_t)W + 2, (cuuint64_t)H + 2, (cuuint64_t)D + 2,
                              (cuuint64_t)B};
  const cuuint64_t s1 = (cuuint64_t)ctot * 2;
  const cuuint64_t strides[4] = {s1, s1 * (W + 2), s1 * (W + 2) * (H + 2), s1 * (W + 2) * (H + 2) * (D + 2)};
  const cuuint32_t box[5] = {32, (cuuint32_t)wbox, (cuuint32_t)hbox, (cuuint32_t)dbox, 1};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void *>(ptr), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// 2-D map of rows of 32 BF16 (64 bytes), box of box_rows rows, 64-byte swizzle
bool make_map_rows32(CUtensorMap *map, const void *ptr, long long rows, int box_rows) {
  EncodeTiled enc = encode_fn();
  if (!enc) return false;
  const cuuint64_t dims[2] = {32, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {64};
  const cuuint32_t box[2] = {32, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// ---- weight gradients ------------------------------------------------------------
// dW[tap][co][ci] = sum_u dY[u - off(tap)][co] * X[u][ci] over all voxels u
// of all samples.  Both operands are channel-major with K = voxels flattened
// over the padded volume: row pitch Wp (a multiple of 8, >= W + 2), plane
// (H + 2) * Wp, sample stride pstride (a multiple of 64).  X's copy has a
// zero halo, so halo positions add nothing; dY's three copies S_dx (dx =
// 0, 1, 2) carry the periodic halo and the x part of the tap offset, so the
// y and z parts are aligned flat shifts of the TMA box.  Taps are stacked
// along M (128 rows = taps x output channels); K is split over blocks into
// FP32 partial sums, added in a fixed order afterwards.
struct WgradArgs {
  int cin, cout, co_rows, taps_per_tile, co_tiles;
  int ntile;
  int Wp;
  int plane;
  long long k_tiles;
  int splits;
  int tmem_cols;
  float *partial;  // [splits][27][cout][cin]
};

constexpr int kWgTileA = 128 * 128;  // 128 rows x 64 K x 2 B
constexpr int kWgTileB = 256 * 128;  // up to 256 rows
constexpr int kWgSmem = kStages * (kWgTileA + kWgTileB) + 1024;

// B stages hold ntile rows of 128 bytes (the dynamic shared memory is sized
// by ntile), so layers with up to 64 input channels fit two blocks per SM.
__global__ void __launch_bounds__(128, 2)
k_wgrad(const __grid_constant__ CUtensorMap a0, const __grid_constant__ CUtensorMap a1,
        const __grid_constant__ CUtensorMap a2, const __grid_constant__ CUtensorMap tb, WgradArgs w, int *err) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t pad = (1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u;
  uint8_t *tA = smem_raw + pad;
  uint8_t *tB = tA + kStages * kWgTileA;
  const int tile_b = w.ntile * 128;  // bytes of one B stage (a multiple of 2048)
  __shared__ uint64_t full[kStages], empty[kStages], done;
  __shared__ uint32_t tmem_base;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int group = blockIdx.x / w.co_tiles, cot = blockIdx.x % w.co_tiles;
  const int tap0 = group * w.taps_per_tile, co0 = cot * w.co_rows, ci0 = blockIdx.y * w.ntile;
  // K tiles z, z + splits, z + 2 splits, ... (z = blockIdx.z): the blocks
  // of one launch work through one run of consecutive tiles at a time, so
  // the windows that other taps read again (up to a plane further on) are
  // still in L2
  const long long kz = blockIdx.z;
  const int nk = kz < w.k_tiles ? (int)((w.k_tiles - kz + w.splits - 1) / w.splits) : 0;
  const uint32_t bytes_a = 128u * 128u, bytes_b = (uint32_t)w.ntile * 128u;
  if (warp == 0) {
    tc::tmem_alloc(&tmem_base, (uint32_t)w.tmem_cols);
    tc::tmem_relinquish();
  }
  if (threadIdx.x == 32) {
    for (int s = 0; s < kStages; s++) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(&done, 1);
    tc::fence_mbar_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  bool ok = true;
  int issued = 0;
  if (threadIdx.x == 0) {
    for (int kt = 0; kt < nk; kt++) {
      const int s = kt % kStages;
      if (kt >= kStages && !tc::mbar_wait(&empty[s], ((kt / kStages) - 1) & 1, kWaitLimit)) {
        ok = false;
        break;
      }
      const int k0 = (int)((kz + (long long)kt * w.splits) * 64);
      tc::mbar_expect_tx(&full[s], bytes_a + bytes_b);
      for (int tl = 0; tl < w.taps_per_tile; tl++) {
        const int tap = tap0 + tl < 27 ? tap0 + tl : 26;  // rows past tap 26 are discarded
        const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
        const int x = k0 - (dy - 1) * w.Wp - (dz - 1) * w.plane;
        const CUtensorMap *am = dx == 0 ? &a0 : (dx == 1 ? &a1 : &a2);
        tc::tma_load_2d(tA + s * kWgTileA + tl * w.co_rows * 128, am, &full[s], x, co0);
      }
      tc::tma_load_2d(tB + s * tile_b, &tb, &full[s], k0, ci0);
      issued = kt + 1;
    }
  } else if (threadIdx.x == 32) {
    const uint32_t idesc = tc::idesc_bf16(128, w.ntile);
    for (int kt = 0; kt < nk; kt++) {
      const int s = kt % kStages;
      if (!tc::mbar_wait(&full[s], (kt / kStages) & 1, kWaitLimit)) {
        ok = false;
        break;
      }
      tc::fence_after_sync();
      const uint64_t ad = tc::smem_desc(tA + s * kWgTileA, tc::kSwizzle128, 128);
      const uint64_t bd = tc::smem_desc(tB + s * tile_b, tc::kSwizzle128, 128);
#pragma unroll
      for (int kk = 0; kk < 4; kk++) tc::mma_bf16(tmem, ad + 2 * kk, bd + 2 * kk, idesc, (kt | kk) != 0);
      tc::mma_commit(&empty[s]);
    }
    tc::mma_commit(&done);
  }
  __syncwarp();
  const bool okd = __all_sync(0xffffffffu, tc::mbar_wait(&done, 0, kWaitLimit));
  tc::fence_after_sync();
  if (okd) {
    const int r = warp * 32 + lane;
    const int tap = tap0 + r / w.co_rows, co = co0 + r % w.co_rows;
    float *dst = w.partial + (((long long)blockIdx.z * 27 + tap) * w.cout + co) * w.cin + ci0;
#pragma unroll 1
    for (int c = 0; c < w.ntile; c += 8) {
      float v[8];
      tc::tmem_ld8(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
      if (nk == 0) {
#pragma unroll
        for (int i = 0; i < 8; i++) v[i] = 0.0f;
      }
      if (tap < 27) {
        ((float4 *)(dst + c))[0] = make_float4(v[0], v[1], v[2], v[3]);
        ((float4 *)(dst + c))[1] = make_float4(v[4], v[5], v[6], v[7]);
      }
    }
  }
  if (!ok || !okd) atomicExch(err, 1);
  if (threadIdx.x == 0) {
    for (int kt = issued > kStages ? issued - kStages : 0; kt < issued; kt++)
      if (!tc::mbar_wait(&full[kt % kStages], (kt / kStages) & 1, kWaitLimit)) atomicExch(err, 2);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, (uint32_t)w.tmem_cols);
}

// ---- weight gradients, taps stacked along N ----------------------------------
// The same sum with the y/z part of the tap offset moved to the input:
// dW[tap][co][ci] = sum_v S_dx[v][co] * X[v + s][ci], s = (dy - 1) * Wp +
// (dz - 1) * plane (v = u - s; X is zero outside its interior and TMA fills
// zeros outside the array, so the terms are the same).  Per K tile of 64
// flat positions a block then loads the three dY copies once (M: dx blocks
// of cout rows, 128 rows = up to 3 copies, a 4th block of 32 rows for cout =
// 32 is never loaded and its accumulator rows are dropped) and the input
// window at nt shifts s (N: nt taps x cc input channels, up to 288 rows in
// two MMAs), instead of 27 shifted dY tiles against one input tile: the
// operand bytes staged per FLOP drop 2.7x for 32 channels, and every MMA
// is 128 x 144 instead of 128 x 32.
struct WgradNArgs {
  int cin, cout;
  int dpm;        // dx copies per M tile
  int nt;         // (dy, dz) taps per block
  int groups;     // tap groups: ceil(9 / nt)
  int cc;         // input channels per block (cin, or a divisor of it)
  int ci_chunks;  // cin / cc
  int n_rows;     // nt * cc: accumulator columns
  int n_mma;      // columns per MMA (n_rows split into equal parts of <= 256)
  int Wp, plane;
  long long k_tiles;
  int splits;
  int tmem_cols;
  float *partial;  // [splits][27][cout][cin]
  // one TMA box per stage and operand where the layout allows it: the dpm
  // dY copies as one 3-D box (copies equally spaced in memory), the nt
  // input windows as one 4-D box (nt = 9: dy, dz = 0..2; nt = 3: dy =
  // 0..2 at one dz) of a view with strides Wp and plane along dy and dz;
  // the 4-D box is used where all its windows lie inside the array
  int a3, b4;
  long long b4_dim0;  // first-axis extent of the window view
  // dY copies in K-tile blocks [tile][3][cout][64] (slbc_tc_cmajor_tiles):
  // a0 boxes dpm * cout rows of a tile, a1 boxes cout rows
  int a_tiles;
};

constexpr int kWgnMaxRows = 288;
constexpr int kWgnSmem = kStages * (kWgTileA + kWgnMaxRows * 128) + 1024;

// Block decomposition of k_wgrad_n for (cin, cout); false when it does not
// apply (cout not 32, 64 or 128).
bool wgrad_n_plan(int cin, int cout, WgradNArgs &w) {
  if (!(cout == 32 || cout == 64 || cout == 128) || cin < 16 || cin % 16) return false;
  w.cin = cin;
  w.cout = cout;
  w.dpm = std::min(128 / cout, 3);
  int cc = cin;
  if (cc > 256) {
    cc = 0;
    for (int c = 256; c >= 16; c -= 16)
      if (cin % c == 0) { cc = c; break; }
    if (!cc) return false;
  }
  int groups = (9 * cc + kWgnMaxRows - 1) / kWgnMaxRows, nt = (9 + groups - 1) / groups;
  while (nt * cc > kWgnMaxRows) {
    groups++;
    nt = (9 + groups - 1) / groups;
  }
  w.cc = cc;
  w.ci_chunks = cin / cc;
  w.nt = nt;
  w.groups = groups;
  w.n_rows = nt * cc;
  const int parts = (w.n_rows + 255) / 256;
  if (w.n_rows % (16 * parts)) return false;
  w.n_mma = w.n_rows / parts;
  w.tmem_cols = 32;
  while (w.tmem_cols < w.n_rows) w.tmem_cols *= 2;
  return true;
}

int wgrad_n_ctas(const WgradNArgs &w) { return ((3 + w.dpm - 1) / w.dpm) * w.groups * w.ci_chunks; }

__global__ void __launch_bounds__(128, 1)
k_wgrad_n(const __grid_constant__ CUtensorMap a0, const __grid_constant__ CUtensorMap a1,
          const __grid_constant__ CUtensorMap a2, const __grid_constant__ CUtensorMap tb,
          const __grid_constant__ CUtensorMap a_all, const __grid_constant__ CUtensorMap b_win, WgradNArgs w,
          int *err) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t pad = (1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u;
  uint8_t *tA = smem_raw + pad;
  uint8_t *tB = tA + kStages * kWgTileA;
  const int tile_b = w.n_rows * 128;  // bytes of one B stage (a multiple of 2048)
  __shared__ uint64_t full[kStages], empty[kStages], done;
  __shared__ uint32_t tmem_base;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int chunk = blockIdx.x % w.ci_chunks;
  const int g = (blockIdx.x / w.ci_chunks) % w.groups;
  const int mt = blockIdx.x / (w.ci_chunks * w.groups);
  const int ci0 = chunk * w.cc;
  // K tiles z, z + splits, z + 2 splits, ... (z = blockIdx.z): the blocks
  // of one launch work through one run of consecutive tiles at a time, so
  // the windows that other taps read again (up to a plane further on) are
  // still in L2
  const long long kz = blockIdx.z;
  const int nk = kz < w.k_tiles ? (int)((w.k_tiles - kz + w.splits - 1) / w.splits) : 0;
  // bytes landing per stage: the dY copies and input windows actually loaded
  int a_blocks = 0, b_taps = 0;
  for (int d = 0; d < w.dpm; d++) a_blocks += mt * w.dpm + d < 3;
  for (int t = 0; t < w.nt; t++) b_taps += g * w.nt + t < 9;
  const uint32_t bytes = (uint32_t)(a_blocks * w.cout * 128 + b_taps * w.cc * 128);
  if (warp == 0) {
    tc::tmem_alloc(&tmem_base, (uint32_t)w.tmem_cols);
    tc::tmem_relinquish();
  }
  if (threadIdx.x == 32) {
    for (int s = 0; s < kStages; s++) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(&done, 1);
    tc::fence_mbar_init();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  bool ok = true;
  int issued = 0;
  if (threadIdx.x == 0) {
    for (int kt = 0; kt < nk; kt++) {
      const int s = kt % kStages;
      if (kt >= kStages && !tc::mbar_wait(&empty[s], ((kt / kStages) - 1) & 1, kWaitLimit)) {
        ok = false;
        break;
      }
      const int k0 = (int)((kz + (long long)kt * w.splits) * 64);
      tc::mbar_expect_tx(&full[s], bytes);
      if (w.a_tiles) {
        if (a_blocks == w.dpm) {
          tc::tma_load_3d(tA + s * kWgTileA, &a0, &full[s], 0, mt * w.dpm * w.cout, k0 >> 6);
        } else {
          for (int d = 0; d < a_blocks; d++)
            tc::tma_load_3d(tA + s * kWgTileA + d * w.cout * 128, &a1, &full[s], 0, (mt * w.dpm + d) * w.cout, k0 >> 6);
        }
      } else if (w.a3 && a_blocks == w.dpm) {
        tc::tma_load_3d(tA + s * kWgTileA, &a_all, &full[s], k0, 0, mt * w.dpm);
      } else {
        for (int d = 0; d < w.dpm; d++) {
          const int dx = mt * w.dpm + d;
          if (dx >= 3) break;
          const CUtensorMap *am = dx == 0 ? &a0 : (dx == 1 ? &a1 : &a2);
          tc::tma_load_2d(tA + s * kWgTileA + d * w.cout * 128, am, &full[s], k0, 0);
        }
      }
      // first window of the group: dy = 0 at the group's first dz
      const long long xw = (long long)k0 - w.Wp + ((g * w.nt) / 3 - 1) * (long long)w.plane;
      if (w.b4 && b_taps == w.nt && xw >= 0 && xw + 64 <= w.b4_dim0) {
        tc::tma_load_4d(tB + s * tile_b, &b_win, &full[s], (int)xw, ci0, 0, 0);
      } else {
        for (int t = 0; t < w.nt; t++) {
          const int yz = g * w.nt + t;
          if (yz >= 9) break;
          const int dy = yz % 3, dz = yz / 3;
          // may start before 0 or end past the array: TMA fills zeros there
          const int x = k0 + (dy - 1) * w.Wp + (dz - 1) * w.plane;
          tc::tma_load_2d(tB + s * tile_b + t * w.cc * 128, &tb, &full[s], x, ci0);
        }
      }
      issued = kt + 1;
    }
  } else if (threadIdx.x == 32) {
    const uint32_t idesc = tc::idesc_bf16(128, w.n_mma);
    const int parts = w.n_rows / w.n_mma;
    for (int kt = 0; kt < nk; kt++) {
      const int s = kt % kStages;
      if (!tc::mbar_wait(&full[s], (kt / kStages) & 1, kWaitLimit)) {
        ok = false;
        break;
      }
      tc::fence_after_sync();
      const uint64_t ad = tc::smem_desc(tA + s * kWgTileA, tc::kSwizzle128, 128);
      for (int j = 0; j < parts; j++) {
        const uint64_t bd = tc::smem_desc(tB + s * tile_b + j * w.n_mma * 128, tc::kSwizzle128, 128);
#pragma unroll
        for (int kk = 0; kk < 4; kk++)
          tc::mma_bf16(tmem + (uint32_t)(j * w.n_mma), ad + 2 * kk, bd + 2 * kk, idesc, (kt | kk) != 0);
      }
      tc::mma_commit(&empty[s]);
    }
    tc::mma_commit(&done);
  }
  __syncwarp();
  const bool okd = __all_sync(0xffffffffu, tc::mbar_wait(&done, 0, kWaitLimit));
  tc::fence_after_sync();
  if (okd) {
    const int r = warp * 32 + lane;
    const int d = r / w.cout, co = r % w.cout;
    const int dx = mt * w.dpm + d;
    const bool row_ok = d < w.dpm && dx < 3;
#pragma unroll 1
    for (int c = 0; c < w.n_rows; c += 8) {
      float v[8];
      tc::tmem_ld8(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);  // whole warp
      if (nk == 0) {
#pragma unroll
        for (int i = 0; i < 8; i++) v[i] = 0.0f;
      }
      const int t = c / w.cc, yz = g * w.nt + t;
      if (row_ok && yz < 9) {
        const int tap = (yz / 3) * 9 + (yz % 3) * 3 + dx;
        float *dst = w.partial + (((long long)blockIdx.z * 27 + tap) * w.cout + co) * w.cin + ci0 + c % w.cc;
        ((float4 *)dst)[0] = make_float4(v[0], v[1], v[2], v[3]);
        ((float4 *)dst)[1] = make_float4(v[4], v[5], v[6], v[7]);
      }
    }
  }
  if (!ok || !okd) atomicExch(err, 1);
  if (threadIdx.x == 0) {
    for (int kt = issued > kStages ? issued - kStages : 0; kt < issued; kt++)
      if (!tc::mbar_wait(&full[kt % kStages], (kt / kStages) & 1, kWaitLimit)) atomicExch(err, 2);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, (uint32_t)w.tmem_cols);
}

// dw[i] = sum over splits of partial[s][i], in split order
__global__ void k_sum_splits(const float *partial, long long n, int splits, float *dw) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float v = 0.0f;
    for (int s = 0; s < splits; s++) v += partial[(long long)s * n + i];
    dw[i] = v;
  }
}

// Channel-major flat copy of channels [coff, coff + nch) of a padded
// channels-last buffer: dst[c][n * pstride + (z * (H + 2) + y) * Wp + x] =
// src[n][z][y][x - shift][coff + c] for 0 <= x - shift <= W + 1 (0 beyond;
// zero_halo: interior voxels only, every halo position 0); with ncopy > 0
// the 64-position rows go to K-tile blocks instead, dst[t][copy][c][64]
// for t = flat position / 64 (the three x-shifted copies of an output
// gradient side by side per tile: one contiguous 12 KB block of DRAM per
// 32-channel tile for the weight gradient's A operand).  A block moves
// 64 consecutive flat positions x 64 channels through shared memory, so
// both the channel runs it reads and the position runs it writes are
// 128-byte rows.
__global__ void __launch_bounds__(256) k_cmajor(const __nv_bfloat16 *src, int B, int D, int H, int W, int ctot,
                                                int coff, int nch, int Wp, long long pstride, int shift,
                                                int zero_halo, int copy, int ncopy, __nv_bfloat16 *dst) {
  __shared__ __nv_bfloat16 tile[64][64 + 8];
  const long long plane = (long long)(H + 2) * Wp;
  const long long per_sample = (long long)(D + 2) * plane;
  const long long total = (long long)B * pstride;
  const long long ntiles = total / 64;
  const int nck = (nch + 63) / 64;
  for (long long work = blockIdx.x; work < ntiles * nck; work += gridDim.x) {
    const long long t = work / nck;
    const int c0 = (int)(work % nck) * 64;
    const int cw = nch - c0 < 64 ? nch - c0 : 64;
    // load: 64 positions x cw channels, 8 channels (16 B) per thread access
    for (int a = threadIdx.x; a < 64 * 8; a += blockDim.x) {
      const int pos = a / 8, cv = a % 8;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (cv * 8 < cw) {
        const long long e = t * 64 + pos;
        const int n = (int)(e / pstride);
        const long long f = e % pstride;
        if (f < per_sample) {
          const int z = (int)(f / plane);
          const long long r = f % plane;
          const int y = (int)(r / Wp);
          const int x = (int)(r % Wp) - shift;
          bool in = x >= 0 && x <= W + 1;
          if (zero_halo) in = in && x >= 1 && x <= W && y >= 1 && y <= H && z >= 1 && z <= D;
          if (in)
            v = *(const uint4 *)(src + ((((long long)n * (D + 2) + z) * (H + 2) + y) * (W + 2) + x) * ctot + coff +
                                 c0 + cv * 8);
        }
      }
      const __nv_bfloat16 *vb = (const __nv_bfloat16 *)&v;
#pragma unroll
      for (int i = 0; i < 8; i++) tile[cv * 8 + i][pos] = vb[i];
    }
    __syncthreads();
    // store: per channel 64 positions = 128 B, 16 B per thread access
    for (int a = threadIdx.x; a < 64 * 8; a += blockDim.x) {
      const int c = a / 8, pv = a % 8;
      if (c >= cw) continue;
      // channel-major row, or (ncopy > 0) row c of copy `copy` in the
      // block of K tile t: [t][copy][c][64]
      const long long o = ncopy ? ((t * ncopy + copy) * nch + c0 + c) * 64 : (long long)(c0 + c) * total + t * 64;
      *(uint4 *)(dst + o + pv * 8) = *(const uint4 *)&tile[c][pv * 8];
    }
    __syncthreads();
  }
}

// 2-D map: rows x cols BF16 (cols contiguous), box 64 x box_rows (128-byte swizzle)
bool make_map_k64(CUtensorMap *map, const void *ptr, long long rows, long long cols, int box_rows) {
  return make_map_2d(map, ptr, rows, cols, box_rows);
}

// 3 equally spaced copies (copy_bytes apart) of rows x cols BF16: box of 64
// columns x rows x ncopy copies
bool make_map_copies(CUtensorMap *map, const void *ptr, long long rows, long long cols, long long copy_bytes,
                     int ncopy) {
  EncodeTiled enc = encode_fn();
  if (!enc) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)cols, (cuuint64_t)rows, 3};
  const cuuint64_t strides[2] = {(cuuint64_t)cols * 2, (cuuint64_t)copy_bytes};
  const cuuint32_t box[3] = {64, (cuuint32_t)rows, (cuuint32_t)ncopy};
  const cuuint32_t estr[3] = {1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void *>(ptr), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// K-tile blocks [ntiles][rows][64] BF16: box of 64 x box_rows x 1
bool make_map_tiles(CUtensorMap *map, const void *ptr, long long rows, long long ntiles, int box_rows) {
  EncodeTiled enc = encode_fn();
  if (!enc) return false;
  const cuuint64_t dims[3] = {64, (cuuint64_t)rows, (cuuint64_t)ntiles};
  const cuuint64_t strides[2] = {128, (cuuint64_t)rows * 128};
  const cuuint32_t box[3] = {64, (cuuint32_t)box_rows, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void *>(ptr), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Shifted windows of rows x cols BF16 (row-major, channel rows): element
// (x, c, dy, dz) = ptr[c * cols + x + dy * Wp + dz * plane]; the first axis
// ends (ny - 1) * Wp + (nz - 1) * plane short of cols, so no window reaches
// past its row.  Box: 64 x box_rows x ny x nz.
bool make_map_windows(CUtensorMap *map, const void *ptr, long long rows, long long cols, int Wp, long long plane,
                      int box_rows, int ny, int nz, long long &dim0) {
  EncodeTiled enc = encode_fn();
  if (!enc) return false;
  dim0 = cols - (ny - 1) * (long long)Wp - (nz - 1) * plane;
  if (dim0 < 64) return false;
  const cuuint64_t dims[4] = {(cuuint64_t)dim0, (cuuint64_t)rows, (cuuint64_t)ny, (cuuint64_t)nz};
  const cuuint64_t strides[3] = {(cuuint64_t)cols * 2, (cuuint64_t)Wp * 2, (cuuint64_t)plane * 2};
  const cuuint32_t box[4] = {64, (cuuint32_t)box_rows, (cuuint32_t)ny, (cuuint32_t)nz};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void *>(ptr), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// M tile of 128 voxels for a D x H x W grid: false when the grid does not
// tile (sides powers of two with W * H * D >= 128 do)
bool tile_shape(int D, int H, int W, int &wbox, int &hbox, int &dbox) {
  wbox = W < 128 ? W : 128;
  hbox = H < 128 / wbox ? H : 128 / wbox;
  dbox = 128 / (wbox * hbox);
  return wbox * hbox * dbox == 128 && W % wbox == 0 && H % hbox == 0 && D % dbox == 0 && wbox <= 256 &&
         hbox <= 256 && dbox <= 256;
}

int cmajor_launch(const char *who, const void *src, int B, int D, int H, int W, int ctot, int coff, int nch, int Wp,
                  long long pstride, int shift, int zero_halo, int copy, int ncopy, void *dst, void *stream) {
  if (B < 1 || nch < 1 || coff < 0 || coff + nch > ctot || Wp < W + 2 || Wp % 8 || pstride % 64 ||
      pstride < (long long)(D + 2) * (H + 2) * Wp || shift < -1 || shift > 1)
    return slbc::set_error(std::string(who) + ": bad geometry"), 1;
  if (nch % 8 || coff % 8 || ctot % 8 || !aligned16(src) || !aligned16(dst))
    return slbc::set_error(std::string(who) + ": channels in multiples of 8, 16-byte aligned buffers"), 1;
  const long long work = (long long)B * pstride / 64 * ((nch + 63) / 64);
  const int blocks = (int)std::min<long long>(work, 152LL * 16);
  k_cmajor<<<blocks, 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16 *)src, B, D, H, W, ctot, coff, nch, Wp,
                                                     pstride, shift, zero_halo, copy, ncopy, (__nv_bfloat16 *)dst);
  slbc::count_launch();
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return slbc::set_error(std::string(who) + ": " + cudaGetErrorString(e)), 1;
  return 0;
}

// Both weight-gradient entry points: dY as three channel-major copies (dy0,
// dy1, dy2) or, with dyt, as K-tile blocks of the three copies.
int wgrad_launch(const char *who, const void *dy0, const void *dy1, const void *dy2, const void *dyt, const void *xt,
                 int B, int D, int H, int W, int Wp, long long pstride, int cin, int cout, float *partial,
                 long long partial_floats, int splits, float *dw, void *stream) {
  const std::string me(who);
  WgradArgs w;
  if (cout < 32 || (cout > 128 && cout % 128) || (cout <= 128 && 128 % cout) || cin < 16 || cin % 16)
    return slbc::set_error(me + ": cout must be 32, 64, 128 or a multiple of 128; cin a multiple of 16"), 1;
  if (Wp < W + 2 || Wp % 8 || pstride % 64 || pstride < (long long)(D + 2) * (H + 2) * Wp || splits < 1)
    return slbc::set_error(me + ": bad geometry"), 1;
  if (partial_floats < (long long)splits * 27 * cout * cin)
    return slbc::set_error(me + ": partial buffer too small"), 1;
  if (dyt) dy0 = dy1 = dy2 = dyt;
  if (!aligned16(dy0) || !aligned16(dy1) || !aligned16(dy2) || !aligned16(xt) || !aligned16(partial) ||
      !aligned16(dw))
    return slbc::set_error(me + ": buffers must be 16-byte aligned"), 1;
  const long long cols = (long long)B * pstride;
  WgradNArgs wn;
  const bool plan_n = wgrad_n_plan(cin, cout, wn);
  if (dyt && !plan_n) return slbc::set_error(me + ": K-tile blocks need cout 32, 64 or 128"), 1;
  if (plan_n) {  // taps stacked along N
    wn.Wp = Wp;
    wn.plane = (H + 2) * Wp;
    wn.k_tiles = cols / 64;
    wn.splits = splits;
    wn.partial = partial;
    int *err = tc_err_flag();
    if (!err) return slbc::set_error(me + ": no device error flag"), 1;
    CUtensorMap m0, m1, m2, mb;
    wn.a_tiles = dyt != nullptr;
    if (wn.a_tiles) {
      if (!make_map_tiles(&m0, dyt, 3LL * cout, wn.k_tiles, wn.dpm * cout) ||
          !make_map_tiles(&m1, dyt, 3LL * cout, wn.k_tiles, cout) || !make_map_k64(&mb, xt, cin, cols, wn.cc))
        return slbc::set_error(me + ": tensor map encoding failed"), 1;
      m2 = m0;
    } else if (!make_map_k64(&m0, dy0, cout, cols, cout) || !make_map_k64(&m1, dy1, cout, cols, cout) ||
               !make_map_k64(&m2, dy2, cout, cols, cout) || !make_map_k64(&mb, xt, cin, cols, wn.cc)) {
      return slbc::set_error(me + ": tensor map encoding failed"), 1;
    }
    // single-box forms (each falls back to the per-copy / per-tap boxes
    // when its map cannot be made)
    CUtensorMap ma = m0, mw = mb;
    const long long cstride = (const char *)dy1 - (const char *)dy0;
    wn.a3 = !wn.a_tiles && wn.dpm > 1 && cstride >= (long long)cout * cols * 2 && cstride % 16 == 0 &&
            (const char *)dy2 - (const char *)dy1 == cstride && make_map_copies(&ma, dy0, cout, cols, cstride, wn.dpm);
    wn.b4_dim0 = 0;
    wn.b4 = (wn.nt == 9 || wn.nt == 3) &&
            make_map_windows(&mw, xt, cin, cols, Wp, wn.plane, wn.cc, 3, wn.nt / 3, wn.b4_dim0);
    if (!wn.a3) ma = m0;
    if (!wn.b4) mw = mb;
    static unsigned long long attr_n_done = 0;
    cudaError_t e = smem_opt_in((const void *)k_wgrad_n, kWgnSmem, attr_n_done);
    if (e != cudaSuccess) return slbc::set_error(me + ": " + cudaGetErrorString(e)), 1;
    const dim3 grid((unsigned)wgrad_n_ctas(wn), 1, (unsigned)splits);
    const int smem = kStages * (kWgTileA + wn.n_rows * 128) + 1024;
    k_wgrad_n<<<grid, 128, smem, (cudaStream_t)stream>>>(m0, m1, m2, mb, ma, mw, wn, err);
    slbc::count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return slbc::set_error(me + ": " + cudaGetErrorString(e)), 1;
    const long long n = 27LL * cout * cin;
    k_sum_splits<<<(int)std::min<long long>((n + 255) / 256, 152LL * 8), 256, 0, (cudaStream_t)stream>>>(
        partial, n, splits, dw);
    slbc::count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return slbc::set_error(me + ": " + cudaGetErrorString(e)), 1;
    return 0;
  }
  w.cin = cin; w.cout = cout;
  w.co_rows = cout < 128 ? cout : 128;
  w.taps_per_tile = 128 / w.co_rows;
  w.co_tiles = cout / w.co_rows;
  w.ntile = cin;
  while (w.ntile > 256) w.ntile /= 2;
  if (cin % w.ntile || w.ntile % 16) return slbc::set_error(me + ": cin does not split into N tiles"), 1;
  w.Wp = Wp;
  w.plane = (H + 2) * Wp;
  w.k_tiles = (long long)B * pstride / 64;
  w.splits = splits;
  w.tmem_cols = 32;
  while (w.tmem_cols < w.ntile) w.tmem_cols *= 2;
  w.partial = partial;
  int *err = tc_err_flag();
  if (!err) return slbc::set_error(me + ": no device error flag"), 1;
  CUtensorMap m0, m1, m2, mb;
  if (!make_map_k64(&m0, dy0, cout, cols, w.co_rows) || !make_map_k64(&m1, dy1, cout, cols, w.co_rows) ||
      !make_map_k64(&m2, dy2, cout, cols, w.co_rows) || !make_map_k64(&mb, xt, cin, cols, w.ntile))
    return slbc::set_error(me + ": tensor map encoding failed"), 1;
  static unsigned long long attr_done = 0;
  cudaError_t e = smem_opt_in((const void *)k_wgrad, kWgSmem, attr_done);
  if (e != cudaSuccess) return slbc::set_error(me + ": " + cudaGetErrorString(e)), 1;
  const dim3 grid((unsigned)(((27 + w.taps_per_tile - 1) / w.taps_per_tile) * w.co_tiles), (unsigned)(cin / w.ntile),
                  (unsigned)splits);
  const int smem = kStages * (kWgTileA + w.ntile * 128) + 1024;
  k_wgrad<<<grid, 128, smem, (cudaStream_t)stream>>>(m0, m1, m2, mb, w, err);
  slbc::count_launch();
  e = cudaGetLastError();
  if (e != cudaSuccess) return slbc::set_error(me + ": " + cudaGetErrorString(e)), 1;
  const long long n = 27LL * cout * cin;
  k_sum_splits<<<(int)std::min<long long>((n + 255) / 256, 152LL * 8), 256, 0, (cudaStream_t)stream>>>(
      partial, n, splits, dw);
  slbc::count_launch();
  e = cudaGetLastError();
  if (e != cudaSuccess) return slbc::set_error(me + ": " + cudaGetErrorString(e)), 1;
  return 0;
}

}  // namespace

extern "C" {

int slbc_tc_gemm(const void *A, const void *B, float *D, int M, int N, int K, int ldd, void *stream) {
  if (M <= 0 || N <= 0 || K <= 0 || M % kBM || N % kBN || K % kBK)
    return slbc::set_error("slbc_tc_gemm: M and N must be multiples of 128 and K of 64"), 1;
  if (ldd < N || ldd % 4) return slbc::set_error("slbc_tc_gemm: ldd must be >= N and a multiple of 4"), 1;
  if (!aligned16(A) || !aligned16(B) || !aligned16(D))
    return slbc::set_error("slbc_tc_gemm: A, B and D must be 16-byte aligned"), 1;
  int *err = tc_err_flag();
  if (!err) return slbc::set_error("slbc_tc_gemm: no device error flag"), 1;
  CUtensorMap ta, tb;
  if (!make_map_2d(&ta, A, M, K, kBM) || !make_map_2d(&tb, B, N, K, kBN))
    return slbc::set_error("slbc_tc_gemm: tensor map encoding failed"), 1;
  static unsigned long long attr_done = 0;
  cudaError_t e = smem_opt_in((const void *)k_gemm_bf16, kGemmSmem, attr_done);
  if (e != cudaSuccess) return slbc::set_error(std::string("slbc_tc_gemm: ") + cudaGetErrorString(e)), 1;
  k_gemm_bf16<<<dim3(N / kBN, M / kBM), 128, kGemmSmem, (cudaStream_t)stream>>>(ta, tb, D, ldd, K, err);
  slbc::count_launch();
  e = cudaGetLastError();
  if (e != cudaSuccess) return slbc::set_error(std::string("slbc_tc_gemm: ") + cudaGetErrorString(e)), 1;
  return 0;
}

static int conv3d(const void *in, int B, int D, int H, int W, int in_ctot, int in_coff, int cin, const void *wgt,
                  const float *bias, int cout, void *out, float *out_f32, int out_ctot, int out_coff, int relu,
                  const void *mask, void *stream) {
  ConvArgs a;
  if (!out == !out_f32) return slbc::set_error("slbc_tc_conv3d: exactly one output buffer"), 1;
  if (out_f32 && out_ctot % 4) return slbc::set_error("slbc_tc_conv3d_f32: out_ctot must be a multiple of 4"), 1;
  if (!out) out = out_f32;  // alignment checks below
  if (B < 1 || cin < 32 || cin % 32 || cout < 16 || cout > 256 || cout % 16)
    return slbc::set_error("slbc_tc_conv3d: cin must be a multiple of 32, cout a multiple of 16 up to 256"), 1;
  if (in_ctot % 8 || in_coff % 8 || in_coff + cin > in_ctot || out_ctot % 8 || out_coff % 8 ||
      out_coff + cout > out_ctot)
    return slbc::set_error("slbc_tc_conv3d: channel counts and offsets must be multiples of 8 and fit"), 1;
  if (!tile_shape(D, H, W, a.wbox, a.hbox, a.dbox))
    return slbc::set_error("slbc_tc_conv3d: the grid does not tile into 128-voxel boxes"), 1;
  if (!aligned16(in) || !aligned16(wgt) || !aligned16(out) || (mask && !aligned16(mask)))
    return slbc::set_error("slbc_tc_conv3d: buffers must be 16-byte aligned"), 1;
  int *err = tc_err_flag();
  if (!err) return slbc::set_error("slbc_tc_conv3d: no device error flag"), 1;
  CUtensorMap tx, tw;
  if (!make_map_act(&tx, in, B, D, H, W, in_ctot, a.wbox, a.hbox, a.dbox) ||
      !make_map_rows32(&tw, wgt, 27LL * (cin / 32) * cout, cout))
    return slbc::set_error("slbc_tc_conv3d: tensor map encoding failed"), 1;
  a.D = D; a.H = H; a.W = W;
  a.cin = cin; a.cout = cout; a.in_coff = in_coff;
  a.out_ctot = out_ctot; a.out_coff = out_coff;
  a.relu = relu;
  a.tmem_cols = 32;
  while (a.tmem_cols < cout) a.tmem_cols *= 2;
  a.bias = bias;
  a.mask = (const __nv_bfloat16 *)mask;
  a.out = out_f32 ? nullptr : (__nv_bfloat16 *)out;
  a.out_f32 = out_f32;
  if ((cout == 32 || cout == 64 || cout == 128) && W % 16 == 0 && H % 8 == 0 && D % kHzSlices == 0) {
    // narrow layer: input-reuse tiles of 16 x 8 x 2 voxels
    CUtensorMap th;
    if (!make_map_act(&th, in, B, D, H, W, in_ctot, 16, 10, kHzSlices + 2))
      return slbc::set_error("slbc_tc_conv3d: tensor map encoding failed"), 1;
    a.tmem_cols = kHzSlices * cout;  // 64, 128 or 256 columns
    static unsigned long long attr_hz[2] = {0, 0};
    const int nst = hz_stages(cout), smem = hz_smem(cout);
    const void *fn = nst == 3 ? (const void *)k_conv_halo<3> : (const void *)k_conv_halo<2>;
    // one opt-in per instantiation, at the largest size it launches with
    cudaError_t eh = smem_opt_in(fn, nst == 3 ? hz_smem(32) : hz_smem(128), attr_hz[nst == 3 ? 0 : 1]);
    if (eh != cudaSuccess) return slbc::set_error(std::string("slbc_tc_conv3d: ") + cudaGetErrorString(eh)), 1;
    const dim3 grid((unsigned)((W / 16) * (H / 8) * (D / kHzSlices)), (unsigned)B);
    if (nst == 3)
      k_conv_halo<3><<<grid, 128, smem, (cudaStream_t)stream>>>(th, tw, a, err);
    else
      k_conv_halo<2><<<grid, 128, smem, (cudaStream_t)stream>>>(th, tw, a, err);
    slbc::count_launch();
    eh = cudaGetLastError();
    if (eh != cudaSuccess) return slbc::set_error(std::string("slbc_tc_conv3d: ") + cudaGetErrorString(eh)), 1;
    return 0;
  }
  static unsigned long long attr_done[3] = {0, 0, 0};
  const int nst = conv_stages(cout), smem = conv_smem(nst, cout);
  const void *fn = nst == 8 ? (const void *)k_conv_fwd<8> : (nst == 6 ? (const void *)k_conv_fwd<6> : (const void *)k_conv_fwd<4>);
  cudaError_t e = smem_opt_in(fn, kConvSmemMax, attr_done[nst == 8 ? 0 : (nst == 6 ? 1 : 2)]);
  if (e != cudaSuccess) return slbc::set_error(std::string("slbc_tc_conv3d: ") + cudaGetErrorString(e)), 1;
  const dim3 grid((unsigned)((long long)D * H * W / 128), (unsigned)B);
  if (nst == 8)
    k_conv_fwd<8><<<grid, 128, smem, (cudaStream_t)stream>>>(tx, tw, a, err);
  else if (nst == 6)
    k_conv_fwd<6><<<grid, 128, smem, (cudaStream_t)stream>>>(tx, tw, a, err);
  else
    k_conv_fwd<4><<<grid, 128, smem, (cudaStream_t)stream>>>(tx, tw, a, err);
  slbc::count_launch();
  e = cudaGetLastError();
  if (e != cudaSuccess) return slbc::set_error(std::string("slbc_tc_conv3d: ") + cudaGetErrorString(e)), 1;
  return 0;
}

int slbc_tc_conv3d(const void *in, int B, int D, int H, int W, int in_ctot, int in_coff, int cin, const void *wgt,
                   const float *bias, int cout, void *out, int out_ctot, int out_coff, int relu, const void *mask,
                   void *stream) {
  return conv3d(in, B, D, H, W, in_ctot, in_coff, cin, wgt, bias, cout, out, nullptr, out_ctot, out_coff, relu, mask,
                stream);
}

int slbc_tc_conv3d_f32(const void *in, int B, int D, int H, int W, int in_ctot, int in_coff, int cin,
                       const void *wgt, const float *bias, int cout, float *out, int out_ctot, int out_coff,
                       void *stream) {
  return conv3d(in, B, D, H, W, in_ctot, in_coff, cin, wgt, bias, cout, nullptr, out, out_ctot, out_coff, 0, nullptr,
                stream);
}

int slbc_tc_halo(void *buf, int B, int D, int H, int W, int ctot, int coff, int nch, void *stream) {
  if (B < 1 || D < 1 || H < 1 || W < 1 || ctot % 8 || coff % 8 || nch % 8 || nch < 8 || coff + nch > ctot)
    return slbc::set_error("slbc_tc_halo: channel counts and offsets must be multiples of 8 and fit"), 1;
  if (!aligned16(buf)) return slbc::set_error("slbc_tc_halo: buffer must be 16-byte aligned"), 1;
  const long long per = 2LL * (H + 2) * (W + 2) + 2LL * D * (W + 2) + 2LL * D * H;
  const long long total = (long long)B * per * (nch / 8);
  const int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 16);
  k_halo<<<blocks, 256, 0, (cudaStream_t)stream>>>((__nv_bfloat16 *)buf, B, D, H, W, ctot, coff, nch);
  slbc::count_launch();
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return slbc::set_error(std::string("slbc_tc_halo: ") + cudaGetErrorString(e)), 1;
  return 0;
}

int slbc_tc_cmajor(const void *src, int B, int D, int H, int W, int ctot, int coff, int nch, int Wp,
                   long long pstride, int shift, int zero_halo, void *dst, void *stream) {
  return cmajor_launch("slbc_tc_cmajor", src, B, D, H, W, ctot, coff, nch, Wp, pstride, shift, zero_halo, 0, 0, dst,
                       stream);
}

int slbc_tc_cmajor_tiles(const void *src, int B, int D, int H, int W, int ctot, int coff, int nch, int Wp,
                         long long pstride, int shift, int copy, int ncopy, void *dst, void *stream) {
  if (ncopy < 1 || copy < 0 || copy >= ncopy)
    return slbc::set_error("slbc_tc_cmajor_tiles: copy must lie in [0, ncopy)"), 1;
  return cmajor_launch("slbc_tc_cmajor_tiles", src, B, D, H, W, ctot, coff, nch, Wp, pstride, shift, 0, copy, ncopy,
                       dst, stream);
}

int slbc_tc_wgrad_splits(int cin, int cout, long long k_tiles, long long max_splits) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    sms = 152;
  WgradNArgs wn;
  long long want;
  // as many splits as fill the SMs in one wave: a block left over for a
  // second wave would take as long as the whole first one
  if (wgrad_n_plan(cin, cout, wn)) {
    const int ctas = wgrad_n_ctas(wn);  // one block per SM
    want = sms / ctas;
  } else {  // two blocks per SM
    const int co_rows = cout < 128 ? cout : 128;
    int ntile = cin;
    while (ntile > 256) ntile /= 2;
    const int blocks = ((27 + 128 / co_rows - 1) / (128 / co_rows)) * (cout / co_rows) * (cin / ntile);
    want = 2 * sms / blocks;
  }
  want = std::min(want, std::max(1LL, k_tiles / 8));
  want = std::min(want, max_splits);
  return (int)std::max(1LL, want);
}

int slbc_tc_wgrad(const void *dy0, const void *dy1, const void *dy2, const void *xt, int B, int D, int H, int W,
                  int Wp, long long pstride, int cin, int cout, float *partial, long long partial_floats, int splits,
                  float *dw, void *stream) {
  return wgrad_launch("slbc_tc_wgrad", dy0, dy1, dy2, nullptr, xt, B, D, H, W, Wp, pstride, cin, cout, partial,
                      partial_floats, splits, dw, stream);
}

int slbc_tc_wgrad_tiles(const void *dyt, const void *xt, int B, int D, int H, int W, int Wp, long long pstride,
                        int cin, int cout, float *partial, long long partial_floats, int splits, float *dw,
                        void *stream) {
  if (!dyt) return slbc::set_error("slbc_tc_wgrad_tiles: no dY blocks"), 1;
  return wgrad_launch("slbc_tc_wgrad_tiles", nullptr, nullptr, nullptr, dyt, xt, B, D, H, W, Wp, pstride, cin, cout,
                      partial, partial_floats, splits, dw, stream);
}

// Synchronises the device and returns (and clears) the tensor-core kernels'
// error flag: 0 fine, 1 a pipeline wait gave up, 2 a load never landed.
int slbc_tc_status(void) {
  int *err = tc_err_flag();
  if (!err) return -1;
  if (cudaDeviceSynchronize() != cudaSuccess) return -1;
  int v = 0;
  if (cudaMemcpy(&v, err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  if (v) cudaMemset(err, 0, sizeof(int));
  return v;
}

}  // extern "C"
