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
};

constexpr int kConvTileA = 128 * 64;       // 128 voxels x 32 channels x 2 B
constexpr int kConvTileB = 256 * 64;       // up to 256 output channels x 32 x 2 B
constexpr int kConvSmem = kStages * (kConvTileA + kConvTileB) + 1024;

__global__ void __launch_bounds__(128, 1)
k_conv_fwd(const __grid_constant__ CUtensorMap tx, const __grid_constant__ CUtensorMap tw, ConvArgs a, int *err) {
  extern __shared__ uint8_t smem_raw[];
  const uint32_t pad = (1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u;
  uint8_t *tA = smem_raw + pad;
  uint8_t *tB = tA + kStages * kConvTileA;
  __shared__ uint64_t full[kStages], empty[kStages], done;
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
      const int tap = kt / nck, ck = kt - tap * nck;
      const int dz = tap / 9, dy = (tap / 3) % 3, dx = tap % 3;
      tc::mbar_expect_tx(&full[s], (uint32_t)kConvTileA + bytes_b);
      tc::tma_load_5d(tA + s * kConvTileA, &tx, &full[s], a.in_coff + ck * 32, x0 + dx, y0 + dy, z0 + dz, n);
      tc::tma_load_2d(tB + s * kConvTileB, &tw, &full[s], 0, kt * a.cout);
      issued = kt + 1;
    }
  } else if (threadIdx.x == 32) {
    const uint32_t idesc = tc::idesc_bf16(128, a.cout);
    for (int kt = 0; kt < nk; kt++) {
      const int s = kt % kStages;
      if (!tc::mbar_wait(&full[s], (kt / kStages) & 1, kWaitLimit)) {
        ok = false;
        break;
      }
      tc::fence_after_sync();
      const uint64_t ad = tc::smem_desc(tA + s * kConvTileA, tc::kSwizzle64, 64);
      const uint64_t bd = tc::smem_desc(tB + s * kConvTileB, tc::kSwizzle64, 64);
      tc::mma_bf16(tmem, ad, bd, idesc, kt != 0);
      tc::mma_bf16(tmem, ad + 2, bd + 2, idesc, 1);
      tc::mma_commit(&empty[s]);
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
      uint4 o;
      __nv_bfloat162 *ob = (__nv_bfloat162 *)&o;
#pragma unroll
      for (int i = 0; i < 4; i++) ob[i] = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
      *(uint4 *)(dst + c) = o;
    }
  }
  if (!ok || !okd) atomicExch(err, 1);
  if (threadIdx.x == 0) {
    for (int kt = issued > kStages ? issued - kStages : 0; kt < issued; kt++)
      if (!tc::mbar_wait(&full[kt % kStages], (kt / kStages) & 1, kWaitLimit)) atomicExch(err, 2);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, (uint32_t)a.tmem_cols);
}

// Periodic halo of channels [coff, coff + nch) (nch a multiple of 8): every
// halo voxel gets its wrapped interior voxel.
__global__ void k_halo(__nv_bfloat16 *buf, int B, int D, int H, int W, int ctot, int coff, int nch) {
  const long long P = (long long)(D + 2) * (H + 2) * (W + 2);
  const int nv = nch / 8;
  const long long total = (long long)B * P * nv;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int cv = (int)(e % nv);
    const long long v = e / nv;
    const int n = (int)(v / P);
    long long r = v % P;
    const int x = (int)(r % (W + 2));
    r /= (W + 2);
    const int y = (int)(r % (H + 2)), z = (int)(r / (H + 2));
    if (x >= 1 && x <= W && y >= 1 && y <= H && z >= 1 && z <= D) continue;
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

// M tile of 128 voxels for a D x H x W grid: false when the grid does not
// tile (sides powers of two with W * H * D >= 128 do)
bool tile_shape(int D, int H, int W, int &wbox, int &hbox, int &dbox) {
  wbox = W < 128 ? W : 128;
  hbox = H < 128 / wbox ? H : 128 / wbox;
  dbox = 128 / (wbox * hbox);
  return wbox * hbox * dbox == 128 && W % wbox == 0 && H % hbox == 0 && D % dbox == 0 && wbox <= 256 &&
         hbox <= 256 && dbox <= 256;
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
  static std::once_flag attr;
  cudaError_t e = cudaSuccess;
  std::call_once(attr, [&] {
    e = cudaFuncSetAttribute(k_gemm_bf16, cudaFuncAttributeMaxDynamicSharedMemorySize, kGemmSmem);
  });
  if (e != cudaSuccess) return slbc::set_error(std::string("slbc_tc_gemm: ") + cudaGetErrorString(e)), 1;
  k_gemm_bf16<<<dim3(N / kBN, M / kBM), 128, kGemmSmem, (cudaStream_t)stream>>>(ta, tb, D, ldd, K, err);
  slbc::count_launch();
  e = cudaGetLastError();
  if (e != cudaSuccess) return slbc::set_error(std::string("slbc_tc_gemm: ") + cudaGetErrorString(e)), 1;
  return 0;
}

int slbc_tc_conv3d(const void *in, int B, int D, int H, int W, int in_ctot, int in_coff, int cin, const void *wgt,
                   const float *bias, int cout, void *out, int out_ctot, int out_coff, int relu, const void *mask,
                   void *stream) {
  ConvArgs a;
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
  a.out = (__nv_bfloat16 *)out;
  static std::once_flag attr;
  cudaError_t e = cudaSuccess;
  std::call_once(attr, [&] {
    e = cudaFuncSetAttribute(k_conv_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, kConvSmem);
  });
  if (e != cudaSuccess) return slbc::set_error(std::string("slbc_tc_conv3d: ") + cudaGetErrorString(e)), 1;
  k_conv_fwd<<<dim3((unsigned)((long long)D * H * W / 128), (unsigned)B), 128, kConvSmem, (cudaStream_t)stream>>>(
      tx, tw, a, err);
  slbc::count_launch();
  e = cudaGetLastError();
  if (e != cudaSuccess) return slbc::set_error(std::string("slbc_tc_conv3d: ") + cudaGetErrorString(e)), 1;
  return 0;
}

int slbc_tc_halo(void *buf, int B, int D, int H, int W, int ctot, int coff, int nch, void *stream) {
  if (B < 1 || D < 1 || H < 1 || W < 1 || ctot % 8 || coff % 8 || nch % 8 || nch < 8 || coff + nch > ctot)
    return slbc::set_error("slbc_tc_halo: channel counts and offsets must be multiples of 8 and fit"), 1;
  if (!aligned16(buf)) return slbc::set_error("slbc_tc_halo: buffer must be 16-byte aligned"), 1;
  const long long total = (long long)B * (D + 2) * (H + 2) * (W + 2) * (nch / 8);
  const int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 16);
  k_halo<<<blocks, 256, 0, (cudaStream_t)stream>>>((__nv_bfloat16 *)buf, B, D, H, W, ctot, coff, nch);
  slbc::count_launch();
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return slbc::set_error(std::string("slbc_tc_halo: ") + cudaGetErrorString(e)), 1;
  return 0;
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
