// Tensor-core kernels of the learned warm start (BF16 inputs, FP32
// accumulation in TMEM, tcgen05.mma issued by one thread, operands staged by
// TMA through a 4-stage mbarrier pipeline).
//
// slbc_tc_gemm: D[M x N] (FP32, row-major, leading dimension ldd) =
// A[M x K] * B[N x K]^T with A and B BF16, row-major (K contiguous).  The
// weight gradients of the network's convolutions are this product.
#include <cstring>
#include <mutex>

#include "slbc_internal.cuh"
#include "slbc_tc.cuh"

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
