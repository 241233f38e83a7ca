// Mean-flow sums without any device allocation (slbc_vsum_noalloc).
//
// Some callers of this library cannot allocate device memory at the point
// where they need the mean flow: a solver embedded in a host application
// that owns all device memory through its own pool, or a time-stepping loop
// that must not call cudaMalloc (cudaMalloc can synchronise the whole device
// and can fail under memory pressure in the middle of a run).  This entry
// point takes the populations, flags and output buffer from the caller and
// keeps its only intermediate data -- one partial sum per reduction block --
// in the file-scope device array below, which every GPU that loads the
// library holds until the process exits.
//
// Compiled with -fmad=false, like the FP64 kernels, so the sums equal those
// of slbc_vsum when the same number of reduction blocks is used.
#include <cstring>
#include <mutex>

#include "slbc_internal.cuh"
#include "slbc_kernels.cuh"

namespace {

constexpr int kMaxBlocks = SLBC_VSUM_NOALLOC_MAX_BLOCKS;
constexpr int kMaxDevices = 64;

// Partial sums: 5 per block.  Every element a call reads is written by the
// same call first, so nothing needs clearing between calls.
static __device__ __align__(256) double g_vsum_scratch[5 * kMaxBlocks];

// Device address of g_vsum_scratch, cached per device together with the id
// of the CUDA context it was looked up in (the host-side name is only a
// stand-in and must never be passed to a kernel).  Context ids are unique for
// the life of the process, so after a cudaDeviceReset, or with another
// context bound on the same device, the address is looked up again instead
// of reusing one from a context that no longer exists.
struct ScratchEntry {
  unsigned long long ctx_id;
  void *addr;
};
ScratchEntry g_scratch[kMaxDevices];
std::mutex g_scratch_lock;

// cuCtxGetCurrent / cuCtxGetId through the runtime's driver entry-point
// query, so the library needs no link-time dependency on libcuda.
typedef int (*CtxGetCurrentFn)(void **);
typedef int (*CtxGetIdFn)(void *, unsigned long long *);

bool current_context_id(unsigned long long *id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    looked_up = true;
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (CtxGetCurrentFn)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (CtxGetIdFn)f;
  }
  if (get_current == nullptr || get_id == nullptr) return false;
  void *ctx = nullptr;
  if (get_current(&ctx) != 0 || ctx == nullptr) return false;
  return get_id(ctx, id) == 0;
}

int scratch_for_current_device(double **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    slbc::set_error(std::string("slbc_vsum_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    return 1;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    slbc::set_error("slbc_vsum_noalloc: device index out of range");
    return 1;
  }
  std::lock_guard<std::mutex> guard(g_scratch_lock);
  unsigned long long ctx = 0;
  if (g_scratch[dev].addr != nullptr && current_context_id(&ctx) && ctx == g_scratch[dev].ctx_id) {
    *out = (double *)g_scratch[dev].addr;
    return 0;
  }
  void *p = nullptr;
  e = cudaGetSymbolAddress(&p, g_vsum_scratch);  // makes the device's primary context current if none is
  if (e != cudaSuccess || p == nullptr) {
    slbc::set_error(std::string("slbc_vsum_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    return 1;
  }
  // cache only what can be validated later; otherwise look it up every call
  g_scratch[dev].addr = current_context_id(&ctx) ? p : nullptr;
  g_scratch[dev].ctx_id = ctx;
  *out = (double *)p;
  return 0;
}

template <typename T>
cudaError_t launch(const void *pop, long long npad, int layout, const unsigned short *flags,
                   int esi, int esj, int esk, double rho0, double fac, double bx, double by,
                   double bz, const void *bf, const double *psi, int nblocks, double *scratch,
                   double *out, cudaStream_t st) {
  slbc::PopArgs<T> p;
  p.pop = (T *)pop;
  p.npad = npad;
  p.flags = (const uint16_t *)flags;
  p.esi = esi; p.esj = esj; p.esk = esk;
  slbc::k_vsum<T><<<nblocks, slbc::kReduceThreads, 0, st>>>(p, layout, rho0, fac, bf == nullptr,
                                                             bx, by, bz, (const T *)bf, psi, scratch);
  slbc::count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  slbc::k_final_sum_tree<5><<<1, 256, 0, st>>>(scratch, nblocks, out);
  slbc::count_launch();
  return cudaGetLastError();
}

}  // namespace

extern "C" int slbc_vsum_noalloc(const void *pop, long long npad, int precision, int layout,
                                 const unsigned short *flags, int esi, int esj, int esk,
                                 double rho0, double fac, double bx, double by, double bz,
                                 const void *bf, const double *psi, int nblocks, double *out,
                                 void *stream) {
  if (nblocks < 1 || nblocks > kMaxBlocks) {
    slbc::set_error("slbc_vsum_noalloc: nblocks must be between 1 and " + std::to_string(kMaxBlocks) +
                    " (the size of its static scratch), got " + std::to_string(nblocks));
    return 1;
  }
  if (pop == nullptr || flags == nullptr || out == nullptr) {
    slbc::set_error("slbc_vsum_noalloc: pop, flags and out must be device pointers");
    return 1;
  }
  if (esi < 1 || esj < 1 || esk < 1 || (long long)esi * esj * esk >= (1LL << 31)) {
    slbc::set_error("slbc_vsum_noalloc: lattice sides must be >= 1 with fewer than 2^31 nodes");
    return 1;
  }
  if (npad < (long long)esi * esj * esk) {
    slbc::set_error("slbc_vsum_noalloc: npad is smaller than the number of nodes");
    return 1;
  }
  if (layout < SLBC_LAYOUT_N || layout > SLBC_LAYOUT_C1 || (precision != 0 && precision != 1)) {
    slbc::set_error("slbc_vsum_noalloc: precision must be 0 or 1 and layout 0, 1 or 2");
    return 1;
  }
  double *scratch = nullptr;
  if (scratch_for_current_device(&scratch)) return 1;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = precision == 0
      ? launch<double>(pop, npad, layout, flags, esi, esj, esk, rho0, fac, bx, by, bz, bf, psi,
                       nblocks, scratch, out, st)
      : launch<float>(pop, npad, layout, flags, esi, esj, esk, rho0, fac, bx, by, bz, bf, psi,
                      nblocks, scratch, out, st);
  if (e != cudaSuccess) {
    slbc::set_error(std::string("slbc_vsum_noalloc: ") + cudaGetErrorString(e));
    return (int)e;
  }
  return 0;
}
