// Sphere rasterisation on the GPU (the node tests of many insertsph calls
// at once; reference src/lbobjs.c:204-232 for one sphere).
//
// For n spheres (r, x, y, z) inserted in order, insertsph gives every node
// with rsq = (i-x)^2 + (j-y)^2 + (k-z)^2 < r^2 to the sphere, a later sphere
// taking the node over from an earlier one.  Here one block per sphere walks
// the sphere's bounding box; per node the highest sphere index that covers
// it is kept (atomicMax), which is the sphere that holds it after all n
// insertions; per sphere the number of nodes it covers (insertsph's ns,
// which decides whether the object is kept) and whether any of them was
// already taken -- by an object before the call or by an earlier sphere of
// the call (insertsph's "overlaps").  The products, differences and sums of
// rsq are explicitly rounded (no multiply-add contraction) in the order the
// reference writes them, so the node sets equal the host's exactly.
#include <cmath>
#include <string>

#include "slbc_internal.cuh"

namespace {

__device__ __forceinline__ void sphere_box(const double *s, int n, int dim, int axis, int &lo, int &hi) {
  const double c = s[1 + axis], r = fabs(s[0]);
  lo = 0;
  hi = dim - 1;
  if (isfinite(s[0]) && isfinite(s[1]) && isfinite(s[2]) && isfinite(s[3])) {
    const double a = floor(c - r) - 1.0, b = ceil(c + r) + 1.0;
    lo = a < 0.0 ? 0 : (a > dim - 1 ? dim : (int)a);
    hi = b > dim - 1 ? dim - 1 : (b < 0.0 ? -1 : (int)b);
  }
}

__device__ __forceinline__ bool covers(const double *s, int i, int j, int k) {
  const double di = __dsub_rn((double)i, s[1]), dj = __dsub_rn((double)j, s[2]), dk = __dsub_rn((double)k, s[3]);
  const double rsq = __dadd_rn(__dadd_rn(__dmul_rn(di, di), __dmul_rn(dj, dj)), __dmul_rn(dk, dk));
  return rsq < __dmul_rn(s[0], s[0]);
}

// pass 1: per node the last covering sphere, per sphere its node count
__global__ void k_raster(const double *sph, int nsph, int esi, int esj, int esk, int *last, int *count) {
  const int s = blockIdx.x;
  if (s >= nsph) return;
  const double *sp = sph + 4 * s;
  int lo[3], hi[3];
  sphere_box(sp, nsph, esi, 0, lo[0], hi[0]);
  sphere_box(sp, nsph, esj, 1, lo[1], hi[1]);
  sphere_box(sp, nsph, esk, 2, lo[2], hi[2]);
  const long long ni = hi[0] - lo[0] + 1, nj = hi[1] - lo[1] + 1, nk = hi[2] - lo[2] + 1;
  if (ni <= 0 || nj <= 0 || nk <= 0) return;
  int c = 0;
  for (long long e = threadIdx.x; e < ni * nj * nk; e += blockDim.x) {
    const int i = lo[0] + (int)(e / (nj * nk)), j = lo[1] + (int)((e / nk) % nj), k = lo[2] + (int)(e % nk);
    if (!covers(sp, i, j, k)) continue;
    atomicMax(last + ((long long)i * esj + j) * esk + k, s);
    c++;
  }
  if (c) atomicAdd(count + s, c);
}

// pass 1b: per node the first covering sphere (for the overlap flags)
__global__ void k_raster_first(const double *sph, int nsph, int esi, int esj, int esk, int *first) {
  const int s = blockIdx.x;
  if (s >= nsph) return;
  const double *sp = sph + 4 * s;
  int lo[3], hi[3];
  sphere_box(sp, nsph, esi, 0, lo[0], hi[0]);
  sphere_box(sp, nsph, esj, 1, lo[1], hi[1]);
  sphere_box(sp, nsph, esk, 2, lo[2], hi[2]);
  const long long ni = hi[0] - lo[0] + 1, nj = hi[1] - lo[1] + 1, nk = hi[2] - lo[2] + 1;
  if (ni <= 0 || nj <= 0 || nk <= 0) return;
  for (long long e = threadIdx.x; e < ni * nj * nk; e += blockDim.x) {
    const int i = lo[0] + (int)(e / (nj * nk)), j = lo[1] + (int)((e / nk) % nj), k = lo[2] + (int)(e % nk);
    if (covers(sp, i, j, k)) atomicMin(first + ((long long)i * esj + j) * esk + k, s);
  }
}

// pass 2: a sphere overlaps when one of its nodes was taken before the call
// or is covered by an earlier sphere
__global__ void k_raster_overlap(const double *sph, int nsph, int esi, int esj, int esk, const int *first,
                                 const unsigned char *taken, unsigned char *overlap) {
  const int s = blockIdx.x;
  if (s >= nsph) return;
  const double *sp = sph + 4 * s;
  int lo[3], hi[3];
  sphere_box(sp, nsph, esi, 0, lo[0], hi[0]);
  sphere_box(sp, nsph, esj, 1, lo[1], hi[1]);
  sphere_box(sp, nsph, esk, 2, lo[2], hi[2]);
  const long long ni = hi[0] - lo[0] + 1, nj = hi[1] - lo[1] + 1, nk = hi[2] - lo[2] + 1;
  if (ni <= 0 || nj <= 0 || nk <= 0) return;
  int o = 0;
  for (long long e = threadIdx.x; e < ni * nj * nk; e += blockDim.x) {
    const int i = lo[0] + (int)(e / (nj * nk)), j = lo[1] + (int)((e / nk) % nj), k = lo[2] + (int)(e % nk);
    const long long x = ((long long)i * esj + j) * esk + k;
    if (covers(sp, i, j, k) && (taken[x] || first[x] < s)) o = 1;
  }
  if (__syncthreads_or(o) && threadIdx.x == 0) overlap[s] = 1;
}

__global__ void k_fill_int(int *p, long long n, int v) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    p[e] = v;
}

}  // namespace

extern "C" int slbc_raster_spheres(int esi, int esj, int esk, int nsph, const double *sph,
                                   const unsigned char *taken, int *last, int *count, unsigned char *overlap) {
  if (esi < 1 || esj < 1 || esk < 1 || (long long)esi * esj * esk >= (1LL << 31) || nsph < 0) {
    slbc::set_error("slbc_raster_spheres: bad lattice or sphere count");
    return 1;
  }
  const long long n = (long long)esi * esj * esk;
  double *d_sph = nullptr;
  int *d_last = nullptr, *d_first = nullptr, *d_count = nullptr;
  unsigned char *d_taken = nullptr, *d_over = nullptr;
  cudaError_t e = cudaSuccess;
  auto ok = [&](cudaError_t r) { if (e == cudaSuccess) e = r; return e == cudaSuccess; };
  const int fill_blocks = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
  if (ok(cudaMalloc(&d_last, n * sizeof(int))) && ok(cudaMalloc(&d_first, n * sizeof(int))) &&
      ok(cudaMalloc(&d_taken, (size_t)n)) && ok(cudaMalloc(&d_sph, (size_t)(nsph > 0 ? nsph : 1) * 4 * sizeof(double))) &&
      ok(cudaMalloc(&d_count, (size_t)(nsph > 0 ? nsph : 1) * sizeof(int))) &&
      ok(cudaMalloc(&d_over, (size_t)(nsph > 0 ? nsph : 1)))) {
    k_fill_int<<<fill_blocks, 256>>>(d_last, n, -1);
    k_fill_int<<<fill_blocks, 256>>>(d_first, n, 0x7fffffff);
    slbc::count_launch(2);
    if (ok(cudaGetLastError()) && ok(cudaMemcpy(d_taken, taken, (size_t)n, cudaMemcpyHostToDevice)) && nsph > 0 &&
        ok(cudaMemcpy(d_sph, sph, (size_t)nsph * 4 * sizeof(double), cudaMemcpyHostToDevice)) &&
        ok(cudaMemset(d_count, 0, (size_t)nsph * sizeof(int))) && ok(cudaMemset(d_over, 0, (size_t)nsph))) {
      k_raster<<<nsph, 256>>>(d_sph, nsph, esi, esj, esk, d_last, d_count);
      k_raster_first<<<nsph, 256>>>(d_sph, nsph, esi, esj, esk, d_first);
      k_raster_overlap<<<nsph, 256>>>(d_sph, nsph, esi, esj, esk, d_first, d_taken, d_over);
      slbc::count_launch(3);
      if (ok(cudaGetLastError()) && ok(cudaMemcpy(count, d_count, (size_t)nsph * sizeof(int), cudaMemcpyDeviceToHost)))
        ok(cudaMemcpy(overlap, d_over, (size_t)nsph, cudaMemcpyDeviceToHost));
    }
    if (e == cudaSuccess) ok(cudaMemcpy(last, d_last, n * sizeof(int), cudaMemcpyDeviceToHost));
  }
  cudaFree(d_last); cudaFree(d_first); cudaFree(d_taken); cudaFree(d_sph); cudaFree(d_count); cudaFree(d_over);
  if (e != cudaSuccess) {
    slbc::set_error(std::string("slbc_raster_spheres: ") + cudaGetErrorString(e));
    return (int)e;
  }
  return 0;
}
