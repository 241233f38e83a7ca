// Internal definitions shared by the CUDA translation units of the GB300
// SunlightLB device layer: the D3Q15 link table, the device state of one
// lattice, and the per-precision launcher interface.
#pragma once

#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "slb_device.h"

namespace slbc {

// ---------------------------------------------------------------------------
// D3Q15 link table (reference src/lbmisc.c:87-104):
//   q  : 0  1  2  3  4  5  6  7  8  9 10 11 12 13 14
//   cx : 0  1 -1  0  0  0  0  1 -1  1 -1  1 -1  1 -1
//   cy : 0  0  0  1 -1  0  0  1  1 -1 -1  1  1 -1 -1
//   cz : 0  0  0  0  0  1 -1  1  1  1  1 -1 -1 -1 -1
//   w  : 16 8  8  8  8  8  8  1  1  1  1  1  1  1  1
// Written as constexpr functions so they fold to immediates in unrolled
// device loops and still work for run-time q.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int CX(int q) {
  return (q == 1 || q == 7 || q == 9 || q == 11 || q == 13) ? 1
       : (q == 2 || q == 8 || q == 10 || q == 12 || q == 14) ? -1 : 0;
}
__host__ __device__ constexpr int CY(int q) {
  return (q == 3 || q == 7 || q == 8 || q == 11 || q == 12) ? 1
       : (q == 4 || q == 9 || q == 10 || q == 13 || q == 14) ? -1 : 0;
}
__host__ __device__ constexpr int CZ(int q) {
  return (q == 5 || q == 7 || q == 8 || q == 9 || q == 10) ? 1
       : (q == 6 || q == 11 || q == 12 || q == 13 || q == 14) ? -1 : 0;
}
__host__ __device__ constexpr int OPP(int q) {
  return q == 0 ? 0 : (q <= 6 ? ((q & 1) ? q + 1 : q - 1) : 21 - q);
}

// Per-node flag word: bit 15 = solid node; bit q (1..14) = the link between
// the node x and its upstream neighbour x - c_q joins a fluid and a solid
// node (a bounce-back link).  The bit serves the population arriving along
// q and, equally, the population leaving along opp(q).
constexpr uint16_t FLAG_SOLID = 0x8000u;
constexpr uint16_t FLAG_LINKS = 0x7FFEu;

// Launch shape of the fused step (chosen by the autotuner per parity).
// npt = kStepVec4 selects the 128-bit form (FP32 populations, esk a
// multiple of 4): 4 nodes along k per thread, block_k threads per block.
constexpr int kStepVec4 = -4;
constexpr int kV4Threads = 128;  // threads per block of the 4-wide form
struct StepConfig {
  int npt = 0;      // rows along j per thread (1, 2 or 4), or kStepVec4; 0 = not tuned
  int block_k = 0;  // threads along k (threads per block for kStepVec4)
};

// Device state of one lattice.
struct Lattice {
  int esi = 0, esj = 0, esk = 0;
  int precision = 0;          // 0 FP64, 1 FP32, 2 BF16
  long long nnodes = 0;
  long long npad = 0;         // stride between population arrays (elements)
  void *pop = nullptr;        // 15 * npad elements
  void *scratch = nullptr;    // second population buffer (separate phases)
  uint16_t *flags = nullptr;  // per node
  int layout = SLBC_LAYOUT_N;
  // geometry
  int nobj = 0;
  long long nbnd = 0;
  int *bnd_node = nullptr;    // solid boundary nodes, sorted (object, node)
  int *bnd_obj = nullptr;
  double *bnd_f = nullptr;    // 3 * nbnd node forces (x block, y block, z block)
  int npiece = 0;             // distribf work pieces
  int *piece_obj = nullptr, *piece_lo = nullptr, *piece_hi = nullptr;
  double *piece_sum = nullptr;  // 6 * npiece
  double *obj_pos = nullptr;    // 3 * nobj
  double *obj_ft = nullptr;     // 6 * nobj
  unsigned char *ads = nullptr; // adsorption byte per node
  // per fluid node, bit q: the link from x - c_q is a boundary link from an
  // adsorbing solid node (rebuilt when ads_version moved on)
  uint16_t *ads_links = nullptr;
  long ads_version = 0, ads_links_version = -1;
  int *objidx = nullptr;        // object index per node (-1 fluid)
  int *move_buf = nullptr;      // changed-node list of slbc_move_sphere (count, then pairs)
  long move_cap = 0;
  // parameters
  slbc_params par{};
  int bf_uniform = 1;
  double bf_const[3] = {0.0, 0.0, 0.0};
  void *bf = nullptr;         // 3 * npad of the population type, when not uniform
  void *uw = nullptr;         // 3 * npad of the population type: wall velocity
  // reductions
  double *partials = nullptr;
  int npartials = 0;
  double *host_out = nullptr; // pinned, small
  // staging for host transfers
  double *staging = nullptr;
  long long staging_nodes = 0;
  // moment propagation: density snapshot (FP64, and FP32 for FP32 tracers)
  double *mp_rho64 = nullptr;
  float *mp_rho32 = nullptr;
  // 1/rho in FP32 for the FP32 tracer update, rebuilt when the snapshot
  // changes (mp_rho_gen counts snapshots)
  float *mp_rinv32 = nullptr;
  unsigned long long mp_rho_gen = 1, mp_rinv_gen = 0;
  // counts changes of the populations (steps, uploads, phases, warm starts)
  unsigned long long state_version = 0;
  // FP32 tracer on a frozen flow: per-node stencil coefficients
  // (mp_coef[q*npad + x], q = 0 the node itself), valid for mp_coef_key;
  // mp_last_key is the state seen by the previous FP32 tracer update
  float *mp_coef = nullptr;
  unsigned long long mp_coef_key[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  unsigned long long mp_last_key[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  bool mp_coef_valid = false;
  // BF16 paired-deviation storage: post-collision moments (drho, ru), two
  // float4 buffers, and the deviation scale; the paired deviations are two
  // copies of one 16-byte vector per node in pop.  mom_cur selects the
  // current copy of both; a step writes the other one.
  void *mom[2] = {nullptr, nullptr};
  int mom_cur = 0;
  int graph_mom = 0;
  double bf16_scale = 1.0;
  // execution
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaGraphExec_t graph = nullptr;
  int graph_steps = 0;
  unsigned long long generation = 1;  // bumped when anything the step reads changes
  unsigned long long graph_generation = 0;
  StepConfig tuned[2];        // [0] even step, [1] odd step
  int tune_state = 0;         // 0 not tuned, 1 tuned, -1 tuning disabled
};

// whether the 128-bit form of the fused step applies to a lattice
struct Lattice;
bool vec4_ok(const Lattice &L);

// Arguments shared by the population kernels.
template <typename T>
struct PopArgs {
  T *pop;
  long long npad;
  const uint16_t *flags;
  int esi, esj, esk;
};

template <typename T>
struct StepArgs {
  PopArgs<T> p;
  T omega, comega, rho0;
  int stokes, skip_solid, moving;
  int bf_uniform;
  T bfx, bfy, bfz;
  const T *bf;   // 3 * npad when not uniform
  const T *uw;   // 3 * npad wall velocities when moving
};

struct ForceArgs {
  long long nbnd;
  const int *bnd_node;
  double *f;     // 3 * nbnd
};

struct MoveArgs;

// Per-precision launchers (defined in slbc_f64.cu / slbc_f32.cu).
// Device side of a batch of lattices advanced by one persistent launch.
// Lattices of one batch launch share whether walls move and whether the
// body force is uniform (the kernel is compiled for each combination); a
// batch step makes one launch per combination present.
// Two ways to run it: mode 0 (tiles), one launch per class and step over the
// packed cell index of all lattices, steps replayed from a CUDA graph;
// mode 1 (persistent), one launch per class for all the steps, every block
// owning whole lattices.
struct BatchState {
  std::vector<Lattice *> lats;
  int precision = 1;
  int mode = 0;
  int sms = 0;
  int nworkers = 0;                 // blocks of the last persistent launch
  void *doms = nullptr;             // BatchDom<T> per lattice
  int *work_off = nullptr, *work = nullptr;  // persistent: lattices of each block (CSR)
  int2 *tiles = nullptr;            // tiles: (lattice, first cell), grouped by class
  long long tiles_cap = 0;
  // tiles per (class, starting parity): class = 2 * moving + uniform force,
  // group g holds the domains whose first step has parity g (odd0 = g)
  int class_tiles[4][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
};

#define SLBC_DECLARE_LAUNCHERS(SUFFIX)                                          \
  cudaError_t launch_batch_##SUFFIX(BatchState &B, int nsteps);                 \
  cudaError_t launch_velocity_##SUFFIX(Lattice &L, double fac, float *u, float *drho); \
  cudaError_t prepare_tiles_##SUFFIX(BatchState &B);                             \
  cudaError_t launch_tiles_##SUFFIX(BatchState &B, int step);                    \
  cudaError_t launch_step_##SUFFIX(Lattice &L, int odd);                        \
  cudaError_t launch_force_##SUFFIX(Lattice &L);                                \
  cudaError_t launch_vsum_##SUFFIX(Lattice &L, double fac, const double *psi,   \
                                   double *partials, int nblocks);              \
  cudaError_t launch_put_##SUFFIX(Lattice &L, const double *stage,              \
                                  long long x0, long long n);                   \
  cudaError_t launch_get_##SUFFIX(Lattice &L, double *stage, long long x0,      \
                                  long long n);                                 \
  cudaError_t launch_put_host_##SUFFIX(Lattice &L, const double *host);         \
  cudaError_t launch_get_host_##SUFFIX(Lattice &L, double *host);               \
  cudaError_t launch_swap_##SUFFIX(Lattice &L);                                 \
  cudaError_t launch_to_natural_##SUFFIX(Lattice &L);                           \
  cudaError_t launch_bbl_##SUFFIX(Lattice &L, int with_force);                  \
  cudaError_t launch_propagate_##SUFFIX(Lattice &L);                            \
  cudaError_t launch_collide_##SUFFIX(Lattice &L);                              \
  cudaError_t launch_setvel_##SUFFIX(Lattice &L, const double *stage,           \
                                     long long x0, long long n, int has_rho,    \
                                     int skip_solid);                           \
  cudaError_t launch_mp_rhoinit_##SUFFIX(Lattice &L);                           \
  cudaError_t launch_move_sphere_##SUFFIX(Lattice &L, const MoveArgs &m,       \
                                          int with_uw);                         \
  cudaError_t launch_vacf_sums_##SUFFIX(Lattice &L, double *p, const double *p2, \
                                        const double *psi, double pmean,        \
                                        int axis, double *partials, int nblocks); \
  cudaError_t launch_mp_step_##SUFFIX(Lattice &L, const void *p_in, void *p_out, \
                                      int tp_f64, double alpha, double adprob,  \
                                      int moving, const double *objstate,       \
                                      float *lo_in, float *lo_out, int *lo_live);

SLBC_DECLARE_LAUNCHERS(f64)
SLBC_DECLARE_LAUNCHERS(f32)

// BF16 paired-deviation storage (slbc_bf16.cu): the operations it supports
cudaError_t launch_step_bf16(Lattice &L, int odd);
cudaError_t launch_pair_step(Lattice &L, int planes);  // no swap of the state copies
int bf16_default_planes(const Lattice &L);
cudaError_t launch_put_bf16(Lattice &L, const double *stage, long long x0, long long n, int *unpaired);
cudaError_t launch_get_bf16(Lattice &L, double *stage, long long x0, long long n);
cudaError_t launch_vsum_bf16(Lattice &L, double fac, const double *psi, double *partials, int nblocks);
cudaError_t launch_force_bf16(Lattice &L);
cudaError_t launch_setvel_bf16(Lattice &L, const double *stage, long long x0, long long n, int has_rho,
                               int skip_solid);
cudaError_t launch_collide_bf16(Lattice &L);
cudaError_t launch_mp_rhoinit_bf16(Lattice &L);

// 1/rho of the density snapshot for FP32 tracers, rebuilt when stale
// (slbc_core.cu)
cudaError_t ensure_mp_rinv(Lattice &L);
// column sums of the tracer stencil set to 1 (mass conservation)
cudaError_t launch_mp_coef_norm(Lattice &L);
// one FP32 tracer update from the lattice's stencil coefficients
cudaError_t launch_mp_apply(Lattice &L, const float *pin, const float *lin, float *pout, float *lout, dim3 grid,
                            dim3 block, int planes);

// Launch bookkeeping and error text (defined in slbc_core.cu)
void count_launch(int n = 1);
void set_error(const std::string &msg);
int reduction_blocks(const Lattice &L);
constexpr int kReduceThreads = 256;

}  // namespace slbc
