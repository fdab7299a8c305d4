// The device integrator: one group of cells per thread block, one cell per
// thread, the whole interval of fastode.solvers.Algorithm.solve
// (fastode/solvers.py:305-415) on the device.
//
// Mapping. FP64 is the bound on GB300 (about 1 TFLOP/s against 74 TFLOP/s
// FP32), and a double-precision warp instruction costs the same issue slot
// whether one lane or all 32 are active. Every lane therefore integrates its
// own cell with the same instruction stream: the mechanism's pattern, the
// elimination schedule and the step sequence are shared by the group, so the
// warp never diverges and no FP64 slot is wasted on masked lanes.
//
// Memory. Per-cell working arrays (LU factors, Jacobian values, stage
// vectors) live in a global scratch slot laid out item-major with cells
// fastest, so a warp reads one 256-byte line per item. The dense work row of
// the elimination and the solve vector live in shared memory, indexed
// [species][lane].
//
// Arithmetic order. The stage combinations, the error norm and the
// controller follow the reference's NumPy expressions operation by operation
// with explicit round-to-nearest intrinsics (no contraction into FMA), so the
// step sequence reproduces the reference whenever the two LUs agree to
// roundoff; the LU, the triangular solves and the sparse map to Jacobian
// values use FMA.
#include <cuda_runtime.h>

#include "rosenbrock.cuh"
#include "smem_attribute.h"

namespace fo {

// __maxnreg__(255): a block of at most 256 threads still fits one SM's
// register file, and eight single-warp groups per SM (the compact kernel's
// shared-memory limit) fit too. Left to itself ptxas gave this kernel 128
// registers, and the triangular solves' register-buffered chunks paid for it
// (one interval of 65,536 cells took 18% longer).
__global__ void __maxnreg__(255) solve_kernel(SolveParams p) {
  extern __shared__ double smem[];
  double* red = smem;       // 32 doubles
  double* w = smem + 32;    // n * lanes
  double* scr = p.scratch + (int64_t)blockIdx.x * p.slot_doubles;
  if (p.queue == nullptr) {
    solve_group(p, blockIdx.x, scr, w, red);
    return;
  }
  __shared__ int next;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) next = atomicAdd(p.queue, 1);
    __syncthreads();
    const int g = next;
    if (g >= p.ngroups) break;
    solve_group(p, g, scr, w, red);
  }
}

// ---- standalone evaluations (fastode/chem.py:86-102) ------------------------

__global__ void eval_kernel(SolveParams p, int C, int want_jac, double* out) {
  const int L = blockDim.x, lane = threadIdx.x;
  const int64_t cell = (int64_t)blockIdx.x * L + lane;
  Lane ln;
  ln.lane = lane;
  ln.L = L;
  ln.active = cell < C;
  ln.cell = ln.active ? cell : (C - 1);
  double* scr = p.scratch + (int64_t)blockIdx.x * p.slot_doubles;
  const int n = p.t.n;
  double* Y = scr + p.sl.y * L;
  for (int i = 0; i < n; ++i) SCR(Y, i) = p.Y[ln.cell * p.ycs + (int64_t)__ldg(p.t.perm + i) * p.yss];
  if (!want_jac) {
    double* f = scr + p.sl.f0 * L;
    eval_rhs(p, ln, Y, scr + p.sl.r * L, f);
    if (ln.active)
      for (int i = 0; i < n; ++i) out[ln.cell * p.ycs + (int64_t)__ldg(p.t.perm + i) * p.yss] = SCR(f, i);
  } else {
    double* negj = scr + p.sl.negj * L;
    eval_negjac(p, ln, Y, scr + p.sl.d * L, negj);
    if (ln.active)
      for (int e = 0; e < p.t.nnzj; ++e) out[ln.cell * p.t.nnzj + __ldg(p.t.j_src + e)] = -SCR(negj, e);
  }
}

#undef SCR
#undef WROW

// ---- launch wrappers ----------------------------------------------------------

cudaError_t launch_solve(const SolveParams& p, int grid, size_t smem, cudaStream_t stream) {
  static SmemAttribute attribute(reinterpret_cast<const void*>(solve_kernel));
  cudaError_t e = attribute.ensure(smem);
  if (e != cudaSuccess) return e;
  solve_kernel<<<grid, p.lanes, smem, stream>>>(p);
  return cudaGetLastError();
}

// Several mechanisms in one persistent launch: the batch table lives in the
// workspace, items [starts[b], starts[b+1]) of the queue are the groups of
// batch b, and each block integrates whatever group it pulls next.
__global__ void __maxnreg__(255) solve_multi_kernel(const SolveParams* __restrict__ batches, int nb,
                                                          const int32_t* __restrict__ starts, int32_t* queue,
                                                          double* scratch, int64_t slot_doubles) {
  extern __shared__ double smem[];
  double* red = smem;
  double* w = smem + 32;
  double* scr = scratch + (int64_t)blockIdx.x * slot_doubles;
  __shared__ int next;
  __shared__ SolveParams params;
  int current = -1;
  const int total = starts[nb];
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) next = atomicAdd(queue, 1);
    __syncthreads();
    const int item = next;
    if (item >= total) break;
    int b = 0;
    while (b + 1 < nb && item >= starts[b + 1]) ++b;
    load_batch_params(batches, b, current, params);
    solve_group(params, item - starts[b], scr, w, red);
  }
}

cudaError_t launch_solve_multi(const SolveParams* batches, int nb, const int32_t* starts, int32_t* queue,
                               double* scratch, int64_t slot_doubles, int grid, int lanes, size_t smem,
                               cudaStream_t stream) {
  static SmemAttribute attribute(reinterpret_cast<const void*>(solve_multi_kernel));
  cudaError_t e = attribute.ensure(smem);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(queue, 0, sizeof(int32_t), stream);
  if (e != cudaSuccess) return e;
  solve_multi_kernel<<<grid, lanes, smem, stream>>>(batches, nb, starts, queue, scratch, slot_doubles);
  return cudaGetLastError();
}

cudaError_t launch_eval(const SolveParams& p, int C, int want_jac, double* out, cudaStream_t stream) {
  const int blocks = (C + p.lanes - 1) / p.lanes;
  eval_kernel<<<blocks, p.lanes, 0, stream>>>(p, C, want_jac, out);
  return cudaGetLastError();
}

}  // namespace fo
