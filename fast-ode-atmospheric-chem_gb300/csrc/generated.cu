// The integrator kernel of the generated variant (FO_VARIANT_GENERATED).
//
// This translation unit is compiled once, at build time, as relocatable
// device code (nvcc -rdc=true -cubin); it calls fo_gen_factor and
// fo_gen_solve, which a plan generates for its own mechanism (codegen.cpp).
// jit.cpp links the two with nvJitLink into one module per mechanism and
// launches fo_generated_solve_kernel from it. The step loops, stages, norm,
// controller and projection are the shared device functions of
// rosenbrock.cuh; only the factorization and the solves are the mechanism's.
//
// One warp per group (32 lanes, the generated code's operand stride), and at
// most 128 registers per thread, so that sixteen groups are resident per SM:
// the generated factorization needs no shared memory, and with one group per
// warp 2,048 groups of the 65,536-cell workload fit on the GPU at once.
#define FO_LINK_GENERATED 1

#include <cuda_runtime.h>

#include "adjoint.cuh"
#include "rosenbrock.cuh"

extern "C" __global__ void __launch_bounds__(32, 16) fo_generated_solve_kernel(fo::SolveParams p) {
  extern __shared__ double smem[];
  double* red = smem;       // 32 doubles
  double* w = smem + 32;    // the projection's work row (constrained mechanisms only)
  double* scr = p.scratch + (int64_t)blockIdx.x * p.slot_doubles;
  if (p.queue == nullptr) {
    fo::solve_group(p, blockIdx.x, scr, w, red);
  } else {
    __shared__ int next;
    for (;;) {
      __syncthreads();
      if (threadIdx.x == 0) next = atomicAdd(p.queue, 1);
      __syncthreads();
      const int g = next;
      if (g >= p.ngroups) break;
      fo::solve_group(p, g, scr, w, red);
    }
  }
  fo::rounds_drain(p.rounds);
}

// Several mechanisms in one persistent launch (the generated form of
// solve_multi_kernel): items [starts[b], starts[b+1]) of the queue are the
// groups of batch b, whose parameters carry the mechanism's index in this
// module; each block integrates whatever group it pulls next.
extern "C" __global__ void __launch_bounds__(32, 16)
    fo_generated_multi_kernel(const fo::SolveParams* __restrict__ batches, int nb, const int32_t* __restrict__ starts,
                              int32_t* queue, double* scratch, int64_t slot_doubles) {
  extern __shared__ double smem[];
  double* red = smem;
  double* w = smem + 32;
  double* scr = scratch + (int64_t)blockIdx.x * slot_doubles;
  __shared__ int next;
  __shared__ fo::SolveParams params;
  int current = -1;
  unsigned int* const rounds = batches[0].rounds;   // the same words in every batch
  const int total = starts[nb];
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) next = atomicAdd(queue, 1);
    __syncthreads();
    const int item = next;
    if (item >= total) break;
    int b = 0;
    while (b + 1 < nb && item >= starts[b + 1]) ++b;
    fo::load_batch_params(batches, b, current, params);
    fo::solve_group(params, item - starts[b], scr, w, red);
  }
  fo::rounds_drain(rounds);
}

// The discrete adjoint of one interval (adjoint.cuh) on the mechanism's
// generated factorization, solves and transposed solves.
extern "C" __global__ void __launch_bounds__(32, 16) fo_generated_adjoint_kernel(fo::AdjParams a) {
  extern __shared__ double smem[];
  fo::adjoint_group(a, smem + 32);
}
