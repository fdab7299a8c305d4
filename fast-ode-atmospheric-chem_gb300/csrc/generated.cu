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

#include "rosenbrock.cuh"

extern "C" __global__ void __launch_bounds__(32, 16) fo_generated_solve_kernel(fo::SolveParams p) {
  extern __shared__ double smem[];
  double* red = smem;       // 32 doubles
  double* w = smem + 32;    // the projection's work row (constrained mechanisms only)
  double* scr = p.scratch + (int64_t)blockIdx.x * p.slot_doubles;
  if (p.queue == nullptr) {
    fo::solve_group(p, blockIdx.x, scr, w, red);
    return;
  }
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
