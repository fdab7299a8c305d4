// The discrete adjoint kernel with the table-driven factorization and solves
// (the device functions and the method are in adjoint.cuh; generated.cu has
// the same kernel on a mechanism's generated code).
#include <cuda_runtime.h>

#include "adjoint.cuh"
#include "smem_attribute.h"

namespace fo {

__global__ void __maxnreg__(255) adjoint_kernel(AdjParams a) {
  extern __shared__ double smem[];
  adjoint_group(a, smem + 32);
}

cudaError_t launch_adjoint(const AdjParams& a, int grid, int lanes, size_t smem, cudaStream_t stream) {
  static SmemAttribute attribute(reinterpret_cast<const void*>(adjoint_kernel));
  cudaError_t e = attribute.ensure(smem);
  if (e != cudaSuccess) return e;
  adjoint_kernel<<<grid, lanes, smem, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace fo
