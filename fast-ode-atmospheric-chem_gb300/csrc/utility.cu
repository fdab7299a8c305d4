// Rate constants on the device and the FP64 roofline probe.
//
// fo_rate_constants: thermal rate constants k = A exp(-E/T) [M]^power, the
// synthetic workloads' form of the Arrhenius rows of fastode/ts1.py:76-79 with
// the third-body density folded in as fastode/ts1.py:100-102 folds it.
// fo_update_photolysis: photolysis columns J * f(t) at an interval start, the
// device form of the photolysis patch in fastode/ts1.py:204-214 (the factor is
// the diurnal cosine max(0, cos(phase + omega t)) per cell).
// fo_photolysis_factor: the same columns from per-cell factors f[c] computed by
// the caller, k = J * f as one IEEE product, so a caller whose factors came
// from the host gets the host's rate constants bit for bit.
// fo_fp64_fma_rate: a DFMA throughput kernel that states the FP64 roofline
// denominator on the device the integrator runs on.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "fastode_gb300.h"

namespace {

__global__ void rate_constants_kernel(int C, int R, const double* __restrict__ A, const double* __restrict__ E,
                                      const double* __restrict__ power, const double* __restrict__ T,
                                      const double* __restrict__ M, double* __restrict__ k, int64_t kcs,
                                      int64_t krs) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)C * R) return;
  const int c = (int)(idx % C);
  const int j = (int)(idx / C);
  double v = A[j] * exp(-E[j] / T[c]);
  if (power != nullptr && power[j] != 0.0) v = v * pow(M[c], power[j]);
  k[(int64_t)c * kcs + (int64_t)j * krs] = v;
}

__global__ void photolysis_kernel(int C, int nphoto, const int32_t* __restrict__ rxn, const double* __restrict__ J,
                                  const double* __restrict__ phase, double omega_t, double* __restrict__ k,
                                  int64_t kcs, int64_t krs) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)C * nphoto) return;
  const int c = (int)(idx % C);
  const int p = (int)(idx / C);
  const double f = cos(phase[c] + omega_t);
  k[(int64_t)c * kcs + (int64_t)rxn[p] * krs] = J[p] * (f > 0.0 ? f : 0.0);
}

__global__ void photolysis_clock_kernel(int C, int nphoto, const int32_t* __restrict__ rxn,
                                        const double* __restrict__ J, const double* __restrict__ phase, double omega,
                                        const double* __restrict__ t_dev, double* __restrict__ k, int64_t kcs,
                                        int64_t krs) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)C * nphoto) return;
  const int c = (int)(idx % C);
  const int p = (int)(idx / C);
  const double f = cos(phase[c] + omega * t_dev[0]);
  k[(int64_t)c * kcs + (int64_t)rxn[p] * krs] = J[p] * (f > 0.0 ? f : 0.0);
}

__global__ void photolysis_factor_kernel(int C, int nphoto, const int32_t* __restrict__ rxn,
                                         const double* __restrict__ J, const double* __restrict__ f,
                                         double* __restrict__ k, int64_t kcs, int64_t krs) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)C * nphoto) return;
  const int c = (int)(idx % C);
  const int p = (int)(idx / C);
  k[(int64_t)c * kcs + (int64_t)rxn[p] * krs] = __dmul_rn(J[p], f[c]);
}

__global__ void advance_clock_kernel(double* t_dev, double dt) { t_dev[0] += dt; }

// Eight independent FMA chains per thread; every warp is full.
__global__ void fma_rate_kernel(double* out, int iters) {
  double a0 = 0.5, a1 = 1.0, a2 = 1.5, a3 = 2.0, a4 = 2.5, a5 = 3.0, a6 = 3.5, a7 = 4.0;
  const double x = 1.0 + 1.0e-9 * threadIdx.x, y = 0.999999;
  for (int i = 0; i < iters; ++i) {
    a0 = fma(a0, y, x); a1 = fma(a1, y, x); a2 = fma(a2, y, x); a3 = fma(a3, y, x);
    a4 = fma(a4, y, x); a5 = fma(a5, y, x); a6 = fma(a6, y, x); a7 = fma(a7, y, x);
  }
  out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

thread_local std::string g_err;

}  // namespace

extern "C" {

int fo_rate_constants(int32_t C, int32_t R, const double* A, const double* E, const double* power, const double* T,
                      const double* M, double* k, int64_t k_cell_stride, int64_t k_reaction_stride, void* stream) {
  if (C < 0 || R < 0 || !A || !E || !T || !k || (power && !M)) return FO_E_INVALID;
  const int64_t total = (int64_t)C * R;
  if (total == 0) return FO_OK;
  const int block = 256;
  rate_constants_kernel<<<(unsigned)((total + block - 1) / block), block, 0, (cudaStream_t)stream>>>(
      C, R, A, E, power, T, M, k, k_cell_stride, k_reaction_stride);
  return cudaGetLastError() == cudaSuccess ? FO_OK : FO_E_CUDA;
}

int fo_update_photolysis(int32_t C, int32_t nphoto, const int32_t* rxn, const double* J, const double* phase,
                         double omega, double t, double* k, int64_t k_cell_stride, int64_t k_reaction_stride,
                         void* stream) {
  if (C < 0 || nphoto < 0 || (nphoto > 0 && (!rxn || !J || !phase || !k))) return FO_E_INVALID;
  const int64_t total = (int64_t)C * nphoto;
  if (total == 0) return FO_OK;
  const int block = 256;
  photolysis_kernel<<<(unsigned)((total + block - 1) / block), block, 0, (cudaStream_t)stream>>>(
      C, nphoto, rxn, J, phase, omega * t, k, k_cell_stride, k_reaction_stride);
  return cudaGetLastError() == cudaSuccess ? FO_OK : FO_E_CUDA;
}

int fo_photolysis_factor(int32_t C, int32_t nphoto, const int32_t* rxn, const double* J, const double* f,
                         double* k, int64_t k_cell_stride, int64_t k_reaction_stride, void* stream) {
  if (C < 0 || nphoto < 0 || (nphoto > 0 && C > 0 && (!rxn || !J || !f || !k))) return FO_E_INVALID;
  const int64_t total = (int64_t)C * nphoto;
  if (total == 0) return FO_OK;
  const int block = 256;
  photolysis_factor_kernel<<<(unsigned)((total + block - 1) / block), block, 0, (cudaStream_t)stream>>>(
      C, nphoto, rxn, J, f, k, k_cell_stride, k_reaction_stride);
  return cudaGetLastError() == cudaSuccess ? FO_OK : FO_E_CUDA;
}

int fo_update_photolysis_clock(int32_t C, int32_t nphoto, const int32_t* rxn, const double* J, const double* phase,
                               double omega, const double* t_dev, double* k, int64_t k_cell_stride,
                               int64_t k_reaction_stride, void* stream) {
  if (C < 0 || nphoto < 0 || !t_dev || (nphoto > 0 && (!rxn || !J || !phase || !k))) return FO_E_INVALID;
  const int64_t total = (int64_t)C * nphoto;
  if (total == 0) return FO_OK;
  const int block = 256;
  photolysis_clock_kernel<<<(unsigned)((total + block - 1) / block), block, 0, (cudaStream_t)stream>>>(
      C, nphoto, rxn, J, phase, omega, t_dev, k, k_cell_stride, k_reaction_stride);
  return cudaGetLastError() == cudaSuccess ? FO_OK : FO_E_CUDA;
}

int fo_advance_clock(double* t_dev, double dt, void* stream) {
  if (!t_dev) return FO_E_INVALID;
  advance_clock_kernel<<<1, 1, 0, (cudaStream_t)stream>>>(t_dev, dt);
  return cudaGetLastError() == cudaSuccess ? FO_OK : FO_E_CUDA;
}

int fo_fp64_fma_rate(double* fma_per_second) {
  if (!fma_per_second) return FO_E_INVALID;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return FO_E_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return FO_E_CUDA;
  const int block = 256, grid = sms * 8, iters = 4096;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * (size_t)grid * block) != cudaSuccess) return FO_E_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0, 0);
    fma_rate_kernel<<<grid, block>>>(out, iters);
    cudaEventRecord(e1, 0);
    cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return FO_E_CUDA;
  *fma_per_second = 8.0 * iters * (double)grid * block / (best * 1e-3);
  return FO_OK;
}

}  // extern "C"
